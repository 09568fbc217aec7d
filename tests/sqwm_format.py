"""Test infrastructure: an independent numpy restatement of the compiled-map file format (.sqwm version 11,
src/common/bsp_map_save_load.rs:20-300, struct layouts of src/common/bsp_map_compact.rs and
lightmap_compression.rs) for checking the C++ reader and writer, and a pure-numpy restatement of the
lightmap compression arithmetic (f32 throughout) that pins the oracle's."""
import numpy as np

HEADER_BYTES = 8 + 32 * 12
PLANE = [("vec", "<f4", 3), ("dist", "<f4")]
LUMPS = [
    ("nodes", np.dtype([("children", "<u4", 2)] + PLANE)),
    ("leafs", np.dtype([("first_polygon", "<u4"), ("num_polygons", "<u4"), ("first_leaf_portal", "<u4"),
                        ("num_leaf_portals", "<u4")])),
    ("polygons", np.dtype([("first_vertex", "<u4"), ("num_vertices", "<u4"), ("plane", "<f4", 4),
                           ("tex_coord_equation", "<f4", (2, 4)), ("tex_coord_min", "<i4", 2), ("tex_coord_max", "<i4", 2),
                           ("lightmap_data_offset", "<u4"), ("texture", "<u4")])),
    ("portals", np.dtype([("leafs", "<u4", 2), ("plane", "<f4", 4), ("first_vertex", "<u4"), ("num_vertices", "<u4")])),
    ("leafs_portals", np.dtype("<u4")),
    ("vertices", np.dtype(("<f4", 3))),
    ("textures", np.dtype("S64")),
    ("submodels", np.dtype([("root_node", "<u4"), ("first_polygon", "<u4"), ("num_polygons", "<u4")])),
    ("submodels_bsp_nodes", np.dtype([("plane", "<f4", 4), ("first_polygon", "<u4"), ("num_polygons", "<u4"),
                                      ("children", "<u4", 2)])),
    ("entities", np.dtype([("first_key_value_pair", "<u4"), ("num_key_value_pairs", "<u4"), ("submodel_index", "<u4")])),
    ("key_value_pairs", np.dtype([("key", "<u2", 2), ("value", "<u2", 2)])),
    ("strings_data", np.dtype("u1")),
    ("lightmaps_data", np.dtype(("u1", 4))),
    ("directional_lightmaps_data", np.dtype(("u1", 13))),
    ("light_grid_header", np.dtype([("grid_cell_size", "<f4", 3), ("grid_start", "<f4", 3), ("grid_size", "<u4", 3)])),
    ("light_grid_columns", np.dtype([("start_z", "<u4"), ("first_sample", "<u4"), ("num_samples", "<u4")])),
    ("light_grid_samples", np.dtype(("u1", 32))),
]


def lump_table(data):
    return np.frombuffer(data[8:HEADER_BYTES], "<u4").reshape(32, 3)


def parse(data):
    """{lump name: numpy array} of a file image (the raw, still compressed, lightmap records)."""
    assert data[:4] == b"SqwM" and int.from_bytes(data[4:8], "little") == 11
    table = lump_table(data)
    out = {}
    for i, (name, dt) in enumerate(LUMPS):
        off, size, count = (int(v) for v in table[i])
        assert size == dt.itemsize, (name, size, dt.itemsize)
        out[name] = np.frombuffer(data[off:off + size * count], dt).copy()
    return out


def serialize(lumps):
    """A file image of {lump name: array} (missing lumps empty), lumps back to back after the header."""
    header = bytearray(HEADER_BYTES)
    header[:4] = b"SqwM"
    header[4:8] = (11).to_bytes(4, "little")
    body = bytearray()
    for i, (name, dt) in enumerate(LUMPS):
        a = np.ascontiguousarray(lumps.get(name, np.zeros(0, dt)), dtype=dt)
        entry = np.array([HEADER_BYTES + len(body), dt.itemsize, a.shape[0]], "<u4")
        header[8 + i * 12:20 + i * 12] = entry.tobytes()
        body += a.tobytes()
    return bytes(header + body)


def _fmax(a, b):
    return np.where(np.isnan(a), b, np.where(np.isnan(b), a, np.maximum(a, b))).astype(np.float32)


def _fmin(a, b):
    return np.where(np.isnan(a), b, np.where(np.isnan(b), a, np.minimum(a, b))).astype(np.float32)


def compress_color(c):
    """CompressedColor::compress over (n, 3) float32 -> (n, 4) uint8."""
    c = np.asarray(c, np.float32).reshape(-1, 3)
    with np.errstate(invalid="ignore", over="ignore"):
        m = _fmax(_fmax(c[:, 0], c[:, 1]), c[:, 2])
        scale = _fmin(_fmax(np.ceil(m).astype(np.float32), np.float32(1)), np.float32(255))
        mul = (np.float32(255) / scale).astype(np.float32)
        v = _fmin(_fmax((c * mul[:, None]).astype(np.float32), np.float32(0)), np.float32(255))
    return np.concatenate([np.trunc(v).astype(np.uint8), scale.astype(np.uint8)[:, None]], axis=1)


def decompress_color(r):
    r = np.asarray(r, np.uint8).reshape(-1, 4)
    mul = (r[:, 3].astype(np.float32) / np.float32(255)).astype(np.float32)
    return (r[:, :3].astype(np.float32) * mul[:, None]).astype(np.float32)


def compress_vector(v):
    v = np.asarray(v, np.float32).reshape(-1, 3)
    a = np.abs(v)
    with np.errstate(invalid="ignore", over="ignore"):
        m = _fmax(_fmax(a[:, 0], a[:, 1]), a[:, 2])
        scale = _fmin(_fmax(np.ceil(m).astype(np.float32), np.float32(1)), np.float32(255))
        mul = (np.float32(127) / scale).astype(np.float32)
        q = _fmin(_fmax((v * mul[:, None]).astype(np.float32), np.float32(-127)), np.float32(127))
    return np.concatenate([np.trunc(q).astype(np.int8).view(np.uint8), scale.astype(np.uint8)[:, None]], axis=1)


def decompress_vector(r):
    r = np.asarray(r, np.uint8).reshape(-1, 4)
    mul = (r[:, 3].astype(np.float32) / np.float32(127)).astype(np.float32)
    return (r[:, :3].view(np.int8).astype(np.float32) * mul[:, None]).astype(np.float32)
