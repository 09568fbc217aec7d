"""Compiled maps (.sqwm version 11) and lightmap compression on the CPU: known answers of the compression
(lightmap_compression.rs:48-130), the oracle against an independent numpy restatement, the C++ writer's
file against an independent reader of the format (bsp_map_save_load.rs:20-300), writer -> reader round
trips, and the reader's errors."""
import math

import numpy as np
import pytest

import oracle
import sqwm_format as fmt
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.usefixtures("built_libs")

f32 = np.float32


def test_color_compression_known_answers():
    # max 1 -> scale 1, multiplier 255; max 300 -> scale 255 (clamped), multiplier 1; all zero -> scale 1;
    # a NaN component is ignored by the max and clamps to 0
    rgb = np.array([[1.0, 0.5, 0.25], [300.0, 2.0, -1.0], [0.0, 0.0, 0.0], [math.nan, 3.5, 1.0]], np.float32)
    want = np.array([[255, 127, 63, 1], [255, 2, 0, 255], [0, 0, 0, 1], [0, 223, 63, 4]], np.uint8)
    assert np.array_equal(oracle.compress_lightmaps(rgb), want)
    assert np.array_equal(fmt.compress_color(rgb), want)
    back = oracle.decompress_lightmaps(want)
    assert back[0, 0] == f32(255) * (f32(1) / f32(255)) and back[1, 0] == f32(255) and back[2, 0] == 0.0
    assert back[3, 1] == f32(223) * (f32(4) / f32(255))


def test_vector_and_directional_known_answers():
    el = np.zeros(3, abi.DIR_LIGHTMAP_ELEMENT)
    el["light_direction_vector_scaled"] = [[0.5, -0.25, 0.0], [-200.0, 100.0, 0.0], [0.001, 0.0, 0.0]]
    el["directional_light_deviation"] = [0.5, 2.0, -1.0]
    el["ambient_light"] = [[1.0, 1.0, 1.0], [0, 0, 0], [2, 1, 0]]
    rec = oracle.compress_directional_lightmaps(el)
    # direction: scale 1, multiplier 127 -> (63, -31, 0); scale 200, multiplier 0.635 -> (-127, 63, 0)
    assert list(rec[0, 4:8].view(np.int8)[:3]) == [63, -31, 0] and rec[0, 7] == 1
    assert list(rec[1, 4:7].view(np.int8)) == [-127, 63, 0] and rec[1, 7] == 200
    # deviation x 255, clamped to [0, 255], truncated
    assert list(rec[:, 8]) == [127, 255, 0]
    back = oracle.decompress_directional_lightmaps(rec)
    # 0.001 x 127 truncates to 0: the zero direction becomes (0, 0, 1/1024)
    assert list(back["light_direction_vector_scaled"][2]) == [0.0, 0.0, f32(1.0 / 1024.0)]
    assert back["directional_light_deviation"][0] == f32(127) / f32(255)


def test_oracle_against_numpy_restatement():
    rng = np.random.default_rng(5)
    n = 20000
    rgb = (rng.standard_exponential((n, 3)) * rng.choice([0.01, 1.0, 30.0, 400.0], (n, 1))).astype(np.float32)
    rgb[::97] *= -1
    rgb[::101, 1] = np.nan
    rgb[::103] = 0
    rec = oracle.compress_lightmaps(rgb)
    assert np.array_equal(rec, fmt.compress_color(rgb))
    rnd = rng.integers(0, 256, (n, 4), dtype=np.uint8)
    assert np.array_equal(oracle.decompress_lightmaps(rnd).view(np.uint32), fmt.decompress_color(rnd).view(np.uint32))
    el = np.zeros(n, abi.DIR_LIGHTMAP_ELEMENT)
    el["ambient_light"] = rgb
    el["directional_light_color"] = rgb[::-1]
    el["light_direction_vector_scaled"] = (rng.standard_normal((n, 3)) * rng.choice([0.002, 1.0, 50.0, 600.0], (n, 1)))
    el["directional_light_deviation"] = rng.uniform(-0.2, 1.2, n)
    drec = oracle.compress_directional_lightmaps(el)
    assert np.array_equal(drec[:, 0:4], fmt.compress_color(el["ambient_light"]))
    assert np.array_equal(drec[:, 4:8], fmt.compress_vector(el["light_direction_vector_scaled"]))
    assert np.array_equal(drec[:, 9:13], fmt.compress_color(el["directional_light_color"]))
    rd = rng.integers(0, 256, (n, 13), dtype=np.uint8)
    rd[::7, 4:7] = 0  # zero directions
    rd[::11, 7] = 0   # zero scale
    got = oracle.decompress_directional_lightmaps(rd)
    assert np.array_equal(got["ambient_light"].view(np.uint32), fmt.decompress_color(rd[:, 0:4]).view(np.uint32))
    d = fmt.decompress_vector(rd[:, 4:8])
    zero = (d * d).sum(axis=1) <= 0
    d[zero] = [0.0, 0.0, f32(1.0 / 1024.0)]
    assert np.array_equal(got["light_direction_vector_scaled"].view(np.uint32), d.view(np.uint32))
    assert np.array_equal(got["directional_light_deviation"], (rd[:, 8].astype(np.float32) / f32(255)).astype(np.float32))


DIR_MAP = dict(host.SMALL_MAP, directional_lightmaps=1)


@pytest.fixture(scope="module")
def saved(tmp_path_factory):
    scene = host.Scene(**DIR_MAP)
    path = tmp_path_factory.mktemp("maps") / "small.sqwm"
    scene.save_map(str(path))
    yield scene, path, path.read_bytes()
    scene.close()


def test_writer_file_layout(saved):
    """The C++ writer's file read by the independent reader: geometry as the scene holds it, lightmaps as
    the oracle compresses the scene's f32 lightmaps, lumps back to back."""
    scene, _, data = saved
    lumps = fmt.parse(data)
    info = scene.info()
    assert (lumps["nodes"].size, lumps["leafs"].size, lumps["polygons"].size, lumps["portals"].size) == \
        (info.nodes, info.leafs, info.polygons, info.portals)
    polys, verts = host.Frame(scene).map_data()
    p = lumps["polygons"]
    assert np.array_equal(p["plane"], polys["plane"]) and np.array_equal(p["tex_coord_equation"], polys["tex_coord_equation"])
    for k in ("tex_coord_min", "tex_coord_max", "first_vertex", "num_vertices", "lightmap_data_offset", "texture"):
        assert np.array_equal(p[k], polys[k]), k
    assert np.array_equal(lumps["vertices"], verts)
    st = scene.static_data()
    assert np.array_equal(lumps["lightmaps_data"], oracle.compress_lightmaps(st.lightmaps))
    assert np.array_equal(lumps["directional_lightmaps_data"], oracle.compress_directional_lightmaps(st.directional_lightmaps))
    assert lumps["textures"].size == info.materials and lumps["textures"][0].startswith(b"generated/")
    table = fmt.lump_table(data)
    ends = [fmt.HEADER_BYTES] + [int(o + s * c) for o, s, c in table[:17]]
    assert all(int(table[i][0]) == ends[i] for i in range(17)) and ends[-1] == len(data)


def test_reader_round_trip(saved):
    """Reading the file back: the same geometry, lightmaps decoded as the oracle decodes the file's
    records, the compressed records kept as the file holds them, the player start as the first camera
    position; writing the loaded map again gives the same geometry lumps."""
    scene, path, data = saved
    lumps = fmt.parse(data)
    loaded = host.Scene.load_map(str(path), **DIR_MAP)
    from_bytes = host.Scene.load_map(data, **DIR_MAP)
    try:
        st = loaded.static_data()
        assert np.array_equal(st.lightmaps.reshape(-1).view(np.uint32),
                              oracle.decompress_lightmaps(lumps["lightmaps_data"]).reshape(-1).view(np.uint32))
        want_d = oracle.decompress_directional_lightmaps(lumps["directional_lightmaps_data"])
        assert st.directional_lightmaps.tobytes() == want_d.tobytes()
        simple, directional = loaded.compressed_lightmaps()
        assert np.array_equal(simple, lumps["lightmaps_data"]) and np.array_equal(directional, lumps["directional_lightmaps_data"])
        assert from_bytes.static_data().lightmaps.tobytes() == st.lightmaps.tobytes()
        polys0, verts0 = host.Frame(scene).map_data()
        polys1, verts1 = host.Frame(loaded).map_data()
        for k in ("plane", "tex_coord_equation", "basis_u", "basis_v", "basis_start", "basis_normal", "tex_coord_min",
                  "tex_coord_max", "first_vertex", "num_vertices", "lightmap_data_offset", "texture"):
            assert np.array_equal(polys0[k], polys1[k]), k
        assert np.array_equal(verts0, verts1)
        fr = host.Frame(loaded).prepare(0, host.frame_options(640, 480, abi.SW_PIXEL_C32, directional=True))
        start = fmt.parse(data)
        assert fr.surfaces.size > 0
        origin = None
        kv, strings = start["key_value_pairs"], start["strings_data"].tobytes()
        for e in start["entities"]:
            pairs = {strings[k[0]:k[0] + k[1]]: strings[v[0]:v[0] + v[1]]
                     for k, v in kv[e["first_key_value_pair"]:e["first_key_value_pair"] + e["num_key_value_pairs"]]}
            if pairs.get(b"classname") == b"info_player_start":
                origin = [float(x) for x in pairs[b"origin"].split()]
        assert origin is not None and np.allclose(list(fr.params.cam_pos), origin)
        again = str(path) + ".2"
        loaded.save_map(again)
        lumps2 = fmt.parse(open(again, "rb").read())
        for k in ("nodes", "leafs", "polygons", "portals", "leafs_portals", "vertices"):
            assert lumps2[k].tobytes() == lumps[k].tobytes(), k
    finally:
        loaded.close()
        from_bytes.close()


def test_loaded_map_camera_path(saved):
    """The camera path through leafs and portals stays inside the map: every frame sees polygons."""
    _, _, data = saved
    loaded = host.Scene.load_map(data, **dict(DIR_MAP, num_frames=128))
    try:
        fr = host.Frame(loaded)
        opts = host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=True)
        seen = [fr.prepare(fi, opts).surfaces.size for fi in range(0, 128, 4)]
        assert min(seen) > 0, seen
    finally:
        loaded.close()


def _with(lumps, **changes):
    out = {k: v.copy() for k, v in lumps.items()}
    out.update(changes)
    return fmt.serialize(out)


def test_reader_errors(saved):
    _, _, data = saved
    lumps = fmt.parse(data)
    cases = [
        (data[:100], "header"),
        (b"XqwM" + data[4:], "bad id"),
        (data[:4] + (10).to_bytes(4, "little") + data[8:], "version: 10"),
        (data[:len(data) - 10], "past the end"),
    ]
    p = lumps["polygons"].copy()
    p["texture"][5] = lumps["textures"].size
    cases.append((_with(lumps, polygons=p), "texture out of range"))
    n = lumps["nodes"].copy()
    n["children"][0][0] = n.size - 1
    cases.append((_with(lumps, nodes=n), "not before its parent"))
    lf = lumps["leafs"].copy()
    lf["first_polygon"][1] = lf["first_polygon"][0]
    cases.append((_with(lumps, leafs=lf), "two leafs"))
    p = lumps["polygons"].copy()
    k = int(np.nonzero(p["lightmap_data_offset"])[0][-1])
    p["lightmap_data_offset"][k] = lumps["directional_lightmaps_data"].shape[0] - 1
    cases.append((_with(lumps, polygons=p), "lightmap out of range"))
    pt = lumps["portals"].copy()
    pt["leafs"][0][1] = lumps["leafs"].size
    cases.append((_with(lumps, portals=pt), "leaf out of range"))
    for blob, msg in cases:
        with pytest.raises(gpu.SwError, match=msg):
            host.Scene.load_map(blob, **DIR_MAP)
    # a lump of the wrong element size reads as empty (read_lump): here the nodes, so no BSP tree
    bad = bytearray(data)
    bad[8 + 4:8 + 8] = (25).to_bytes(4, "little")
    with pytest.raises(gpu.SwError, match="no BSP tree"):
        host.Scene.load_map(bytes(bad), **DIR_MAP)
    with pytest.raises(gpu.SwError, match="can't open"):
        host.Scene.load_map("/nonexistent/map.sqwm", **DIR_MAP)
    # options that need the generator's rooms
    with pytest.raises(gpu.SwError, match="generated scenes only"):
        host.Scene.load_map(data, **dict(DIR_MAP, num_models=4))
