"""CPU tests of the shadowed-light preparation (host) and of the oracle's depth rasteriser.

The host half follows prepare_dynamic_lights / build_shadow_maps (partial_renderer.rs:398-592): cube
maps for the shadowed lights that touch a visible leaf, 64..256 texels by distance, allocated light by
light, six sides each; the oracle's DepthRasterizer (rasterizer.rs:1295-1474) is checked against a
second, independent float32 restatement on small polygons."""
import math

import numpy as np
import pytest

import oracle
from sqwheel import abi, host


@pytest.fixture(scope="module")
def shadow_scene(built_libs):
    return host.Scene(**dict(host.SMALL_MAP, num_dynamic_lights=4, shadowed_lights=2))


def expected_size(light, cam_pos, quality):
    # partial_renderer.rs:440-462 (f32 arithmetic; `as u32` truncates)
    pos = np.array(light["position"], np.float32)
    dist = np.float32(np.linalg.norm(np.float32(cam_pos) - pos))
    closest = np.float32(dist - np.float32(light["radius"]))
    if closest <= 0:
        return 256
    target = np.float32(np.float32(128.0) * np.float32(light["radius"]) / closest)
    e = max(float(np.float32(math.log2(target)) + np.float32(quality)), 0.0)
    return int(min(max(1 << min(int(e), 31), 64), 256))


@pytest.mark.parametrize("quality", [0.0, -1.0, 1.0])
def test_shadow_allocation(shadow_scene, quality):
    fr = host.Frame(shadow_scene)
    for fi in (0, 20, 56, 60, 100):
        fr.prepare(fi, host.frame_options(640, 480, abi.SW_PIXEL_C64, directional=False, shadows_quality=quality))
        sh = fr.light_shadows
        assert sh.size == fr.lights.size
        offset = 0
        for li in range(sh.size):
            if li >= 2:
                assert sh[li]["kind"] == abi.SW_SHADOW_NONE  # only the first shadowed_lights lights
                continue
            if sh[li]["kind"] == abi.SW_SHADOW_NONE:
                continue  # a light whose sphere touches no visible leaf gets no maps
            assert sh[li]["kind"] == abi.SW_SHADOW_CUBE
            assert sh[li]["offset"] == offset
            assert sh[li]["size"] == expected_size(fr.lights[li], fr.params.cam_pos, quality)
            offset += 6 * int(sh[li]["size"]) ** 2
        assert fr.shadow_texels == offset
        # every depth draw lies in one side of one map
        sides = [(int(s["offset"]) + k * int(s["size"]) ** 2, int(s["size"])) for s in sh if s["kind"] == abi.SW_SHADOW_CUBE
                 for k in range(6)]
        starts = {o: size for o, size in sides}
        for d in fr.depth_draws:
            assert int(d["map_offset"]) in starts and starts[int(d["map_offset"])] == d["map_size"]
            assert 3 <= d["vertex_count"] <= abi.SW_MAX_POLYGON_VERTICES
            assert d["first_vertex"] + d["vertex_count"] <= fr.depth_vertices.size


def test_shadow_maps_cover_closed_rooms(shadow_scene):
    """Inside a closed map every direction from a light meets a wall: all six sides of a map are covered
    (but for the odd crack between adjacent polygons) with positive inverse depths."""
    fr = host.Frame(shadow_scene)
    fr.prepare(0, host.frame_options(640, 480, abi.SW_PIXEL_C64, directional=False))
    storage = np.zeros(fr.shadow_texels, np.float32)
    oracle.shadow_maps(fr.depth_draws, fr.depth_vertices, storage)
    assert (storage == 0).mean() < 1e-3
    assert (storage[storage != 0] > 0).all()


def restated_fill(depth, size, verts, eq):
    """An independent float32 restatement of DepthRasterizer::fill_polygon for convex clockwise polygons
    (whole-pixel rows only: every vertex y at a pixel centre offset, so no thin-line part)."""
    n = len(verts)
    lo = min(range(n), key=lambda i: (verts[i][1], i))
    half = 1 << 15
    li = ri = lo
    cur_y = verts[lo][1]
    while True:
        nli = (li + n - 1) % n
        nri = (ri + 1) % n
        (lx, ly), (nlx, nly), (rx, ry), (nrx, nry) = verts[li], verts[nli], verts[ri], verts[nri]
        dyl, dyr = nly - ly, nry - ry
        next_y = min(nly, nry)
        if dyl > half and dyr > half:
            dxl = int(np.int64(nlx - lx) * 65536 // dyl) if (nlx - lx) >= 0 else -int((-(np.int64(nlx - lx) * 65536)) // dyl)
            dxr = int(np.int64(nrx - rx) * 65536 // dyr) if (nrx - rx) >= 0 else -int((-(np.int64(nrx - rx) * 65536)) // dyr)
            xl0 = lx + ((dxl * (cur_y - ly)) >> 16)
            xr0 = rx + ((dxr * (cur_y - ry)) >> 16)
            y0 = max((cur_y + half) >> 16, 0)
            y1 = min((next_y + half) >> 16, size)
            dstart = (y0 << 16) + half - cur_y
            xl = xl0 + ((dstart * dxl) >> 16) + half
            xr = xr0 + ((dstart * dxr) >> 16) + half
            line = np.float32(np.float32(np.float32(y0) * eq[1]) + np.float32(np.float32(0.5) * np.float32(eq[0] + eq[1])))
            line = np.float32(line + eq[2])
            for y in range(y0, y1):
                xs, xe = max(xl >> 16, 0), min(xr >> 16, size)
                if xs < xe:
                    v = np.float32(line + np.float32(np.float32(xs) * eq[0]))
                    for x in range(xs, xe):
                        depth[y * size + x] = v
                        v = np.float32(v + eq[0])
                xl += dxl
                xr += dxr
                line = np.float32(line + eq[1])
        if nli == nri:
            break
        if verts[nri][1] < verts[nli][1]:
            ri = nri
        else:
            li = nli
        cur_y = next_y


def test_oracle_depth_rasteriser_against_restatement(built_libs):
    rng = np.random.default_rng(5)
    size = 24
    for trial in range(40):
        # a convex clockwise quad with vertices at pixel centres (y = k + 0.5) so every part spans whole rows
        cx, cy = rng.uniform(6, 18, 2)
        r = rng.uniform(3, 9)
        angles = np.sort(rng.uniform(0, 2 * np.pi, 4))[::-1]
        verts = []
        for a in angles:
            x = int((cx + r * np.cos(a)) * 65536)
            y = (int(cy + r * np.sin(a)) << 16) + (1 << 15)
            verts.append((x, y))
        if len({v[1] for v in verts}) < 4:
            continue
        eq = np.array(rng.uniform(-1e-3, 1e-3, 2).tolist() + [rng.uniform(0.01, 0.1)], np.float32)
        want = np.full(size * size, -1.0, np.float32)
        restated_fill(want, size, verts, eq)
        d = np.zeros(1, abi.DEPTH_DRAW)
        d[0]["vertex_count"] = 4
        d[0]["map_size"] = size
        d[0]["depth_eq"] = eq
        v = np.array(verts, dtype=[("x", "<i4"), ("y", "<i4")]).view(abi.VERTEX16)
        got = np.full(size * size, -1.0, np.float32)
        oracle.shadow_maps(d, v, got)
        assert np.array_equal(want.view(np.uint32), got.view(np.uint32)), f"trial {trial}"


def test_projector_circle_known_answer(built_libs):
    """make_shadow_map_circle on a 16x16 map: row y keeps [dx, 16 - dx) with dx = 8 - min(ceil(sqrt(64 -
    (y - 8)^2)), 8) (light.rs:135-156); the rest becomes 1e24."""
    import math
    storage = np.zeros(300, np.float32)
    oracle.shadow_map_circle(storage, 40, 16)
    m = storage[40:40 + 256].reshape(16, 16)
    for y in range(16):
        dx = 8 - min(math.ceil(math.sqrt(max(64 - (y - 8) ** 2, 0))), 8)
        row = np.zeros(16, np.float32)
        row[:dx] = 1e24
        row[16 - dx:] = 1e24
        assert np.array_equal(m[y], row), y
    assert not storage[:40].any() and not storage[40 + 256:].any()


def test_projector_lights_narrow_light_lists(built_libs):
    """A projector's cone (the five pyramid planes) leaves polygons outside it without the light, which
    the same light as an unshadowed point light would reach; its map size follows the reference's
    formula (partial_renderer.rs:462-513)."""
    base = dict(host.SMALL_MAP, num_dynamic_lights=4)
    plain = host.Scene(**base)
    proj = host.Scene(**dict(base, projector_lights=4))
    fp, fq = host.Frame(plain), host.Frame(proj)
    opts = host.frame_options(640, 480, abi.SW_PIXEL_C64, directional=False)
    fewer = 0
    for fi in (0, 12, 40):
        fp.prepare(fi, opts)
        fq.prepare(fi, opts)
        assert fp.surfaces.size == fq.surfaces.size
        lp, lq = fp.surfaces["num_lights"].sum(), fq.surfaces["num_lights"].sum()
        assert lq <= lp
        fewer += int(lp - lq)
        for m in fq.light_shadows:
            if m["kind"] == abi.SW_SHADOW_PROJECTOR:
                assert 32 <= m["size"] <= 1024 and (int(m["size"]) & (int(m["size"]) - 1)) == 0
                assert abs(np.linalg.norm(m["basis_z"]) - 1.0) < 1e-5
    assert fewer > 0
