"""The light grid (bsp_map_compact.rs:162-188) and fetch_light_from_grid (triangle_models_rendering.rs:582-700)
on the CPU: the host's fetch equals a numpy restatement (trilinear mix of the up to 8 existing non-zero
samples, renormalised when the weights sum below 0.995) at seeded positions inside, on the edges of and
outside the grid; a scene without a grid fetches zero; the grid survives a .sqwm save and load (samples
through the map's compressed form); models and sprites of a grid-lit map take their light from it, so
their vertices differ from the unlit map's."""
import numpy as np
import pytest

from sqwheel import abi, host

pytestmark = pytest.mark.usefixtures("built_libs")

GRID_MAP = dict(host.SMALL_MAP, num_models=4, num_sprites=12, num_portals=3, portals_depth=1, light_grid=1)


def np_fetch(header, cols, samples, pos):
    f32 = np.float32
    cell, start, size = header["cell_size"], header["start"], header["size"].astype(np.int64)
    if (size == 0).any() or (cell == 0).any() or cols.size == 0 or samples.size == 0:
        return np.zeros(24, f32)
    gp = (np.asarray(pos, f32) - start) / cell
    gi = np.floor(gp).astype(np.int64)
    total = np.zeros(24, f32)
    factor = f32(0)
    for dx in (0, 1):
        x = gi[0] + dx
        if x < 0 or x >= size[0]:
            continue
        fx = f32(1) - abs(gp[0] - f32(x))
        for dy in (0, 1):
            y = gi[1] + dy
            if y < 0 or y >= size[1]:
                continue
            start_z, first, n = (int(v) for v in cols[x + y * size[0]])
            if n == 0:
                continue
            fy = f32(1) - abs(gp[1] - f32(y))
            for dz in (0, 1):
                z = gi[2] + dz
                if z < 0 or z >= size[2] or z < start_z or z >= start_z + n:
                    continue
                s = samples[first + z - start_z]
                if not s.any():
                    continue
                fz = f32(1) - abs(gp[2] - f32(z))
                w = f32(fx * fy * fz)
                total = (total + s * w).astype(f32)
                factor = f32(factor + w)
    if factor <= 0:
        return np.zeros(24, f32)
    if factor < f32(0.995):
        total = (total * (f32(1) / factor)).astype(f32)
    return total


@pytest.fixture(scope="module")
def grid_scene():
    s = host.Scene(**GRID_MAP)
    yield s
    s.close()


def test_grid_well_formed(grid_scene):
    header, cols, samples = grid_scene.light_grid()
    assert cols.shape[0] == int(header["size"][0]) * int(header["size"][1]) > 0
    used = cols[cols[:, 2] > 0]
    assert used.shape[0] > 0 and (used[:, 2] < cols.shape[0]).all()
    assert ((used[:, 1].astype(np.int64) + used[:, 2]) <= samples.shape[0]).all()
    zero = ~samples.any(axis=1)
    assert zero.any() and (~zero).any(), "some zero samples (solid space) and some lit ones"


def test_fetch_matches_restatement(grid_scene):
    header, cols, samples = grid_scene.light_grid()
    rng = np.random.default_rng(11)
    lo = header["start"] - header["cell_size"]
    hi = header["start"] + header["cell_size"] * (header["size"].astype(np.float32) + 1)
    points = [rng.uniform(lo, hi).astype(np.float32) for _ in range(400)]
    # exactly on grid points and cell edges, and far outside
    for k in range(40):
        ix = rng.integers(0, header["size"], 3)
        points.append((header["start"] + header["cell_size"] * ix).astype(np.float32))
    points += [np.array([1e9, 0, 0], np.float32), np.array([-1e9, -1e9, -1e9], np.float32)]
    lit = 0
    for p in points:
        want = np_fetch(header, cols, samples, p)
        got = grid_scene.fetch_light(p)
        assert np.array_equal(want.view(np.uint32), got.view(np.uint32)), (p, want, got)
        lit += int(got.any())
    assert lit > 100


def test_no_grid_fetches_zero():
    s = host.Scene(**dict(GRID_MAP, light_grid=0))
    try:
        _, cols, samples = s.light_grid()
        assert cols.size == 0 and samples.size == 0
        assert not s.fetch_light([100.0, 100.0, 50.0]).any()
    finally:
        s.close()


def frames(scene, count=6):
    fr = host.Frame(scene)
    opts = host.frame_options(320, 180, abi.SW_PIXEL_C32, directional=False)
    out = []
    for fi in range(0, 64, 64 // count):
        fr.prepare(fi, opts)
        out.append((fr.vertices.copy(), fr.tri_vertices.copy(), fr.views.copy()))
    return out


def test_grid_survives_map_round_trip(grid_scene, tmp_path):
    path = tmp_path / "grid.sqwm"
    grid_scene.save_map(str(path))
    loaded = host.Scene(str(path), **dict(GRID_MAP, num_models=0, num_sprites=0, num_portals=0))
    try:
        h0, c0, s0 = grid_scene.light_grid()
        h1, c1, s1 = loaded.light_grid()
        assert np.array_equal(c0, c1)
        for k in h0:
            assert np.array_equal(h0[k], h1[k])
        # samples go through the map's compressed form (lightmap_compression.rs): close, not equal
        assert s0.shape == s1.shape
        np.testing.assert_allclose(s1, s0, rtol=0.02, atol=0.02)
    finally:
        loaded.close()


def test_models_and_sprites_lit_from_grid(grid_scene):
    unlit = host.Scene(**dict(GRID_MAP, light_grid=0))
    try:
        a, b = frames(grid_scene), frames(unlit)
        differ = sum(int(not np.array_equal(x[1], y[1])) for x, y in zip(a, b))
        assert differ > 0, "model/sprite vertex lights do not depend on the grid"
    finally:
        unlit.close()


def test_stress_configuration_prepares():
    """The stress configuration's map (128 rooms, portals, decals, sprites, 200 grid-lit models): frames
    of its camera path carry portal views and model triangles, and the map has a light grid."""
    s = host.Scene(**host.STRESS_MAP)
    try:
        info = s.info()
        assert info.polygons > 60000
        _, cols, samples = s.light_grid()
        assert cols.size > 0 and samples.size > 0
        fr = host.Frame(s)
        opts = host.frame_options(960, 540, abi.SW_PIXEL_C64, directional=True)
        views = tris = 0
        for fi in (0, 37, 74, 208, 224):
            fr.prepare(fi, opts)
            views += len(fr.views)
            tris += fr.model_triangles
        assert views > 0 and tris > 0
    finally:
        s.close()
