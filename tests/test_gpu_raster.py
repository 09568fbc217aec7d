"""GPU parity of the tile-binned rasteriser against the oracle's single-thread path: coverage, polygon
order and texel addresses bit-exact, all three interpolation modes and five blend modes, Color32 and
Color64, tiles cut by the frame edges."""
import numpy as np
import pytest

import oracle
import scenes
from sqwheel import abi, gpu, synth

pytestmark = pytest.mark.gpu


def render_both(arena, draws, verts, w, h, fmt, clear=False, init=None):
    fp = gpu.frame_params(w, h, fmt, (0, 0, 0), clear_background=clear)
    dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
    want = np.zeros((h, w), dt) if init is None else init.copy()
    if clear:
        oracle.clear_background(fp, want)
    bad = oracle.rasterize(draws, verts, arena, fp, want)
    st = synth.BatchedSurfaces(seed=1, count=1, max_side=8)
    r = gpu.GpuRenderer(st.static_data())
    try:
        if init is not None:
            r.set_framebuffer(init, fmt)
        r.frame_begin(fp)
        r.set_surfaces(arena)
        r.submit_draws(draws, verts)
        got = np.zeros((h, w), dt)
        r.render(got)
        stats = r.stats()
    finally:
        r.close()
    return want, got, bad, stats


def assert_frames_equal(want, got):
    if np.array_equal(want, got):
        return
    ys, xs = np.nonzero(want != got)
    raise AssertionError(f"{ys.size} pixels differ, first at (x={xs[0]}, y={ys[0]}): want {want[ys[0], xs[0]]:#x} "
                         f"got {got[ys[0], xs[0]]:#x}")


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
@pytest.mark.parametrize("mode", [abi.SW_RASTER_FULL_PERSPECTIVE, abi.SW_RASTER_LINE_Z_CORRECTED, abi.SW_RASTER_AFFINE])
def test_raster_modes_bit_exact(gpu_ok, fmt, mode):
    w, h = 333, 207  # not a multiple of the tile size
    arena, draws, verts = scenes.make_raster_scene(100 + mode + 3 * fmt, w, h, 50, modes=(mode,), pixel_format=fmt)
    want, got, bad, stats = render_both(arena, draws, verts, w, h, fmt)
    assert bad == 0 and stats.bad_texel_fetches == 0
    assert (want != 0).mean() > 0.9
    assert_frames_equal(want, got)


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
def test_raster_blend_order_bit_exact(gpu_ok, fmt):
    """Every blend mode, heavy overdraw: painter's order must be preserved exactly."""
    w, h = 256, 192
    arena, draws, verts = scenes.make_raster_scene(7 + fmt, w, h, 120, blends=(0, 1, 2, 3, 4), pixel_format=fmt)
    rng = np.random.default_rng(3)
    init = rng.integers(0, 1 << 62, (h, w), dtype=np.uint64)
    if fmt == abi.SW_PIXEL_C32:
        init = init.astype(np.uint32)
    want, got, _, _ = render_both(arena, draws, verts, w, h, fmt, init=init)
    assert_frames_equal(want, got)


def test_raster_clear_background(gpu_ok):
    w, h = 100, 60
    arena, draws, verts = scenes.make_raster_scene(21, w, h, 3, pixel_format=abi.SW_PIXEL_C32)
    want, got, _, _ = render_both(arena, draws[:1], verts, w, h, abi.SW_PIXEL_C32, clear=True)
    assert (want == 0x00201008).any()
    assert_frames_equal(want, got)


def test_raster_thin_and_degenerate(gpu_ok):
    """Sub-pixel slivers through the single-line branch (rasterizer.rs:220-254) and empty polygons."""
    w, h = 64, 64
    arena = np.arange(1, 16 * 16 + 1, dtype=np.uint32)
    F = 65536
    polys = [
        [(10 * F, 20 * F + F // 4), (50 * F, 20 * F + F // 3), (30 * F, 20 * F + F // 2 + F // 8)],  # dy < 0.5
        [(5 * F, 5 * F), (5 * F, 5 * F), (5 * F, 5 * F)],  # a point
        [(0, 0), (63 * F, 0), (63 * F, 63 * F), (0, 63 * F)],  # full frame
        [(-5 * F, 30 * F), (70 * F, 31 * F), (20 * F, 40 * F)],  # crosses the frame edges
    ]
    verts, draws = [], []
    for i, p in enumerate(polys):
        d = np.zeros((), abi.DRAW_CMD)
        d["first_vertex"] = len(verts)
        d["vertex_count"] = len(p)
        d["mode"] = abi.SW_RASTER_AFFINE
        d["blend"] = abi.SW_BLEND_AVERAGE if i else abi.SW_BLEND_NONE
        d["depth_eq"] = (0.0, 0.0, 0.01)
        d["tc_eq"] = (0.002, 0.0, 0.0, 0.002, 0.0, 0.0)
        d["tex_size"] = (16, 16)
        draws.append(d)
        verts.extend(p)
    draws = np.array(draws, abi.DRAW_CMD)
    verts = np.array(verts, abi.VERTEX16)
    want, got, bad, _ = render_both(arena, draws, verts, w, h, abi.SW_PIXEL_C32)
    assert bad == 0
    assert_frames_equal(want, got)


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
def test_many_small_draws_binned(gpu_ok, fmt):
    """Over 10k small draws with heavy overdraw and every blend mode, on a frame of many bins (the tile
    pass scans each bin's ordered draw list): bit-exact, painter's order kept across bins."""
    w, h = 700, 450  # bins cut by the frame edges
    arena, draws, verts = scenes.make_small_draws(77 + fmt, w, h, 12000, pixel_format=fmt)
    assert draws.size > 10000
    rng = np.random.default_rng(5)
    init = rng.integers(0, 1 << 62, (h, w), dtype=np.uint64)
    if fmt == abi.SW_PIXEL_C32:
        init = init.astype(np.uint32)
    want, got, bad, stats = render_both(arena, draws, verts, w, h, fmt, init=init)
    assert bad == 0 and stats.bad_texel_fetches == 0
    assert_frames_equal(want, got)
