"""Triangle draws (Rasterizer::fill_triangle, rasterizer.rs:731-1292: models, decals, sprites) on the GPU
against the oracle, bit for bit: interleaved with polygon draws in painter's order, every blend mode,
both pixel formats, thin and degenerate triangles, through the per-call API and the frame graph."""
import numpy as np
import pytest

import oracle
import scenes
from sqwheel import abi, gpu, synth

pytestmark = pytest.mark.gpu


def workload(seed, w, h, fmt, num_quads=60, num_tris=400):
    arena, poly_draws, verts = scenes.make_raster_scene(seed, w, h, num_quads, blends=(0, 1, 2, 3, 4), pixel_format=fmt)
    lite, tri_draws, tv = scenes.make_triangle_draws(seed + 1, w, h, num_tris)
    draws = scenes.interleave(poly_draws, tri_draws, seed + 2)
    return arena, draws, verts, lite, tv


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
def test_triangles_bit_exact(gpu_ok, fmt):
    w, h = 640, 400
    arena, draws, verts, lite, tv = workload(3 + fmt, w, h, fmt)
    st = synth.BatchedSurfaces(seed=1, count=1, max_side=8)
    fp = gpu.frame_params(w, h, fmt, (0, 0, 0))
    dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
    r = gpu.GpuRenderer(st.static_data())
    try:
        r.set_lite_textures(lite)
        r.frame_begin(fp)
        r.set_surfaces(arena)
        r.submit_draws_ex(draws, verts, tv)
        got = np.zeros((h, w), dt)
        r.render(got)
        want = np.zeros((h, w), dt)
        assert oracle.rasterize(draws, verts, arena, fp, want, tri_vertices=tv, lite=lite) == 0
        assert np.array_equal(want, got), f"{(want != got).sum()} pixels differ"
        assert r.stats().bad_texel_fetches == 0
    finally:
        r.close()


@pytest.mark.parametrize("blend", [0, 1, 2, 3, 4])
def test_triangle_blends_graph(gpu_ok, blend):
    """Only triangles, one blend mode each, through sw_draw_frame (one CUDA graph), colour64."""
    w, h = 320, 240
    lite, draws, tv = scenes.make_triangle_draws(40 + blend, w, h, 300, blends=(blend,))
    st = synth.BatchedSurfaces(seed=1, count=1, max_side=8)
    fp = gpu.frame_params(w, h, abi.SW_PIXEL_C64, (0, 0, 0))
    r = gpu.GpuRenderer(st.static_data())
    try:
        r.set_lite_textures(lite)
        got = np.zeros((h, w), np.uint64)
        want = np.zeros((h, w), np.uint64)
        for _ in range(2):  # the frame buffer carries over between frames
            r.draw_frame(r.frame_input(fp, None, None, 0, draws, None, dst=got, tri_vertices=tv))
            assert oracle.rasterize(draws, None, None, fp, want, tri_vertices=tv, lite=lite) == 0
            assert np.array_equal(want, got), f"{(want != got).sum()} pixels differ"
        assert r.stats().bad_texel_fetches == 0
    finally:
        r.close()


def test_triangle_validation(gpu_ok):
    w, h = 64, 64
    lite, draws, tv = scenes.make_triangle_draws(7, w, h, 4)
    st = synth.BatchedSurfaces(seed=1, count=1, max_side=8)
    fp = gpu.frame_params(w, h, abi.SW_PIXEL_C32, (0, 0, 0))
    r = gpu.GpuRenderer(st.static_data())
    try:
        r.frame_begin(fp)
        r.set_surfaces(np.zeros(16, np.uint32))
        with pytest.raises(gpu.SwError, match="lite textures"):
            r.submit_draws_ex(draws, None, tv)  # no lite textures uploaded yet
        r.set_lite_textures(lite)
        r.submit_draws_ex(draws, None, tv)
        bad = draws.copy()
        bad["first_vertex"][2] = tv.size - 2
        with pytest.raises(gpu.SwError, match="triangle vertices"):
            r.submit_draws_ex(bad, None, tv)
        bad = draws.copy()
        bad["tex_source"][1] = abi.SW_TEXSRC_SURFACE
        with pytest.raises(gpu.SwError, match="texture source"):
            r.submit_draws_ex(bad, None, tv)
        bad = draws.copy()
        bad["tex_offset"][0] = lite.size
        with pytest.raises(gpu.SwError, match="lite textures"):
            r.submit_draws_ex(bad, None, tv)
    finally:
        r.close()


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
def test_model_frames(gpu_ok, fmt):
    """Whole frames of a map with animated triangle models (drawn after their leaf's polygons) through
    the C++ host renderer and one frame graph, against the oracle's frames from the same host arrays."""
    from sqwheel import host
    scene = host.Scene(**dict(host.SMALL_MAP, num_models=40))
    st = scene.static_data()
    lite = scene.lite_textures()
    hr = host.HostRenderer(scene)
    fr = host.Frame(scene)
    dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
    opts = host.frame_options(640, 480, fmt, directional=False)
    want = np.zeros((480, 640), dt)
    try:
        for fi in (0, 10, 11, 30, 47):
            fr.prepare(fi, opts)
            assert fr.model_triangles > 0 or fi == 30
            arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want, tri_vertices=fr.tri_vertices, lite=lite) == 0
            got = np.zeros((480, 640), dt)
            hr.render_frame(fi, opts, out=got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
    finally:
        hr.close()


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
def test_decal_and_sprite_frames(gpu_ok, fmt):
    """Whole frames with decals (cut out of the polygons they cover, subdivided, lightmap-lit:
    draw_polygon_decals) and sprites (every orientation, tessellated near the camera: draw_sprite) among
    animated models, through the host renderer and one frame graph, against the oracle's frames from
    the same host arrays."""
    from sqwheel import host
    scene = host.Scene(**dict(host.SMALL_MAP, num_models=8, num_sprites=60, num_decals=300, num_dynamic_lights=3))
    st = scene.static_data()
    lite = scene.lite_textures()
    hr = host.HostRenderer(scene)
    fr = host.Frame(scene)
    dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
    opts = host.frame_options(640, 480, fmt, directional=False)
    want = np.zeros((480, 640), dt)
    triangles = 0
    try:
        for fi in (0, 6, 20, 21, 40, 55):
            fr.prepare(fi, opts)
            triangles += fr.model_triangles
            arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want, tri_vertices=fr.tri_vertices, lite=lite) == 0
            got = np.zeros((480, 640), dt)
            hr.render_frame(fi, opts, out=got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
        assert triangles > 200
    finally:
        hr.close()
