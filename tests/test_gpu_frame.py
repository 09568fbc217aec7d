"""Whole frames through the GPU path vs the oracle, both fed by the same host-side frame preparation:
surface arena, rasterised frame, tonemapped frame and exposure sequence bit-exact."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu


def run_frames(scene, frames, w, h, fmt, directional, post=False, clear=False):
    st = scene.static_data()
    fr = host.Frame(scene)
    r = gpu.GpuRenderer(st)
    t32, t64, _, _ = scene.skybox()
    sky = None
    if t32.size:
        r.set_skybox(t32, t64)
        sky = t64 if fmt == abi.SW_PIXEL_C64 else t32
    exposure = 1.0
    cfg = abi.PostConfig.default()
    try:
        for fi in frames:
            fr.prepare(fi, host.frame_options(w, h, fmt, directional=directional, clear_background=clear))
            want_arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8)
            r.frame_begin(fr.params, fr.lights)
            r.submit_surfaces(fr.surfaces, fr.total_texels)
            got_arena = r.read_surfaces(fr.total_texels, fmt)
            assert np.array_equal(want_arena, got_arena), f"frame {fi}: surfaces differ"
            dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
            want = np.zeros((h, w), dt)
            if clear:
                oracle.clear_background(fr.params, want)
            bad = oracle.rasterize(fr.draws, fr.vertices, want_arena, fr.params, want, skybox=sky)
            assert bad == 0
            assert sky is None or fr.skybox_draws > 0
            r.submit_draws(fr.draws, fr.vertices)
            got = np.zeros((h, w), dt)
            r.render(got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
            if post:
                want_ldr, exposure_next, _ = oracle.postprocess(cfg, want, 1.0 / 60.0, (1.0, 1.0, 1.0), exposure)
                got_ldr = np.zeros((h, w), np.uint32)
                r.postprocess(cfg, 1.0 / 60.0, (1.0, 1.0, 1.0), out=got_ldr)
                assert np.array_equal(want_ldr, got_ldr), f"frame {fi}: tonemapped frame differs"
                assert r.exposure() == np.float32(exposure_next)
                exposure = exposure_next
        assert r.stats().bad_texel_fetches == 0
    finally:
        r.close()


def test_small_map_frames_c32(gpu_ok):
    scene = host.Scene(**host.SMALL_MAP)
    run_frames(scene, [0, 7, 21, 40, 63], 640, 480, abi.SW_PIXEL_C32, directional=False)


def test_full_map_frames_hdr_with_postprocess(gpu_ok):
    """Directional lightmaps, normal maps, dielectric and metal specular, 8 moving lights, Color64 +
    bloom + tonemap + exposure, at a reduced resolution so the single-thread oracle stays fast."""
    scene = host.Scene(**dict(host.FULL_MAP, grid_x=4, grid_y=4))
    run_frames(scene, [0, 30, 31, 32, 90], 480, 270, abi.SW_PIXEL_C64, directional=True, post=True)


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
def test_sky_map_frames(gpu_ok, fmt):
    """draw_skybox: the skybox sides (HDR brightness 2) behind open ceilings, rotating, drawn first."""
    scene = host.Scene(**host.SKY_MAP)
    run_frames(scene, [0, 5, 23, 47, 63], 400, 300, fmt, directional=False, post=fmt == abi.SW_PIXEL_C64)


def test_sky_map_missing_side_and_validation(gpu_ok):
    scene = host.Scene(**dict(host.SKY_MAP, skybox_missing_side=5, skybox_size=64))
    # the sky's top is missing: those pixels keep the background (cleared here, draw_background)
    run_frames(scene, [3, 31], 320, 240, abi.SW_PIXEL_C32, directional=False, clear=True)
    # a skybox draw needs sw_set_skybox; an unknown texture source is rejected
    st = scene.static_data()
    fr = host.Frame(scene).prepare(3, host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False))
    r = gpu.GpuRenderer(st)
    try:
        r.frame_begin(fr.params, fr.lights)
        r.submit_surfaces(fr.surfaces, fr.total_texels)
        with pytest.raises(gpu.SwError, match="skybox"):
            r.submit_draws(fr.draws, fr.vertices)
        t32, t64, _, _ = scene.skybox()
        r.set_skybox(t32, t64)
        bad = fr.draws.copy()
        bad["tex_source"][0] = 2
        with pytest.raises(gpu.SwError, match="texture source"):
            r.submit_draws(bad, fr.vertices)
        r.submit_draws(fr.draws, fr.vertices)
    finally:
        r.close()


def test_host_renderer_sky_map(gpu_ok):
    """The C++ host renderer uploads the scene's skybox itself (swh_renderer_create)."""
    scene = host.Scene(**host.SKY_MAP)
    hr = host.HostRenderer(scene)
    try:
        opts = host.frame_options(320, 240, abi.SW_PIXEL_C64, directional=False)
        hr.prepare_frame(17, opts)
        got = np.zeros((240, 320), np.uint64)
        hr.draw_frame(got)
    finally:
        hr.close()
    st = scene.static_data()
    fr = host.Frame(scene).prepare(17, opts)
    assert fr.skybox_draws > 0
    arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=4)
    want = np.zeros((240, 320), np.uint64)
    oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want, skybox=scene.skybox()[1])
    assert np.array_equal(want, got)


def test_host_renderer_draw_frame_models(gpu_ok):
    """The per-call host path (swh_renderer_prepare_frame + swh_renderer_draw_frame) with triangle models,
    sprites and decals: their triangle draws and vertices reach the rasteriser; equal to the oracle."""
    scene = host.Scene(**dict(host.SMALL_MAP, num_models=3, model_triangles=600, num_sprites=8, num_decals=16))
    hr = host.HostRenderer(scene)
    opts = host.frame_options(320, 240, abi.SW_PIXEL_C64, directional=False)
    st = scene.static_data()
    lite = scene.lite_textures()
    fr = host.Frame(scene)
    tris = 0
    try:
        for fi in (5, 21, 40):
            hr.prepare_frame(fi, opts)
            got = np.zeros((240, 320), np.uint64)
            hr.draw_frame(got)
            fr.prepare(fi, opts)
            tris += fr.model_triangles
            arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=4)
            want = np.zeros((240, 320), np.uint64)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want, tri_vertices=fr.tri_vertices,
                                    lite=lite) == 0
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
    finally:
        hr.close()
    assert tris > 0


def test_host_renderer_render_frame_graph(gpu_ok):
    """swh_renderer_render_frame: host work + the whole frame as one graph with postprocess, the result
    copied straight into a registered host buffer; equal to the oracle's frame and tonemap."""
    scene = host.Scene(**host.SMALL_MAP)
    hr = host.HostRenderer(scene)
    cfg = abi.PostConfig.default()
    opts = host.frame_options(320, 240, abi.SW_PIXEL_C64, directional=False)
    out = np.zeros((240, 320), np.uint32)
    try:
        hr.register_host_buffer(out)
        with pytest.raises(gpu.SwError):
            hr.register_host_buffer(out[10:20])  # overlaps a registered buffer
        hr.render_frame(12, opts, out=out, post=cfg)
        got_registered = out.copy()
        hr.unregister_host_buffer(out)
        with pytest.raises(gpu.SwError):
            hr.unregister_host_buffer(out)
    finally:
        hr.close()
    st = scene.static_data()
    fr = host.Frame(scene).prepare(12, opts)
    arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=4)
    hdr = np.zeros((240, 320), np.uint64)
    oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, hdr)
    want, _, _ = oracle.postprocess(cfg, hdr, 1.0 / 60.0, (1.0, 1.0, 1.0), 1.0)
    assert np.array_equal(want, got_registered)


def test_host_renderer_matches_python_driven_path(gpu_ok):
    """swh_renderer_* (C++ host driving the C ABI) renders the same frame as the step-by-step path."""
    scene = host.Scene(**host.SMALL_MAP)
    hr = host.HostRenderer(scene)
    try:
        opts = host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False)
        hr.prepare_frame(12, opts)
        got = np.zeros((240, 320), np.uint32)
        hr.draw_frame(got)
    finally:
        hr.close()
    st = scene.static_data()
    fr = host.Frame(scene).prepare(12, opts)
    arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=4)
    want = np.zeros((240, 320), np.uint32)
    oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want)
    assert np.array_equal(want, got)
