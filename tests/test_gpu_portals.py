"""Portals on the GPU (sw_draw_frame with nested views) against the oracle: whole frames of a map with a
mirror, a camera screen mixed with a texture and a parallax window, two nested levels, dynamic and
shadowed lights, in both pixel formats (and through the HDR postprocess), equal the oracle's frames
composed view by view (each portal texture rendered, mixed, then sampled by the frame's portal draws),
also with models, sprites and portal textures lit from a light grid; the depth limit (black portals mixed with their texture) likewise; malformed views are refused."""
import ctypes

import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu

PORTAL_MAP = dict(host.SMALL_MAP, num_portals=3, portals_depth=2, num_dynamic_lights=3, shadowed_lights=1)
FRAMES = list(range(28, 64, 2))


def oracle_frame(scene, fr, storage, w, h, fmt):
    """The frame composed by the oracle: surfaces of every view, the views in order, then the frame."""
    st = scene.static_data()
    lite = scene.lite_textures()
    if fr.shadow_texels:
        if storage.size < fr.shadow_texels:
            storage = np.concatenate([storage, np.zeros(fr.shadow_texels - storage.size, np.float32)])
        oracle.shadow_maps(fr.depth_draws, fr.depth_vertices, storage)
    shadows = fr.light_shadows if fr.shadow_texels else None
    arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8,
                                  shadows=shadows, shadow_texels=storage if fr.shadow_texels else None)
    if len(fr.views):
        oracle.render_views(fr.views, fr.draws, fr.vertices, arena, fr.params, tri_vertices=fr.tri_vertices, lite=lite)
    want = np.zeros((h, w), np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32)
    oracle.clear_background(fr.params, want)
    assert oracle.rasterize(fr.draws[:fr.main_draws], fr.vertices, arena, fr.params, want, tri_vertices=fr.tri_vertices,
                            lite=lite) == 0
    return want, storage


@pytest.mark.parametrize("fmt,depth,grid", [(abi.SW_PIXEL_C32, 2, 0), (abi.SW_PIXEL_C64, 2, 0), (abi.SW_PIXEL_C32, 0, 0),
                                            (abi.SW_PIXEL_C64, 1, 1)])
def test_portal_frames(gpu_ok, fmt, depth, grid):
    """grid=1: a light-grid map with models and sprites, all of them and the portal textures lit from the grid."""
    extra = dict(light_grid=1, num_models=3, num_sprites=10) if grid else {}
    scene = host.Scene(**dict(PORTAL_MAP, portals_depth=depth, **extra))
    fr = host.Frame(scene)
    hr = host.HostRenderer(scene)
    w, h = 640, 360
    opts = host.frame_options(w, h, fmt, directional=False, clear_background=True)
    storage = np.zeros(0, np.float32)
    views = nested = 0
    try:
        for fi in FRAMES:  # in order: the shadow-map storage carries over
            fr.prepare(fi, opts)
            views += len(fr.views)
            nested += int((fr.views["num_draws"] > 0).sum()) if len(fr.views) else 0
            want, storage = oracle_frame(scene, fr, storage, w, h, fmt)
            got = np.zeros_like(want)
            hr.render_frame(fi, opts, out=got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
        assert views > 0
        assert (nested > 0) == (depth > 0)
    finally:
        hr.close()
        scene.close()


def test_portal_frames_postprocessed(gpu_ok):
    """Colour64 portal frames through bloom and tonemap, exposure carried from frame to frame."""
    scene = host.Scene(**PORTAL_MAP)
    fr = host.Frame(scene)
    hr = host.HostRenderer(scene)
    w, h = 640, 360
    opts = host.frame_options(w, h, abi.SW_PIXEL_C64, directional=False, clear_background=True)
    cfg = abi.PostConfig.default()
    storage = np.zeros(0, np.float32)
    exposure = 1.0
    try:
        assert gpu.load_library().sw_set_exposure(hr.context(), ctypes.c_float(exposure)) == abi.SW_OK
        seen = 0
        for fi in FRAMES[::2]:
            fr.prepare(fi, opts)
            seen += len(fr.views)
            hdr, storage = oracle_frame(scene, fr, storage, w, h, abi.SW_PIXEL_C64)
            want, exposure, _ = oracle.postprocess(cfg, hdr, 1.0 / 60.0, [1.0, 1.0, 1.0], exposure)
            got = np.zeros((h, w), np.uint32)
            hr.render_frame(fi, opts, out=got, post=cfg, frame_duration_s=1.0 / 60.0)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
        assert seen > 0
    finally:
        hr.close()
        scene.close()


def test_malformed_views_refused(gpu_ok):
    scene = host.Scene(**PORTAL_MAP)
    fr = host.Frame(scene)
    glib = gpu.load_library()
    hr = host.HostRenderer(scene)
    w, h = 640, 360
    opts = host.frame_options(w, h, abi.SW_PIXEL_C32, directional=False)
    try:
        fi = next(f for f in FRAMES if (fr.prepare(f, opts) or True) and len(fr.views))
        ctx = hr.context()
        base = fr.views.copy()

        def frame_input(views, main_draws):
            fin = abi.FrameInput()
            fin.params = fr.params
            fin.num_lights, fin.lights = fr.lights.size, abi.ptr(fr.lights)
            fin.surfaces, fin.num_surfaces, fin.total_texels = abi.ptr(fr.surfaces), fr.surfaces.size, fr.total_texels
            fin.num_draws, fin.draws = fr.draws.size, abi.ptr(fr.draws)
            fin.vertices, fin.num_vertices = abi.ptr(fr.vertices), fr.vertices.size
            fin.num_views, fin.views, fin.main_draws = views.size, abi.ptr(views), main_draws
            return fin

        good = frame_input(base, fr.main_draws)
        assert glib.sw_draw_frame(ctx, ctypes.byref(good)) == abi.SW_OK
        cases = []
        v = base.copy(); v[0]["target_offset"] = fr.total_texels; cases.append((v, fr.main_draws, b"target outside"))
        v = base.copy(); v[0]["width"] = 0; cases.append((v, fr.main_draws, b"bad size"))
        v = base.copy(); v[0]["first_draw"] = 0; v[0]["num_draws"] = max(1, int(v[0]["num_draws"])); cases.append((v, fr.main_draws, b"draws outside"))
        v = base.copy(); cases.append((v, fr.draws.size + 1, b"main_draws"))
        v = base.copy(); v[0]["mix_blend"] = 7; v[0]["mix_size"] = [4, 4]; cases.append((v, fr.main_draws, b"texture mix"))
        v = base.copy(); v[0]["mix_blend"] = 0; v[0]["mix_size"] = [4, 4]; v[0]["mix_offset"] = 1 << 40
        cases.append((v, fr.main_draws, b"texture mix"))
        v = base.copy(); v[0]["clear_background"] = 3; cases.append((v, fr.main_draws, b"clear_background"))
        for views, main_draws, msg in cases:
            fin = frame_input(views, main_draws)
            assert glib.sw_draw_frame(ctx, ctypes.byref(fin)) == abi.SW_ERR_INVALID_ARGUMENT, msg
            assert msg in glib.sw_last_error(ctx), (msg, glib.sw_last_error(ctx))
        assert glib.sw_draw_frame(ctx, ctypes.byref(good)) == abi.SW_OK  # the context still renders
    finally:
        hr.close()
        scene.close()
