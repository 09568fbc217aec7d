"""Shadowed dynamic lights (cube shadow maps) through the GPU path against the oracle: the depth maps
(DepthRenderer + DepthRasterizer, drawn into a storage that persists between frames), surfaces lit
through them (cube_shadow_map_fetch), and whole frames through both preparation paths - bit-exact."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu

SHADOW_MAP = dict(host.SMALL_MAP, num_dynamic_lights=4, shadowed_lights=2)


def test_shadow_maps_and_surfaces(gpu_ok):
    """Per frame: the GPU's storage equals the oracle's (both start at zero and are never cleared, so a
    frame's uncovered texels keep the previous frame's values), and the surfaces built with the frame's
    shadow maps equal the oracle's."""
    scene = host.Scene(**SHADOW_MAP)
    st = scene.static_data()
    fr = host.Frame(scene)
    r = gpu.GpuRenderer(st)
    storage = np.zeros(0, np.float32)
    shadowed_texels = 0
    try:
        frames = [(0, abi.SW_PIXEL_C64), (9, abi.SW_PIXEL_C32), (30, abi.SW_PIXEL_C64), (31, abi.SW_PIXEL_C64)]
        frames += [(f, abi.SW_PIXEL_C64) for f in range(40, 64, 4)]
        for fi, fmt in frames:
            fr.prepare(fi, host.frame_options(640, 480, fmt, directional=True, shadows_quality=-1.0 if fi == 31 else 0.0))
            assert fr.depth_draws.size > 0 and (fr.light_shadows["kind"] == abi.SW_SHADOW_CUBE).sum() >= 1
            if storage.size < fr.shadow_texels:
                storage = np.concatenate([storage, np.zeros(fr.shadow_texels - storage.size, np.float32)])
            oracle.shadow_maps(fr.depth_draws, fr.depth_vertices, storage)
            r.build_shadow_maps(fr.depth_draws, fr.depth_vertices, fr.shadow_texels)
            got = r.read_shadow_maps(storage.size)
            assert np.array_equal(got.view(np.uint32), storage.view(np.uint32)), \
                f"frame {fi}: {(got != storage).sum()} shadow-map texels differ"
            want = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8,
                                         shadows=fr.light_shadows, shadow_texels=storage)
            r.set_light_shadows(fr.light_shadows)
            r.frame_begin(fr.params, fr.lights)
            r.submit_surfaces(fr.surfaces, fr.total_texels)
            assert np.array_equal(want, r.read_surfaces(fr.total_texels, fmt)), f"frame {fi}: surfaces differ"
            plain = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8)
            shadowed_texels += int((plain != want).sum())
        # box rooms are convex: only lights shining through doorways and corridors leave texels in shadow
        assert shadowed_texels > 0
    finally:
        r.close()


@pytest.mark.parametrize("gpu_prep", [True, False])
def test_shadowed_frames_through_the_renderer(gpu_ok, gpu_prep):
    """render_frame with shadowed lights (shadow maps built before the frame's graph) equals the oracle's
    frame from the host's preparation and shadow maps."""
    scene = host.Scene(**SHADOW_MAP)
    st = scene.static_data()
    fr = host.Frame(scene)
    hr = host.HostRenderer(scene)
    hr.set_gpu_prep(gpu_prep)
    w, h = 640, 480
    opts = host.frame_options(w, h, abi.SW_PIXEL_C64, directional=True, clear_background=True)
    storage = np.zeros(0, np.float32)
    try:
        for fi in [3, 56, 60]:
            fr.prepare(fi, opts)
            if storage.size < fr.shadow_texels:
                storage = np.concatenate([storage, np.zeros(fr.shadow_texels - storage.size, np.float32)])
            oracle.shadow_maps(fr.depth_draws, fr.depth_vertices, storage)
            arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8,
                                          shadows=fr.light_shadows, shadow_texels=storage)
            want = np.zeros((h, w), np.uint64)
            oracle.clear_background(fr.params, want)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want) == 0
            got = np.zeros((h, w), np.uint64)
            hr.render_frame(fi, opts, out=got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
    finally:
        hr.close()


def test_shadow_inputs_are_validated(gpu_ok):
    scene = host.Scene(**SHADOW_MAP)
    fr = host.Frame(scene).prepare(0, host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False))
    r = gpu.GpuRenderer(scene.static_data())
    try:
        bad = fr.depth_draws.copy()
        bad[0]["map_offset"] = fr.shadow_texels  # past the storage
        with pytest.raises(gpu.SwError):
            r.build_shadow_maps(bad, fr.depth_vertices, fr.shadow_texels)
        r.build_shadow_maps(fr.depth_draws, fr.depth_vertices, fr.shadow_texels)
        sh = fr.light_shadows.copy()
        sh[0]["size"] = 4096  # too large
        with pytest.raises(gpu.SwError):
            r.set_light_shadows(sh)
        r.set_light_shadows(fr.light_shadows)
        r.set_light_shadows(None)
    finally:
        r.close()


@pytest.mark.parametrize("quality", [0.0, 1.0])
def test_shadow_maps_prepared_on_the_gpu(gpu_ok, quality):
    """sw_build_shadow_maps_view (each side's leafs from the host, their polygons' depth draws prepared on
    the GPU) leaves the storage that the host-prepared depth draws leave, texel for texel, frame after
    frame; the host halves agree on the maps."""
    scene = host.Scene(**dict(host.FULL_MAP, shadowed_lights=4))
    fr, fv = host.Frame(scene), host.Frame(scene)
    hr = host.HostRenderer(scene)  # its context holds the map (sw_set_map)
    glib = gpu.load_library()
    opts = host.frame_options(1280, 720, abi.SW_PIXEL_C64, directional=True, shadows_quality=quality)
    storage = np.zeros(0, np.float32)
    try:
        for fi in (0, 7, 70, 140, 141, 250):
            fr.prepare(fi, opts)
            fv.prepare_view(fi, opts)
            assert fv.depth_draws.size == 0 and fv.shadow_sides.size == 6 * (fv.light_shadows["kind"] == abi.SW_SHADOW_CUBE).sum()
            assert fv.light_shadows.tobytes() == fr.light_shadows.tobytes() and fv.shadow_texels == fr.shadow_texels
            if storage.size < fr.shadow_texels:
                storage = np.concatenate([storage, np.zeros(fr.shadow_texels - storage.size, np.float32)])
            oracle.shadow_maps(fr.depth_draws, fr.depth_vertices, storage)
            s, lf = fv.shadow_sides, fv.shadow_leafs
            assert glib.sw_build_shadow_maps_view(hr.context(), abi.ptr(s), s.size, abi.ptr(lf), lf.size,
                                                  fv.shadow_texels) == abi.SW_OK
            got = np.zeros(storage.size, np.float32)
            assert glib.sw_read_shadow_maps(hr.context(), abi.ptr(got), got.size) == abi.SW_OK
            assert np.array_equal(got.view(np.uint32), storage.view(np.uint32)), \
                f"frame {fi}: {(got != storage).sum()} of {storage.size} texels differ"
        # invalid lists are rejected before anything runs
        bad = lf.copy()
        bad[0]["side"] = s.size
        assert glib.sw_build_shadow_maps_view(hr.context(), abi.ptr(s), s.size, abi.ptr(bad), bad.size,
                                              fv.shadow_texels) == abi.SW_ERR_INVALID_ARGUMENT
        bad = s.copy()
        bad[0]["map_offset"] = fv.shadow_texels
        assert glib.sw_build_shadow_maps_view(hr.context(), abi.ptr(bad), bad.size, abi.ptr(lf), lf.size,
                                              fv.shadow_texels) == abi.SW_ERR_INVALID_ARGUMENT
    finally:
        hr.close()
