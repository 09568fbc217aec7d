"""Failure detection without a GPU fault: bad inputs injected on the host are rejected with an error
status before anything is uploaded or launched, and the context renders correctly afterwards.

Injected: a NaN or infinite camera (position, view matrices), a light with a NaN, a zero-size frame
buffer, and malformed map data (polygons whose vertices, texture or lightmap fall outside the uploaded
arrays, texture mips outside the texel array)."""
import ctypes
import math

import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu

W, H = 320, 240


def counters(r):
    s = r.stats()
    return (s.surfaces, s.surface_texels, s.draws, s.pixel_writes, s.upload_bytes)


def oracle_frame(scene, fr):
    st = scene.static_data()
    arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=4)
    want = np.zeros((H, W), np.uint32)
    oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want)
    return want


def test_non_finite_camera_and_lights_rejected(gpu_ok):
    scene = host.Scene(**host.SMALL_MAP)
    fr = host.Frame(scene).prepare(12, host.frame_options(W, H, abi.SW_PIXEL_C32, directional=False))
    r = gpu.GpuRenderer(scene.static_data())
    try:
        before = counters(r)
        for bad in (math.nan, math.inf, -math.inf):
            p = abi.FrameParams.from_buffer_copy(fr.params)
            p.cam_pos[1] = bad
            with pytest.raises(gpu.SwError, match="non-finite camera"):
                r.frame_begin(p, fr.lights)
            with pytest.raises(gpu.SwError, match="non-finite camera"):
                r.draw_frame(r.frame_input(p, fr.lights, fr.surfaces, fr.total_texels, fr.draws, fr.vertices,
                                           dst=np.zeros((H, W), np.uint32)))
        if fr.lights.size:
            lights = fr.lights.copy()
            lights["position"][0, 2] = math.nan
            with pytest.raises(gpu.SwError, match="non-finite"):
                r.frame_begin(fr.params, lights)
        assert counters(r) == before, "a rejected frame uploaded or launched something"
        # the context is still usable: the same frame with the good camera equals the oracle's
        got = np.zeros((H, W), np.uint32)
        r.draw_frame(r.frame_input(fr.params, fr.lights, fr.surfaces, fr.total_texels, fr.draws, fr.vertices, dst=got))
        assert np.array_equal(got, oracle_frame(scene, fr))
    finally:
        r.close()


def test_non_finite_view_matrices_rejected(gpu_ok):
    """sw_draw_frame_view with an infinite view matrix or a NaN planes matrix."""
    scene = host.Scene(**host.SMALL_MAP)
    glib = gpu.load_library()
    hr = host.HostRenderer(scene)
    fr = host.Frame(scene)
    opts = host.frame_options(W, H, abi.SW_PIXEL_C32, directional=False)
    try:
        ctx = hr.context()
        for field, bad in (("view_matrix", math.inf), ("planes_matrix", math.nan)):
            vin = fr.prepare_view(5, opts)
            getattr(vin, field)[5] = bad
            s0 = abi.Stats()
            glib.sw_get_stats(ctx, ctypes.byref(s0))
            assert glib.sw_draw_frame_view(ctx, ctypes.byref(vin)) == abi.SW_ERR_INVALID_ARGUMENT
            assert b"non-finite camera" in glib.sw_last_error(ctx)
            s1 = abi.Stats()
            glib.sw_get_stats(ctx, ctypes.byref(s1))
            assert (s0.upload_bytes, s0.draws, s0.surfaces) == (s1.upload_bytes, s1.draws, s1.surfaces)
        out = np.zeros((H, W), np.uint32)
        hr.render_frame(5, opts, out=out)
        fr.prepare(5, opts)
        assert np.array_equal(out, oracle_frame(scene, fr))
    finally:
        hr.close()


def test_zero_size_framebuffer_rejected(gpu_ok):
    scene = host.Scene(**host.SMALL_MAP)
    fr = host.Frame(scene).prepare(3, host.frame_options(W, H, abi.SW_PIXEL_C32, directional=False))
    r = gpu.GpuRenderer(scene.static_data())
    hr = host.HostRenderer(scene)
    try:
        before = counters(r)
        for w, h in ((0, H), (W, 0), (0, 0)):
            p = abi.FrameParams.from_buffer_copy(fr.params)
            p.width, p.height = w, h
            with pytest.raises(gpu.SwError, match="bad frame size"):
                r.frame_begin(p, fr.lights)
            with pytest.raises(gpu.SwError, match="bad frame size"):
                r.draw_frame(r.frame_input(p, fr.lights, fr.surfaces, fr.total_texels, fr.draws, fr.vertices))
        with pytest.raises(gpu.SwError):
            r.set_framebuffer(np.zeros((0, 16), np.uint64), abi.SW_PIXEL_C64)
        assert counters(r) == before
        # the host renderer refuses zero-size options before any host or GPU work
        with pytest.raises(gpu.SwError):
            hr.render_frame(3, host.frame_options(0, H, abi.SW_PIXEL_C32, directional=False), out=np.zeros((1, 1), np.uint32))
    finally:
        r.close()
        hr.close()


def test_malformed_map_rejected(gpu_ok):
    """Map data that points outside the uploaded arrays is rejected at upload (sw_set_map, sw_create)."""
    scene = host.Scene(**host.SMALL_MAP)
    glib = gpu.load_library()
    hr = host.HostRenderer(scene)
    try:
        ctx = hr.context()
        polys, verts = host.Frame(scene).map_data()
        assert glib.sw_set_map(ctx, abi.ptr(polys), polys.size, abi.ptr(verts), verts.shape[0]) == abi.SW_OK
        k = int(np.nonzero(polys["flags"] & 4)[0][0])  # a polygon with a lit diffuse layer (SW_POLY_DIFFUSE_LAYER)
        assert polys["lightmap_data_offset"][k] != 0
        for field, value, msg in (("first_vertex", verts.shape[0], b"vertices out of range"),
                                  ("texture", 1 << 20, b"bad texture"),
                                  ("lightmap_data_offset", 0xFFFFFF00, b"lightmap out of range"),
                                  ("blending_mode", 9, b"bad blending mode")):
            bad = polys.copy()
            bad[field][k] = value
            rc = glib.sw_set_map(ctx, abi.ptr(bad), bad.size, abi.ptr(verts), verts.shape[0])
            assert rc == abi.SW_ERR_INVALID_ARGUMENT, field
            assert msg in glib.sw_last_error(ctx), (field, glib.sw_last_error(ctx))
    finally:
        hr.close()
    # texture mips outside the texel array
    st = scene.static_data()
    mips = st.texture_mips.copy()
    mips["offset"][3] = st.texels.size
    bad_static = gpu.StaticData(st.texels, mips, st.emissive_pixels, st.emissive_mips, st.lightmaps,
                                st.directional_lightmaps)
    with pytest.raises(gpu.SwError):
        gpu.GpuRenderer(bad_static)
