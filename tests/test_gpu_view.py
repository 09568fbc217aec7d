"""GPU-side surface and draw preparation (sw_draw_frame_view) against the host's preparation.

The host path (FramePrep::prepare: prepare_polygons_surfaces, build_polygons_surfaces, draw_tree) is the
restatement the oracle tests pin; the GPU path must produce the same surface descriptors, draw commands
and vertices bit for bit, and therefore the same frames."""
import ctypes

import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu


def prepared_equal(scene, frames, w, h, fmt, directional=True, mip_bias=0.0):
    """For each frame: the descriptors, draws and vertices the GPU prepared equal the host's, and the two
    renderers (GPU preparation, host preparation) give the same frame."""
    hr_gpu = host.HostRenderer(scene)
    hr_host = host.HostRenderer(scene)
    hr_host.set_gpu_prep(False)
    fr = host.Frame(scene)
    dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
    opts = host.frame_options(w, h, fmt, directional=directional, mip_bias=mip_bias)
    try:
        for fi in frames:
            fr.prepare(fi, opts)
            got = np.zeros((h, w), dt)
            want = np.zeros((h, w), dt)
            hr_gpu.render_frame(fi, opts, out=got)
            hr_host.render_frame(fi, opts, out=want)
            k, s, d, v = hr_gpu.read_view_prep()
            assert k.error == 0
            assert k.num_surfaces == fr.surfaces.size and k.total_texels == fr.total_texels, f"frame {fi}: surface count"
            assert np.array_equal(s.view(np.uint8), fr.surfaces.view(np.uint8)), f"frame {fi}: surface descriptors differ"
            assert k.num_draws == fr.draws.size and k.num_vertices == fr.vertices.size, f"frame {fi}: draw count"
            assert np.array_equal(d.view(np.uint8), fr.draws.view(np.uint8)), f"frame {fi}: draws differ"
            assert np.array_equal(v.view(np.uint8), fr.vertices.view(np.uint8)), f"frame {fi}: vertices differ"
            assert np.array_equal(got, want), f"frame {fi}: {(got != want).sum()} pixels differ"
    finally:
        hr_gpu.close()
        hr_host.close()


def test_view_prep_small_map_c32(gpu_ok):
    scene = host.Scene(**host.SMALL_MAP)
    prepared_equal(scene, [0, 7, 21, 40, 63, 100, 150], 640, 480, abi.SW_PIXEL_C32, directional=False)


def test_view_prep_full_map_c64(gpu_ok):
    """64-room map at 1920x1080: directional lightmaps, 8 moving lights (light lists), specular materials."""
    scene = host.Scene(**host.FULL_MAP)
    prepared_equal(scene, list(range(0, 256, 17)), 1920, 1080, abi.SW_PIXEL_C64)


def test_view_prep_sky_map(gpu_ok):
    """Sky polygons stay on the host (their bounds place the skybox draws, which come first)."""
    scene = host.Scene(**host.SKY_MAP)
    prepared_equal(scene, [0, 5, 30, 61, 90], 800, 600, abi.SW_PIXEL_C64)


def test_view_prep_scrolling_textures(gpu_ok):
    """Scrolling materials (get_texture_shift >> mip in the descriptors' tc start and basis start), other
    mips included; and the frames against the oracle's through the host-prepared descriptors."""
    scene = host.Scene(**dict(host.SMALL_MAP, scrolling_materials=12, emissive_frac=0.3))
    prepared_equal(scene, [0, 1, 45, 123, 1000, 99999], 640, 480, abi.SW_PIXEL_C64)
    prepared_equal(scene, [7, 500], 640, 480, abi.SW_PIXEL_C32, directional=False, mip_bias=1.5)
    st = scene.static_data()
    fr = host.Frame(scene)
    hr = host.HostRenderer(scene)
    opts = host.frame_options(640, 480, abi.SW_PIXEL_C64, directional=True, clear_background=True)
    try:
        for fi in (90, 777):
            fr.prepare(fi, opts)
            arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8)
            want = np.zeros((480, 640), np.uint64)
            oracle.clear_background(fr.params, want)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want) == 0
            got = np.zeros((480, 640), np.uint64)
            hr.render_frame(fi, opts, out=got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
    finally:
        hr.close()


def test_view_prep_framed_animations(gpu_ok):
    """Materials cycling through texture frames (the mapping table advances once per frame; every
    renderer and frame here sees the same sequence), with scrolling on some of them."""
    scene = host.Scene(**dict(host.FULL_MAP, animated_materials=10, scrolling_materials=4))
    prepared_equal(scene, [0, 1, 15, 16, 30, 31, 45, 60, 200, 201], 1280, 720, abi.SW_PIXEL_C64)


def test_view_prep_mip_bias_and_emissive(gpu_ok):
    """Other mips (bias 1.5) and the emissive layer's descriptors."""
    scene = host.Scene(**dict(host.SMALL_MAP, emissive_frac=0.5, num_dynamic_lights=4))
    prepared_equal(scene, [3, 33, 77], 640, 480, abi.SW_PIXEL_C64, mip_bias=1.5)


def test_view_prep_postprocessed_sequence(gpu_ok):
    """render_frame with bloom + tonemap into a registered host buffer: the GPU-prepared sequence equals the
    host-prepared one frame by frame (exposure state included), and the tonemapped frame equals the
    oracle's postprocess of the oracle-rasterised frame."""
    scene = host.Scene(**host.FULL_MAP)
    w, h = 1280, 720
    opts = host.frame_options(w, h, abi.SW_PIXEL_C64, directional=True)
    cfg = abi.PostConfig.default()
    hr_gpu = host.HostRenderer(scene)
    hr_host = host.HostRenderer(scene)
    hr_host.set_gpu_prep(False)
    out_gpu = np.zeros((h, w), np.uint32)
    out_host = np.zeros((h, w), np.uint32)
    hr_gpu.register_host_buffer(out_gpu)
    try:
        for fi in [2, 40, 41, 42, 120]:
            hr_gpu.render_frame(fi, opts, out=out_gpu, post=cfg)
            hr_host.render_frame(fi, opts, out=out_host, post=cfg)
            assert np.array_equal(out_gpu, out_host), f"frame {fi}: {(out_gpu != out_host).sum()} pixels differ"
        st = gpu.load_library()
        e = [ctypes.c_float(), ctypes.c_float()]
        st.sw_get_exposure(hr_gpu.context(), ctypes.byref(e[0]))
        st.sw_get_exposure(hr_host.context(), ctypes.byref(e[1]))
        assert e[0].value == e[1].value
    finally:
        hr_gpu.unregister_host_buffer(out_gpu)
        hr_gpu.close()
        hr_host.close()


def test_view_prep_against_oracle_frame(gpu_ok):
    """The GPU-prepared frame equals the oracle's surfaces + rasterisation of the host's preparation."""
    scene = host.Scene(**host.SMALL_MAP)
    st = scene.static_data()
    fr = host.Frame(scene)
    w, h, fmt = 640, 480, abi.SW_PIXEL_C64
    opts = host.frame_options(w, h, fmt, directional=True, clear_background=True)
    hr = host.HostRenderer(scene)
    try:
        for fi in [11, 12, 90]:
            fr.prepare(fi, opts)
            arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8)
            want = np.zeros((h, w), np.uint64)
            oracle.clear_background(fr.params, want)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want) == 0
            got = np.zeros((h, w), np.uint64)
            hr.render_frame(fi, opts, out=got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
    finally:
        hr.close()


def test_view_frame_without_leafs_and_bad_leafs(gpu_ok):
    """No visible leaf: only the background. A leaf outside the map is refused on the host, before any
    launch; the context stays usable."""
    scene = host.Scene(**host.SMALL_MAP)
    hr = host.HostRenderer(scene)
    lib = gpu.load_library()
    ctx = hr.context()
    try:
        fr = host.Frame(scene)
        opts = host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False, clear_background=True)
        vin = fr.prepare_view(5, opts)
        vin.num_leafs = 0
        vin.num_leaf_lights = 0
        out = np.zeros((240, 320), np.uint32)
        vin.dst = ctypes.c_void_p(out.ctypes.data)
        vin.dst_pitch = 320
        vin.dst_is_device = 0
        assert lib.sw_draw_frame_view(ctx, ctypes.byref(vin)) == abi.SW_OK
        assert (out == 0x00201008).all()
        leafs = fr.view_leafs.copy()
        leafs[0]["num_polygons"] = 1 << 30
        vin = fr.prepare_view(5, opts)
        vin.leafs = ctypes.c_void_p(leafs.ctypes.data)
        vin.dst = ctypes.c_void_p(out.ctypes.data)
        vin.dst_pitch = 320
        assert lib.sw_draw_frame_view(ctx, ctypes.byref(vin)) == abi.SW_ERR_INVALID_ARGUMENT
        vin = fr.prepare_view(6, opts)
        vin.dst = ctypes.c_void_p(out.ctypes.data)
        vin.dst_pitch = 320
        assert lib.sw_draw_frame_view(ctx, ctypes.byref(vin)) == abi.SW_OK
    finally:
        hr.close()


def test_view_material_frames_are_validated(gpu_ok):
    """A material frame naming a texture without mips is refused on the host before any launch; the
    context stays usable, and a valid table is accepted."""
    scene = host.Scene(**dict(host.SMALL_MAP, animated_materials=2))
    hr = host.HostRenderer(scene)
    lib = gpu.load_library()
    ctx = hr.context()
    try:
        fr = host.Frame(scene)
        opts = host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False)
        out = np.zeros((240, 320), np.uint32)
        vin = fr.prepare_view(5, opts)
        assert vin.num_material_frames > 0 and vin.material_frames
        frames = np.ctypeslib.as_array(ctypes.cast(vin.material_frames, ctypes.POINTER(ctypes.c_uint8)),
                                       shape=(vin.num_material_frames * abi.MATERIAL_FRAME.itemsize,)).view(abi.MATERIAL_FRAME).copy()
        bad = frames.copy()
        bad[0]["texture"] = 1 << 20
        vin.material_frames = ctypes.c_void_p(bad.ctypes.data)
        vin.dst = ctypes.c_void_p(out.ctypes.data)
        vin.dst_pitch = 320
        assert lib.sw_draw_frame_view(ctx, ctypes.byref(vin)) == abi.SW_ERR_INVALID_ARGUMENT
        vin.material_frames = ctypes.c_void_p(frames.ctypes.data)
        assert lib.sw_draw_frame_view(ctx, ctypes.byref(vin)) == abi.SW_OK
    finally:
        hr.close()
