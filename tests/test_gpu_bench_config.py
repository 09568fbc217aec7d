"""The benchmarked configuration against the oracle, at full size: the 64-room map (seed 2), 1920x1080
Color64 with directional lightmaps, normal maps, specular materials and 8 moving lights, bloom + tonemap,
on the benchmark's own camera-path frames in its order (exposure carried from frame to frame).

Both ways the benchmark drives the library are checked: sw_draw_frame (the host-prepared arrays, one
CUDA graph per frame) and swh_renderer_render_frame (host visibility, GPU-side surface and draw
preparation). For every frame the surface arena, the HDR frame, the tonemapped frame and the next
frame's exposure equal the oracle's bit for bit. The oracle rasterises with one whole-screen clip rect,
the reference's num_threads == 1 path (partial_renderer.rs:1207-1234)."""
import ctypes
import os

import numpy as np
import pytest

import bench
import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu

W, H = bench.W, bench.H
# the benchmark's first eight frames: its warm-up frames and the first timed ones
FRAMES = bench.frame_indices(8)


@pytest.fixture(scope="module")
def scene():
    s = host.Scene(**host.FULL_MAP)
    yield s
    s.close()


@pytest.fixture(scope="module")
def expected(scene):
    """The oracle's surface arena, HDR frame, tonemapped frame and next exposure of every frame."""
    st = scene.static_data()
    fr = host.Frame(scene)
    opts = host.frame_options(W, H, abi.SW_PIXEL_C64, directional=True)
    cfg = abi.PostConfig.default()
    threads = os.cpu_count() or 1
    hdr = np.zeros((H, W), np.uint64)  # the frame buffer carries over from frame to frame
    exposure = 1.0
    out = []
    for fi in FRAMES:
        fr.prepare(fi, opts)
        arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=threads)
        hdr = hdr.copy()
        assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, hdr) == 0
        ldr, exposure_next, _ = oracle.postprocess(cfg, hdr, 1.0 / 60.0, (1.0, 1.0, 1.0), exposure)
        out.append(dict(index=fi, arena=arena, hdr=hdr, ldr=ldr, exposure=np.float32(exposure_next),
                        texels=fr.total_texels))
        exposure = exposure_next
    return out


def check_frame(want, arena, hdr, ldr, exposure):
    fi = want["index"]
    assert np.array_equal(want["arena"], arena), f"frame {fi}: surface arena differs"
    assert np.array_equal(want["hdr"], hdr), f"frame {fi}: {(want['hdr'] != hdr).sum()} HDR pixels differ"
    assert np.array_equal(want["ldr"], ldr), f"frame {fi}: {(want['ldr'] != ldr).sum()} tonemapped pixels differ"
    assert np.float32(exposure) == want["exposure"], f"frame {fi}: exposure {exposure} != {want['exposure']}"


def test_bench_frames_graph(gpu_ok, scene, expected):
    """sw_draw_frame, as the benchmark's measurement pass runs it."""
    r = gpu.GpuRenderer(scene.static_data())
    fr = host.Frame(scene)
    opts = host.frame_options(W, H, abi.SW_PIXEL_C64, directional=True)
    cfg = abi.PostConfig.default()
    ldr = np.zeros((H, W), np.uint32)
    try:
        for want in expected:
            fr.prepare(want["index"], opts)
            r.draw_frame(r.frame_input(fr.params, fr.lights, fr.surfaces, fr.total_texels, fr.draws, fr.vertices,
                                       post_config=cfg, dst=ldr))
            arena = r.read_surfaces(fr.total_texels, abi.SW_PIXEL_C64)
            hdr = r.read_framebuffer(W, H, abi.SW_PIXEL_C64)
            check_frame(want, arena, hdr, ldr, r.exposure())
        assert r.stats().bad_texel_fetches == 0
    finally:
        r.close()


def test_bench_frames_render_frame(gpu_ok, scene, expected):
    """swh_renderer_render_frame with the GPU-side preparation, as the benchmark's e2e loop runs it
    (the Color32 frame written straight into a registered host buffer)."""
    glib = gpu.load_library()
    hr = host.HostRenderer(scene)
    opts = host.frame_options(W, H, abi.SW_PIXEL_C64, directional=True)
    cfg = abi.PostConfig.default()
    ldr = np.zeros((H, W), np.uint32)
    ctx = hr.context()
    try:
        hr.register_host_buffer(ldr)
        for want in expected:
            hr.render_frame(want["index"], opts, out=ldr, post=cfg)
            arena = np.empty(want["texels"], np.uint64)
            assert glib.sw_read_surfaces(ctx, abi.ptr(arena), arena.nbytes) == 0
            hdr = np.empty((H, W), np.uint64)
            assert glib.sw_read_framebuffer(ctx, abi.ptr(hdr), hdr.nbytes) == 0
            e = ctypes.c_float()
            assert glib.sw_get_exposure(ctx, ctypes.byref(e)) == 0
            check_frame(want, arena, hdr, ldr, e.value)
        hr.unregister_host_buffer(ldr)
    finally:
        hr.close()
