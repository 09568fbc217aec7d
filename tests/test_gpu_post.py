"""GPU parity of the HDR postprocessor (bloom + tonemap + auto exposure) and the frame upscaler."""
import ctypes

import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, synth

pytestmark = pytest.mark.gpu


def hdr_frame(rng, w, h, hi=4000):
    lanes = rng.integers(0, hi, (h, w, 4), dtype=np.uint64)
    lanes[..., 3] = rng.integers(0, 2, (h, w)) * 255
    return (lanes[..., 0] | (lanes[..., 1] << 16) | (lanes[..., 2] << 32) | (lanes[..., 3] << 48)).astype(np.uint64)


def config(**kw):
    c = abi.PostConfig.default()
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("scale_log2,linear,sigma", [(1, 0, 1.0), (1, 1, 1.0), (2, 1, 6.0), (3, 0, 3.0), (2, 0, 0.0),
                                                     (1, 1, 25.0)])
def test_postprocess_sequence_bit_exact(gpu_ok, scale_log2, linear, sigma):
    """Four frames in a row: tonemapped pixels and the exposure state match bit for bit."""
    rng = np.random.default_rng(scale_log2 * 10 + linear)
    w, h = 203, 117
    cfg = config(bloom_buffer_scale_log2=scale_log2, linear_bloom_filter=linear, bloom_sigma=sigma)
    st = synth.BatchedSurfaces(seed=1, count=1, max_side=8)
    r = gpu.GpuRenderer(st.static_data())
    exposure = 1.0
    modulate = (1.0, 0.9, 1.1)
    try:
        for frame in range(4):
            hdr = hdr_frame(rng, w, h, hi=600 * (frame + 1))
            want, exposure_next, _ = oracle.postprocess(cfg, hdr, 1.0 / 60.0, modulate, exposure, pitch=w + 5)
            r.set_framebuffer(hdr, abi.SW_PIXEL_C64)
            got = np.zeros((h, w + 5), np.uint32)
            r.postprocess(cfg, 1.0 / 60.0, modulate, out=got, pitch=w + 5)
            assert np.array_equal(want[:, :w], got[:, :w]), f"frame {frame}: {(want[:, :w] != got[:, :w]).sum()} px differ"
            assert r.exposure() == np.float32(exposure_next), (frame, r.exposure(), exposure_next)
            exposure = exposure_next
    finally:
        r.close()


@pytest.mark.parametrize("mode,scale", [(abi.SW_UPSCALE_NEAREST, 2), (abi.SW_UPSCALE_NEAREST, 3), (abi.SW_UPSCALE_AVG2X, 2)])
def test_upscale_bit_exact(gpu_ok, mode, scale):
    rng = np.random.default_rng(scale)
    W, H = 161, 93
    src = rng.integers(0, 1 << 32, (H // scale) * (W // scale), dtype=np.uint64).astype(np.uint32)
    want = oracle.upscale(mode, scale, src, W, H)
    st = synth.BatchedSurfaces(seed=1, count=1, max_side=8)
    r = gpu.GpuRenderer(st.static_data())
    try:
        got = np.zeros((H, W), np.uint32)
        r.upscale(mode, scale, src, got)
    finally:
        r.close()
    assert np.array_equal(want, got)
