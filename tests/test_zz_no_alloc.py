"""The allocation-free postprocessor entry point against the context-based one.

sw_postprocess_noalloc serves callers that cannot call cudaMalloc (engines that own all device memory
through their own pools, frame loops that cannot take cudaMalloc's implicit synchronisation). It takes
device pointers, keeps its scratch in a static device array, and must produce exactly what
sw_postprocess produces for the same frame and exposure. Two calls in a row check that the shared
scratch left behind by the first call does not leak into the second. This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from sqwheel import abi, gpu, synth

pytestmark = pytest.mark.gpu


def hdr_frame(rng, w, h, hi):
    lanes = rng.integers(0, hi, (h, w, 4), dtype=np.uint64)
    lanes[..., 3] = 255
    return (lanes[..., 0] | (lanes[..., 1] << 16) | (lanes[..., 2] << 32) | (lanes[..., 3] << 48)).astype(np.uint64)


# (width, height, bloom_sigma, bloom_buffer_scale_log2, linear filter): bloom at scales 2, 4 and 8, both
# filters, no bloom (the per-line float sums of the scratch array), and frames at the size limit
CASES = [
    (1000, 700, 3.0, 1, 0),
    (1000, 700, 3.0, 1, 1),
    (1920, 1080, 1.0, 1, 0),
    (1920, 1080, 0.0, 1, 0),
    (640, 480, 0.0, 2, 1),
    (800, 600, 6.0, 2, 1),
    (999, 701, 3.0, 3, 0),
]


@pytest.mark.parametrize("w,h,sigma,scale_log2,linear", CASES)
def test_noalloc_matches_context_postprocess(gpu_ok, w, h, sigma, scale_log2, linear):
    import torch

    import oracle
    lib = gpu.load_library()
    rng = np.random.default_rng(17 + linear + 2 * scale_log2 + int(sigma))
    cfg = abi.PostConfig.default()
    cfg.linear_bloom_filter = linear
    cfg.bloom_sigma = sigma
    cfg.bloom_buffer_scale_log2 = scale_log2
    mod = (1.0, 0.8, 1.2)
    st = synth.BatchedSurfaces(seed=1, count=1, max_side=8)
    r = gpu.GpuRenderer(st.static_data())
    try:
        for call, (hi, exposure) in enumerate([(3000, 1.0), (200, 2.5)]):
            hdr = hdr_frame(rng, w, h, hi)
            # Context-based reference result.
            r.set_exposure(exposure)
            r.set_framebuffer(hdr, abi.SW_PIXEL_C64)
            want = np.zeros((h, w), np.uint32)
            r.postprocess(cfg, 1.0 / 60.0, mod, out=want)
            # Allocation-free entry point on device buffers.
            d_hdr = torch.from_numpy(hdr.view(np.int64)).cuda()
            d_dst = torch.zeros((h, w + 3), dtype=torch.int32, device="cuda")
            d_avg = torch.full((4,), -1.0, dtype=torch.float32, device="cuda")
            cmod = (ctypes.c_float * 3)(*mod)
            rc = lib.sw_postprocess_noalloc(ctypes.c_void_p(d_hdr.data_ptr()), w, h, ctypes.byref(cfg), float(exposure), cmod,
                                            ctypes.c_void_p(d_dst.data_ptr()), w + 3, ctypes.c_void_p(d_avg.data_ptr()), None)
            assert rc == abi.SW_OK
            torch.cuda.synchronize()
            got = d_dst.cpu().numpy().view(np.uint32)[:, :w]
            assert np.array_equal(want, got), f"call {call}: {(want != got).sum()} pixels differ"
            # the frame's average colour, which the context turns into its next exposure: the same lanes
            # as the oracle's (whose exposure sequence the context's matches bit for bit)
            _, _, want_avg = oracle.postprocess(cfg, hdr, 1.0 / 60.0, mod, exposure)
            assert np.array_equal(d_avg.cpu().numpy()[:3], want_avg[:3]), (d_avg.cpu().numpy(), want_avg)
    finally:
        r.close()


def test_noalloc_rejects_oversized_frames(gpu_ok):
    import torch
    lib = gpu.load_library()
    cfg = abi.PostConfig.default()
    cmod = (ctypes.c_float * 3)(1.0, 1.0, 1.0)
    d = torch.zeros(16, dtype=torch.int64, device="cuda")
    max_width = 1920  # SW_NOALLOC_MAX_WIDTH; rejected before any device access
    rc = lib.sw_postprocess_noalloc(ctypes.c_void_p(d.data_ptr()), max_width + 1, 8, ctypes.byref(cfg), 1.0, cmod,
                                    ctypes.c_void_p(d.data_ptr()), max_width + 1, None, None)
    assert rc == abi.SW_ERR_LIMIT
    rc = lib.sw_postprocess_noalloc(None, 64, 64, ctypes.byref(cfg), 1.0, cmod, ctypes.c_void_p(d.data_ptr()), 64, None, None)
    assert rc == abi.SW_ERR_INVALID_ARGUMENT
