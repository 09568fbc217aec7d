"""GPU tests of the learned 2x upscaler (include/swlearn.h) against the CPU FP32 oracle
(oracle/upscaler_oracle.py):

  * gradients of the tcgen05 forward/backward kernels vs the oracle on the same bf16-rounded inputs;
  * inference vs the oracle on frames whose sizes are not multiples of the 128 x 4 tiles;
  * the learned mode of sw_upscale through a renderer context;
  * checkpoint save / load (hash and version checked);
  * training on frame pairs rendered by the plain renderer beats the non-learned upscales
    (2x average, nearest) on a map the network never saw;
  * a network forced to emit noise fails the PSNR check and the monitor falls back to the plain path.
"""
import ctypes
import os

import numpy as np
import pytest

import upscaler_oracle as uo
from sqwheel import abi, gpu, host, learned

pytestmark = pytest.mark.gpu


def _frame(rng, h, w, block=8):
    base = rng.integers(0, 256, (h // block + 1, w // block + 1, 3))
    a = np.repeat(np.repeat(base, block, 0), block, 1)[:h, :w] + rng.integers(-20, 21, (h, w, 3))
    a = np.clip(a, 0, 255).astype(np.uint32)
    alpha = rng.integers(0, 256, (h, w)).astype(np.uint32)
    return (a[..., 0] | (a[..., 1] << 8) | (a[..., 2] << 16) | (alpha << 24)).astype(np.uint32)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda:0")


def _lanes(a):
    return np.stack([(a >> s) & 255 for s in (0, 8, 16, 24)], -1).astype(np.int64)


@pytest.fixture(scope="module")
def ups(gpu_ok):
    u = learned.Upscaler(0, seed=5)
    yield u
    u.close()


def test_gradients_match_oracle(ups):
    rng = np.random.default_rng(11)
    lo, hi = _frame(rng, 96, 160), _frame(rng, 192, 320)
    # crops at the frame edge and inside; the oracle uses the same bf16 roundings
    spots = [(0, 0), (32, 32), (160 - 128, 96 - 64)]
    g, loss = ups.gradients([(_dev(lo), _dev(hi), x, y) for x, y in spots])
    go, loss_o = uo.gradients(ups.params(), [(lo, hi, x, y) for x, y in spots])
    assert loss == pytest.approx(loss_o, rel=1e-4)
    off = 0
    for l, (ci, co) in enumerate(uo.LAYERS):
        nw = co * 9 * ci
        for sl in (slice(off, off + nw), slice(off + nw, off + nw + co)):
            rel = np.linalg.norm(g[sl] - go[sl]) / np.linalg.norm(go[sl])
            assert rel < 1e-3, (l, rel)
        off += nw + co


@pytest.mark.parametrize("w,h", [(200, 130), (128, 4), (131, 67)])
def test_inference_matches_oracle(ups, w, h):
    import torch
    rng = np.random.default_rng(w * 1000 + h)
    lo = _frame(rng, h, w)
    out = torch.zeros((2 * h, 2 * w + 6), dtype=torch.int32, device="cuda:0")  # pitch != width
    ups.infer(_dev(lo), out[:, :2 * w])
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    ref = uo.infer(ups.params(), lo)
    d = np.abs(_lanes(got[:, :2 * w]) - _lanes(ref))
    # the only difference is f32 summation order inside the convolutions: a bf16 activation may round
    # the other way, which moves an output byte by at most 1
    assert d.max() <= 1
    assert (d == 0).mean() > 0.999
    assert np.all(got[:, 2 * w:] == 0)  # nothing written past the row


@pytest.mark.parametrize("w,h", [(960, 540), (250, 37), (121, 240), (120, 3)])
def test_fused_inference_equals_layered(ups, w, h):
    """The fused four-layer kernel gives the same bytes as one launch per layer (strip edges, segment
    edges, frame borders, widths that are not multiples of the 120-column strips)."""
    import torch
    rng = np.random.default_rng(w + 7 * h)
    lo = _dev(_frame(rng, h, w))
    a = torch.zeros((2 * h, 2 * w), dtype=torch.int32, device="cuda:0")
    b = torch.zeros_like(a)
    try:
        ups.set_fused(True)
        ups.infer(lo, a)
        ups.check()
        ups.set_fused(False)
        ups.infer(lo, b)
        ups.check()
    finally:
        ups.set_fused(True)
    torch.cuda.synchronize()
    assert torch.equal(a, b), int((a != b).sum())


def test_learned_mode_through_context(ups, gpu_ok):
    import torch
    scene = host.Scene(**host.SMALL_MAP)
    r = host.HostRenderer(scene)
    try:
        ctx = r.context()
        lib = gpu.load_library()
        rng = np.random.default_rng(2)
        lo = _dev(_frame(rng, 60, 80))
        a = torch.zeros((120, 160), dtype=torch.int32, device="cuda:0")
        b = torch.zeros_like(a)
        assert lib.sw_upscale(ctx, abi.SW_UPSCALE_LEARNED, 2, ctypes.c_void_p(lo.data_ptr()), 1,
                              ctypes.c_void_p(a.data_ptr()), 160, 120, 160, 1) != 0  # nothing attached
        assert lib.sw_set_learned_upscaler(ctx, ups.h) == 0
        assert lib.sw_upscale(ctx, abi.SW_UPSCALE_LEARNED, 2, ctypes.c_void_p(lo.data_ptr()), 1,
                              ctypes.c_void_p(a.data_ptr()), 160, 120, 160, 1) == 0
        # host buffers through the same entry point
        host_out = np.zeros((120, 160), np.uint32)
        src = lo.cpu().numpy().view(np.uint32).copy()
        assert lib.sw_upscale(ctx, abi.SW_UPSCALE_LEARNED, 2, abi.ptr(src), 0, abi.ptr(host_out), 160, 120, 160, 0) == 0
        lib.sw_sync(ctx)
        ups.infer(lo, b)
        torch.cuda.synchronize()
        assert torch.equal(a, b)
        assert np.array_equal(host_out, b.cpu().numpy().view(np.uint32))
        assert lib.sw_set_learned_upscaler(ctx, None) == 0
    finally:
        r.close()


def test_checkpoint_roundtrip(ups, tmp_path):
    p0 = ups.params()
    path = str(tmp_path / "ups.bin")
    ups.save(path)
    other = learned.Upscaler(0, seed=99)
    try:
        assert not np.array_equal(other.params(), p0)
        other.load(path)
        assert np.array_equal(other.params(), p0)
        assert other.steps() == ups.steps()
        data = bytearray(open(path, "rb").read())
        data[100] ^= 1
        bad = str(tmp_path / "bad.bin")
        open(bad, "wb").write(bytes(data))
        with pytest.raises(gpu.SwError, match="hash"):
            other.load(bad)
        open(bad, "wb").write(bytes(data[:-9]))
        with pytest.raises(gpu.SwError):
            other.load(bad)
        assert np.array_equal(other.params(), p0)  # a rejected file changes nothing
    finally:
        other.close()


@pytest.fixture(scope="module")
def trained(gpu_ok):
    """A network trained on three small maps the evaluation map is not among, plus the evaluation
    source (the small map's own camera path)."""
    u = learned.Upscaler(0, seed=7)
    srcs = [learned.PairRenderer(host.Scene(**dict(host.SMALL_MAP, seed=s, num_frames=1024)), (320, 240))
            for s in (11, 12, 13)]
    hist = learned.train(u, srcs, 400, crops_per_step=8, lr=1e-3, pool=16, seed=1, log_every=100)
    ev = learned.PairRenderer(host.Scene(**host.SMALL_MAP), (320, 240))
    yield u, ev, hist
    for s in srcs:
        s.close()
    ev.close()
    u.close()


def test_training_beats_non_learned_upscales(trained):
    u, ev, hist = trained
    assert u.steps() == 400
    assert all(np.isfinite(m) for _, m in hist)
    mean, per_frame = learned.evaluate(u, ev, range(0, 64, 4))
    # the learned upscale must beat both methods it replaces on the unseen map, on average and on
    # most frames
    assert mean["learned"] > mean["avg2x"] + 0.3, mean
    assert mean["learned"] > mean["nearest"] + 0.3, mean
    wins = np.mean(np.array(per_frame["learned"]) > np.array(per_frame["avg2x"]))
    assert wins >= 0.75, (wins, per_frame)


def test_noise_network_triggers_fallback(trained):
    import torch
    u, ev, _ = trained
    good = u.params()
    try:
        rng = np.random.default_rng(0)
        u.set_params(rng.normal(0, 1.0, learned.NUM_PARAMS).astype(np.float32))  # emits noise
        m = learned.Monitor(check_interval=4, threshold_db=38.0, fallback_frames=3)
        lo = torch.zeros((ev.lo_h, ev.lo_w), dtype=torch.int32, device="cuda:0")
        hi = torch.zeros((2 * ev.lo_h, 2 * ev.lo_w), dtype=torch.int32, device="cuda:0")
        out = torch.zeros_like(hi)
        plans = []
        for f in range(6):
            p = m.plan()
            plans.append(p)
            if p == learned.PLAN_PLAIN:
                ev.render_hi(f, hi)
                continue
            ev.render_lo(f, lo)
            ev.sync()
            u.infer(lo, out)
            if p == learned.PLAN_LEARNED_CHECKED:
                ev.render_hi(f, hi)
                ev.sync()
                m.report(u.psnr(out, hi))
        assert plans[0] == learned.PLAN_LEARNED_CHECKED
        assert plans[1:4] == [learned.PLAN_PLAIN] * 3
        assert plans[4] == learned.PLAN_LEARNED_CHECKED and plans[5] == learned.PLAN_PLAIN
        assert m.fallbacks == 2 and m.last_psnr_db < 38.0
    finally:
        u.set_params(good)


def test_psnr_kernel(ups):
    import torch
    rng = np.random.default_rng(4)
    a = _frame(rng, 33, 47)
    b = a.copy()
    assert ups.psnr(_dev(a), _dev(b)) == 99.0
    b ^= np.uint32(3)  # b channel off by up to 3, alpha ignored
    d = _lanes(a)[..., :3] - _lanes(b)[..., :3]
    want = 10 * np.log10(255.0 ** 2 / np.mean(d.astype(np.float64) ** 2))
    assert ups.psnr(_dev(a), _dev(b)) == pytest.approx(want, abs=1e-9)


def test_bounded_wait_runs_out_and_recovers(ups):
    """Failure detection without a fault: a kernel waits on an mbarrier that nothing completes (no copy
    or MMA in flight), gives up after a bounded number of polls, records its error code, frees its TMEM
    and returns; the host reads the code, and the upscaler keeps working (same bytes as before)."""
    import torch
    rng = np.random.default_rng(11)
    lo = _dev(_frame(rng, 64, 200))
    before = torch.zeros((128, 400), dtype=torch.int32, device="cuda:0")
    ups.infer(lo, before)
    ups.check()
    for polls in (1, 1 << 10, 1 << 14):
        assert ups.wait_probe(polls) == 5
    ups.check()  # the probe's record was cleared: no kernel failure is reported
    after = torch.zeros_like(before)
    ups.infer(lo, after)
    ups.check()
    torch.cuda.synchronize()
    assert torch.equal(before, after)
    with pytest.raises(gpu.SwError):
        ups.wait_probe(0)
