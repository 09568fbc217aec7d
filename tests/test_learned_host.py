"""CPU checks of the learned upscaler's host side: the FP32 oracle's backward pass against finite
differences (which pins the oracle the GPU gradients are checked with), and the every-Nth-frame PSNR
monitor with fallback to the plain path (sw_monitor_*, pure host logic in libswgpu.so)."""
import numpy as np
import pytest

import upscaler_oracle as uo
from sqwheel import learned


def _frame(rng, h, w):
    a = rng.integers(0, 256, (h, w, 3)).astype(np.uint32)
    return (a[..., 0] | (a[..., 1] << 8) | (a[..., 2] << 16) | (np.uint32(255) << 24)).astype(np.uint32)


def _params(rng):
    p = np.zeros(uo.NUM_PARAMS)
    off = 0
    for ci, co in uo.LAYERS:
        nw = co * 9 * ci
        p[off:off + nw] = rng.normal(0, np.sqrt(2 / (9 * ci)), nw)
        p[off + nw:off + nw + co] = rng.normal(0, 0.05, co)
        off += nw + co
    return p


def test_param_count_matches_header():
    assert uo.NUM_PARAMS == learned.NUM_PARAMS == 22860


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    lo, hi = _frame(rng, 20, 24), _frame(rng, 40, 48)
    p = _params(rng)
    crops = [(lo, hi, 2, 3), (lo, hi, 6, 5)]
    g, loss = uo.gradients(p, crops, crop_w=16, crop_h=12, margin=2, exact=True)
    assert loss == pytest.approx(uo.loss(p, crops, 16, 12, 2), rel=1e-12)
    # every layer's weights and biases, including the first and the last parameter
    idx = list(rng.choice(uo.NUM_PARAMS, 16, replace=False)) + [0, 895, 896, 896 + 9247, 22859]
    for i in idx:
        e = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += e
        pm[i] -= e
        fd = (uo.loss(pp, crops, 16, 12, 2) - uo.loss(pm, crops, 16, 12, 2)) / (2 * e)
        assert abs(g[i] - fd) <= 2e-2 * abs(fd) + 2e-7, (i, g[i], fd)


def test_oracle_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 3.14159265, -2.5e-3, 0.0], np.float32)
    r = uo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # tie (1 + 2^-8) rounds to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] - 3.140625) < 1e-7
    assert r[5] == 0.0
    assert np.all(uo.bf16(r) == r)


def test_monitor_checks_every_nth_frame(built_libs):
    m = learned.Monitor(check_interval=4, threshold_db=38.0, fallback_frames=3)
    plans = []
    for _ in range(9):
        p = m.plan()
        plans.append(p)
        if p == learned.PLAN_LEARNED_CHECKED:
            m.report(40.0)
    C, L = learned.PLAN_LEARNED_CHECKED, learned.PLAN_LEARNED
    # first learned frame is checked, then every 4th
    assert plans == [C, L, L, L, C, L, L, L, C]
    assert m.checks == 3 and m.fallbacks == 0 and m.learned_frames == 9


def test_monitor_falls_back_and_rechecks(built_libs):
    m = learned.Monitor(check_interval=8, threshold_db=38.0, fallback_frames=3)
    assert m.plan() == learned.PLAN_LEARNED_CHECKED
    m.report(30.0)  # below threshold -> plain for 3 frames
    assert [m.plan() for _ in range(3)] == [learned.PLAN_PLAIN] * 3
    assert m.plan() == learned.PLAN_LEARNED_CHECKED  # first frame back is checked
    m.report(float("nan"))  # a NaN PSNR fails too
    assert m.plan() == learned.PLAN_PLAIN
    assert m.fallbacks == 2 and m.failed_checks == 2 and m.plain_frames == 4
    for _ in range(2):
        m.plan()
    assert m.plan() == learned.PLAN_LEARNED_CHECKED
    m.report(45.0)
    assert m.plan() == learned.PLAN_LEARNED
    assert m.last_psnr_db == pytest.approx(45.0)


def test_monitor_rejects_misuse(built_libs):
    with pytest.raises(Exception):
        learned.Monitor(check_interval=0)
    m = learned.Monitor(check_interval=2)
    with pytest.raises(Exception):
        m.report(40.0)  # nothing to report
    assert m.plan() == learned.PLAN_LEARNED_CHECKED
    with pytest.raises(Exception):
        m.plan()  # the checked frame's report is missing
