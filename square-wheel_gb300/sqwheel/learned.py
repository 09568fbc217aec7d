"""Learned 2x upscaler (libswgpu.so, include/swlearn.h): binding, training pairs rendered by the plain
GPU renderer, the training loop, evaluation against the non-learned upscales, and the
every-Nth-frame PSNR monitor with fallback to the plain path.

No counterpart in the reference: its FrameUpscaler (src/square_wheel/frame_upscaler.rs:42-239) has
only the nearest and 2x-averaging upscales this is compared with. Device frames are torch tensors
(device memory only; every operation on them runs in libswgpu.so).
"""
import ctypes
import os

import numpy as np

from . import abi
from .gpu import SwError, load_library

NUM_PARAMS = 22860
CROP_W, CROP_H, CROP_MARGIN, MAX_CROPS = 128, 64, 4, 32
PLAN_LEARNED, PLAN_LEARNED_CHECKED, PLAN_PLAIN = 0, 1, 2


class Crop(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_void_p), ("hi", ctypes.c_void_p), ("lo_width", ctypes.c_uint32),
                ("lo_height", ctypes.c_uint32), ("lo_pitch", ctypes.c_uint32), ("hi_pitch", ctypes.c_uint32),
                ("x", ctypes.c_int32), ("y", ctypes.c_int32)]


class Monitor(ctypes.Structure):
    """SwMonitor: every-Nth-frame PSNR check with fallback to the plain path (host logic, no GPU)."""
    _fields_ = [("check_interval", ctypes.c_uint32), ("fallback_frames", ctypes.c_uint32),
                ("threshold_db", ctypes.c_float), ("frames", ctypes.c_uint64), ("learned_frames", ctypes.c_uint64),
                ("checks", ctypes.c_uint64), ("failed_checks", ctypes.c_uint64), ("fallbacks", ctypes.c_uint64),
                ("plain_frames", ctypes.c_uint64), ("plain_left", ctypes.c_uint32), ("since_check", ctypes.c_uint32),
                ("check_pending", ctypes.c_uint32), ("recheck", ctypes.c_uint32), ("last_psnr_db", ctypes.c_float)]

    def __init__(self, check_interval=16, threshold_db=38.0, fallback_frames=32):
        super().__init__()
        self._lib = load_library()
        r = self._lib.sw_monitor_init(ctypes.byref(self), check_interval, threshold_db, fallback_frames)
        if r != 0:
            raise SwError(f"sw_monitor_init failed ({r})")

    def plan(self):
        p = ctypes.c_uint32()
        r = self._lib.sw_monitor_plan(ctypes.byref(self), ctypes.byref(p))
        if r != 0:
            raise SwError(f"sw_monitor_plan failed ({r})")
        return p.value

    def report(self, psnr_db):
        r = self._lib.sw_monitor_report(ctypes.byref(self), float(psnr_db))
        if r != 0:
            raise SwError(f"sw_monitor_report failed ({r})")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class Upscaler:
    """One network (weights, Adam state, workspaces) on one GPU."""

    def __init__(self, device=0, seed=1):
        self.lib = load_library()
        self.device = device
        self.h = ctypes.c_void_p()
        r = self.lib.sw_upscaler_create(device, seed, ctypes.byref(self.h))
        if r != 0:
            raise SwError(f"sw_upscaler_create failed ({r})")

    def _check(self, r, what):
        if r != 0:
            msg = self.lib.sw_upscaler_last_error(self.h)
            raise SwError(f"{what} failed ({r}): {msg.decode() if msg else ''}")

    def close(self):
        if self.h:
            self.lib.sw_upscaler_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.zeros(NUM_PARAMS, np.float32)
        self._check(self.lib.sw_upscaler_get_params(self.h, abi.ptr(p), NUM_PARAMS), "get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._check(self.lib.sw_upscaler_set_params(self.h, abi.ptr(p), p.size), "set_params")

    @staticmethod
    def crops(items):
        """items: (lo_tensor, hi_tensor, x, y) with (h, w) / (2h, 2w) int32 device tensors."""
        arr = (Crop * len(items))()
        for i, (lo, hi, x, y) in enumerate(items):
            arr[i] = Crop(lo.data_ptr(), hi.data_ptr(), lo.shape[1], lo.shape[0], lo.stride(0), hi.stride(0), x, y)
        return arr

    def gradients(self, items):
        arr = self.crops(items)
        g = np.zeros(NUM_PARAMS, np.float32)
        loss = ctypes.c_float()
        self._check(self.lib.sw_upscaler_gradients(self.h, arr, len(items), abi.ptr(g), ctypes.byref(loss)), "gradients")
        return g, loss.value

    def train_step(self, items, lr, want_mse=False):
        arr = self.crops(items)
        mse = ctypes.c_float()
        self._check(self.lib.sw_upscaler_train_step(self.h, arr, len(items), lr, ctypes.byref(mse) if want_mse else None),
                    "train_step")
        return mse.value if want_mse else None

    def steps(self):
        s = ctypes.c_uint64()
        self._check(self.lib.sw_upscaler_steps(self.h, ctypes.byref(s)), "steps")
        return s.value

    def infer(self, lo, hi, stream=0):
        """lo (h, w) and hi (2h, 2w) int32 device tensors."""
        self._check(self.lib.sw_upscaler_infer(self.h, _ptr(lo), lo.shape[1], lo.shape[0], lo.stride(0), _ptr(hi),
                                               hi.stride(0), ctypes.c_void_p(stream or None)), "infer")

    def set_fused(self, enable):
        self._check(self.lib.sw_upscaler_set_fused(self.h, 1 if enable else 0), "set_fused")

    def check(self):
        """Wait for the device; raises if a kernel gave up on a bounded wait."""
        self._check(self.lib.sw_upscaler_check(self.h), "check")

    def wait_probe(self, max_polls=1 << 14):
        """Runs the bounded-wait failure path on a barrier nothing completes; returns the recorded code."""
        code = ctypes.c_int()
        self._check(self.lib.sw_upscaler_wait_probe(self.h, max_polls, ctypes.byref(code)), "wait_probe")
        return code.value

    def psnr(self, a, b, stream=0):
        out = ctypes.c_double()
        self._check(self.lib.sw_upscaler_psnr(self.h, _ptr(a), a.stride(0), _ptr(b), b.stride(0), a.shape[1], a.shape[0],
                                              ctypes.c_void_p(stream or None), ctypes.byref(out)), "psnr")
        return out.value

    def save(self, path):
        self._check(self.lib.sw_upscaler_save(self.h, os.fsencode(path)), "save")

    def load(self, path):
        self._check(self.lib.sw_upscaler_load(self.h, os.fsencode(path)), "load")


class PairRenderer:
    """Renders the same camera pose at (w, h) and (2w, 2h) with the plain GPU path into device tensors.

    hdr=False: colour32 frames without postprocessing (the small-map configuration);
    hdr=True: colour64 + bloom + tonemap to colour32, exposure pinned to `exposure` for both sizes.
    """

    def __init__(self, scene, lo_size, device=0, hdr=False, exposure=1.0, directional=None):
        import torch
        from . import host
        self.torch = torch
        self.scene = scene
        self.lo_w, self.lo_h = lo_size
        self.hdr = hdr
        self.exposure = exposure
        self.device = device
        self.dev = torch.device(f"cuda:{device}")
        self.glib = load_library()
        fmt = abi.SW_PIXEL_C64 if hdr else abi.SW_PIXEL_C32
        directional = bool(scene.config.directional_lightmaps) if directional is None else directional
        self.opts_lo = host.frame_options(self.lo_w, self.lo_h, fmt, directional=directional)
        self.opts_hi = host.frame_options(2 * self.lo_w, 2 * self.lo_h, fmt, directional=directional)
        self.r_lo = host.HostRenderer(scene, device=device)
        self.r_hi = host.HostRenderer(scene, device=device)
        self.config = abi.PostConfig.default()
        self.mod = (ctypes.c_float * 3)(1.0, 1.0, 1.0)

    def num_frames(self):
        return self.scene.info().frames

    def stream_of(self, r):
        s = ctypes.c_void_p()
        self.glib.sw_get_stream(r.context(), ctypes.byref(s))
        return s.value or 0

    def _render(self, r, opts, index, out, pin_exposure):
        r.prepare_frame(index, opts)
        if not self.hdr:
            r.draw_frame(device_ptr=out.data_ptr(), pitch=out.stride(0))
            return
        r.draw_frame()
        ctx = r.context()
        if pin_exposure:
            self.glib.sw_set_exposure(ctx, self.exposure)
        rc = self.glib.sw_postprocess(ctx, ctypes.byref(self.config), 1.0 / 60.0, self.mod, _ptr(out), out.stride(0), 1)
        if rc != 0:
            raise SwError(f"sw_postprocess failed ({rc}): {self.glib.sw_last_error(ctx).decode()}")

    def render_lo(self, index, out, pin_exposure=True):
        self._render(self.r_lo, self.opts_lo, index, out, pin_exposure)

    def render_hi(self, index, out, pin_exposure=True):
        self._render(self.r_hi, self.opts_hi, index, out, pin_exposure)

    def render_pair(self, index, lo, hi, pin_exposure=True):
        self.render_lo(index, lo, pin_exposure)
        self.render_hi(index, hi, pin_exposure)

    def sync(self):
        for r in (self.r_lo, self.r_hi):
            rc = self.glib.sw_sync(r.context())
            if rc != 0:
                raise SwError(f"sw_sync failed ({rc}): {self.glib.sw_last_error(r.context()).decode()}")

    def close(self):
        self.r_lo.close()
        self.r_hi.close()


def train(ups, sources, steps, crops_per_step=8, lr=1e-3, pool=32, seed=0, log_every=0, log=None,
          checkpoint=None, checkpoint_every=0):
    """Adam training on crops of frame pairs rendered on the fly by the plain renderer.

    sources: list of PairRenderer (one per training map, same lo size). A pool of `pool` pairs is
    rendered first; every step then replaces one pair with a new random pose, so `steps` steps see
    `pool + steps` distinct pairs. Returns the list of (step, mse) logged."""
    torch = sources[0].torch
    rng = np.random.default_rng(seed)
    lo_w, lo_h = sources[0].lo_w, sources[0].lo_h
    dev = sources[0].dev
    lo = torch.zeros((pool, lo_h, lo_w), dtype=torch.int32, device=dev)
    hi = torch.zeros((pool, 2 * lo_h, 2 * lo_w), dtype=torch.int32, device=dev)

    def render(slot):
        src = sources[int(rng.integers(len(sources)))]
        src.render_pair(int(rng.integers(src.num_frames())), lo[slot], hi[slot])
        src.sync()

    for s in range(pool):
        render(s)
    history = []
    start = ups.steps()
    for step in range(steps):
        render(step % pool)
        items = []
        for _ in range(crops_per_step):
            k = int(rng.integers(pool))
            x = int(rng.integers(lo_w - CROP_W + 1))
            y = int(rng.integers(lo_h - CROP_H + 1))
            items.append((lo[k], hi[k], x, y))
        want = bool(log_every) and ((step + 1) % log_every == 0 or step + 1 == steps)
        mse = ups.train_step(items, lr, want_mse=want)
        if want:
            history.append((start + step + 1, mse))
            if log:
                log(start + step + 1, mse)
        if checkpoint and checkpoint_every and (step + 1) % checkpoint_every == 0:
            ups.save(checkpoint)
    return history


def evaluate(ups, src, frames, renderer_ctx=None):
    """Mean PSNR (dB) over `frames` of `src` for learned, 2x-average and nearest upscales of the
    half-resolution frame against the plain full-resolution frame."""
    torch = src.torch
    glib = load_library()
    lo = torch.zeros((src.lo_h, src.lo_w), dtype=torch.int32, device=src.dev)
    hi = torch.zeros((2 * src.lo_h, 2 * src.lo_w), dtype=torch.int32, device=src.dev)
    out = torch.zeros_like(hi)
    ctx = renderer_ctx or src.r_lo.context()
    res = {"learned": [], "avg2x": [], "nearest": []}
    for f in frames:
        src.render_pair(f, lo, hi)
        src.sync()
        ups.infer(lo, out)
        res["learned"].append(ups.psnr(out, hi))
        for name, mode in (("avg2x", abi.SW_UPSCALE_AVG2X), ("nearest", abi.SW_UPSCALE_NEAREST)):
            rc = glib.sw_upscale(ctx, mode, 2, _ptr(lo), 1, _ptr(out), out.shape[1], out.shape[0], out.stride(0), 1)
            if rc != 0:
                raise SwError(f"sw_upscale failed ({rc})")
            glib.sw_sync(ctx)
            res[name].append(ups.psnr(out, hi))
    return {k: float(np.mean(v)) for k, v in res.items()}, res
