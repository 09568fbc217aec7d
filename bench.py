"""Benchmark of the GB300 Square-Wheel world-rendering path.

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload frame|surfaces|upscale|shadows] [--impl gpu|reference]
                [--learn-steps S]

Prints one JSON line (rank 0). A step is one pass of the hot path over one batch of synthetic input.

Workloads
  frame (default, the headline): one 1920x1080 HDR frame of the 64-room map (~32k polygons,
      directional lightmaps, 256x256 textures with mips and normal maps, 25% metal / 25% dielectric
      specular, 8 moving point lights): surface build -> tile raster -> bloom + tonemap + exposure.
      Frames walk the seeded 256-frame camera path. The host's per-frame work (visibility, surface
      preparation, draw setup) is done before the timed region; `value` is frames/s of device time
      (sum of the three stages' CUDA-event times on the library's stream, inputs resident in HBM);
      `e2e` is frames/s through the C ABI from host memory (host visibility + upload + GPU-side surface
      and draw preparation + GPU + 8.3 MB readback); `e2e.host_prepared` the same with the host
      preparing every surface and draw.
      The same frames are then rendered the learned way (960x540 + learned 2x upscale, network trained
      first for --learn-steps steps on two other maps) and reported under "learned" with their PSNR
      against the plain frames.
  surfaces: 4,096 surfaces, sides log-uniform 4..512 texels, mips 0..3, directional lightmaps,
      built in one launch; value in Mtexels/s.
  upscale: the learned 2x upscale alone (960x540 -> 1920x1080); value in frames/s, tensor roofline.
Timing: W >= 3 untimed warm-up steps, K timed steps, each preceded by an L2 flush (a 512 MiB write)
outside the timed span. Multi-GPU: independent replicas (different camera-path offsets), no collective;
value = sum over ranks of frames / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "square-wheel_gb300"))

import numpy as np  # noqa: E402

METRIC = "1080p frames/s: learned 2x upscale vs plain GPU (PSNR>=38 dB); Mtexels/s"
W, H = 1920, 1080


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(ms, world, device="cpu"):
    """The job's time over `world` replicas: the slowest rank's (every rank gets it)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_offset(rank):
    """Camera-path offset of a replica: every rank draws different frames of the same workload."""
    return rank * 11


def frame_indices(n, offset=0):
    """Frames spread over the 256-frame camera path."""
    return [(offset + i * 37) % 256 for i in range(n)]


# ---------------------------------------------------------------------------------------------------------
# frame workload

# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch of each stage's kernels at the
# frame workload, from one `ncu --set full` capture of this command (cold cache: ncu replays every kernel
# alone; the frame's writes are still in L2 when a kernel ends).
STAGE_TRAFFIC = {
    "post": None,
    "raster": None,
    "surf": None,
}


# Kernels one frame launches (either preparation split on the host side): surface build, raster setup,
# raster tiles, bloom blur, tonemap, exposure average.
FRAME_LAUNCHES = 6


def raster_bytes(pixel_writes, w, h):
    """Algorithmic bytes of the tile pass: every span pixel's texel read and frame write (colour64;
    the metric's frames blend nothing) and the bloom downscale's read of the frame, which its epilogue
    performs (the bloom + tonemap formula's first term)."""
    return pixel_writes * (8 + 8) + w * h * 8


def post_bytes(w, h, scale=2):
    """Algorithmic bytes of bloom + tonemap after the downscale: the two blur passes (bloom buffer read
    and written twice), the tonemap's HDR read and Color32 write, and its bloom read. With the
    downscale's W*H*8 in raster_bytes the two stages sum to the bloom + tonemap formula
    W*H*8 + 2*(W/S)(H/S)*8*2 + W*H*(8+4) + (W/S)(H/S)*8."""
    bw, bh = w // scale, h // scale
    return 2 * bw * bh * 8 * 2 + w * h * (8 + 4) + bw * bh * 8


class FrameWorkload:
    name = ("frame: 1920x1080 colour64 + bloom + tonemap, 64-room map (~32k polygons), directional lightmaps, "
            "256^2 textures + normal maps, 25% metal / 25% dielectric, 8 moving point lights")
    unit = "frames/s"

    def __init__(self, frames, offset=0):
        from sqwheel import abi, host
        self.abi = abi
        self.host = host
        self.scene = host.Scene(**host.FULL_MAP)
        self.static = self.scene.static_data()
        self.opts = host.frame_options(W, H, abi.SW_PIXEL_C64, directional=True)
        fr = host.Frame(self.scene)
        self.frames = []
        self.prep_ms = []
        for fi in frame_indices(frames, offset):
            t0 = time.perf_counter()
            fr.prepare(fi, self.opts)
            self.prep_ms.append((time.perf_counter() - t0) * 1e3)
            self.frames.append(dict(index=fi, surfaces=fr.surfaces, draws=fr.draws, vertices=fr.vertices,
                                    lights=fr.lights, params=fr.params, total_texels=fr.total_texels))
        self.config = abi.PostConfig.default()

    def lm_elements(self, f):
        s = f["surfaces"]
        sh = s["lightmap_tc_shift"].astype(np.int64)
        lg = s["lightmap_scale_log2"].astype(np.int64)
        lu = ((s["size"][:, 0] - 1 + sh[:, 0]) >> lg) + 2
        lv = ((s["size"][:, 1] - 1 + sh[:, 1]) >> lg) + 2
        return int((lu * lv).sum())

    def surface_bytes(self, f):
        return f["total_texels"] * (8 + 8) + self.lm_elements(f) * 40

    def half_resolution_frames(self):
        """Host work of the same camera poses at 960x540 (the learned path's render size)."""
        opts = self.host.frame_options(W // 2, H // 2, self.abi.SW_PIXEL_C64, directional=True)
        fr = self.host.Frame(self.scene)
        out = []
        for f in self.frames:
            fr.prepare(f["index"], opts)
            out.append(dict(index=f["index"], surfaces=fr.surfaces, draws=fr.draws, vertices=fr.vertices,
                            lights=fr.lights, params=fr.params, total_texels=fr.total_texels))
        return out


UPSCALER_FLOPS = 2 * (W // 2) * (H // 2) * 9 * (3 * 32 + 32 * 32 + 32 * 32 + 32 * 12)  # algorithmic, per frame
LEARN_MAPS = (21, 22)  # training maps: the full-size configuration with other seeds than the bench map


def run_learned(args, work, r, plain_ldr, local):
    """The learned form of the same frames: 960x540 render + bloom + tonemap, then the learned 2x
    upscale (tcgen05 kernels) to 1920x1080, PSNR against the plain full-resolution frames of the same
    steps. The network is trained first, on frame pairs the plain renderer draws from random poses of
    two other maps of the same configuration (the bench map is not among them)."""
    import torch
    from sqwheel import abi, host, learned
    t0 = time.perf_counter()
    ups = learned.Upscaler(local, seed=1)
    srcs = [learned.PairRenderer(host.Scene(**dict(host.FULL_MAP, seed=s, num_frames=1024)), (W // 2, H // 2),
                                 device=local, hdr=True) for s in LEARN_MAPS]
    learned.train(ups, srcs, args.learn_steps, crops_per_step=16, lr=1e-3, pool=24, seed=5)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    for src in srcs:
        src.close()
    lo_frames = work.half_resolution_frames()
    r.attach_upscaler(ups)
    r.set_exposure(1.0)
    stream = torch.cuda.ExternalStream(r.stream_handle())
    dev = f"cuda:{local}"
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    lo = torch.empty((H // 2, W // 2), dtype=torch.int32, device=dev)
    out = torch.empty((H, W), dtype=torch.int32, device=dev)
    tmp = torch.empty((H, W), dtype=torch.int32, device=dev)
    totals = {"frame_graph": 0.0, "upscale": 0.0}
    psnr = {"learned": [], "avg2x": [], "nearest": []}
    for step, f in enumerate(lo_frames):
        timed = step >= args.warmup
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        # the half-resolution frame as one CUDA graph (as the plain measurement), then the upscale
        r.draw_frame(r.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"], f["vertices"],
                                   post_config=work.config, dst_device_ptr=lo.data_ptr(), pitch=W // 2))
        r.upscale_device(abi.SW_UPSCALE_LEARNED, 2, lo.data_ptr(), out.data_ptr(), W, H, W)
        t = r.timings()
        if not timed:
            continue
        totals["frame_graph"] += t[4]
        totals["upscale"] += t[3]
        psnr["learned"].append(ups.psnr(out, plain_ldr[step], stream=r.stream_handle()))
        for name, mode in (("avg2x", abi.SW_UPSCALE_AVG2X), ("nearest", abi.SW_UPSCALE_NEAREST)):
            r.upscale_device(mode, 2, lo.data_ptr(), tmp.data_ptr(), W, H, W)
            psnr[name].append(ups.psnr(tmp, plain_ldr[step], stream=r.stream_handle()))
    r.attach_upscaler(None)
    ups.close()
    s = args.steps
    ms = sum(totals.values()) / s
    up_ms = totals["upscale"] / s
    return {
        "ms": ms, "upscale_ms": up_ms, "train_s": train_s,
        "stages_ms": {k: round(v / s, 4) for k, v in totals.items()},
        "psnr": psnr,
    }


LEARN_SMALL_MAPS = (11, 12, 13)  # training maps for the 8-room evaluation: other seeds of that configuration


def run_learned_small_map(args, local):
    """The learned path on the map configuration the learned-upscaler benchmark names (the 8-room map of
    the CPU-runnable configuration, its own camera path), at 1920x1080: plain frames (colour64 + bloom +
    tonemap as one CUDA graph) against half-resolution frames (the same graph at 960x540) + the learned
    upscale, each path in its own context (its own exposure sequence), L2 flushed before every frame.
    The network is trained first on frame pairs of three other 8-room maps."""
    import torch
    from sqwheel import abi, gpu, host, learned
    dev = f"cuda:{local}"
    t0 = time.perf_counter()
    ups = learned.Upscaler(local, seed=1)
    srcs = [learned.PairRenderer(host.Scene(**dict(host.SMALL_MAP, seed=s, num_frames=1024)), (W // 2, H // 2),
                                 device=local, hdr=True) for s in LEARN_SMALL_MAPS]
    learned.train(ups, srcs, args.learn_steps, crops_per_step=16, lr=1e-3, pool=24, seed=5)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    for src in srcs:
        src.close()
    scene = host.Scene(**host.SMALL_MAP)
    static = scene.static_data()
    cfg = abi.PostConfig.default()
    plain_r, learned_r = gpu.GpuRenderer(static, device=local), gpu.GpuRenderer(static, device=local)
    for x in (plain_r, learned_r):
        x.enable_timing(True)
    learned_r.attach_upscaler(ups)
    fr = host.Frame(scene)
    hi_opts = host.frame_options(W, H, abi.SW_PIXEL_C64, directional=False)
    lo_opts = host.frame_options(W // 2, H // 2, abi.SW_PIXEL_C64, directional=False)
    plain = torch.empty((H, W), dtype=torch.int32, device=dev)
    lo = torch.empty((H // 2, W // 2), dtype=torch.int32, device=dev)
    out = torch.empty((H, W), dtype=torch.int32, device=dev)
    tmp = torch.empty((H, W), dtype=torch.int32, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    frames = list(range(0, 64, 3))
    warm = 3
    plain_ms, learned_ms = [], []
    psnr = {"learned": [], "avg2x": [], "nearest": []}

    def frame_in(x, opts, fi, dst, pitch):
        fr.prepare(fi, opts)
        return x.frame_input(fr.params, fr.lights, fr.surfaces, fr.total_texels, fr.draws, fr.vertices, post_config=cfg,
                             dst_device_ptr=dst, pitch=pitch)

    for step, fi in enumerate(frames):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        plain_r.draw_frame(frame_in(plain_r, hi_opts, fi, plain.data_ptr(), W))
        tp = plain_r.timings()[4]
        flush.fill_(1.0)
        torch.cuda.synchronize()
        learned_r.draw_frame(frame_in(learned_r, lo_opts, fi, lo.data_ptr(), W // 2))
        learned_r.upscale_device(abi.SW_UPSCALE_LEARNED, 2, lo.data_ptr(), out.data_ptr(), W, H, W)
        t = learned_r.timings()
        torch.cuda.synchronize()
        if step < warm:
            continue
        plain_ms.append(tp)
        learned_ms.append(t[4] + t[3])
        psnr["learned"].append(ups.psnr(out, plain))
        for name, mode in (("avg2x", abi.SW_UPSCALE_AVG2X), ("nearest", abi.SW_UPSCALE_NEAREST)):
            learned_r.upscale_device(mode, 2, lo.data_ptr(), tmp.data_ptr(), W, H, W)
            torch.cuda.synchronize()
            psnr[name].append(ups.psnr(tmp, plain))
    learned_r.attach_upscaler(None)
    plain_r.close()
    learned_r.close()
    ups.close()
    pm, lm = statistics.mean(plain_ms), statistics.mean(learned_ms)
    n = len(psnr["learned"])
    return {
        "map": "8-room map of the CPU-runnable configuration (its own 64-frame camera path, every 3rd frame), "
               "1920x1080, colour64 + bloom + tonemap",
        "plain_frames_per_s": round(1e3 / pm, 2), "learned_frames_per_s": round(1e3 / lm, 2),
        "speedup_vs_plain": round(pm / lm, 3),
        "psnr_db": {"learned_mean": round(float(np.mean(psnr["learned"])), 3),
                    "learned_min": round(float(np.min(psnr["learned"])), 3),
                    "avg2x_mean": round(float(np.mean(psnr["avg2x"])), 3),
                    "nearest_mean": round(float(np.mean(psnr["nearest"])), 3),
                    "frames_at_or_above_38db": f"{sum(x >= 38.0 for x in psnr['learned'])}/{n}"},
        "train": {"steps": args.learn_steps, "crops_per_step": 16, "maps": f"8-room configuration, seeds {list(LEARN_SMALL_MAPS)}",
                  "seconds": round(train_s, 2)},
    }


def run_frame_gpu(args, world, rank, local):
    import torch
    from sqwheel import abi, gpu
    torch.cuda.set_device(local)
    nsteps = args.warmup + args.steps
    work = FrameWorkload(nsteps, offset=replica_offset(rank))
    r = gpu.GpuRenderer(work.static, device=local)
    r.enable_timing(True)
    stream = torch.cuda.ExternalStream(r.stream_handle())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    ldr_frames = torch.empty((len(work.frames), H, W), dtype=torch.int32, device=f"cuda:{local}")
    totals = {"surf": 0.0, "raster": 0.0, "post": 0.0}
    frame_span = 0.0
    texels = 0
    surf_bytes = 0
    pix_before = r.stats().pixel_writes
    pix_writes = 0
    launches = 0

    def frame_input(step, f):
        return r.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"], f["vertices"],
                             post_config=work.config, dst_device_ptr=ldr_frames[step].data_ptr(), pitch=W)

    # autotuner: tile shape of the tile pass and surface-build grid, on the first frame
    if args.autotune_reps > 0:
        tune, tune_ms = r.autotune(frame_input(0, work.frames[0]), reps=args.autotune_reps)
    else:
        tune, tune_ms = r.tuning(), 0.0
    r.set_exposure(1.0)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        # pass 1: the frame's kernels launched directly (the graph's launch sequence without the graph)
        # with CUDA events between the stages on the library's stream: the per-stage rooflines
        r.set_frame_graph(False)
        for step, f in enumerate(work.frames):
            timed = step >= args.warmup
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            r.draw_frame(frame_input(step, f))
            t = r.timings()
            if timed:
                totals["surf"] += t[0]
                totals["raster"] += t[1]
                totals["post"] += t[2]
                frame_span += t[4]
                texels += f["total_texels"]
                surf_bytes += work.surface_bytes(f)
                launches += FRAME_LAUNCHES
            if step == args.warmup - 1:
                pix_before = r.stats().pixel_writes
        pix_writes = r.stats().pixel_writes - pix_before
        r.set_frame_graph(True)
        # pass 2 (the measurement): the same frames through sw_draw_frame, one CUDA graph per frame;
        # device time of the whole graph (uploads, surfaces, raster setup + tiles, postprocess, readback)
        r.set_exposure(1.0)
        graph_ms = []
        for step, f in enumerate(work.frames):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            r.draw_frame(frame_input(step, f))
            t = r.timings()
            if step >= args.warmup:
                graph_ms.append(t[4])
                launches += FRAME_LAUNCHES
        torch.cuda.synchronize()
    gpu_ldr = ldr_frames[:4].cpu().numpy().view(np.uint32).copy()  # for the parity check against the oracle
    stage_sum_ms = (totals["surf"] + totals["raster"] + totals["post"]) / args.steps
    frame_ms = max_over_ranks(statistics.mean(graph_ms), world, f"cuda:{local}")
    value = world * 1e3 / frame_ms

    # e2e: the C++ host renderer drives the C ABI per frame (swh_renderer_render_frame: the host's
    # visibility, light positioning and leaf order, then one graph with the upload from host memory,
    # GPU-side surface and draw preparation, surfaces, raster and postprocess) and the Color32 frame
    # lands in a host buffer the caller registered once. The same loop with the host preparing every
    # surface and draw (the reference's split) is reported beside it.
    from sqwheel import abi, host
    import ctypes

    def e2e_run(gpu_prep, in_flight):
        """Frames/s of swh_renderer_render_frame over the frames in order (every frame's host work, upload,
        GPU work and Color32 frame in host memory): one frame at a time (the median frame), or with two
        frames in flight (the whole sequence, including the last frame's copy-out)."""
        hr = host.HostRenderer(work.scene, device=local)
        hr.set_gpu_prep(gpu_prep)
        hr.set_frames_in_flight(in_flight)
        glib = gpu.load_library()
        glib.sw_set_tuning(hr.context(), ctypes.byref(tune))
        outs = [np.zeros((H, W), np.uint32) for _ in range(in_flight)]
        for o in outs:
            hr.register_host_buffer(o)
        frames = work.frames[: max(4, min(args.steps, 12))]
        for k, f in enumerate(frames):  # warm-up pass: buffers at their capacities, the frame graphs captured
            hr.render_frame(f["index"], work.opts, out=outs[k % in_flight], post=work.config)
        hr.sync()
        s0 = abi.Stats()
        glib.sw_get_stats(hr.context(), ctypes.byref(s0))
        times = []
        t_all = time.perf_counter()
        for k, f in enumerate(frames):
            t0 = time.perf_counter()
            hr.render_frame(f["index"], work.opts, out=outs[k % in_flight], post=work.config)
            times.append((time.perf_counter() - t0) * 1e3)
        hr.sync()
        total_ms = (time.perf_counter() - t_all) * 1e3
        s1 = abi.Stats()
        glib.sw_get_stats(hr.context(), ctypes.byref(s1))
        for o in outs:
            hr.unregister_host_buffer(o)
        hr.close()
        value = 1e3 / statistics.median(times[1:]) if in_flight == 1 else 1e3 * len(frames) / total_ms
        return value, (s1.upload_bytes - s0.upload_bytes) / len(frames), outs[0].nbytes

    e2e_serial, h2d_step, d2h_step = e2e_run(True, 1)
    e2e_val, _, _ = e2e_run(True, 2)
    e2e_host_val, h2d_host_step, _ = e2e_run(False, 2)

    lr = run_learned(args, work, r, ldr_frames, local) if args.learn_steps > 0 else None
    if lr is not None:
        launches += args.steps * (FRAME_LAUNCHES + 1)  # half-resolution frame + the fused upscale kernel
    lr_small = run_learned_small_map(args, local) if args.learn_steps > 0 else None

    peak, peak_kind = peaks()
    s = args.steps
    stage_bytes = {
        "surf": surf_bytes / s,
        "raster": raster_bytes(pix_writes / s, W, H),
        "post": post_bytes(W, H),
    }
    stages = {}
    for k, ms in totals.items():
        ms_per = ms / s
        gbs = stage_bytes[k] / (ms_per / 1e3) / 1e9 if ms_per > 0 else 0.0
        stages[k] = {"ms": round(ms_per, 4), "algorithmic_bytes": int(stage_bytes[k]), "GB/s": round(gbs, 1),
                     "frac_of_measured_hbm": round(gbs / peak, 4)}
    dom = max(totals, key=totals.get)
    kernel_names = {"surf": "surf_build_kernel", "raster": "raster_tiles_kernel (bloom downscale in its epilogue)",
                    "post": "pp_blur_kernel + pp_tonemap_bloom_kernel (+ pp_average_bloom_kernel beside it)"}
    out_line = None
    if rank == 0:
        cpu, parity = cpu_frame_baseline(work, gpu_ldr=gpu_ldr)
        out_line = {
            "metric": METRIC, "value": round(value, 2), "unit": "frames/s", "n_gpus": world, "steps": s,
            "warmup": args.warmup, "ms_per_step": round(frame_ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (lighting) / int (raster)", "data": "synthetic (seeded scene generator)",
            "config": {"workload": work.name, "width": W, "height": H, "pixel_format": "C64",
                       "frames": [f["index"] for f in work.frames[args.warmup:]],
                       "mean_surface_texels": int(texels / s), "mtexels_per_s": round(texels / totals["surf"] / 1e3, 1),
                       "mean_pixel_writes": int(pix_writes / s),
                       "mean_host_prep_ms": round(statistics.mean(work.prep_ms), 3),
                       "l2": "flushed (512 MiB write) before every timed step",
                       "timing": "CUDA-event device time of the frame's CUDA graph (sw_draw_frame: uploads, surface "
                                 "build, raster setup + tiles, bloom + tonemap, exposure readback)",
                       "stage_kernel_sum_ms": round(stage_sum_ms, 4),
                       "per_call_api_frame_span_ms": round(frame_span / s, 4),
                       "tuning": {"raster_tile": int(tune.raster_tile), "surface_blocks_per_sm": int(tune.surface_blocks_per_sm),
                                  "surface_texels_per_thread": int(tune.surface_texels_per_thread),
                                  "autotune_best_ms": round(tune_ms, 4)},
                       "parallelism": f"replicas x{world}"},
            "stages": stages,
            "roofline": {"bound": "hbm", "kernel": kernel_names[dom], "achieved": stages[dom]["GB/s"], "peak": peak,
                         "unit": "GB/s", "frac": stages[dom]["frac_of_measured_hbm"],
                         "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_launch": stages[dom]["algorithmic_bytes"],
                         "traffic": STAGE_TRAFFIC.get(dom)},
            "cpu_baseline": cpu,
            "parity": parity,
            "e2e": {"value": round(e2e_val, 2), "unit": "frames/s", "h2d_bytes_per_step": int(h2d_step),
                    "d2h_bytes_per_step": int(d2h_step),
                    "path": "render_frame: host visibility + GPU-side surface and draw preparation, two frames in "
                            "flight (each frame's copy into a registered host buffer overlaps the next frame)",
                    "one_frame_at_a_time": round(e2e_serial, 2),
                    "host_prepared": {"value": round(e2e_host_val, 2), "unit": "frames/s",
                                      "h2d_bytes_per_step": int(h2d_host_step),
                                      "path": "render_frame with the host preparing every surface and draw, two frames "
                                              "in flight"}},
            "clocks": clocks.summary(),
            "gpu_launches": launches,
        }
        if lr is not None:
            out_line["learned"] = learned_summary(lr, frame_ms, args)
        if lr_small is not None:
            out_line["learned_8_room_map"] = lr_small
        print(json.dumps(out_line), flush=True)
    r.close()
    return out_line


def learned_summary(lr, plain_ms, args):
    p = lr["psnr"]
    tf = UPSCALER_FLOPS / (lr["upscale_ms"] / 1e3) / 1e12
    peak = None
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        peak = float(json.load(open(pp)).get("bf16_tflops", 0)) or None
    kind = "measured bf16_tflops (burst)"
    if peak is None:
        peak, kind = 1900.0, "fallback"
    n = len(p["learned"])
    mon = monitored_sequence(p["learned"], lr["ms"], plain_ms)
    return {
        "what": "960x540 frame (CUDA graph: surfaces, raster, bloom + tonemap) + learned 2x upscale to 1920x1080 "
                "(BF16 tcgen05, FP32 accumulate), same frames as the plain measurement",
        "frames_per_s": round(1e3 / lr["ms"], 2), "ms_per_frame": round(lr["ms"], 4),
        "speedup_vs_plain": round(plain_ms / lr["ms"], 3),
        "with_quality_monitor": mon,
        "stages_ms": lr["stages_ms"],
        "psnr_db": {"learned_mean": round(float(np.mean(p["learned"])), 3),
                    "learned_min": round(float(np.min(p["learned"])), 3),
                    "avg2x_mean": round(float(np.mean(p["avg2x"])), 3),
                    "nearest_mean": round(float(np.mean(p["nearest"])), 3),
                    "frames_at_or_above_38db": f"{sum(x >= 38.0 for x in p['learned'])}/{n}"},
        "upscaler_roofline": {"bound": "tensor", "kernel": "fused_upscale_kernel (one launch, four layers)",
                              "achieved": round(tf, 1), "peak": peak, "unit": "TFLOP/s", "frac": round(tf / peak, 4),
                              "peak_source": kind, "algorithmic_flops_per_launch": UPSCALER_FLOPS},
        "train": {"steps": args.learn_steps, "crops_per_step": 16, "crop": "128x64 half-resolution pixels",
                  "maps": f"full-size configuration, seeds {list(LEARN_MAPS)} (bench map: seed 2)",
                  "seconds": round(lr["train_s"], 2)},
    }


def monitored_sequence(psnr_db, learned_ms, plain_ms, check_interval=16, threshold_db=38.0, fallback_frames=32):
    """What the renderer delivers with the learned path's quality monitor (sw_monitor_*: every 16th
    learned frame also renders the plain frame and checks the PSNR; a check under 38 dB switches to the
    plain path for 32 frames) over the measured frames in their order, each frame's PSNR the one
    measured for it. A learned frame costs the learned path's mean time, a checked one that plus a
    plain frame, a fallback frame the plain path's: frames/s counts only frames actually delivered."""
    from sqwheel import learned
    m = learned.Monitor(check_interval=check_interval, threshold_db=threshold_db, fallback_frames=fallback_frames)
    total = 0.0
    kinds = {"learned": 0, "learned_checked": 0, "plain_fallback": 0}
    for db in psnr_db:
        plan = m.plan()
        if plan == 2:
            total += plain_ms
            kinds["plain_fallback"] += 1
        elif plan == 1:
            total += learned_ms + plain_ms
            kinds["learned_checked"] += 1
            m.report(db)
        else:
            total += learned_ms
            kinds["learned"] += 1
    n = len(psnr_db)
    return {"frames_per_s": round(1e3 * n / total, 2), "speedup_vs_plain": round(plain_ms * n / total, 3),
            "frames": kinds, "failed_checks": int(m.failed_checks),
            "monitor": f"check every {check_interval}th learned frame at {threshold_db} dB, {fallback_frames} plain "
                       f"frames after a failed check"}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def cpu_frame_baseline(work, max_frames=4, gpu_ldr=None):
    """The oracle (C++ restatement of the reference CPU renderer) on the machine's host cores: the same host
    work, surfaces with one task per surface, split_rect rasterisation with one region per thread, and
    the postprocessor single-threaded (the reference's default, use_multithreading = false). Host
    preparation and the oracle's rendering are timed separately.

    gpu_ldr (optional): the GPU's tonemapped frames of the same first frames, exposure sequence started
    at 1.0. They are compared with the oracle's frames of the reference's num_threads == 1 raster path
    (one whole-screen clip rect, partial_renderer.rs:1207-1234: split_rect regions clip spans and move
    texel addresses, so the timed multithreaded raster is not the parity reference); the frame buffer
    carries over from frame to frame as the reference's does. Returns (baseline, parity or None)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    host = work.host
    fr = host.Frame(work.scene)
    ts, prep_ts = [], []
    frames = [f["index"] for f in work.frames[:max_frames]]
    exposure = 1.0
    arenas = []
    for fi in frames:
        t0 = time.perf_counter()
        fr.prepare(fi, work.opts)
        t1 = time.perf_counter()
        arena = oracle.build_surfaces(work.static, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=threads)
        fb = np.zeros((H, W), np.uint64)
        oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, fb, num_threads=threads)
        _, exposure, _ = oracle.postprocess(work.config, fb, 1.0 / 60.0, (1.0, 1.0, 1.0), exposure)
        t2 = time.perf_counter()
        ts.append(t2 - t0)
        prep_ts.append(t1 - t0)
        if gpu_ldr is not None:
            arenas.append((fi, arena))
    v = len(ts) / sum(ts)
    base = {"value": round(v, 3), "unit": "frames/s", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
            "host_prep_ms": round(1e3 * statistics.mean(prep_ts), 3),
            "oracle_ms": round(1e3 * (sum(ts) - sum(prep_ts)) / len(ts), 3),
            "sample": f"{len(frames)} frames {frames} of the same workload; host work + oracle surfaces ({threads} threads) + "
                      f"split_rect raster ({threads} regions) + single-thread postprocess"}
    if gpu_ldr is None:
        return base, None
    mismatched, exposure = 0, 1.0
    fb = np.zeros((H, W), np.uint64)
    for k, (fi, arena) in enumerate(arenas):
        fr.prepare(fi, work.opts)
        oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, fb, num_threads=1)
        ldr, exposure, _ = oracle.postprocess(work.config, fb, 1.0 / 60.0, (1.0, 1.0, 1.0), exposure)
        mismatched += int((ldr != gpu_ldr[k]).sum())
    parity = {"frames": len(arenas), "mismatched_pixels": mismatched,
              "what": "tonemapped 1920x1080 frames of the measured graph pass (the first frames of its sequence) vs "
                      "the oracle (surfaces, num_threads == 1 raster, bloom + tonemap, exposure carried over)"}
    return base, parity


# ---------------------------------------------------------------------------------------------------------
# models workload: the frame with triangle models (the stress configuration's animated models)

def run_models_gpu(args, world, rank, local):
    """value: frames/s of device time of the 1920x1080 colour64 + bloom + tonemap frame of the 64-room map
    with 200 per-vertex animated triangle models (about 2k triangles, 8 keyframes each) drawn after their
    leaf's polygons (host-prepared draw list, one CUDA graph per frame, L2 flushed before each);
    e2e: the same frames through swh_renderer_render_frame with two frames in flight."""
    import ctypes
    import torch
    from sqwheel import abi, gpu, host
    torch.cuda.set_device(local)
    scene = host.Scene(**host.MODEL_MAP)
    static = scene.static_data()
    lite = scene.lite_textures()
    opts = host.frame_options(W, H, abi.SW_PIXEL_C64, directional=True)
    cfg = abi.PostConfig.default()
    fr = host.Frame(scene)
    frames, prep_ms = [], []
    for fi in frame_indices(args.warmup + args.steps, replica_offset(rank)):
        t0 = time.perf_counter()
        fr.prepare(fi, opts)
        prep_ms.append((time.perf_counter() - t0) * 1e3)
        frames.append(dict(index=fi, surfaces=fr.surfaces, draws=fr.draws, vertices=fr.vertices, tri=fr.tri_vertices,
                           lights=fr.lights, params=fr.params, total_texels=fr.total_texels, tris=fr.model_triangles))
    r = gpu.GpuRenderer(static, device=local)
    r.set_lite_textures(lite)
    r.enable_timing(True)
    stream = torch.cuda.ExternalStream(r.stream_handle())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    ldr = torch.empty((H, W), dtype=torch.int32, device=f"cuda:{local}")

    def fin(f):
        return r.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"], f["vertices"],
                             post_config=cfg, dst_device_ptr=ldr.data_ptr(), pitch=W, tri_vertices=f["tri"])

    stage = {"surf": 0.0, "raster": 0.0, "post": 0.0}
    graph_ms = []
    with ClockSampler(local) as clocks:
        r.set_frame_graph(False)
        for step, f in enumerate(frames):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            r.draw_frame(fin(f))
            t = r.timings()
            if step >= args.warmup:
                stage["surf"] += t[0]
                stage["raster"] += t[1]
                stage["post"] += t[2]
        r.set_frame_graph(True)
        r.set_exposure(1.0)
        pix0 = r.stats().pixel_writes
        for step, f in enumerate(frames):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            if step == args.warmup:
                pix0 = r.stats().pixel_writes
            r.draw_frame(fin(f))
            t = r.timings()
            if step >= args.warmup:
                graph_ms.append(t[4])
        torch.cuda.synchronize()
        pix = (r.stats().pixel_writes - pix0) / args.steps
    ms = max_over_ranks(statistics.mean(graph_ms), world, f"cuda:{local}")
    s = args.steps
    tris = statistics.mean(f["tris"] for f in frames[args.warmup:])
    # e2e: host work (models included) + one graph per frame, two frames in flight
    hr = host.HostRenderer(scene, device=local)
    hr.set_frames_in_flight(2)
    glib = gpu.load_library()
    outs = [np.zeros((H, W), np.uint32) for _ in range(2)]
    for o in outs:
        hr.register_host_buffer(o)
    efr = frames[: max(4, min(s, 12))]
    for k, f in enumerate(efr):
        hr.render_frame(f["index"], opts, out=outs[k % 2], post=cfg)
    hr.sync()
    s0 = abi.Stats()
    glib.sw_get_stats(hr.context(), ctypes.byref(s0))
    t0 = time.perf_counter()
    for k, f in enumerate(efr):
        hr.render_frame(f["index"], opts, out=outs[k % 2], post=cfg)
    hr.sync()
    e2e = len(efr) / (time.perf_counter() - t0)
    s1 = abi.Stats()
    glib.sw_get_stats(hr.context(), ctypes.byref(s1))
    for o in outs:
        hr.unregister_host_buffer(o)
    hr.close()
    peak, peak_kind = peaks()
    raster_ms = stage["raster"] / s
    rbytes = raster_bytes(pix, W, H)
    gbs = rbytes / (raster_ms / 1e3) / 1e9
    if rank == 0:
        # CPU: host work + the oracle's surfaces, split_rect raster (polygons and triangles) and
        # postprocess on a bounded sample; parity: the first frames against the oracle's single-thread raster
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        threads = os.cpu_count() or 1
        sample = frames[:3]
        t0 = time.perf_counter()
        exposure = 1.0
        for f in sample:
            fr.prepare(f["index"], opts)
            arena = oracle.build_surfaces(static, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=threads)
            fb = np.zeros((H, W), np.uint64)
            oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, fb, num_threads=threads, tri_vertices=fr.tri_vertices,
                             lite=lite)
            _, exposure, _ = oracle.postprocess(cfg, fb, 1.0 / 60.0, (1.0, 1.0, 1.0), exposure)
        cpu_v = len(sample) / (time.perf_counter() - t0)
        # parity of one frame through the graph path (fresh context, exposure 1.0)
        r2 = gpu.GpuRenderer(static, device=local)
        r2.set_lite_textures(lite)
        f = frames[0]
        got = np.zeros((H, W), np.uint32)
        r2.draw_frame(r2.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"], f["vertices"],
                                     post_config=cfg, dst=got, tri_vertices=f["tri"]))
        r2.close()
        arena = oracle.build_surfaces(static, f["surfaces"], f["lights"], f["params"], f["total_texels"], num_threads=threads)
        fb = np.zeros((H, W), np.uint64)
        oracle.rasterize(f["draws"], f["vertices"], arena, f["params"], fb, tri_vertices=f["tri"], lite=lite)
        want, _, _ = oracle.postprocess(cfg, fb, 1.0 / 60.0, (1.0, 1.0, 1.0), 1.0)
        print(json.dumps({
            "metric": METRIC, "value": round(world * 1e3 / ms, 2), "unit": "frames/s", "n_gpus": world, "steps": s,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (lighting) / int (raster)", "data": "synthetic (seeded scene generator)",
            "config": {"workload": "models: the 1920x1080 colour64 + bloom + tonemap frame of the 64-room map with 200 "
                                   "per-vertex animated triangle models (about 2k triangles, 8 keyframes each)",
                       "mean_model_triangle_draws": int(tris), "mean_pixel_writes": int(pix),
                       "mean_host_prep_ms": round(statistics.mean(prep_ms), 3),
                       "timing": "CUDA-event device time of the frame's CUDA graph (host-prepared draw list)",
                       "l2": "flushed (512 MiB write) before every timed step", "parallelism": f"replicas x{world}"},
            "stages_ms": {k: round(v / s, 4) for k, v in stage.items()},
            "roofline": {"bound": "hbm", "kernel": "raster_tiles_kernel (polygons and triangles, bloom downscale epilogue)",
                         "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4),
                         "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_launch": int(rbytes), "traffic": None},
            "parity": {"frames": 1, "mismatched_pixels": int((want != got).sum())},
            "cpu_baseline": {"value": round(cpu_v, 3), "unit": "frames/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": f"{len(sample)} frames: host work + oracle surfaces, split_rect raster with the "
                                       f"triangles, postprocess"},
            "e2e": {"value": round(e2e, 2), "unit": "frames/s", "h2d_bytes_per_step": int((s1.upload_bytes - s0.upload_bytes) / len(efr)),
                    "d2h_bytes_per_step": int(outs[0].nbytes), "path": "render_frame (host models + host-prepared draws), "
                                                                       "two frames in flight"},
            "clocks": clocks.summary(), "gpu_launches": s * FRAME_LAUNCHES}), flush=True)
    r.close()


STRESS_TRAIN_MAPS = (31, 32)  # training maps for the stress evaluation: its configuration, other seeds, no portals


def run_stress_gpu(args, world, rank, local):
    """The stress configuration: frames of the 128-room map (portals and mirrors two levels deep,
    translucent, alpha-blended and alpha-tested surfaces, 2k decals, sprites, 200 animated models, all lit
    from a seeded light grid) delivered at 3840x2160 colour32 after bloom + tonemap.
    value: frames/s the renderer delivers at 3840x2160 on the learned path under its quality monitor
    (the 1920x1080 frame, learned 2x upscale; every 16th frame checked against the plain 3840x2160 frame
    at 38 dB, 32 plain frames after a failed check), from the device time of each frame's CUDA graph (+
    the upscale); plain: the 3840x2160 frames alone. e2e: the same through swh_renderer_render_frame with
    the host work (visibility, portals, models) and the copy of each delivered frame to pinned host memory."""
    import ctypes
    import torch
    from sqwheel import abi, gpu, host, learned
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    SW, SH = 2 * W, 2 * H
    t0 = time.perf_counter()
    ups = learned.Upscaler(local, seed=1)
    srcs = [learned.PairRenderer(host.Scene(**dict(host.STRESS_MAP, seed=sd, num_portals=0, num_frames=1024)), (W, H),
                                 device=local, hdr=True) for sd in STRESS_TRAIN_MAPS]
    learned.train(ups, srcs, args.learn_steps, crops_per_step=16, lr=1e-3, pool=24, seed=5)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    for src in srcs:
        src.close()
    scene = host.Scene(**host.STRESS_MAP)
    cfg = abi.PostConfig.default()
    glib = gpu.load_library()
    hr = host.HostRenderer(scene, device=local)
    ctx = hr.context()
    assert glib.sw_enable_timing(ctx, 1) == 0
    assert glib.sw_set_learned_upscaler(ctx, ups.h) == 0
    stream = torch.cuda.ExternalStream(hr_stream(glib, ctx))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    full = torch.empty((SH, SW), dtype=torch.int32, device=dev)
    half = torch.empty((H, W), dtype=torch.int32, device=dev)
    up = torch.empty((SH, SW), dtype=torch.int32, device=dev)
    opts_hi = host.frame_options(SW, SH, abi.SW_PIXEL_C64, directional=True)
    opts_lo = host.frame_options(W, H, abi.SW_PIXEL_C64, directional=True)
    t5 = (ctypes.c_float * 5)()

    def timings():
        assert glib.sw_get_timings(ctx, t5) == 0
        return list(t5)

    def render(fi, opts, dst, pitch):
        # exposure pinned to 1.0 so that the plain and the learned frame of a pose are comparable
        assert glib.sw_set_exposure(ctx, ctypes.c_float(1.0)) == 0
        hr.render_frame(fi, opts, device_ptr=dst.data_ptr(), pitch=pitch, post=cfg)

    def upscale():
        assert glib.sw_upscale(ctx, abi.SW_UPSCALE_LEARNED, 2, ctypes.c_void_p(half.data_ptr()), 1,
                               ctypes.c_void_p(up.data_ptr()), SW, SH, SW, 1) == 0

    idx = frame_indices(args.warmup + args.steps, replica_offset(rank))
    plain_ms, learned_ms, psnr, views, tris, launches = [], [], [], 0, 0, 0
    fr = host.Frame(scene)
    with ClockSampler(local) as clocks:
        for step, fi in enumerate(idx):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            render(fi, opts_hi, full, SW)
            tp = timings()[4]
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            render(fi, opts_lo, half, W)
            tl = timings()[4]
            upscale()
            tu = timings()[3]
            if step < args.warmup:
                continue
            plain_ms.append(tp)
            learned_ms.append(tl + tu)
            psnr.append(ups.psnr(up, full, stream=hr_stream(glib, ctx)))
            fr.prepare(fi, opts_hi)
            views += len(fr.views)
            tris += fr.model_triangles
            # per frame: the frame's kernels, per portal view setup / bins / tiles / mix, the texture-effect
            # pass; the two frames of the step (views counted at 3840x2160 for both) and the upscale
            launches += 2 * (FRAME_LAUNCHES + 4 * len(fr.views) + (1 if fr.texture_passes.size else 0)) + 1
    p_ms = statistics.mean(plain_ms)
    l_ms = statistics.mean(learned_ms)
    mon = monitored_sequence(psnr, l_ms, p_ms)
    ms = max_over_ranks(1e3 / mon["frames_per_s"], world, dev)
    # e2e: the host work and a pinned-host copy of every delivered 3840x2160 frame, wall clock
    out = np.zeros((SH, SW), np.uint32)
    hr.register_host_buffer(out)
    pinned = torch.empty((SH, SW), dtype=torch.int32).pin_memory()
    efr = idx[args.warmup:args.warmup + max(4, min(args.steps, 8))]
    e_plain, e_learned = [], []
    for fi in efr[:2]:
        hr.render_frame(fi, opts_hi, out=out, post=cfg)
    hr.sync()
    st0 = abi.Stats()
    assert glib.sw_get_stats(ctx, ctypes.byref(st0)) == 0
    for fi in efr:
        t0 = time.perf_counter()
        hr.render_frame(fi, opts_hi, out=out, post=cfg)
        hr.sync()
        e_plain.append((time.perf_counter() - t0) * 1e3)
    st1 = abi.Stats()
    assert glib.sw_get_stats(ctx, ctypes.byref(st1)) == 0
    h2d = int((st1.upload_bytes - st0.upload_bytes) / len(efr))
    hr.render_frame(efr[0], opts_lo, device_ptr=half.data_ptr(), pitch=W, post=cfg)
    hr.sync()
    for fi in efr:
        t0 = time.perf_counter()
        hr.render_frame(fi, opts_lo, device_ptr=half.data_ptr(), pitch=W, post=cfg)
        upscale()
        assert glib.sw_sync(ctx) == 0
        pinned.copy_(up)  # on torch's own stream: the library's stream ends with its context
        e_learned.append((time.perf_counter() - t0) * 1e3)
    hr.unregister_host_buffer(out)
    del pinned
    e_mon = monitored_sequence(psnr, statistics.mean(e_learned), statistics.mean(e_plain))
    assert glib.sw_set_learned_upscaler(ctx, None) == 0
    if rank == 0:
        # parity of one plain 3840x2160 frame with portals (fresh renderer, exposure 1.0) against the
        # oracle composing its views; the CPU baseline is that oracle frame's time with all host threads
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        threads = os.cpu_count() or 1
        fi = next((f for f in idx if (fr.prepare(f, opts_hi) or True) and len(fr.views)), idx[0])
        # a fresh preparation, as the fresh renderer's: its texture-effect passes generate every effect
        fr = host.Frame(scene)
        fr.prepare(fi, opts_hi)
        static = scene.static_data()
        lite = scene.lite_textures()
        hr2 = host.HostRenderer(scene, device=local)
        got = np.zeros((SH, SW), np.uint32)
        assert glib.sw_set_exposure(hr2.context(), ctypes.c_float(1.0)) == 0
        hr2.render_frame(fi, opts_hi, out=got, post=cfg)
        hr2.close()
        t0 = time.perf_counter()
        work = type(static)(static.texels.copy(), static.texture_mips, static.emissive_pixels.copy(), static.emissive_mips,
                            static.lightmaps, static.directional_lightmaps)
        oracle.apply_texture_passes(fr.texture_passes, fr.texture_shifts, work)
        arena = oracle.build_surfaces(work, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=threads)
        if len(fr.views):
            oracle.render_views(fr.views, fr.draws, fr.vertices, arena, fr.params, tri_vertices=fr.tri_vertices, lite=lite)
        fb = np.zeros((SH, SW), np.uint64)
        oracle.rasterize(fr.draws[:fr.main_draws], fr.vertices, arena, fr.params, fb, num_threads=threads,
                         tri_vertices=fr.tri_vertices, lite=lite)
        oracle.postprocess(cfg, fb, 1.0 / 60.0, (1.0, 1.0, 1.0), 1.0)
        cpu_s = time.perf_counter() - t0
        # parity: the single-region raster (the threaded one clips each draw to its region, which moves
        # the edge walk's start on region borders), as the GPU's
        fb = np.zeros((SH, SW), np.uint64)
        oracle.rasterize(fr.draws[:fr.main_draws], fr.vertices, arena, fr.params, fb, tri_vertices=fr.tri_vertices, lite=lite)
        want, _, _ = oracle.postprocess(cfg, fb, 1.0 / 60.0, (1.0, 1.0, 1.0), 1.0)
        n = len(psnr)
        print(json.dumps({
            "metric": "3840x2160 frames/s delivered: learned 2x upscale from 1920x1080 under the PSNR>=38 dB monitor",
            "value": round(world * mon["frames_per_s"], 2), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (lighting) / int (raster) / bf16 (upscaler)",
            "data": "synthetic (seeded scene generator)",
            "config": {"workload": "stress: 128-room map (16x8), 12 portals (mirrors, cameras, parallax windows, 2 nested "
                                   "levels), translucent / alpha-blended / alpha-tested surfaces, 2000 decals, 64 sprites, "
                                   "200 animated models (about 2k triangles, 8 keyframes) lit from a seeded light grid; "
                                   "3840x2160 colour64 + bloom + tonemap",
                       "mean_portal_views": round(views / n, 2), "mean_model_triangle_draws": int(tris / n),
                       "timing": "CUDA-event device time of each frame's CUDA graph (+ the upscale launch)",
                       "l2": "flushed (512 MiB write) before every timed frame", "parallelism": f"replicas x{world}"},
            "plain_3840x2160": {"frames_per_s": round(1e3 / p_ms, 2), "ms_per_frame": round(p_ms, 4)},
            "learned": {"frames_per_s": round(1e3 / l_ms, 2), "ms_per_frame": round(l_ms, 4),
                        "psnr_db": {"mean": round(float(np.mean(psnr)), 3), "min": round(float(np.min(psnr)), 3),
                                    "frames_at_or_above_38db": f"{sum(x >= 38.0 for x in psnr)}/{n}"},
                        "with_quality_monitor": mon,
                        "train": {"steps": args.learn_steps, "pairs": "1920x1080 -> 3840x2160",
                                  "maps": f"stress configuration without portals, seeds {list(STRESS_TRAIN_MAPS)} "
                                          f"(bench map: seed 5)", "seconds": round(train_s, 2)}},
            "parity": {"frames": 1, "frame_index": int(fi), "portal_views": int(len(fr.views)),
                       "mismatched_pixels": int((want != got).sum())},
            "cpu_baseline": {"value": round(1.0 / cpu_s, 4), "unit": "frames/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": "1 plain 3840x2160 frame: oracle texture effects, surfaces, portal views, "
                                       "split_rect raster with the triangles, postprocess"},
            "e2e": {"value": round(e_mon["frames_per_s"], 2), "unit": "frames/s",
                    "plain_frames_per_s": round(1e3 / statistics.mean(e_plain), 2),
                    "learned_frames_per_s": round(1e3 / statistics.mean(e_learned), 2),
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(out.nbytes),
                    "path": "swh_renderer_render_frame (host visibility, portals and models) per frame, wall clock, "
                            "the delivered frame copied to pinned host memory; monitor applied as for value"},
            "clocks": clocks.summary(), "gpu_launches": launches}), flush=True)
    ups.close()
    hr.close()


def run_small_gpu(args, world, rank, local):
    """The small CPU-runnable configuration: the 8-room map (~2k polygons, 16 128x128 textures, simple
    lightmaps, no dynamic lights) at 640x480 colour32 on its 64-frame camera path. value: frames/s of
    device time of each frame's CUDA graph (host-prepared arrays, L2 flushed before each); e2e: the same
    frames through swh_renderer_render_frame (host visibility + GPU-side preparation, frame into a host
    buffer); cpu_baseline: host work + the oracle with every host thread; parity: the frames against the
    oracle's single-thread raster."""
    import ctypes
    import torch
    from sqwheel import abi, gpu, host
    torch.cuda.set_device(local)
    w, h = 640, 480
    scene = host.Scene(**host.SMALL_MAP)
    static = scene.static_data()
    opts = host.frame_options(w, h, abi.SW_PIXEL_C32, directional=False)
    fr = host.Frame(scene)
    n = scene.info().frames
    idx = [(replica_offset(rank) + k * 5) % n for k in range(args.warmup + args.steps)]
    frames, prep_ms = [], []
    for fi in idx:
        t0 = time.perf_counter()
        fr.prepare(fi, opts)
        prep_ms.append((time.perf_counter() - t0) * 1e3)
        frames.append(dict(index=fi, surfaces=fr.surfaces, draws=fr.draws, vertices=fr.vertices, lights=fr.lights,
                           params=fr.params, total_texels=fr.total_texels))
    r = gpu.GpuRenderer(static, device=local)
    r.enable_timing(True)
    stream = torch.cuda.ExternalStream(r.stream_handle())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    out = torch.empty((len(frames), h, w), dtype=torch.int32, device=f"cuda:{local}")
    graph_ms = []
    with ClockSampler(local) as clocks:
        for step, f in enumerate(frames):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            r.draw_frame(r.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"], f["vertices"],
                                       dst_device_ptr=out[step].data_ptr(), pitch=w))
            t = r.timings()
            if step >= args.warmup:
                graph_ms.append(t[4])
        torch.cuda.synchronize()
    ms = max_over_ranks(statistics.mean(graph_ms), world, f"cuda:{local}")
    gpu_frames = out.cpu().numpy().view(np.uint32)
    r.close()
    # e2e through the C ABI, one frame at a time into a registered host buffer
    hr = host.HostRenderer(scene, device=local)
    glib = gpu.load_library()
    hbuf = np.zeros((h, w), np.uint32)
    hr.register_host_buffer(hbuf)
    for f in frames[: args.warmup]:
        hr.render_frame(f["index"], opts, out=hbuf)
    s0 = abi.Stats()
    glib.sw_get_stats(hr.context(), ctypes.byref(s0))
    t0 = time.perf_counter()
    for f in frames[args.warmup:]:
        hr.render_frame(f["index"], opts, out=hbuf)
    hr.sync()
    e2e = args.steps / (time.perf_counter() - t0)
    s1 = abi.Stats()
    glib.sw_get_stats(hr.context(), ctypes.byref(s1))
    hr.unregister_host_buffer(hbuf)
    hr.close()
    if rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        threads = os.cpu_count() or 1
        # CPU baseline: host work + oracle surfaces (all threads) + split_rect raster (all threads), a
        # bounded sample of the same frames
        sample = frames[:16]
        t0 = time.perf_counter()
        for f in sample:
            fr.prepare(f["index"], opts)
            arena = oracle.build_surfaces(static, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=threads)
            fb = np.zeros((h, w), np.uint32)
            oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, fb, num_threads=threads)
        cpu_v = len(sample) / (time.perf_counter() - t0)
        # parity: every graph frame against the oracle's single-thread raster (the frame buffer carries over)
        want = np.zeros((h, w), np.uint32)
        mism = 0
        for step, f in enumerate(frames):
            arena = oracle.build_surfaces(static, f["surfaces"], f["lights"], f["params"], f["total_texels"], num_threads=threads)
            oracle.rasterize(f["draws"], f["vertices"], arena, f["params"], want)
            mism += int((want != gpu_frames[step]).sum())
        print(json.dumps({
            "metric": METRIC, "value": round(world * 1e3 / ms, 2), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (lighting) / int (raster)", "data": "synthetic (seeded scene generator)",
            "config": {"workload": "small: the 8-room map (~2k polygons, 16 128x128 textures, simple lightmaps, no dynamic "
                                   "lights) at 640x480 colour32, every 5th frame of its 64-frame camera path",
                       "frames": idx[args.warmup:][:8], "mean_surface_texels": int(statistics.mean(f["total_texels"] for f in frames)),
                       "mean_host_prep_ms": round(statistics.mean(prep_ms), 3),
                       "timing": "CUDA-event device time of the frame's CUDA graph (sw_draw_frame)",
                       "l2": "flushed (512 MiB write) before every timed step", "parallelism": f"replicas x{world}"},
            "parity": {"frames": len(frames), "mismatched_pixels": mism},
            "cpu_baseline": {"value": round(cpu_v, 3), "unit": "frames/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": f"{len(sample)} frames: host work + oracle surfaces and split_rect raster, {threads} threads"},
            "e2e": {"value": round(e2e, 2), "unit": "frames/s",
                    "h2d_bytes_per_step": int((s1.upload_bytes - s0.upload_bytes) / args.steps),
                    "d2h_bytes_per_step": int(hbuf.nbytes),
                    "path": "render_frame: host visibility + GPU-side surface and draw preparation, one frame at a time"},
            "clocks": clocks.summary(), "gpu_launches": args.steps * 4}), flush=True)


# ---------------------------------------------------------------------------------------------------------
# surfaces workload

class SurfaceWorkload:
    name = "batched surfaces: 4096 surfaces, sides log-uniform 4-512, mips 0-3, directional lightmaps, C64"

    def __init__(self, seed=3):
        from sqwheel import abi, synth
        self.batch = synth.BatchedSurfaces(seed=seed, count=4096, num_lights=0, pixel_format=abi.SW_PIXEL_C64)


def run_surfaces_gpu(args, world, rank, local):
    import torch
    from sqwheel import gpu
    torch.cuda.set_device(local)
    work = SurfaceWorkload(seed=3 + rank)
    b = work.batch
    r = gpu.GpuRenderer(b.static_data(), device=local)
    fp = gpu.frame_params(W, H, b.pixel_format, b.cam_pos, directional=True)
    r.frame_begin(fp, b.lights)
    r.submit_surfaces(b.surfaces, b.total_texels)
    r.enable_timing(True)
    stream = torch.cuda.ExternalStream(r.stream_handle())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    # the persistent launch replayed as a CUDA graph (sw_rebuild_surfaces with the graph setting on)
    for _ in range(args.warmup):
        r.rebuild_surfaces()
    total = 0.0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            r.rebuild_surfaces()
            total += r.timings()[0]
    ms = max_over_ranks(total / args.steps, world, f"cuda:{local}")
    value = world * b.total_texels / 1e6 / (ms / 1e3)
    gpu_arena = r.read_surfaces(b.total_texels, b.pixel_format)
    # the baseline it is compared against: one launch per surface, same arena
    r.rebuild_surfaces_per_surface()
    per_surface_ms = []
    for _ in range(min(args.steps, 5)):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        r.rebuild_surfaces_per_surface()
        per_surface_ms.append(r.timings()[0])
    per_ms = statistics.mean(per_surface_ms)
    same = bool(np.array_equal(gpu_arena, r.read_surfaces(b.total_texels, b.pixel_format)))
    e2e = []
    for _ in range(3):
        t0 = time.perf_counter()
        r.frame_begin(fp, b.lights)
        r.submit_surfaces(b.surfaces, b.total_texels)
        outa = r.read_surfaces(b.total_texels, b.pixel_format)
        e2e.append(time.perf_counter() - t0)
    peak, peak_kind = peaks()
    alg = b.algorithmic_bytes()
    gbs = alg / (ms / 1e3) / 1e9
    if rank == 0:
        cpu, parity = cpu_surfaces_baseline(work, gpu_arena)
        print(json.dumps({
            "metric": METRIC, "value": round(value, 2), "unit": "Mtexels/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": work.name, "texels_per_step": int(b.total_texels),
                       "materials": "25% metal / 25% dielectric specular, normal maps; no dynamic lights",
                       "timing": "CUDA events around the replayed graph of the persistent surface launch",
                       "l2": "flushed (512 MiB write) before every timed step", "parallelism": f"replicas x{world}"},
            "per_surface_launches": {"ms": round(per_ms, 4), "mtexels_per_s": round(b.total_texels / 1e3 / per_ms, 1),
                                     "persistent_speedup": round(per_ms / ms, 2), "same_arena": same,
                                     "what": f"{b.surfaces.size} launches, one per surface (sw_rebuild_surfaces_per_surface)"},
            "parity": parity,
            "roofline": {"bound": "hbm", "kernel": "surf_build_kernel", "achieved": round(gbs, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(gbs / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                         "algorithmic_bytes_per_launch": int(alg), "traffic": None},
            "cpu_baseline": cpu,
            "e2e": {"value": round(b.total_texels / 1e6 / statistics.median(e2e), 2), "unit": "Mtexels/s",
                    "h2d_bytes_per_step": int(b.surfaces.nbytes + (b.surfaces.size + 1) * 8),
                    "d2h_bytes_per_step": int(outa.nbytes)},
            "clocks": clocks.summary(), "gpu_launches": args.steps}), flush=True)
    r.close()


def cpu_surfaces_baseline(work, gpu_arena=None):
    """The oracle's surface build of the first surfaces (an eighth of the texels) on all host threads;
    with gpu_arena, its texels are compared with the GPU's for those surfaces (the arena lays surfaces
    out in order). Returns (baseline, parity or None)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from sqwheel import gpu
    threads = os.cpu_count() or 1
    b = work.batch
    area = b.surfaces["size"][:, 0].astype(np.int64) * b.surfaces["size"][:, 1]
    cum = np.cumsum(area)
    n = int(np.searchsorted(cum, max(cum[-1] // 8, 1)) + 1)
    sub = b.surfaces[:n].copy()
    sub["out_offset"] = np.concatenate([[0], cum[:n - 1]]).astype(np.uint64)
    texels = int(cum[n - 1])
    fp = gpu.frame_params(64, 64, b.pixel_format, b.cam_pos, directional=b.directional)
    static = b.static_data()
    t0 = time.perf_counter()
    want = oracle.build_surfaces(static, sub, b.lights, fp, texels, num_threads=threads)
    dt = time.perf_counter() - t0
    base = {"value": round(texels / dt / 1e6, 2), "unit": "Mtexels/s", "cores": threads, "kind": "port",
            "cpu_model": cpu_model(),
            "sample": f"{n} of {b.surfaces.size} surfaces ({texels} texels), oracle with {threads} threads"}
    if gpu_arena is None:
        return base, None
    return base, {"surfaces": n, "texels": texels, "mismatched_texels": int((want != gpu_arena[:texels]).sum())}


# ---------------------------------------------------------------------------------------------------------
# shadows workload: shadowed dynamic lights (cube shadow maps) on the 1080p frame of the 64-room map

def run_shadows_gpu(args, world, rank, local):
    """value: shadow-map builds per second of device time (sw_build_shadow_maps_view over the frame's cube
    sides and their leafs, already on the host; L2 flushed before each); e2e: whole 1080p frames with the
    first `--shadowed-lights` of the 8 dynamic lights shadowed, through swh_renderer_render_frame."""
    import ctypes
    import torch
    from sqwheel import abi, gpu, host
    torch.cuda.set_device(local)
    scene = host.Scene(**dict(host.FULL_MAP, shadowed_lights=args.shadowed_lights))
    opts = host.frame_options(W, H, abi.SW_PIXEL_C64, directional=True)
    cfg = abi.PostConfig.default()
    frames = [((k * 37 + 11 * rank) % 256) for k in range(max(args.steps, 4) + args.warmup)]
    hr = host.HostRenderer(scene, device=local)  # its context holds the map
    glib = gpu.load_library()
    ctx = hr.context()
    fr = host.Frame(scene)
    lists = []
    for fi in frames:
        fr.prepare_view(fi, opts)
        lists.append((fr.shadow_sides.copy(), fr.shadow_leafs.copy(), fr.shadow_texels))
    stream = torch.cuda.ExternalStream(hr_stream(glib, ctx))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def build(k):
        sd, lf, n = lists[k]
        rc = glib.sw_build_shadow_maps_view(ctx, abi.ptr(sd), sd.size, abi.ptr(lf), lf.size, n)
        assert rc == abi.SW_OK, rc

    for k in range(args.warmup):
        build(k)
    ms_list = []
    with ClockSampler(local) as clocks:
        for k in range(args.warmup, args.warmup + args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                build(k)
                e1.record(stream)
            e1.synchronize()
            ms_list.append(e0.elapsed_time(e1))
    ms = max_over_ranks(statistics.mean(ms_list), world, f"cuda:{local}")
    # algorithmic bytes of one build: every covered texel once (8-byte read-modify-write in L2) plus each
    # candidate's polygon record and vertices
    texels = statistics.mean(int(n) for _, _, n in lists[args.warmup:])
    cands = statistics.mean(int(lf["num_polygons"].sum()) for _, lf, _ in lists[args.warmup:])
    alg = texels * 16 + cands * (abi.MAP_POLYGON.itemsize + 6 * 12)
    peak, peak_kind = peaks()
    gbs = alg / (ms / 1e3) / 1e9

    def e2e_run(shadowed):
        r2 = host.HostRenderer(host.Scene(**dict(host.FULL_MAP, shadowed_lights=shadowed)), device=local)
        out = np.zeros((H, W), np.uint32)
        r2.register_host_buffer(out)
        for fi in frames[:4]:
            r2.render_frame(fi, opts, out=out, post=cfg)
        times, up = [], 0
        for fi in frames[args.warmup:]:
            s0, s1 = abi.Stats(), abi.Stats()
            glib.sw_get_stats(r2.context(), ctypes.byref(s0))
            t0 = time.perf_counter()
            r2.render_frame(fi, opts, out=out, post=cfg)
            times.append(time.perf_counter() - t0)
            glib.sw_get_stats(r2.context(), ctypes.byref(s1))
            up += s1.upload_bytes - s0.upload_bytes
        r2.unregister_host_buffer(out)
        r2.close()
        return 1.0 / statistics.median(times), up / len(times), out.nbytes

    e2e_val, h2d, d2h = e2e_run(args.shadowed_lights)
    e2e_plain, _, _ = e2e_run(0)
    if rank == 0:
        # CPU: the host's depth-draw preparation (the reference's DepthRenderer restated in C++) and the
        # oracle's DepthRasterizer over those draws, one thread, a bounded sample of the frames
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        sample = frames[args.warmup:args.warmup + 4]
        storage = np.zeros(0, np.float32)
        t0 = time.perf_counter()
        for fi in sample:
            fr.prepare(fi, opts)
            if storage.size < fr.shadow_texels:
                storage = np.concatenate([storage, np.zeros(fr.shadow_texels - storage.size, np.float32)])
            oracle.shadow_maps(fr.depth_draws, fr.depth_vertices, storage)
        cpu_val = len(sample) / (time.perf_counter() - t0)
        print(json.dumps({
            "metric": METRIC, "value": round(world * 1e3 / ms, 1), "unit": "shadow-map builds/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 depth / fixed16 edges", "data": "synthetic (seeded)",
            "config": {"workload": f"cube shadow maps of the 1920x1080 colour64 frame, 64-room map, "
                                   f"{args.shadowed_lights} of 8 dynamic lights shadowed",
                       "texels_per_step": int(texels), "candidate_polygons_per_step": int(cands),
                       "l2": "flushed (512 MiB write) before every timed step", "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "kernel": "shadow_view_kernel", "achieved": round(gbs, 2), "peak": peak,
                         "unit": "GB/s", "frac": round(gbs / peak, 5), "peak_source": f"{peak_kind} hbm_gbs",
                         "algorithmic_bytes_per_launch": int(alg), "traffic": None,
                         "note": "latency-bound: a few MB per launch"},
            "cpu_baseline": {"value": round(cpu_val, 2), "unit": "shadow-map builds/s", "cores": 1, "kind": "port",
                             "sample": f"{len(sample)} frames: host depth-draw preparation + oracle DepthRasterizer"},
            "e2e": {"value": round(e2e_val, 1), "unit": "frames/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "without_shadows": round(e2e_plain, 1)},
            "clocks": clocks.summary(), "gpu_launches": args.steps}), flush=True)
    hr.close()


def hr_stream(glib, ctx):
    import ctypes
    s = ctypes.c_void_p()
    rc = glib.sw_get_stream(ctx, ctypes.byref(s))
    assert rc == 0, rc
    return s.value or 0


# ---------------------------------------------------------------------------------------------------------
# upscale workload (the learned upscaler alone)

def bf16_peak():
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        v = float(json.load(open(pp)).get("bf16_tflops", 0))
        if v > 0:
            return v, "measured bf16_tflops (burst)"
    return 1900.0, "fallback"


def run_upscale_gpu(args, world, rank, local):
    """Learned 2x upscale of a 960x540 Color32 frame to 1920x1080 by the fused four-layer tcgen05 kernel
    (one launch per step; the layer-by-layer form, five launches, is timed beside it), inputs resident
    in HBM, L2 flushed between steps."""
    import ctypes

    import torch
    from sqwheel import abi, gpu, host, learned
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    # a tonemapped half-resolution frame of the full-size map as input
    src = learned.PairRenderer(host.Scene(**host.FULL_MAP), (W // 2, H // 2), device=local, hdr=True)
    lo = torch.empty((H // 2, W // 2), dtype=torch.int32, device=dev)
    src.render_lo(37 + rank, lo)
    src.sync()
    src.close()
    ups = learned.Upscaler(local, seed=1)
    hi = torch.empty((H, W), dtype=torch.int32, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    # a stream of our own: its handle is non-zero, so the upscaler runs on it (NULL selects the
    # upscaler's internal stream) and the events bracket exactly its kernels
    st = torch.cuda.Stream(device=dev)

    def timed(steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(st):
            for _ in range(args.warmup):
                flush.fill_(1.0)
                ups.infer(lo, hi, stream=st.cuda_stream)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clocks, torch.cuda.stream(st):
            for i in range(steps):
                flush.fill_(1.0)
                ev[i][0].record(st)
                ups.infer(lo, hi, stream=st.cuda_stream)
                ev[i][1].record(st)
            torch.cuda.synchronize()
        ups.check()
        return sum(a.elapsed_time(b) for a, b in ev) / steps, clocks

    ups.set_fused(False)
    layered_ms, _ = timed(min(args.steps, 20))
    ups.set_fused(True)
    ms, clocks = timed(args.steps)
    ms = max_over_ranks(ms, world, dev)
    # e2e: through the C ABI (sw_upscale, learned mode) from and to host memory
    r = gpu.GpuRenderer(host.Scene(**host.SMALL_MAP).static_data(), device=local)
    r.attach_upscaler(ups)
    lo_h = lo.cpu().numpy().view(np.uint32).copy()
    out_h = np.zeros((H, W), np.uint32)
    e2e = []
    for i in range(max(4, min(args.steps, 16))):
        t0 = time.perf_counter()
        r.upscale(abi.SW_UPSCALE_LEARNED, 2, lo_h, out_h)
        if i:
            e2e.append(time.perf_counter() - t0)
    r.attach_upscaler(None)
    r.close()
    peak, kind = bf16_peak()
    tf = UPSCALER_FLOPS / (ms / 1e3) / 1e12
    if rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import upscaler_oracle
        p = ups.params()
        t0 = time.perf_counter()
        upscaler_oracle.infer(p, lo_h[:135])
        cpu_s = (time.perf_counter() - t0) * 4
        print(json.dumps({
            "metric": METRIC, "value": round(world * 1e3 / ms, 2), "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)", "data": "synthetic (seeded)",
            "config": {"workload": "learned 2x upscale 960x540 -> 1920x1080 (4-layer 3x3 CNN, 32 channels, pixel shuffle)",
                       "input": "tonemapped 960x540 frame of the 64-room map", "weights": "seeded initialisation",
                       "l2": "flushed (512 MiB write) before every timed step", "parallelism": f"replicas x{world}"},
            "layer_by_layer_ms": round(layered_ms, 5),
            "roofline": {"bound": "tensor", "kernel": "fused_upscale_kernel (one launch, four layers)", "achieved": round(tf, 1),
                         "peak": peak, "unit": "TFLOP/s", "frac": round(tf / peak, 4), "peak_source": kind,
                         "algorithmic_flops_per_launch": UPSCALER_FLOPS, "traffic": None},
            "cpu_baseline": {"value": round(1.0 / cpu_s, 4), "unit": "frames/s", "cores": 1, "kind": "port",
                             "sample": "a quarter frame (135 of 540 rows) through the numpy FP32 oracle, scaled x4"},
            "e2e": {"value": round(1.0 / statistics.median(e2e), 2), "unit": "frames/s",
                    "h2d_bytes_per_step": int(lo_h.nbytes), "d2h_bytes_per_step": int(out_h.nbytes)},
            "clocks": clocks.summary(), "gpu_launches": args.steps}), flush=True)
    ups.close()


# ---------------------------------------------------------------------------------------------------------

def run_reference(args, world, rank):
    """The reference's CPU path restated in C++ (the Rust reference cannot be built here), all host
    threads, one frame per step (host work + surfaces + split_rect raster + postprocess)."""
    if rank != 0:
        return
    if args.workload == "surfaces":
        work = SurfaceWorkload(seed=3)
        vals = [cpu_surfaces_baseline(work)[0] for _ in range(args.warmup + args.steps)][args.warmup:]
        c = vals[-1]
        v = statistics.median(x["value"] for x in vals)
        unit = "Mtexels/s"
        ms = None
    else:
        work = FrameWorkload(args.warmup + args.steps)
        # Each step: one frame of the same workload (bounded: the whole run stays within minutes).
        work_frames = work.frames
        ts = []
        for i in range(len(work_frames)):
            work.frames = work_frames[i:i + 1]
            c, _ = cpu_frame_baseline(work, max_frames=1)
            if i >= args.warmup:
                ts.append(1.0 / c["value"])
        v = len(ts) / sum(ts)
        unit = "frames/s"
        ms = 1e3 * statistics.median(ts)
        c["sample"] = f"{len(ts)} frames, one per step; " + c["sample"].split("; ", 1)[1]
    out = {"metric": METRIC, "impl": "reference", "value": round(v, 3), "unit": unit, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3) if ms else None,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (lighting) / int (raster)",
           "data": "synthetic (seeded)", "config": {"workload": work.name},
           "cpu_baseline": {"value": round(v, 3), "unit": unit, "cores": c["cores"], "kind": "port", "sample": c["sample"],
                            "cpu_model": cpu_model()},
           "e2e": {"value": round(v, 3), "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="frame", choices=["frame", "surfaces", "upscale", "shadows", "models", "small",
                                                                          "stress"])
    ap.add_argument("--shadowed-lights", type=int, default=2, help="shadows workload: shadowed dynamic lights (of 8)")
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--autotune-reps", type=int, default=5,
                    help="frames per configuration of the autotuner before the frame measurement (0: keep the default)")
    ap.add_argument("--learn-steps", type=int, default=20000,
                    help="training steps of the learned upscaler before its measurement (0: skip it)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    try:
        if args.workload == "surfaces":
            run_surfaces_gpu(args, world, rank, local)
        elif args.workload == "upscale":
            run_upscale_gpu(args, world, rank, local)
        elif args.workload == "shadows":
            run_shadows_gpu(args, world, rank, local)
        elif args.workload == "models":
            run_models_gpu(args, world, rank, local)
        elif args.workload == "small":
            run_small_gpu(args, world, rank, local)
        elif args.workload == "stress":
            run_stress_gpu(args, world, rank, local)
        else:
            run_frame_gpu(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
