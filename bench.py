"""Benchmark of the GB300 Square-Wheel rendering path.

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload frame|surfaces] [--impl gpu|reference]

Prints one JSON line (rank 0). A step is one pass of the hot path over one batch of synthetic input:
  surfaces: the batched-surface workload (4,096 surfaces, sides log-uniform 4..512 texels, mips 0..3,
            directional lightmaps, normal-mapped dielectric/metal materials) built in one launch.
Timing: W untimed warm-up steps, then K steps, each preceded by an L2 flush (a 512 MiB write) outside
the timed span; device time from CUDA events on the library's stream, summed over the K steps.
Multi-GPU: the workload is replicated (independent surface batches per rank, no collective); value is
the sum over ranks of units / max-over-ranks time.
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
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
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
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_surfaces_baseline(work, max_seconds=20.0):
    """Oracle (C++ restatement of the reference CPU surface builder, one task per surface on all host
    threads) on a bounded sample of the same surface batch."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from sqwheel import abi, gpu
    threads = os.cpu_count() or 1
    b = work.batch
    # Sample: the first surfaces of the batch up to ~1/8 of its texels.
    area = b.surfaces["size"][:, 0].astype(np.int64) * b.surfaces["size"][:, 1]
    cum = np.cumsum(area)
    n = int(np.searchsorted(cum, max(cum[-1] // 8, 1)) + 1)
    sub = b.surfaces[:n].copy()
    sub["out_offset"] = np.concatenate([[0], cum[:n - 1]]).astype(np.uint64)
    texels = int(cum[n - 1])
    fp = gpu.frame_params(64, 64, b.pixel_format, b.cam_pos, directional=b.directional)
    static = b.static_data()
    t0 = time.perf_counter()
    reps = 0
    while True:
        oracle.build_surfaces(static, sub, b.lights, fp, texels, num_threads=threads)
        reps += 1
        if time.perf_counter() - t0 > min(max_seconds, 3.0) or reps >= 3:
            break
    dt = (time.perf_counter() - t0) / reps
    return {"value": texels / dt / 1e6, "unit": "Mtexels/s", "cores": threads, "kind": "port",
            "sample": f"{n} of {b.surfaces.size} surfaces ({texels} texels), {reps} reps, oracle with {threads} threads"}


class SurfaceWorkload:
    name = "batched surfaces: 4096 surfaces, sides log-uniform 4-512, mips 0-3, directional lightmaps, C64"

    def __init__(self, seed=3):
        from sqwheel import abi, synth
        self.batch = synth.BatchedSurfaces(seed=seed, count=4096, num_lights=0, pixel_format=abi.SW_PIXEL_C64)

    def setup(self, renderer):
        from sqwheel import gpu
        b = self.batch
        self.fp = gpu.frame_params(1920, 1080, b.pixel_format, b.cam_pos, directional=True)
        renderer.frame_begin(self.fp, b.lights)
        renderer.submit_surfaces(b.surfaces, b.total_texels)
        renderer.sync()

    def device_step(self, renderer):
        renderer.rebuild_surfaces()
        return 1  # kernel launches

    def e2e_step(self, renderer):
        """Through the C ABI with host buffers: upload descriptors, build, read the arena back."""
        b = self.batch
        renderer.frame_begin(self.fp, b.lights)
        renderer.submit_surfaces(b.surfaces, b.total_texels)
        out = renderer.read_surfaces(b.total_texels, b.pixel_format)
        h2d = b.surfaces.nbytes + (b.surfaces.size + 1) * 8
        return h2d, out.nbytes

    def units(self):
        return self.batch.total_texels / 1e6  # Mtexels per step

    unit = "Mtexels/s"

    def algorithmic_bytes(self):
        return self.batch.algorithmic_bytes()


def run_gpu(args):
    import torch
    from sqwheel import gpu
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    work = SurfaceWorkload(seed=3 + rank)
    r = gpu.GpuRenderer(work.batch.static_data(), device=local)
    work.setup(r)
    stream = torch.cuda.ExternalStream(r.stream_handle())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    for _ in range(args.warmup):
        work.device_step(r)
    r.sync()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    total_ms = 0.0
    launches = 0
    barrier()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                launches += work.device_step(r)
                e1.record(stream)
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
        barrier()
    ms_per_step = total_ms / args.steps
    if world > 1:
        t = torch.tensor([ms_per_step], device=f"cuda:{local}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_per_step = float(t.item())
    value = work.units() * world / (ms_per_step / 1e3)

    # End to end through the C ABI with host buffers.
    e2e_ms = []
    h2d = d2h = 0
    for _ in range(max(1, min(args.steps, 5))):
        barrier()
        t0 = time.perf_counter()
        h2d, d2h = work.e2e_step(r)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_val = work.units() / (statistics.median(e2e_ms) / 1e3)

    peak, peak_kind = peaks()
    alg = work.algorithmic_bytes()
    achieved = alg / (ms_per_step / 1e3) / 1e9
    out = None
    if rank == 0:
        cpu = cpu_surfaces_baseline(work)
        out = {
            "metric": METRIC, "value": round(value, 2), "unit": work.unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": work.name, "surfaces": int(work.batch.surfaces.size),
                       "texels_per_step": int(work.batch.total_texels), "pixel_format": "C64",
                       "l2": "flushed (512 MiB write) before every timed step", "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "kernel": "surf_build_kernel", "achieved": round(achieved, 1),
                         "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_launch": int(alg),
                         "traffic": None},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_val, 2), "unit": work.unit, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "clocks": clocks.summary(),
            "gpu_launches": launches,
        }
        print(json.dumps(out), flush=True)
    r.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return out


def run_reference(args):
    """The reference's CPU path, restated in C++ (the Rust reference cannot be built here), on all host
    threads, on bounded samples of the same workload."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    work = SurfaceWorkload(seed=3)
    vals = []
    for _ in range(args.warmup):
        cpu_surfaces_baseline(work, max_seconds=5.0)
    t_steps = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        c = cpu_surfaces_baseline(work, max_seconds=5.0)
        t_steps.append(time.perf_counter() - t0)
        vals.append(c["value"])
    v = statistics.median(vals)
    out = {"metric": METRIC, "impl": "reference", "value": round(v, 3), "unit": "Mtexels/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * statistics.median(t_steps), 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded)", "config": {"workload": work.name},
           "cpu_baseline": {"value": round(v, 3), "unit": "Mtexels/s", "cores": c["cores"], "kind": "port",
                            "sample": c["sample"]},
           "e2e": {"value": round(v, 3), "unit": "Mtexels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
