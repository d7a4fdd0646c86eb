"""Benchmark of the HairMSNN per-path-vertex hot path on GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--workload render|vertex]

Workloads (synthetic, seeded):
  render  full wavefront render of procedural straight hair: 10k strands x
          64 cubic B-spline control points, head ellipsoid, sky + directional
          light, 512x512, path_v1=1, path_v2=40, BETA=1, online cache
          training 2^16 records/frame.  One step = one frame (1 spp, as the
          reference's render loop: G-buffer paths + train + infer + compose).
          metric: paths/s.
  vertex  2^18 hair-vertex queries: BSDF eval + BSDF importance sample +
          cache-network inference (Freq-12 / OneBlob-32 / Identity -> 5x64).
          metric: vertex queries/s.

One JSON line is printed by rank 0.  `value` times the kernels with inputs
resident in HBM (vertex: CUDA events per step on the launching stream, L2
flushed between steps outside the events; render: CUDA events around K
pipelined frames on the submitting stream, no flush: each frame in flight
streams its own ~90 MB of path state past the 129 MB L2); `e2e` times the same step
through the public API with pinned host inputs copied in and results copied
out inside the timed region.  Multi-GPU runs are independent replicas (the path has no
exchange step on one box).
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
sys.path.insert(0, ROOT)

def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(path):
        p = json.load(open(path))
        return {"hbm_gbs": p["hbm_gbs"], "bf16_tflops": p["bf16_tflops"],
                "bf16_tflops_sustained": p.get("bf16_tflops_sustained", p["bf16_tflops"]),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for i, nm in enumerate(names):
                if f[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws, device="cuda"):
    """The largest of the ranks' x (x itself on one rank): the job's time is
    its slowest rank's."""
    if ws <= 1:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args):
    """--impl reference: the reference's per-pixel path on the host cores,
    with the oracle alone, which reproduces the reference's own integrator
    bit for bit (the host build of the reference's code under oracle/_ref
    needs the reference checkout, which the GPU host does not have).  No
    product library is loaded: the scene comes from the oracle's generator
    (hairmsnn_gb300.render only supplies the config dict; the package loads
    its library lazily).  Rank 0 only; no GPU work.
      render: the same frame work as the GPU arm per pixel (CpuFrameSample:
              G-buffer paths, cache inference, cache training gradient) over
              a band of pixels per step;
      vertex: BSDF eval + sample and the cache's FP32 inference over a batch
              of the same queries per step."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np
    import bench_workloads as bw
    from oracle import pyoracle as po
    threads = host_threads()
    if args.workload == "vertex":
        from oracle import mlp_oracle as mo
        n = 1 << 14
        wo, wi, t, h, u = po.gen_bsdf_queries(0, n)
        cfg = mo.Config(open(os.path.join(ROOT, "hairmsnn_gb300", "configs", "c1_cache_w64.json")).read(), 16, 3)
        params = np.random.default_rng(0).normal(scale=0.1, size=cfg.n_params)
        x = np.random.default_rng(1).uniform(0, 1, (n, 16)).astype(np.float32)

        def step():
            po.hair_eval(wo.T, wi.T, t.T, h, threads=threads)
            po.hair_sample(wo.T, t.T, h, u.T, threads=threads)
            po.mlp_forward_host(cfg, params, x, threads=threads)
            return n
        metric, unit = bw.VertexWorkload.metric, bw.VertexWorkload.unit
        sample = f"{n} queries per step (oracle: BSDF and FP32 MLP inference in C++ on {threads} threads)"
        cfgd = {"workload": bw.VertexWorkload.workload_name, "sample": "bounded: queries_per_step of the workload",
                "queries_per_step": n}
    else:
        from hairmsnn_gb300.render import straight_hair_scene  # the config dict only
        cpu = bw.CpuFrameSample(straight_hair_scene(512, 512), 1 << 16, threads)
        step = cpu.step
        metric, unit = bw.RenderBenchWorkload.metric, bw.RenderBenchWorkload.unit
        sample = f"bands of {cpu.n} pixels of the 512x512 frame (1 spp) per step: {cpu.what}"
        cfgd = {"workload": bw.RenderBenchWorkload.workload_name,
                "sample": "bounded: pixels_per_step of the frame per step, bands advancing over the frame",
                "pixels_per_step": cpu.n}
    for _ in range(args.warmup):
        step()
    times, units = [], 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        units += step()
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = units / sum(times)
    line = {"impl": "reference", "metric": metric, "value": round(value, 2), "unit": unit, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfgd,
            "cpu_baseline": {"value": round(value, 2), "unit": unit, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 2), "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200,
                    help="timed steps (render: 200 frames, about a second of device time)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("HM_BENCH_WORKLOAD", "render"),
                    choices=["render", "vertex", "precision", "quality", "batch", "diff"])
    ap.add_argument("--fit-steps", type=int, default=200,
                    help="diff workload: Adam steps of the sigma_a recovery reported after the timing")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="render workload: skip the other configurations' figures (vertex batch, precision sweep, "
                         "equal-accuracy relMSE, ablation)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from hairmsnn_gb300 import build
    build.build()
    import bench_workloads as bw
    wl = bw.make_workload(args.workload, torch)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        wl.step()
    torch.cuda.synchronize()

    # ---- device-resident timed region
    sampler = ClockSampler(local if ws > 1 else 0)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    seg_ms = None
    if hasattr(wl, "timed_region"):
        ms = wl.timed_region(args.steps, flush)
    else:
        ne = wl.n_events()
        all_events = [[torch.cuda.Event(enable_timing=True) for _ in range(ne)] for _ in range(args.steps)]
        for k in range(args.steps):
            flush.fill_(k & 0xFF)  # > L2 write between steps, outside the step events
            wl.step(all_events[k])
        torch.cuda.synchronize()
        step_ms = [ev[0].elapsed_time(ev[-1]) for ev in all_events]
        seg_ms = [statistics.mean(ev[i].elapsed_time(ev[i + 1]) for ev in all_events) for i in range(ne - 1)]
        ms = statistics.mean(step_ms)
    if ws > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    launches = wl.kernels_per_step * args.steps
    ms = max_over_ranks(ms, ws)
    units = wl.units_per_step() * ws
    value = units / (ms * 1e-3)

    # ---- end-to-end through the public API (pinned host in/out in the timed region)
    e2e_steps = max(3, args.steps // 2)
    if hasattr(wl, "e2e_region"):
        wl.e2e_region(2)
        e2e_ms = wl.e2e_region(e2e_steps)
    else:
        for _ in range(2):
            wl.e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            wl.e2e_step()
        torch.cuda.synchronize()
        e2e_ms = 1e3 * (time.perf_counter() - t0) / e2e_steps
    e2e_ms = max_over_ranks(e2e_ms, ws)

    if rank != 0:
        return 0
    pk = peaks()
    roof = wl.roofline(seg_ms, pk)
    line = {"metric": wl.metric, "value": round(value, 2), "unit": wl.unit, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": getattr(wl, "dtype", "f32"),
            "data": "synthetic (seeded procedural scene / queries)",
            "config": wl.config(),
            "e2e": {"value": round(wl.units_per_step() * ws / (e2e_ms * 1e-3), 2), "unit": wl.unit,
                    "h2d_bytes_per_step": wl.h2d_bytes, "d2h_bytes_per_step": wl.d2h_bytes},
            "gpu_launches": launches,
            "roofline": roof, "clocks": clocks}
    if hasattr(wl, "paths_per_step"):
        line["paths_per_s"] = round(wl.paths_per_step() * ws / (ms * 1e-3), 1)
    if hasattr(wl, "fit") and args.fit_steps > 0:
        err = wl.fit(args.fit_steps)
        line["fit"] = {"adam_steps": args.fit_steps, "sigma_a_rel_error_max": round(float(err.max()), 5),
                       "sigma_a_rel_error_mean": round(float(err.mean()), 5), "start": "sigma_a x 0.5 or 1.5"}
    if hasattr(wl, "extras") and type(wl).__name__ == "RenderBenchWorkload" and not args.no_extras:
        line["other_configs"] = wl.extras(pk)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = wl.cpu_baseline(host_threads())
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
