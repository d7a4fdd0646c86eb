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
pipelined frames on the submitting stream, a 256 MiB L2-flush write before
each frame's submission inside the region); `e2e` times the same step
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

N_VERTEX = 1 << 18
MLP_FLOP_W64 = 2 * (209 * 64 + 4 * 64 * 64 + 64 * 3)  # 59,904 per query
BSDF_EVAL_BYTES = 40 + 16
BSDF_SAMPLE_BYTES = 44 + 28


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


# ============================================================ vertex workload
class VertexWorkload:
    name = "vertex"
    dtype = "f32 (BSDF); f16 cache MLP with f32 accumulation"
    metric = "hair-vertex queries/s (BSDF eval + importance sample + cache-MLP inference)"
    unit = "queries/s"

    def __init__(self, torch, n=N_VERTEX):
        import numpy as np
        import hairmsnn_gb300 as hm
        from hairmsnn_gb300 import mlp
        self.torch, self.hm, self.n = torch, hm, n
        self.wo, self.wi, self.t, self.h, self.u = hm.gen_bsdf_queries(0, n)
        rng = np.random.default_rng(0)
        x = np.zeros((n, 16), np.float32)
        x[:, 0:3] = rng.uniform(-1, 1, (n, 3))
        x[:, 3:7] = rng.uniform(0, 1, (n, 4))
        x[:, 7] = rng.uniform(-1, 1, n)
        x[:, 8:11] = [0.06, 0.1, 0.2]
        x[:, 11:13] = 0.3
        self.x_host = torch.from_numpy(x).pin_memory()
        self.x = self.x_host.cuda()
        # the chosen form: FP16 operands on tcgen05 with FP32 accumulation,
        # the encoding fused into the network kernel
        self.net = mlp.TinyMLP("c1_cache_w64.json", 16, 3, precision="fp16", seed=0)
        self.out = torch.empty((n, 3), device="cuda")
        self.net.inference(self.x, self.out)  # packs the FP16 weights once
        self.kernels_per_step = 4  # eval, sample, encode, MLP
        # pinned host copies for the end-to-end leg
        self.host_in = [a.cpu().pin_memory() for a in (self.wo, self.wi, self.t, self.h, self.u)]
        self.h2d_bytes = sum(a.numel() * 4 for a in self.host_in) + self.x_host.numel() * 4
        self.d2h_bytes = (3 * n + n + 3 * n + 3 * n + n) * 4 + n * 3 * 4
        self.host_out = [torch.empty(s, dtype=torch.float32).pin_memory()
                         for s in ((3, n), (n,), (3, n), (3, n), (n,), (n, 3))]

    def step(self, events=None):
        hm = self.hm
        ev = events
        if ev: ev[0].record()
        f, pdf = hm.bsdf_eval(self.wo, self.wi, self.t, self.h)
        if ev: ev[1].record()
        wi2, f2, pdf2 = hm.bsdf_sample(self.wo, self.t, self.h, self.u)
        if ev: ev[2].record()
        self.net.inference(self.x, self.out)
        if ev: ev[3].record()
        return f, pdf, wi2, f2, pdf2

    def e2e_step(self):
        torch = self.torch
        dev = [a.to("cuda", non_blocking=True) for a in self.host_in]
        xd = self.x_host.to("cuda", non_blocking=True)
        f, pdf = self.hm.bsdf_eval(dev[0], dev[1], dev[2], dev[3])
        wi2, f2, pdf2 = self.hm.bsdf_sample(dev[0], dev[2], dev[3], dev[4])
        out = self.net.inference(xd)
        for h, d in zip(self.host_out, (f, pdf, wi2, f2, pdf2, out)):
            h.copy_(d, non_blocking=True)
        torch.cuda.current_stream().synchronize()

    def n_events(self):
        return 4

    def units_per_step(self):
        return self.n

    def roofline(self, seg_ms, pk):
        """seg_ms: mean ms of [eval, sample, mlp]; dominant = the longest."""
        n = self.n
        segs = {
            "bsdf_eval_kernel": ("hbm", BSDF_EVAL_BYTES * n / (seg_ms[0] * 1e-3) / 1e9, pk["hbm_gbs"], "GB/s",
                                 seg_ms[0]),
            "bsdf_sample_kernel": ("hbm", BSDF_SAMPLE_BYTES * n / (seg_ms[1] * 1e-3) / 1e9, pk["hbm_gbs"], "GB/s",
                                   seg_ms[1]),
            "tc_encode_kernel + mlp_tc_fwd_kernel<FP16, 64>": ("tensor", MLP_FLOP_W64 * n / (seg_ms[2] * 1e-3) / 1e12,
                                                                pk["bf16_tflops"], "TFLOP/s", seg_ms[2]),
        }
        name = max(segs, key=lambda k: segs[k][4])
        bound, ach, peak, unit, ms = segs[name]
        return {"kernel": name, "bound": bound, "achieved": round(ach, 3), "peak": peak, "unit": unit,
                "frac": round(ach / peak, 5), "traffic": None,
                "note": f"peak = {pk['source']} ({'HBM copy' if bound == 'hbm' else 'cuBLAS bf16 burst'})",
                "per_kernel_ms": {k: round(v[4], 4) for k, v in segs.items()}}

    workload_name = ("vertex: 2^18 hair-vertex queries, BSDF eval+sample (alpha=2deg, beta_m=beta_n=0.3, "
                     "sigma_a=(0.06,0.1,0.2)) + cache MLP Freq12/OneBlob32/Identity->5x64 FP16 on tcgen05 "
                     "(FP32 accumulation)")

    def config(self):
        return {"workload": self.workload_name,
                "queries": self.n, "l2": "flushed between timed steps (256 MiB write)",
                "parallelism": "replicas"}

    def cpu_baseline(self, threads, budget_s=10.0):
        """Oracle port in C++ on the host threads: BSDF eval + sample and the
        cache network's FP32 inference (hm_oracle_mlp.cpp), bounded sample."""
        from oracle import mlp_oracle as mo
        from oracle import pyoracle as po
        n = 1 << 14
        wo, wi, t, h, u = po.gen_bsdf_queries(0, n)
        cfg = mo.Config(self.net.config_text, 16, 3)
        params = self.net.params()
        x = self.x_host[:n].numpy()
        reps, t0 = 0, time.perf_counter()
        while True:
            po.hair_eval(wo.T, wi.T, t.T, h, threads=threads)
            po.hair_sample(wo.T, t.T, h, u.T, threads=threads)
            po.mlp_forward_host(cfg, params, x, threads=threads)
            reps += 1
            el = time.perf_counter() - t0
            if el > budget_s or reps >= 50:
                break
        return {"value": round(reps * n / el, 1), "unit": self.unit, "cores": threads, "kind": "port",
                "sample": f"{reps} x {n} queries (eval + sample and FP32 MLP inference, C++ on {threads} threads)"}


# ========================================================= precision workload
class PrecisionWorkload:
    """Cache-network precision sweep: 2^20 hair-vertex queries (the vertex
    workload's 16-D inputs), Freq12/OneBlob32/Identity -> 5 hidden layers of
    64 or 128 -> 3, FP32 SIMT against FP16/BF16/E4M3 tensor-core inference
    (FP32 accumulation).  One step = one inference pass of the chosen form
    (FP16, width 64) over the 2^20 queries; the sweep reports every
    precision and width with its error against the FP64 oracle."""
    name = "precision"
    metric = "cache-MLP inference queries/s (2^20 queries, width 64, FP16 tensor cores)"
    unit = "queries/s"
    WIDTHS = (64, 128)
    PRECS = ("fp32", "fp16", "bf16", "fp8")

    def __init__(self, torch, n=1 << 20):
        import numpy as np
        from hairmsnn_gb300 import mlp
        self.torch, self.np, self.mlp, self.n = torch, np, mlp, n
        rng = np.random.default_rng(0)
        x = np.zeros((n, 16), np.float32)
        x[:, 0:3] = rng.uniform(-1, 1, (n, 3))
        x[:, 3:7] = rng.uniform(0, 1, (n, 4))
        x[:, 7] = rng.uniform(-1, 1, n)
        x[:, 8:11] = [0.06, 0.1, 0.2]
        x[:, 11:13] = 0.3
        self.x_np = x
        self.targets = rng.lognormal(0.0, 1.5, (n, 3)).astype(np.float32)
        self.x_host = torch.from_numpy(x).pin_memory()
        self.x = self.x_host.cuda()
        self.out = torch.empty((n, 3), device="cuda")
        self.host_out = torch.empty((n, 3), dtype=torch.float32).pin_memory()
        self.net = mlp.TinyMLP("c1_cache_w64.json", 16, 3, precision="fp16", seed=0)
        self.kernels_per_step = 1
        self.h2d_bytes = n * 16 * 4
        self.d2h_bytes = n * 3 * 4

    def step(self, events=None):
        if events: events[0].record()
        self.net.inference(self.x, self.out)
        if events: events[1].record()

    def e2e_step(self):
        xd = self.x_host.to("cuda", non_blocking=True)
        out = self.net.inference(xd)
        self.host_out.copy_(out, non_blocking=True)
        self.torch.cuda.current_stream().synchronize()

    def n_events(self):
        return 2

    def units_per_step(self):
        return self.n

    @staticmethod
    def flops(width):
        # algorithmic: 209 encoded features, 4 hidden-to-hidden layers, 3 outputs
        return 2 * (209 * width + 4 * width * width + width * 3)

    def _time(self, fn, reps=10):
        torch = self.torch
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        for _ in range(3):
            fn()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in ev:
            flush.fill_(1)
            a.record()
            fn()
            b.record()
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / reps

    def sweep(self, pk):
        np, torch = self.np, self.torch
        from oracle import mlp_oracle as mo
        sub = 8192
        xs = self.x_np[:sub]
        out = {}
        for w in self.WIDTHS:
            cfg = f"c1_cache_w{w}.json"
            ref = None
            for prec in self.PRECS:
                net = self.mlp.TinyMLP(cfg, 16, 3, precision=prec, seed=0)
                if ref is None:
                    oc = mo.Config(net.config_text, 16, 3)
                    ref = mo.forward(oc, net.params().astype(np.float64), xs)[0][:, :3]
                y = torch.empty((self.n, 3), device="cuda")
                ms = self._time(lambda: net.inference(self.x, y))
                tgt = torch.from_numpy(self.targets[:1 << 16]).cuda()
                xin = self.x[:1 << 16]
                tms = self._time(lambda: net.training_step(xin, tgt), reps=5)
                got = y[:sub].cpu().numpy().astype(np.float64)
                err = got - ref
                rms_ref = float(np.sqrt(np.mean(ref ** 2)))
                tf = self.flops(w) * self.n / (ms * 1e-3) / 1e12
                out[f"w{w}_{prec}"] = {
                    "inference_ms": round(ms, 4), "queries_per_s": round(self.n / (ms * 1e-3), 1),
                    "tflops": round(tf, 2), "frac_of_bf16_peak": round(tf / pk["bf16_tflops"], 4),
                    "training_step_ms_2^16": round(tms, 4),
                    "err_rms_rel": float(f"{np.sqrt(np.mean(err ** 2)) / rms_ref:.3e}"),
                    "err_max_rel": float(f"{np.abs(err).max() / rms_ref:.3e}")}
                net.close()
        return out

    def roofline(self, seg_ms, pk):
        ms = seg_ms[0]
        tf = self.flops(64) * self.n / (ms * 1e-3) / 1e12
        return {"kernel": "mlp_tc_fwd_kernel<FP16, 64> (encoding fused)", "bound": "tensor",
                "achieved": round(tf, 3), "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": round(tf / pk["bf16_tflops"], 5), "traffic": None,
                "flop_per_query": self.flops(64),
                "note": f"peak = dense bf16 cuBLAS burst ({pk['source']}); FP16 has the same tensor rate",
                "sweep": self.sweep(pk)}

    def config(self):
        return {"workload": "precision: 2^20 hair-vertex queries, cache MLP Freq12/OneBlob32/Identity (224) -> "
                            "5x64 -> 3, FP16 operands on tcgen05, FP32 accumulation; sweep over widths 64/128 and "
                            "FP32/FP16/BF16/E4M3 with errors against the FP64 oracle on 8192 queries",
                "queries": self.n, "l2": "flushed between timed steps (256 MiB write)",
                "parallelism": "replicas"}

    def cpu_baseline(self, threads, budget_s=10.0):
        np = self.np
        from oracle import mlp_oracle as mo
        oc = mo.Config(self.net.config_text, 16, 3)
        params = self.net.params().astype(np.float64)
        n = 1 << 14
        reps, t0 = 0, time.perf_counter()
        while True:
            mo.forward(oc, params, self.x_np[:n])
            reps += 1
            el = time.perf_counter() - t0
            if el > budget_s or reps >= 50:
                break
        return {"value": round(reps * n / el, 1), "unit": self.unit, "cores": threads, "kind": "port",
                "sample": f"{reps} x {n} queries, FP64 numpy forward of the same network"}


def make_workload(name, torch):
    if name == "vertex":
        return VertexWorkload(torch)
    if name == "precision":
        return PrecisionWorkload(torch)
    if name == "batch":
        from hairmsnn_gb300 import render as _r
        return _r.BatchBenchWorkload(torch)
    if name == "diff":
        from hairmsnn_gb300 import render as _r
        return _r.DiffBenchWorkload(torch)
    if name == "quality":
        from hairmsnn_gb300 import render as _r
        return _r.RenderQualityWorkload(torch)
    from hairmsnn_gb300 import render as _r  # noqa: F401  (render workload)
    return _r.RenderBenchWorkload(torch)


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args):
    """--impl reference: the reference's CPU-side restatement (oracle port) of
    the same workload on all host threads; no GPU work."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np
    from oracle import pyoracle as po
    threads = host_threads()
    n = 1 << 14
    wo, wi, t, h, u = po.gen_bsdf_queries(0, n)
    if args.workload == "vertex":
        from oracle import mlp_oracle as mo
        cfg_text = open(os.path.join(ROOT, "hairmsnn_gb300", "configs", "c1_cache_w64.json")).read()
        cfg = mo.Config(cfg_text, 16, 3)
        params = np.random.default_rng(0).normal(scale=0.1, size=cfg.n_params)
        x = np.random.default_rng(1).uniform(0, 1, (n, 16)).astype(np.float32)

        def step():
            po.hair_eval(wo.T, wi.T, t.T, h, threads=threads)
            po.hair_sample(wo.T, t.T, h, u.T, threads=threads)
            po.mlp_forward_host(cfg, params, x, threads=threads)
        units, metric, unit = n, VertexWorkload.metric, VertexWorkload.unit
        sample = f"{n} queries per step (oracle port: BSDF and FP32 MLP inference in C++ on {threads} threads)"
        cfgd = {"workload": VertexWorkload.workload_name, "sample": "bounded: queries_per_step of the workload",
                "queries_per_step": n}
    else:
        from hairmsnn_gb300 import build as hb
        from hairmsnn_gb300 import render as hr
        hb.build()
        cfg = hr.straight_hair_scene(512, 512)
        scene = hr.Scene(cfg)  # host-only parse + generation
        osc = po.OracleScene.from_library(scene)
        P, R = 512 * 512, 1 << 16
        n = 8192
        state = {"p0": (256 * 512), "frame": 0}

        def step():
            osc.render_pixels(1, beta=1, accum_id=state["frame"], every_nth=P // R, n_train=R, p0=state["p0"], n=n,
                              threads=threads)
            state["p0"] = (state["p0"] + n) % (P - n)
            state["frame"] += 1
        units = n
        metric, unit = hr.RenderBenchWorkload.metric, hr.RenderBenchWorkload.unit
        sample = (f"{n} pixels (1 spp) per step of the 512x512 render: the reference's per-pixel path code "
                  f"(rayGenCam / msnnPathTrace / msnnTrainingPath, oracle port) on {threads} threads; "
                  f"cache network not included")
        cfgd = {"workload": hr.RenderBenchWorkload.workload_name,
                "sample": "bounded: pixels_per_step of the frame per step", "pixels_per_step": n}
    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = units / (ms * 1e-3)
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
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("HM_BENCH_WORKLOAD", "render"),
                    choices=["render", "vertex", "precision", "quality", "batch", "diff"])
    ap.add_argument("--fit-steps", type=int, default=200,
                    help="diff workload: Adam steps of the sigma_a recovery reported after the timing")
    ap.add_argument("--no-cpu-baseline", action="store_true")
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
    wl = make_workload(args.workload, torch)
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
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = wl.cpu_baseline(host_threads())
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
