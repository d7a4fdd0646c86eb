"""Workloads of bench.py (benchmark harness, not part of the shipped package).

Each workload times one step of the HairMSNN hot path on the GPU through the
library's public API and, for its `cpu_baseline` leg only, runs the oracle
(oracle/, the CPU restatement of the reference's algorithm) on the host
cores.  The shipped package hairmsnn_gb300/ never imports the oracle.

  render     one 512x512 frame (1 spp) of the full HairMSNN render
  vertex     2^18 hair-vertex queries: BSDF eval + sample + cache inference
  precision  cache-network inference, FP32/FP16/BF16/E4M3 sweep at 2^20
  quality    relMSE of HairMSNN / NRC / PT at 16 spp vs a converged reference
  batch      64 uneven curly-hair scenes rendered as one
  diff       path-replay gradient of an image loss (appearance fit)
"""
import json
import os
import statistics
import time

import numpy as np

from hairmsnn_gb300.render import (IMAGE_CACHE, IMAGE_FINAL, IMAGE_SHORT, MSNN, NRC, PT, BatchRenderer, Renderer,
                                   Scene, _default_cache_config, batch_scene_configs, curly_hair_diff_scene,
                                   diff_materials, relmse, straight_hair_scene)

ROOT = os.path.dirname(os.path.abspath(__file__))
N_VERTEX = 1 << 18
MLP_FLOP_W64 = 2 * (209 * 64 + 4 * 64 * 64 + 64 * 3)  # 59,904 per query
BSDF_EVAL_BYTES = 40 + 16
BSDF_SAMPLE_BYTES = 44 + 28


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
        self.kernels_per_step = 3  # eval, sample, cache network (warp-specialised: encoding overlapped)
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
            "mlp_tc_fused_kernel<FP16, 64>": ("tensor", MLP_FLOP_W64 * n / (seg_ms[2] * 1e-3) / 1e12,
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
        return {"kernel": "mlp_tc_fused_kernel<FP16, 64> (warp-specialised: encoding overlapped with the layers)",
                "bound": "tensor",
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


RAY_RECORD_BYTES = 32 + 16   # ray (origin, direction as float4 pairs) + hit record
NODE_BYTES = 224              # one 8-wide BVH node: eight child boxes + child codes
PRIM_BYTES = 64               # one segment's 4 control points (or a triangle's vertex data)
# DRAM bytes per ray of the shadow-ray traversal launch timed by
# RenderBenchWorkload.shadow_launch (one launch over a 512x512 frame's shadow
# rays), and the counters that bind it, from one ncu capture of that launch
# (profiles/shadow_trace_launch_512.md).
SHADOW_DRAM_BYTES_PER_RAY = 340  # 193.0 MB for 568,386 rays
SHADOW_NCU_COUNTERS = {"lanes_active_per_instruction": 12.9, "issue_active_pct": 46.4,
                       "alu_pipe_active_pct": 42.3, "l1tex_throughput_pct": 63.2, "warps_active_pct": 33.5,
                       "long_scoreboard_stalls_per_issue": 6.39, "l2_hit_rate_pct": 87.3,
                       "dram_throughput_pct": 3.3,
                       "source": "profiles/shadow_trace_launch_512.md (ncu --set full, cold caches)"}


class RenderBenchWorkload:
    """bench.py workload: one frame (1 spp) of the full HairMSNN render per
    step, in the chosen form: FP16 cache network on the tensor cores
    (training and inference), frames in flight, graph replay, autotuned
    launch shapes, two BVH leaves per segment."""

    name = "render"
    metric = "paths/s (HairMSNN full wavefront render, 512x512, 1 spp/frame, online cache training 2^16/frame)"
    unit = "paths/s"
    cache_precision = 1  # FP16 (tcgen05); its relMSE equals the FP32 cache's (quality workload)
    dtype = "f32 (traversal, shading, FP64 sums); f16 cache MLP with f32 accumulation"

    def __init__(self, torch, width=512, height=512, train_records=1 << 16, frames_in_flight=0):
        self.torch = torch
        self.width, self.height, self.train_records = width, height, train_records
        self.frames_in_flight = frames_in_flight
        self.cfg = straight_hair_scene(width, height)
        self.scene = Scene(self.cfg)
        self.scene.build()
        self.r = Renderer(self.scene, MSNN, beta=1, train_records=train_records, train=True,
                          precision=self.cache_precision, frames_in_flight=frames_in_flight)
        self.tuning = self.r.autotune(frames=16)  # 6 frames per candidate picked less stable shapes (4% slower)
        self.P = width * height
        self.h2d_bytes = 0
        self.d2h_bytes = self.P * 3 * 8
        self.stage_ms = []
        self.launches = []
        self.read_stream = torch.cuda.Stream()
        self.host_sums = [torch.empty((height, width, 3), dtype=torch.float64, pin_memory=True) for _ in range(2)]

    def step(self, events=None):
        """One frame enqueued (frames run pipelined on the renderer's own streams)."""
        self.r.frame()
        self.launches.append(self.r.timings().kernel_launches)

    def timed_region(self, steps, flush):
        """Device time of `steps` pipelined frames: an event on the submitting
        stream before the first frame, the renderer's completion joined back
        (hm_render_wait) before the closing event.  No L2 flush: every frame
        streams its own path state (about 90 MB per frame in flight at
        512x512, several frames in flight) past the 129 MB L2, and a flush
        kernel on the submitting stream would run beside the frames in
        flight rather than between them."""
        torch = self.torch
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for k in range(steps):
            self.step()
        self.r.wait()
        t1.record()
        torch.cuda.synchronize()
        self.last_ms = t0.elapsed_time(t1) / steps
        return self.last_ms

    @property
    def kernels_per_step(self):
        return int(round(np.mean(self.launches[-8:]))) if self.launches else 0

    def e2e_region(self, steps):
        """Wall time per frame through the public API with the result read back
        every frame: hm_render_frame, then hm_render_read_async of the FP64
        image sums into pinned host memory on a separate stream (the next
        frame's accumulation waits for that copy); host synchronisation at
        both ends."""
        import time
        torch = self.torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(steps):
            self.r.frame()
            self.r.read_async(self.host_sums[k & 1], IMAGE_FINAL, stream=self.read_stream)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        self.host_img = self.host_sums[(steps - 1) & 1].numpy() / self.r.stats().frames
        return 1e3 * el / steps

    def e2e_step(self):
        self.r.frame()
        self.r.read_async(self.host_sums[0], IMAGE_FINAL, stream=self.read_stream)

    def n_events(self):
        return 2

    def units_per_step(self):
        return self.P

    def profile_frames(self, n=4):
        """Synchronous instrumented frames (per-stage CUDA events on the frame's
        stream) for the stage breakdown and the roofline."""
        self.r.instrument(timing=True, counting=False)
        for _ in range(n):
            self.r.frame()
            self.stage_ms.append(self.r.timings().as_dict())
        self.r.instrument(timing=False, counting=False)

    def counted_frame(self):
        """One untimed frame with traversal work counters."""
        self.r.instrument(timing=True, counting=True)
        self.r.frame()
        t = self.r.timings()
        self.r.instrument(timing=False, counting=False)
        return t

    def plain_form(self, frames=20):
        if getattr(self, "_plain_ms", None) is None:
            self._plain_ms = self._plain_form(frames)
        return self._plain_ms

    def _plain_form(self, frames=20):
        """The plain FP32 wavefront form on the same scene and GPU: FP32 cache,
        one frame in flight, kernel-by-kernel launches, default launch
        shapes, one BVH leaf per segment.  Pipelined frame time."""
        torch = self.torch
        cfg = dict(self.cfg)
        cfg["integrator"] = dict(cfg["integrator"], segment_splits=1)
        sc = Scene(cfg)
        r = Renderer(sc, MSNN, beta=1, train_records=self.train_records, train=True, precision=0,
                     frames_in_flight=1)
        r.set_graphs(False)
        for _ in range(3):
            r.frame()
        r.wait()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(frames):
            r.frame()
        r.wait()
        t1.record()
        torch.cuda.synchronize()
        ms = t0.elapsed_time(t1) / frames
        r.close()
        sc.close()
        return ms

    def shadow_launch(self, pk, reps=5):
        """The dominant kernel timed alone, in the same process: one launch of
        the persistent any-hit traversal (the shadow-ray stage's kernel, fed
        from a ray array) over every shadow ray of one 512x512 frame of this
        workload, in the frame's order (bounce by bounce, light samples, then
        BSDF samples, pixel order).  The rays come from the per-path ray log
        of a frame rendered with one frame in flight, whose traversal work
        counters count exactly these rays; CUDA events on the launching
        stream, a 256 MiB write before each launch flushes L2.  Algorithmic
        bytes = rays x 48 B + 8-wide nodes visited x 224 B + primitives
        tested x 64 B."""
        torch = self.torch
        r = Renderer(self.scene, MSNN, beta=1, train_records=self.train_records, train=True,
                     precision=self.cache_precision, frames_in_flight=1)
        vertices = self.scene.info().path_v2 + 1
        r.set_path_log(vertices)
        r.instrument(timing=True, counting=True)
        r.frame()
        c = r.timings()
        log = r.read_path_log()
        r.close()
        kind = log[:, :, 7].view(np.int32)
        order = []
        for k in range(vertices):
            for kd in (1, 2):
                order.append(np.nonzero(kind[:, 3 * k + kd] == kd)[0] * log.shape[1] + 3 * k + kd)
        idx = np.concatenate(order)
        flat = log.reshape(-1, 12)[idx]
        # the frame's extension rays (vertex by vertex, pixel order) for the closest-hit launch
        eidx = np.concatenate([np.nonzero(kind[:, 3 * k] == 0)[0] * log.shape[1] + 3 * k for k in range(vertices)])
        eflat = log.reshape(-1, 12)[eidx]
        del log
        vis = flat[:, 0].view(np.int32)
        org = torch.from_numpy(np.ascontiguousarray(flat[:, 8:11])).cuda()
        dirs = torch.from_numpy(np.ascontiguousarray(flat[:, 4:7])).cuda()
        n = len(flat)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        hits = self.scene.trace(org, dirs, any_hit=True)
        same = float(((hits[:, 1].cpu().numpy().view(np.int32) < 0) == (vis == 1)).mean())
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for k, (a, b) in enumerate(ev):
            flush.fill_(k & 0xFF)
            a.record()
            self.scene.trace(org, dirs, any_hit=True)
            b.record()
        torch.cuda.synchronize()
        ms = statistics.median(a.elapsed_time(b) for a, b in ev)
        alg = n * RAY_RECORD_BYTES + c.shadow_nodes * NODE_BYTES + c.shadow_prims * PRIM_BYTES
        ach = alg / (ms * 1e-3) / 1e9
        # the other traversal kernel, the same way: the frame's extension rays in one closest-hit launch
        eorg = torch.from_numpy(np.ascontiguousarray(eflat[:, 8:11])).cuda()
        edir = torch.from_numpy(np.ascontiguousarray(eflat[:, 4:7])).cuda()
        ehits = self.scene.trace(eorg, edir, any_hit=False)
        esame = float((ehits[:, 1].cpu().numpy().view(np.int32) == eflat[:, 0].view(np.int32)).mean())
        for k, (a, b) in enumerate(ev):
            flush.fill_(k & 0xFF)
            a.record()
            self.scene.trace(eorg, edir, any_hit=False)
            b.record()
        torch.cuda.synchronize()
        ems = statistics.median(a.elapsed_time(b) for a, b in ev)
        ealg = len(eflat) * RAY_RECORD_BYTES + c.extend_nodes * NODE_BYTES + c.extend_prims * PRIM_BYTES
        extension = {"kernel": "persistent_trace_kernel<closest hit> (extension rays of the same frame, one launch)",
                     "launch_ms": round(ems, 4), "rays": len(eflat), "algorithmic_bytes": int(ealg),
                     "achieved": round(ealg / (ems * 1e-3) / 1e9, 2),
                     "frac": round(ealg / (ems * 1e-3) / 1e9 / pk["hbm_gbs"], 4),
                     "hit_primitive_equal_to_frame": round(esame, 6),
                     "per_ray": {"nodes": round(c.extend_nodes / max(1, c.extension_rays), 2),
                                 "prims": round(c.extend_prims / max(1, c.extension_rays), 2)}}
        return {"kernel": "persistent_trace_kernel<any hit> (shadow rays of one frame, one launch)",
                "bound": "hbm", "achieved": round(ach, 2), "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": round(ach / pk["hbm_gbs"], 4),
                "traffic": int(n * SHADOW_DRAM_BYTES_PER_RAY),
                "traffic_basis": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of this launch "
                                  f"({SHADOW_DRAM_BYTES_PER_RAY} B per ray), scaled by the rays"),
                "launch_ms": round(ms, 4), "rays": n, "rays_counted_in_frame": int(c.shadow_rays),
                "visibility_equal_to_frame": round(same, 6),
                "algorithmic_bytes": int(alg),
                "per_ray": {"nodes": round(c.shadow_nodes / max(1, c.shadow_rays), 2),
                            "prims": round(c.shadow_prims / max(1, c.shadow_rays), 2)},
                "binding_counters": SHADOW_NCU_COUNTERS,
                "extension_launch": extension,
                "note": ("algorithmic bytes as in the frame's counted shadow stage; the 90 MB BVH and 10 MB of "
                         "curves are mostly L2-resident, so the DRAM traffic is far below them; the bound is the "
                         "latency of the node loads with a third of the warp slots occupied and the L1 the busiest "
                         "unit (binding_counters); peak = HBM copy ("
                         + pk["source"] + ")")}

    def roofline(self, seg_ms, pk):
        keys = ["extend_ms", "shade_ms", "shadow_ms", "compact_ms", "train_ms", "infer_ms", "compose_ms",
                "camera_ms", "finalize_ms"]
        if not self.stage_ms:
            self.profile_frames()
        n = max(1, min(len(self.stage_ms), 16))
        mean = {k: float(np.mean([s[k] for s in self.stage_ms[-n:]])) for k in keys}
        out = {"stage_ms_per_frame_synchronous": {k: round(v, 4) for k, v in mean.items()},
               "stage_note": "synchronous instrumented frames (one frame at a time), after the timed region; "
                             "the timed frames overlap eight at a time"}
        out.update(self.shadow_launch(pk))
        if type(self) is RenderBenchWorkload:
            plain = self.plain_form()
            chosen = self.last_ms if getattr(self, "last_ms", None) else None
            out["plain_fp32_wavefront_form"] = {
                "ms_per_frame": round(plain, 3), "paths_per_s": round(self.P / (plain * 1e-3), 1),
                "chosen_form_speedup": round(plain / chosen, 3) if chosen else None,
                "what": "FP32 cache, 1 frame in flight, kernel-by-kernel launches, default launch shapes, "
                        "1 BVH leaf per segment; same scene and GPU"}
        return out

    def _frame_ms(self, r, frames=20):
        torch = self.torch
        for _ in range(3):
            r.frame()
        r.wait()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(frames):
            r.frame()
        r.wait()
        t1.record()
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / frames

    def _timed_frames(self, r, n):
        torch = self.torch
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(n):
            r.frame()
        r.wait()
        t1.record()
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / n

    def quality(self, spp=None, ref_spp=None, pretrain_passes=None):
        """relMSE at `spp` of HairMSNN (each cache precision), PT, NRC and
        HairMSNN after scene-sample training, against a converged PT image of
        the same scene (frames 16 .. 16 + ref_spp of one PT run); frame times
        and the PT sample count needed for the same error."""
        spp = spp or getattr(self, "spp", 16)
        ref_spp = ref_spp or getattr(self, "ref_spp", 1024)
        pretrain_passes = pretrain_passes or getattr(self, "pretrain_passes", 256)
        pt = Renderer(self.scene, PT, frames_in_flight=self.frames_in_flight)
        pt_ms = self._timed_frames(pt, spp)
        pt_img = pt.read(IMAGE_FINAL)
        ref_ms = self._timed_frames(pt, ref_spp)
        total = pt.read(IMAGE_FINAL) * (spp + ref_spp)
        ref = (total - pt_img * spp) / ref_spp
        pt.close()
        by_prec = {}
        for name, prec in (("fp32", 0), ("fp16", 1), ("bf16", 2), ("fp8", 3)):
            ms = Renderer(self.scene, MSNN, beta=1, train_records=self.train_records, train=True,
                          precision=prec, frames_in_flight=self.frames_in_flight)
            t_ms = self._timed_frames(ms, spp)
            img = ms.read(IMAGE_FINAL)
            ms.close()
            by_prec[name] = {"relmse": round(relmse(img, ref), 6), "ms_per_frame": round(t_ms, 3)}
            if name == "fp32":
                ms_ms, ms_img = t_ms, img
        # the reference's initial training before the first frame (one second
        # of scene-sample passes there; a fixed pass count here)
        ms = Renderer(self.scene, MSNN, beta=1, train_records=self.train_records, train=True,
                      frames_in_flight=self.frames_in_flight)
        torch = self.torch
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        ms.pretrain(pretrain_passes)
        t1.record()
        torch.cuda.synchronize()
        pre_ms = t0.elapsed_time(t1)
        t_pre = self._timed_frames(ms, spp)
        e_pre = relmse(ms.read(IMAGE_FINAL), ref)
        ms.close()
        # the reference's comparison renderer: NRC with online training
        # (65536 records per frame, c = 0.01), same frames
        nrc = Renderer(self.scene, NRC, train=True, frames_in_flight=self.frames_in_flight)
        nrc_ms = self._timed_frames(nrc, spp)
        e_nrc = relmse(nrc.read(IMAGE_FINAL), ref)
        nrc.close()
        e_pt, e_ms = relmse(pt_img, ref), relmse(ms_img, ref)
        eq_spp = spp * e_pt / e_ms
        return {"spp": spp, "reference_spp": ref_spp, "reference_ms_per_frame": round(ref_ms, 3),
                "msnn": {"relmse": round(e_ms, 6), "ms_per_frame": round(ms_ms, 3),
                         "paths_per_s": round(self.P / (ms_ms * 1e-3), 1)},
                "pt": {"relmse": round(e_pt, 6), "ms_per_frame": round(pt_ms, 3),
                       "paths_per_s": round(self.P / (pt_ms * 1e-3), 1)},
                "nrc": {"relmse": round(e_nrc, 6), "ms_per_frame": round(nrc_ms, 3),
                        "paths_per_s": round(self.P / (nrc_ms * 1e-3), 1),
                        "pt_spp_for_same_relmse": round(spp * e_pt / e_nrc, 2),
                        "speedup_at_equal_relmse": round((spp * e_pt / e_nrc) * pt_ms / (spp * nrc_ms), 3)},
                "msnn_by_cache_precision": by_prec,
                "msnn_after_scene_sample_training": {
                    "passes": pretrain_passes, "training_ms": round(pre_ms, 1), "relmse": round(e_pre, 6),
                    "ms_per_frame": round(t_pre, 3), "pt_spp_for_same_relmse": round(spp * e_pt / e_pre, 2),
                    "speedup_at_equal_relmse": round((spp * e_pt / e_pre) * pt_ms / (spp * t_pre), 3)},
                "pt_spp_for_msnn_relmse": round(eq_spp, 2),
                "speedup_at_equal_relmse": round(eq_spp * pt_ms / (spp * ms_ms), 3)}

    def extras(self, pk):
        """The other configurations' figures, measured in the same run: the
        2^18-query vertex batch (BSDF eval + sample + FP16 cache inference)
        with its kernels' rooflines, the cache precision sweep at 2^20
        queries (time, TFLOP/s, training step, error against the FP64
        oracle), the equal-accuracy comparison of the chosen and plain forms
        (relMSE at 16 spp against a converged PT image), the ablation of the
        chosen form, the 64-scene batch and the differentiable fit's
        gradient evaluation."""
        torch = self.torch
        out = {}
        vw = VertexWorkload(torch)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        for _ in range(3):
            vw.step()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(vw.n_events())] for _ in range(10)]
        for k, ev in enumerate(evs):
            flush.fill_(k & 0xFF)
            vw.step(ev)
        torch.cuda.synchronize()
        seg = [statistics.mean(ev[i].elapsed_time(ev[i + 1]) for ev in evs) for i in range(vw.n_events() - 1)]
        step_ms = statistics.mean(ev[0].elapsed_time(ev[-1]) for ev in evs)
        out["vertex_2^18"] = {"queries_per_s": round(vw.n / (step_ms * 1e-3), 1), "ms_per_step": round(step_ms, 4),
                              "roofline": vw.roofline(seg, pk), "workload": vw.workload_name}
        pw = PrecisionWorkload(torch)
        out["precision_2^20"] = pw.sweep(pk)
        out["quality_16spp"] = self.quality(16, 1024, 256)
        plain = self.plain_form()
        q = out["quality_16spp"]
        out["equal_accuracy"] = {
            "chosen_form": {"relmse": q["msnn_by_cache_precision"]["fp16"]["relmse"],
                            "ms_per_frame": round(self.last_ms, 3) if getattr(self, "last_ms", None) else None},
            "plain_fp32_form": {"relmse": q["msnn_by_cache_precision"]["fp32"]["relmse"],
                                "ms_per_frame": round(plain, 3)},
            "relmse_ratio_chosen_to_plain": round(q["msnn_by_cache_precision"]["fp16"]["relmse"]
                                                  / q["msnn_by_cache_precision"]["fp32"]["relmse"], 4),
            "speedup": round(plain / self.last_ms, 3) if getattr(self, "last_ms", None) else None}
        out["ablation"] = self.ablation()
        out["batch_64_scenes"] = self.batch_extra()
        out["diff_gradient"] = self.diff_extra()
        return out

    def batch_extra(self, warmup=2, frames=5):
        """The 64-scene batch (BatchBenchWorkload): pipelined frames timed with
        CUDA events, then the same through the public API with the image
        sums read back every frame."""
        torch = self.torch
        import time
        t0 = time.perf_counter()
        bw = BatchBenchWorkload(torch)
        for _ in range(warmup):
            bw.step()
        bw.r.wait()
        ms = bw.timed_region(frames, None)
        e2e_ms = bw.e2e_region(max(2, frames // 2))
        out = {"metric": bw.metric, "paths_per_s": round(bw.P / (ms * 1e-3), 1), "ms_per_frame": round(ms, 3),
               "e2e_paths_per_s": round(bw.P / (e2e_ms * 1e-3), 1), "frames": frames, **bw.stats_scenes,
               "launch_shapes": {k: v for k, v in bw.tuning.items() if k != "ms_per_frame"},
               "scene_setup_s": round(bw.setup_s, 1), "total_s": round(time.perf_counter() - t0, 1)}
        bw.r.close()
        del bw
        torch.cuda.synchronize()
        return out

    def diff_extra(self, warmup=1, steps=3):
        """The differentiable-fit workload (DiffBenchWorkload): gradient
        evaluations timed with CUDA events (no Adam fit here)."""
        torch = self.torch
        import time
        t0 = time.perf_counter()
        dw = DiffBenchWorkload(torch)
        for _ in range(warmup):
            dw.step()
        ms = dw.timed_region(steps, None)
        e2e_ms = dw.e2e_region(2)
        g = dw.last_grad
        out = {"metric": dw.metric, "evaluations_per_s": round(1e3 / ms, 4), "ms_per_evaluation": round(ms, 2),
               "e2e_evaluations_per_s": round(1e3 / e2e_ms, 4),
               "paths_per_s": round(dw.paths_per_step() / (ms * 1e-3), 1), "steps": steps,
               "gradient_finite": bool(np.isfinite(g).all()), "total_s": round(time.perf_counter() - t0, 1)}
        dw.r.close()
        del dw
        torch.cuda.synchronize()
        return out

    def ablation(self):
        """Which choice gives the speed-up: the chosen form with one factor
        changed at a time (same scene, same GPU, pipelined frames)."""
        out = {}
        variants = [("chosen", {}), ("fp32_cache", {"precision": 0}), ("one_frame_in_flight", {"fif": 1}),
                    ("no_graph_replay", {"graphs": False}), ("one_leaf_per_segment", {"split": 1}),
                    ("untuned_launch_shapes", {"tune": False})]
        scenes = {2: self.scene}
        for name, v in variants:
            split = v.get("split", 2)
            if split not in scenes:
                cfg = dict(self.cfg)
                cfg["integrator"] = dict(cfg["integrator"], segment_splits=split)
                scenes[split] = Scene(cfg)
            r = Renderer(scenes[split], MSNN, beta=1, train_records=self.train_records, train=True,
                         precision=v.get("precision", self.cache_precision),
                         frames_in_flight=v.get("fif", self.frames_in_flight))
            if v.get("tune", True):
                r.autotune(frames=16)
            r.set_graphs(v.get("graphs", True))
            ms = self._frame_ms(r)
            out[name] = {"ms_per_frame": round(ms, 3), "paths_per_s": round(self.P / (ms * 1e-3), 1)}
            r.close()
        base = out["chosen"]["ms_per_frame"]
        for name in out:
            out[name]["slowdown_vs_chosen"] = round(out[name]["ms_per_frame"] / base, 3)
        return out

    workload_name = ("render: straight procedural hair 10k strands x 64 B-spline CPs (610k segments, 2 BVH "
                     "leaves each), 20k-tri head, Preetham sky T=3 + directional (3,3,3), 512x512, "
                     "path_v1=1, path_v2=40, BETA=1, cache HashGrid/OneBlob MLP 64x2 in FP16 on tcgen05 "
                     "(training and inference; FP32 master weights), 2^16 training records/frame")

    def config(self):
        return {"workload": self.workload_name,
                "cache_precision": "fp16" if self.cache_precision == 1 else "fp32",
                "pixels": self.P, "train_records": self.train_records,
                "l2": "inputs larger than L2: each frame in flight streams its own ~90 MB path state, with "
                      "several frames in flight, past the 129 MB L2 (scene: 8-wide BVH 90 MB + curves 10 MB); "
                      "no flush kernel",
                "frames_in_flight": self.r.depth(),
                "launch_shapes": {k: v for k, v in self.tuning.items() if k != "ms_per_frame"},
                "parallelism": "replicas"}

    def cpu_baseline(self, threads, budget_s=20.0):
        """The per-frame work of the render on the host cores (CpuFrameSample,
        the oracle alone), over a bounded sample of the frame's pixels."""
        cpu = CpuFrameSample(self.cfg, self.train_records, threads)
        t0 = time.perf_counter()
        done = 0
        while time.perf_counter() - t0 < budget_s:
            done += cpu.step()
        el = time.perf_counter() - t0
        return {"value": round(done / el, 1), "unit": self.unit, "cores": threads, "kind": "port",
                "sample": f"{done} pixels (1 spp) of the same frame, in bands of {cpu.n}: {cpu.what}"}


class CpuFrameSample:
    """One frame's HairMSNN work per pixel on the host, with the oracle alone
    (no shipped library): the scene from the oracle's procedural generator
    (the same arrays as the library's), the reference's G-buffer pass
    (rayGenCam / msnnPathTrace / msnnTrainingPath, the oracle's C++
    restatement pinned to the reference's own integrator), the cache's
    inference over the pixels and its training gradient over the training
    pixels' records (the oracle's C++ FP32 transcription of the network).
    Each step renders the next band of `n` pixels of the frame (wrapping
    around, frame number advancing), so successive steps cover the whole
    frame in proportion."""

    def __init__(self, cfg, train_records, threads, n=16384):
        from oracle import mlp_oracle as mo
        from oracle import pyoracle as po
        self.po, self.threads, self.n = po, threads, n
        self.o = po.procedural_scene(cfg)
        self.P = self.o.width * self.o.height
        self.R = train_records
        self.every = max(1, self.P // train_records)
        text = open(os.path.join(ROOT, "hairmsnn_gb300", "configs", "hairmsnn_cache.json")).read()
        self.oc = mo.Config(text, 12, 3)
        self.params = np.random.default_rng(0).normal(scale=0.05, size=self.oc.n_params)
        self.p0 = 0
        self.frame = 0
        self.what = (f"oracle rayGenCam / msnnPathTrace / msnnTrainingPath (C++) + the cache's inference over the "
                     f"band and its training gradient over the band's training records (C++ FP32), "
                     f"{threads} threads; scene from the oracle's own generator")

    def step(self):
        po, n = self.po, min(self.n, self.P - self.p0)
        col, nn_in, tr, fl = self.o.render_pixels(1, beta=1, accum_id=self.frame, every_nth=self.every,
                                                  n_train=self.R, p0=self.p0, n=n, threads=self.threads)
        po.mlp_forward_host(self.oc, self.params, nn_in, threads=self.threads)
        tmask = (fl & 4) != 0
        if tmask.any():
            po.mlp_grad_host(self.oc, self.params, nn_in[tmask], tr[tmask], threads=self.threads)
        self.p0 += n
        if self.p0 >= self.P:
            self.p0, self.frame = 0, self.frame + 1
        return n


class RenderQualityWorkload(RenderBenchWorkload):
    """HairMSNN (BETA=1, online cache training) against plain path tracing and
    the reference's NRC comparison renderer (online training, 65536 records
    per frame) on the render workload's scene: relMSE of each at 16 spp against a
    converged PT reference of the same scene, their frame times, and the PT
    sample count (and time) needed to reach HairMSNN's relMSE, assuming PT's
    relMSE falls as 1/spp (it is unbiased).  The reference uses frames
    16 .. 16 + ref_spp of one PT run, so it shares no random numbers with
    the 16-spp estimates (the path RNG is seeded by the frame index, as in
    the reference).  The HairMSNN relMSE is also reported with the cache's
    inference in FP16, BF16 and E4M3 on the tensor cores (training FP32).
    One step = one HairMSNN frame, as the render workload."""

    name = "quality"
    metric = "paths/s at fixed relMSE vs PT (HairMSNN BETA=1, 512x512, 16 spp, online cache training 2^16/frame)"

    def __init__(self, torch, width=512, height=512, train_records=1 << 16, spp=16, ref_spp=1024,
                 pretrain_passes=256):
        super().__init__(torch, width, height, train_records)
        self.spp, self.ref_spp, self.pretrain_passes = spp, ref_spp, pretrain_passes

    def roofline(self, seg_ms, pk):
        out = super().roofline(seg_ms, pk)
        out["quality"] = self.quality()
        return out

    def config(self):
        c = super().config()
        c["workload"] = "quality: " + c["workload"] + f"; relMSE at {self.spp} spp vs PT {self.ref_spp} spp"
        return c



class BatchBenchWorkload(RenderBenchWorkload):
    """bench.py workload: one frame (1 spp) of each of 64 uneven scenes,
    rendered as one batch with one shared FP32 cache network (width 64)."""

    dtype = "f32"

    name = "batch"
    metric = "paths/s (64 concurrent HairMSNN scenes, 128^2..1024^2, 2k-50k curly strands, one shared cache)"
    unit = "paths/s"

    def __init__(self, torch, n_scenes=64, train_records=1 << 16):
        import time
        self.torch = torch
        self.train_records = train_records
        t0 = time.perf_counter()
        cfgs, self.betas = batch_scene_configs(n_scenes)
        self.scenes = [Scene(c) for c in cfgs]
        for sc in self.scenes:
            sc.build()
        self.setup_s = time.perf_counter() - t0
        self.r = BatchRenderer(self.scenes, MSNN, betas=self.betas, train_records=train_records, train=True)
        self.tuning = self.r.autotune(frames=1)
        self.P = self.r.pixels
        self.h2d_bytes = 0
        self.d2h_bytes = self.P * 3 * 8
        self.stage_ms = []
        self.launches = []
        self.read_stream = torch.cuda.Stream()
        self.host_sums = [torch.empty((self.P, 3), dtype=torch.float64, pin_memory=True) for _ in range(2)]
        self.n_scenes = n_scenes
        infos = [sc.info() for sc in self.scenes]
        self.stats_scenes = {"pixels": self.P, "segments": int(sum(i.n_segments for i in infos)),
                             "strands": int(sum(i.n_strands for i in infos))}

    def e2e_region(self, steps):
        import time
        torch = self.torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(steps):
            self.r.frame()
            self.r.read_async(self.host_sums[k & 1], IMAGE_FINAL, stream=self.read_stream)
        torch.cuda.synchronize()
        return 1e3 * (time.perf_counter() - t0) / steps

    def config(self):
        return {"workload": f"batch: {self.n_scenes} scenes (seeded), sides 128/256/512/1024, log-uniform 2k-50k "
                            "curly strands (helix r 2-8 mm, pitch 5-20 mm, 48-128 CPs), BETA 0..10, sigma_a "
                            "U[0.02,0.5]^3, one shared FP32 cache (HashGrid/OneBlob MLP 64x2), 2^16 records/frame",
                **self.stats_scenes, "frames_in_flight": self.r.depth(), "scene_setup_s": round(self.setup_s, 1),
                "launch_shapes": {k: v for k, v in self.tuning.items() if k != "ms_per_frame"},
                "l2": "inputs larger than L2 (path state of tens of millions of paths); no flush kernel",
                "parallelism": "replicas"}

    def cpu_baseline(self, threads, budget_s=20.0):
        return {"value": None, "unit": self.unit, "cores": threads, "kind": "port",
                "sample": "not run for the batch workload (see the render workload's CPU baseline)"}



class DiffBenchWorkload:
    """bench.py workload: one gradient evaluation per step of the
    differentiable appearance fit.  A step renders 64 frames (1 spp each) of
    20k curly strands at 256x256, HairMSNN with BETA=2 and the cache frozen
    (hm_render_diff_forward), forms the L2 image loss against a target
    rendered at the true materials, and replays the paths
    (hm_render_diff_backward) for dL/d(sigma_a, beta_m, beta_n, alpha) of 4
    strand groups and dL/dW of the cache.  The target is rendered once with
    the same frame seeds; the materials start with sigma_a 50% off."""

    name = "diff"
    metric = ("gradient evaluations/s (path replay: dL/d(material) of 4 strand groups + dL/dW, 20k curly strands, "
              "256x256, 64 spp, BETA=2)")
    unit = "gradient evaluations/s"

    def __init__(self, torch, width=256, height=256, spp=64, strands=20000, groups=4, pretrain_passes=64):
        self.torch = torch
        self.width, self.height, self.spp, self.groups = width, height, spp, groups
        self.cfg, self.truth = curly_hair_diff_scene(width, height, strands=strands, groups=groups)
        self.scene = Scene(self.cfg)
        self.scene.build()
        self.scene.set_group_materials(self.truth)
        self.r = Renderer(self.scene, MSNN, beta=2, train_records=1 << 14, train=True)
        self.tuning = self.r.autotune(frames=4)
        self.r.pretrain(pretrain_passes)
        self.P = width * height
        self.n = self.P * 3
        self.r.diff_forward(spp)
        self.target = (self.r.device_sums(5) / spp).clone()
        self.target_host = self.target.cpu().numpy()
        self.start = self.truth.copy()
        self.start[:, 0:3] *= np.where(np.random.default_rng(11).random((groups, 3)) < 0.5, 0.5, 1.5)
        self.scene.set_group_materials(self.start)
        self.h2d_bytes = self.P * 3 * 4
        self.d2h_bytes = self.P * 3 * 8 + groups * 6 * 8
        self.launches = []
        self.adj_host = torch.empty((height, width, 3), dtype=torch.float32, pin_memory=True)
        self.adj_dev = torch.empty((height, width, 3), dtype=torch.float32, device="cuda")

    def gradient(self):
        """One gradient evaluation on the device: forward, adjoint, replay."""
        self.r.diff_forward(self.spp)
        img = self.r.device_sums(5) / self.spp
        adj = ((2.0 / self.n) * (img - self.target)).float()
        return self.r.diff_backward(adj)

    def step(self, events=None):
        self.last_grad = self.gradient()

    def timed_region(self, steps, flush):
        """CUDA events on the submitting stream around `steps` evaluations;
        every evaluation streams 64 frames of path state (about 20 MB per
        frame at 256x256, several in flight) and 4.2M cache queries through
        the backward, far past the 129 MB L2: no flush kernel."""
        torch = self.torch
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(steps):
            self.step()
        t1.record()
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / steps

    def e2e_region(self, steps):
        """Through the public API with host buffers: forward, image read to the
        host (FP64), adjoint on the host, copied in from pinned memory,
        replay returning the gradients to the host."""
        import time
        torch = self.torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            self.r.diff_forward(self.spp)
            img = self.r.read()
            self.adj_host.numpy()[...] = (2.0 / self.n) * (img - self.target_host)
            self.adj_dev.copy_(self.adj_host, non_blocking=True)
            self.last_grad = self.r.diff_backward(self.adj_dev)
        torch.cuda.synchronize()
        return 1e3 * (time.perf_counter() - t0) / steps

    @property
    def kernels_per_step(self):
        # forward frames (bounce loop, cache inference, compose) + replay frames
        # (bounce loop, cache adjoint, two gradient sums) + group duals, total,
        # cache forward + backward
        rounds = 3  # BETA + 1 vertices at BETA = 2
        md = self.r.cache().info()
        # cache forward (encode, layers) + backward (fused dgrad, loss sum,
        # per-layer weight-gradient partials and reduction, hash-grid scatter
        # and conversion)
        mlp = 2 + 2 + 2 * (md.n_hidden_layers + 1) + 2
        fwd = 1 + 7 * rounds + 1 + 2 + 1
        rep = 1 + 7 * rounds + 3
        return self.spp * (fwd + rep) + 2 + mlp

    def units_per_step(self):
        return 1

    def paths_per_step(self):
        return 2 * self.P * self.spp

    def fit(self, steps=200, lr=0.05):
        """Adam on log(sigma_a) of every group from the +-50% start; returns
        the final relative error per component (the other materials fixed)."""
        torch = self.torch
        x = torch.tensor(np.log(self.start[:, 0:3].astype(np.float64)), requires_grad=True)
        opt = torch.optim.Adam([x], lr=lr)
        for _ in range(steps):
            m = self.truth.copy()
            m[:, 0:3] = np.exp(x.detach().numpy())
            self.scene.set_group_materials(m)
            g = self.gradient()
            opt.zero_grad()
            x.grad = torch.from_numpy(g[:, 0:3] * m[:, 0:3])
            opt.step()
        self.scene.set_group_materials(self.start)
        got = np.exp(x.detach().numpy())
        return np.abs(got - self.truth[:, 0:3]) / self.truth[:, 0:3]

    def roofline(self, seg_ms, pk):
        """Traversal of the forward frames (instrumented, one frame at a time)
        and the split of an evaluation into forward, replay and cache backward."""
        torch = self.torch
        self.r.instrument(timing=True, counting=False)
        self.r.diff_forward(4)
        t = self.r.timings().as_dict()
        self.r.instrument(timing=True, counting=True)
        self.r.diff_forward(1)
        c = self.r.timings()
        self.r.instrument(timing=False, counting=False)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        self.r.diff_forward(self.spp)
        ev[1].record()
        img = self.r.device_sums(5) / self.spp
        self.r.diff_backward(((2.0 / self.n) * (img - self.target)).float())
        ev[2].record()
        torch.cuda.synchronize()
        dominant = "extend_ms" if t["extend_ms"] >= t["shadow_ms"] else "shadow_ms"
        if dominant == "extend_ms":
            rays, nodes, prims = c.extension_rays, c.extend_nodes, c.extend_prims
        else:
            rays, nodes, prims = c.shadow_rays, c.shadow_nodes, c.shadow_prims
        alg = rays * RAY_RECORD_BYTES + nodes * NODE_BYTES + prims * PRIM_BYTES
        ach = alg / (t[dominant] * 1e-3) / 1e9
        return {"kernel": dominant.replace("_ms", "_kernel") + " (forward frames)", "bound": "hbm",
                "achieved": round(ach, 2), "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": round(ach / pk["hbm_gbs"], 4), "traffic": None,
                "evaluation_split_ms": {"forward_64_frames": round(ev[0].elapsed_time(ev[1]), 3),
                                        "replay_and_cache_backward": round(ev[1].elapsed_time(ev[2]), 3)},
                "stage_ms_per_forward_frame": {k: round(t[k], 4) for k in ("extend_ms", "shade_ms", "shadow_ms",
                                                                           "compact_ms", "infer_ms")},
                "rays_per_forward_frame": {"extension": int(c.extension_rays), "shadow": int(c.shadow_rays)},
                "algorithmic_bytes_per_frame": int(alg),
                "note": ("algorithmic bytes = rays x 48 B + 8-wide BVH nodes visited x 224 B + primitives tested "
                         "x 64 B, counted in an untimed forward frame; the replay re-traces the same rays. "
                         "Peak " + pk["source"])}

    def config(self):
        return {"workload": "diff: 20k curly procedural strands x 96 B-spline CPs (helix r 5 mm, pitch 10 mm), "
                            "20k-tri head, sky + directional light, 256x256, 64 spp per evaluation, HairMSNN BETA=2, "
                            "cache FP32 (frozen, 64 scene-sample training passes), 4 azimuthal strand groups; "
                            "L2 image loss against a target at the true materials (same frame seeds)",
                "pixels": self.P, "spp": self.spp, "groups": self.groups,
                "paths_per_evaluation": self.paths_per_step(),
                "l2": "inputs larger than L2: 64 frames of path state and 4.2M cache queries per evaluation",
                "launch_shapes": {k: v for k, v in self.tuning.items() if k != "ms_per_frame"},
                "parallelism": "replicas"}

    def cpu_baseline(self, threads, budget_s=20.0):
        """The reference has no gradient path.  Baseline: central finite
        differences on the host, the way to differentiate it as it is: one
        gradient of 4 groups x 6 parameters = 49 forward renders of 256x256 x
        64 spp, each timed as the oracle's reference-structured integrator
        (rayGenCam / msnnPathTrace G-buffer pass) on a bounded pixel sample."""
        import time
        from oracle import pyoracle as po
        o = po.OracleScene.from_library(self.scene)
        n = 4096
        t0 = time.perf_counter()
        done = 0
        p0 = (self.height // 2) * self.width
        while True:
            o.render_pixels(1, beta=2, accum_id=done // self.P, every_nth=self.P, n_train=0, p0=p0, n=n,
                            threads=threads)
            done += n
            p0 = (p0 + n) % (self.P - n)
            if time.perf_counter() - t0 > budget_s:
                break
        rate = done / (time.perf_counter() - t0)
        renders = 2 * self.groups * 6 + 1
        value = rate / (self.P * self.spp * renders)
        return {"value": value, "unit": self.unit, "cores": threads, "kind": "port",
                "sample": f"{done} pixels (1 spp) of the oracle's forward integrator on {threads} threads "
                          f"({rate:.0f} paths/s); a finite-difference gradient = {renders} renders of "
                          f"{self.P} pixels x {self.spp} spp; cache not included"}


def make_workload(name, torch):
    if name == "vertex":
        return VertexWorkload(torch)
    if name == "precision":
        return PrecisionWorkload(torch)
    if name == "batch":
        return BatchBenchWorkload(torch)
    if name == "diff":
        return DiffBenchWorkload(torch)
    if name == "quality":
        return RenderQualityWorkload(torch)
    return RenderBenchWorkload(torch)
