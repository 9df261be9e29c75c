"""Benchmark: ROI fits/s of the GB300 B-spline fitter on the batched 3D workload.

Workload (one "step"): 1,000,000 synthetic 3D astigmatic ROIs mixing 11x11,
13x13 and 17x17 pixels in the ratio 1:2:1, 30 LM iterations, fit type 6 - the
batched 3D configuration the headline metric is quoted on. Inputs are seeded
synthetic data (no public dataset exists for this path) and are larger than L2
(~0.7 GB of pixels), so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl gb300 (default) prints one JSON line with
  value: fits/s with the ROIs resident in HBM (CUDA events on the launch stream),
  e2e:   fits/s through the public call (host buffers, copies in the timed region),
  roofline: the fitter kernel against the measured FP32 FMA peak,
  cpu_baseline: the oracle port of the reference CPU fitter on the host cores.
--impl reference times the reference's CPU method (the bit-exact oracle port,
all host threads) on a bounded sample of the same workload.
Multi-GPU runs are independent replicas (every ROI is independent): each rank
fits its own copy of the workload, rank 0 prints the aggregate.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "gpu-based-b-spline-fitter_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "ROI fits/s (3D 13px, 5D 17px) and p50/p99 latency: serving vs plain, 1 GB300"
N_ROIS = 1_000_000
SIZES = (11, 13, 17)
ITERATIONS = 30


def aggregate_ranks(ms, n_local, world, device=None):
    """Whole-job figure of a replicated step: every rank fits its own copy of
    the workload, so the job processes n_local * world fits in the slowest
    rank's time (max over ranks). Returns (max ms, fits/s)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, n_local * world / (ms * 1e-3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region:
    one nvidia-smi process streaming a line every 50 ms, started before the
    region (so its start-up does not fall inside it), each line stamped on
    arrival; the summary keeps the lines that arrived between entering and
    leaving the region (the nearest one when the region is shorter than the
    sampling period)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 50

    def __init__(self, index=0):
        self.index = index
        self.lines = []  # (arrival time, fields)
        self.samples = []
        self._p = None
        self._t = None
        self.t0 = self.t1 = None

    def _read(self):
        for line in self._p.stdout:
            f = [x.strip() for x in line.strip().split(",")]
            if len(f) >= 8:
                self.lines.append((time.time(), f))

    def __enter__(self):
        try:
            self._p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            deadline = time.time() + 5.0
            while not self.lines and time.time() < deadline:
                time.sleep(0.01)
        except Exception:
            self._p = None
        self.t0 = time.time()
        return self

    def __exit__(self, *a):
        self.t1 = time.time()
        if self._p is not None:
            time.sleep(self.PERIOD_MS * 1.5e-3)
            self._p.terminate()  # the process started above
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()
            self._t.join(timeout=5)
        inside = [f for t, f in self.lines if self.t0 <= t <= self.t1 + self.PERIOD_MS * 1e-3]
        if not inside and self.lines:
            mid = 0.5 * (self.t0 + self.t1)
            inside = [min(self.lines, key=lambda x: abs(x[0] - mid))[1]]
        self.samples = inside

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 4 + i and s[4 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples), "period_ms": self.PERIOD_MS}


def make_workload(n=N_ROIS, sizes=SIZES, iterations=ITERATIONS):
    from bsfit import workloads as W
    if len(sizes) == 1:
        return [W.workload_3d(n, s=sizes[0], iterations=iterations, stream=2)]
    return W.workload_3d_mixed(n, sizes=sizes, ratio=(1, 2, 1), iterations=iterations)


def bench_kernel_only(args):
    """Profiling case: warm-up plus timed fits of one workload, nothing else.
    3D (default): one plain launch per size group, or with --batched one
    persistent batched launch per step; --model 5d: fit type 8 on --rois ROIs
    of 17 px; --model 4pi: the 4Pi fit of --rois ROIs of four 13 px channels;
    --model 3d64: the FP64 reference-precision kernel on --rois 3D ROIs of 13 px;
    --model 4d: fit type 7 on --rois ROIs of 13 px. --precision parity runs the
    double-float kernels on the 3D (13 px), 4D and 5D cases. 3D only: --variant
    V --wpb W forces a tuner configuration (e.g. the two-ROIs-per-warp variants
    3 to 5); --eval runs the evaluation kernel alone, at the fitted parameters."""
    import torch
    import bsfit
    from bsfit import workloads as W
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    launches = args.warmup + args.steps
    prec = args.precision
    if prec == "parity" and args.model in ("3d", "4d", "5d"):
        w = {"3d": lambda: W.workload_3d(args.rois, s=13, stream=9),
             "4d": lambda: W.workload_4d(args.rois, sizes=(13,), stream=6)[0],
             "5d": lambda: W.workload_5d(args.rois, s=17, stream=7)}[args.model]()
        m = bsfit.Model(w.fittype, w.coeff, coeff3=w.coeff3, init_p=w.init_p)
        r = torch.from_numpy(w.rois).to(dev)
        with torch.cuda.stream(stream):
            for _ in range(launches):
                m.fit_torch(r, w.iterations, stream=stream, precision="parity")
        stream.synchronize()
        print(json.dumps({"profile_case": True, "model": args.model, "precision": "parity",
                          "rois": len(w.rois), "launches": launches}))
        return 0
    if args.model == "5d":
        w5 = W.workload_5d(args.rois, s=17, stream=7)
        m5 = bsfit.Model(8, w5.coeff, coeff3=w5.coeff3, init_p=w5.init_p)
        r5 = torch.from_numpy(w5.rois).to(dev)
        with torch.cuda.stream(stream):
            for _ in range(launches):
                m5.fit_torch(r5, w5.iterations, stream=stream)
        stream.synchronize()
        print(json.dumps({"profile_case": True, "model": "5d", "rois": len(w5.rois),
                          "launches": launches}))
        return 0
    if args.model == "4d":
        w4 = W.workload_4d(args.rois, sizes=(13,), stream=6)[0]
        m4 = bsfit.Model(7, w4.coeff, init_p=w4.init_p)
        r4 = torch.from_numpy(w4.rois).to(dev)
        with torch.cuda.stream(stream):
            for _ in range(launches):
                m4.fit_torch(r4, w4.iterations, stream=stream)
        stream.synchronize()
        print(json.dumps({"profile_case": True, "model": "4d", "rois": len(w4.rois),
                          "launches": launches}))
        return 0
    if args.model == "3d64":
        w6 = W.workload_3d(args.rois, s=13, stream=9)
        m6 = bsfit.Model(6, w6.coeff)
        r6 = torch.from_numpy(w6.rois).to(dev)
        with torch.cuda.stream(stream):
            for _ in range(launches):
                m6.fit_f64_torch(r6, w6.iterations, stream=stream)
        stream.synchronize()
        print(json.dumps({"profile_case": True, "model": "3d64", "rois": len(w6.rois),
                          "launches": launches}))
        return 0
    if args.model == "4pi":
        w4 = W.workload_4pi(args.rois, s=13, stream=8)
        m4 = bsfit.Model4Pi(w4.coeff, w4.extra["phase_shift"])
        cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        r4, z4, p4, d4 = (cu(w4.rois), cu(w4.extra["init_z"]), cu(w4.extra["init_phi"]),
                          cu(w4.extra["dT"]))
        with torch.cuda.stream(stream):
            for _ in range(launches):
                m4.fit_torch(r4, w4.iterations, z4, p4, dT=d4, stream=stream)
        stream.synchronize()
        print(json.dumps({"profile_case": True, "model": "4pi", "rois": w4.n_fits,
                          "launches": launches}))
        return 0
    groups = make_workload(args.rois, tuple(args.sizes), args.iterations)
    if args.variant is not None:
        # a forced launch configuration (the tuner's variant and warps per block)
        from bsfit import tuning as T
        for g in groups:
            T._set(6, g.roi_size, args.variant, args.wpb)
    work = []
    for g in groups:
        m = bsfit.Model(6, g.coeff)
        r = torch.from_numpy(g.rois).to(dev)
        o = (torch.empty((6, len(g.rois)), device=dev), torch.empty((5, len(g.rois)), device=dev),
             torch.empty((len(g.rois),), device=dev))
        work.append((m, r, o, g))
    if args.eval:
        # the evaluation kernel alone: one untimed fit per size group, then
        # launches of one evaluation per ROI at the fitted parameters
        with torch.cuda.stream(stream):
            ths = []
            for m, r, o, g in work:
                m.fit_torch(r, g.iterations, out=o, stream=stream)
                ths.append(o[0][:5].contiguous())
            for _ in range(launches):
                for (m, r, o, g), th in zip(work, ths):
                    m.eval_torch(r, th, stream=stream)
        stream.synchronize()
        print(json.dumps({"profile_case": True, "eval": True, "rois": sum(len(g.rois) for g in groups),
                          "sizes": args.sizes, "launches": launches * len(work)}))
        return 0
    batch = bsfit.Batch([(m, r, g.iterations) for m, r, o, g in work]) if args.batched else None
    with torch.cuda.stream(stream):
        for _ in range(launches):
            if batch is not None:
                batch.run(stream=stream)
            else:
                for m, r, o, g in work:
                    m.fit_torch(r, g.iterations, out=o, stream=stream)
    stream.synchronize()
    n = sum(len(g.rois) for g in groups)
    per_step = 1 if batch is not None else len(groups)
    # ROI evaluations per step (iterations + 2 per ROI: the initial pass and the
    # CRLB pass), the unit of an instruction count per evaluation
    outs = batch.outputs if batch is not None else [o for m, r, o, g in work]
    evals = sum(float((o[0][5].double() + 2.0).sum().item()) for o in outs) if launches else 0.0
    print(json.dumps({"profile_case": True, "rois": n, "sizes": args.sizes,
                      "batched": bool(args.batched), "launches": launches * per_step,
                      "evaluations_per_step": evals}))
    return 0


def cpu_sample(groups, per_group_frac=0.016):
    """A bounded, proportional sample of the workload for the CPU runs."""
    return [(g.rois[: max(1, int(len(g.rois) * per_group_frac))], g) for g in groups]


def run_cpu(groups, threads, frac):
    from oracle.oracle import Oracle
    o = Oracle()
    n = 0
    t0 = time.perf_counter()
    for rois, g in cpu_sample(groups, frac):
        o.fit(rois, g.fittype, g.iterations, g.coeff, precision="f32", threads=threads)
        n += len(rois)
    dt = time.perf_counter() - t0
    return n, dt


def bench_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    groups = make_workload()
    threads = os.cpu_count() or 1
    frac = 0.008
    for _ in range(args.warmup):
        run_cpu(groups, threads, frac / 4)
    tot_n, tot_t = 0, 0.0
    for _ in range(args.steps):
        n, dt = run_cpu(groups, threads, frac)
        tot_n += n
        tot_t += dt
    v = tot_n / tot_t
    sample = (f"{int(N_ROIS * frac)} ROIs per step ({frac:.1%} of the 1M-ROI 11/13/17 mix), "
              f"oracle port of the reference CPU fitter (FP32, bit-exact), OpenMP over ROIs")
    line = {"metric": METRIC, "value": v, "unit": "fits/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": "3d_batched_1M_11-13-17", "rois": N_ROIS, "fit_type": 6,
                       "iterations": ITERATIONS, "parallelism": "replicas"},
            "cpu_baseline": {"value": v, "unit": "fits/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "fits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_ref_gpu:
        line["reference_gpu_kernel"] = bench_reference_gpu(groups)
    print(json.dumps(line))
    return 0


def bench_reference_gpu(groups):
    """Informational: the reference's own CUDA kernels (one thread per ROI, 64
    per block, as its mex launches them) on this GPU, device-resident ROIs, CUDA
    events. Their throughput grows with the ROI count until every SM holds its
    maximum of 64-thread blocks, so each model gets enough ROIs to fill the GPU:
    3D 200,000 of the step's 13 px ROIs, 4D 80,000 of 13 px, 5D 38,912 of 17 px
    (four blocks per SM); one timed launch after a warm-up on a slice."""
    try:
        import torch
        from oracle import ref_gpu
        if not (torch.cuda.is_available() and ref_gpu.available()):
            return {"unavailable": "no GPU or the reference PTX is not built"}
        from bsfit import workloads as W
        dev = torch.device("cuda", 0)
        r = ref_gpu.RefGPU()
        stream = torch.cuda.Stream(dev)
        out = {}
        g13 = next(g for g in groups if g.roi_size == 13)
        w4 = W.workload_4d(80000, sizes=(13,), stream=402)[0]
        w5 = W.workload_5d(38912, s=17, stream=403)
        cases = [("3d_13px", 6, g13.rois[:200000], g13), ("4d_13px", 7, w4.rois, w4),
                 ("5d_17px", 8, w5.rois, w5)]
        for key, ft, rois, wl in cases:
            d_r = torch.from_numpy(np.ascontiguousarray(rois)).to(dev)
            d_c = r.padded_table(wl.coeff, dev)
            d_c3 = r.padded_table(wl.coeff3, dev) if ft == 8 else None
            ip = None
            if ft in (7, 8):
                ip = torch.from_numpy(np.asarray(wl.init_p, np.float32)).to(dev)
            dims = list(reversed(wl.coeff.shape))
            with torch.cuda.stream(stream):
                r.fit(ft, d_r[: max(64, len(rois) // 16)], wl.iterations, d_c, dims, d_c3, ip,
                      stream=stream)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                r.fit(ft, d_r, wl.iterations, d_c, dims, d_c3, ip, stream=stream)
                b.record(stream)
            stream.synchronize()
            out[key] = len(rois) / (a.elapsed_time(b) * 1e-3)
        out["workloads"] = ("3D: 200000 ROIs of the step's 13 px group, 30 iterations; 4D: "
                            "80000 ROIs 13 px, 60 iterations; 5D: 38912 ROIs 17 px, 60 iterations "
                            "(enough ROIs to fill the GPU with one thread per ROI)")
        out["unit"] = "fits/s"
        out["kernels"] = "GPUmleFit_LM_EMCCD.cu kernel_bsplineMLEFit_*, 64 threads per block"
        return out
    except Exception as e:  # informational figure: report why it is missing
        return {"unavailable": f"{type(e).__name__}: {e}"[:300]}


def bench_serving(args, dev, seed=11):
    """Mixed-model acquisition stream through the serving form, against the
    plain per-call form (one synchronous GPUmleFit_LM_multiD call per frame).

    Frames: 3D 13 px (60%), 4D 13 px (25%), 5D 17 px (15%) models, frame sizes
    log-uniform in 2k-50k ROIs (2k-8k for 5D). The stream is run saturated (all
    frames submitted at once) for throughput, then replayed with Poisson
    arrivals at ~70% of the saturated rate for latency. A second stream of 10k
    ROI 3D frames at the same load gives the per-frame latency."""
    import bsfit
    from bsfit import workloads as W
    rng = np.random.default_rng(seed)
    pools = {"3d": W.workload_3d(200000, s=13, stream=21),
             "4d": W.workload_4d(60000, sizes=(13,), stream=22)[0],
             "5d": W.workload_5d(12000, s=17, stream=23)}
    models = {k: bsfit.Model(w.fittype, w.coeff, coeff3=w.coeff3, init_p=w.init_p) for k, w in pools.items()}
    frames = []
    for _ in range(args.serve_frames):
        kind = rng.choice(["3d", "4d", "5d"], p=[0.6, 0.25, 0.15])
        hi = 8000 if kind == "5d" else 50000
        n = int(np.exp(rng.uniform(np.log(2000), np.log(hi))))
        w = pools[kind]
        o = int(rng.integers(0, len(w.rois) - n))
        frames.append((kind, w, np.ascontiguousarray(w.rois[o:o + n])))
    n_rois = sum(len(f[2]) for f in frames)

    def run_stream(srv, frame_list, gaps):
        srv.reset_stats()
        t0 = time.perf_counter()
        ids = []
        for (kind, w, r), gap in zip(frame_list, gaps):
            if gap > 0:
                target = time.perf_counter() + gap
                while time.perf_counter() < target:
                    srv.poll()
            ids.append(srv.submit([(models[kind], r, w.iterations)]))
        for rid in ids:
            srv.wait(rid, timeout=300.0)
        el = time.perf_counter() - t0
        return el, srv.stats()

    srv = bsfit.Server(max_inflight=4, arena_bytes=4 << 30)
    run_stream(srv, frames[:4], [0] * 4)  # warm-up
    sat_s, sat = run_stream(srv, frames, [0] * len(frames))
    rate = 0.7 * len(frames) / sat_s
    gaps = rng.exponential(1.0 / rate, len(frames))
    gaps[0] = 0
    load_s, loaded = run_stream(srv, frames, gaps)
    # 10k-ROI 3D frames at the same load
    w3 = pools["3d"]
    f10 = [("3d", w3, np.ascontiguousarray(w3.rois[i * 10000:(i + 1) * 10000])) for i in range(20)]
    s10_s, s10 = run_stream(srv, f10, [0] * len(f10))
    g10 = rng.exponential(len(f10) / (0.7 * len(f10) / s10_s) / len(f10), len(f10))
    g10[0] = 0
    _, l10 = run_stream(srv, f10, g10)
    # 10k-ROI frames drawn from the mixed stream (3D 60%, 4D 25%, 5D 15%) at
    # 70% of their saturated rate: per-frame latencies, by model too
    fm = []
    for i in range(40):
        kind = rng.choice(["3d", "4d", "5d"], p=[0.6, 0.25, 0.15])
        w = pools[kind]
        o = int(rng.integers(0, len(w.rois) - 10000))
        fm.append((kind, w, np.ascontiguousarray(w.rois[o:o + 10000])))
    unit_gaps = rng.exponential(1.0, len(fm))
    unit_gaps[0] = 0

    def mixed10k(srv, offered_s=None):
        """Saturated pass, then the frames with Poisson arrivals at 70% of the
        saturated rate (of offered_s, a saturated time, when given: the same
        arrivals for two servers)."""
        sm_s, _ = run_stream(srv, fm, [0] * len(fm))
        gm = unit_gaps * (offered_s or sm_s) / (0.7 * len(fm))
        srv.reset_stats()
        pending = []
        for (kind, w, r), gap in zip(fm, gm):
            if gap > 0:
                target = time.perf_counter() + gap
                while time.perf_counter() < target:
                    srv.poll()
            pending.append((kind, time.perf_counter(), srv.submit([(models[kind], r, w.iterations)])))
        for kind, ts, rid in pending:
            srv.wait(rid, timeout=300.0)
        mixed_stats = srv.stats()
        lat_map = srv.latencies()
        lat_by = [lat_map.get(rid) for _, _, rid in pending]
        lat_by = None if any(x is None for x in lat_by) else lat_by
        return sm_s, mixed_frame_summary(fm, lat_by, mixed_stats, sm_s)

    fm_sat_s, mixed = mixed10k(srv)
    srv.close()
    # merged admission: a free slot takes up to 4 queued requests into one launch
    srv = bsfit.Server(max_inflight=4, arena_bytes=4 << 30, merge=4)
    run_stream(srv, frames[:4], [0] * 4)  # warm-up
    msat_s, _ = run_stream(srv, frames, [0] * len(frames))
    merged = {"merge": 4, "fits_per_s": n_rois / msat_s,
              "frame10k_mixed": mixed10k(srv, fm_sat_s)[1]}
    srv.close()
    # priority launches: short requests on high-priority streams, long launches
    # whose blocks retire as they finish (the same arrivals as above)
    srv = bsfit.Server(max_inflight=4, arena_bytes=4 << 30, priority=True)
    run_stream(srv, frames[:4], [0] * 4)  # warm-up
    psat_s, _ = run_stream(srv, frames, [0] * len(frames))
    prio = {"fits_per_s": n_rois / psat_s, "frame10k_mixed": mixed10k(srv, fm_sat_s)[1]}
    srv.close()
    # both: priority launches and merged admission of requests of one level
    srv = bsfit.Server(max_inflight=4, arena_bytes=4 << 30, merge=4, priority=True)
    run_stream(srv, frames[:4], [0] * 4)  # warm-up
    bsat_s, _ = run_stream(srv, frames, [0] * len(frames))
    prio["merged"] = {"merge": 4, "fits_per_s": n_rois / bsat_s,
                      "frame10k_mixed": mixed10k(srv, fm_sat_s)[1]}
    srv.close()
    # plain per-call form
    t0 = time.perf_counter()
    for kind, w, r in frames:
        kw = {}
        if w.init_p is not None:
            kw["initP"] = w.init_p
        if w.coeff3 is not None:
            kw["coeff3"] = w.coeff3
        bsfit.GPUmleFit_LM_multiD(r, w.fittype, w.iterations, w.coeff, **kw)
    plain_s = time.perf_counter() - t0
    return {"stream": f"{len(frames)} frames, {n_rois} ROIs: 3D 13px 60%, 4D 13px 25%, 5D 17px 15%, "
                      f"2k-50k ROIs per frame (2k-8k for 5D)",
            "fits_per_s": n_rois / sat_s, "plain_fits_per_s": n_rois / plain_s,
            "speedup_vs_plain": plain_s / sat_s,
            "load": 0.7, "p50_ms": loaded["p50_ms"], "p99_ms": loaded["p99_ms"],
            "loaded_fits_per_s": n_rois / load_s,
            "frame10k_3d": {"p50_ms": l10["p50_ms"], "p99_ms": l10["p99_ms"], "load": 0.7,
                            "saturated_p50_ms": s10["p50_ms"]},
            "frame10k_mixed": mixed, "merged": merged, "priority": prio,
            "max_inflight": 4, "arena_bytes": 4 << 30}


def mixed_frame_summary(frames, lat_ms, stats, sat_s):
    """Latency summary of the mixed 10k-ROI frames: overall p50 / p99, the
    fraction of frames within 5 ms, and per model (lat_ms: per-request
    latencies in submission order from the server, when available)."""
    out = {"frames": len(frames), "load": 0.7, "p50_ms": stats["p50_ms"], "p99_ms": stats["p99_ms"],
           "saturated_fits_per_s": 10000 * len(frames) / sat_s}
    if lat_ms is not None and len(lat_ms) == len(frames):
        lat = np.asarray(lat_ms, float)
        out["frac_within_5ms"] = float(np.mean(lat <= 5.0))
        for kind in ("3d", "4d", "5d"):
            sel = np.array([f[0] == kind for f in frames])
            if sel.any():
                out[kind] = {"frames": int(sel.sum()), "p50_ms": float(np.median(lat[sel])),
                             "p99_ms": float(np.quantile(lat[sel], 0.99))}
    return out


def synthetic_movie(F=64, H=512, W=512, per_frame=150, seed=31, offset=100.0, conversion=0.5):
    """ADU frames (F, W, H) = MATLAB [H, W, F]: Poisson background 12 e- and
    astigmatic emitters (1000-5000 e-, z uniform +-600 nm) at random positions."""
    from bsfit import workloads as W_
    rng = np.random.default_rng(seed)
    frames = np.empty((F, W, H), np.float32)
    for f in range(F):
        lam = np.full((W, H), 12.0)
        xs = rng.uniform(8, W - 8, per_frame)
        ys = rng.uniform(8, H - 8, per_frame)
        zs = rng.uniform(-600, 600, per_frame)
        ns = np.exp(rng.uniform(np.log(1000), np.log(5000), per_frame))
        sx, sy = W_.astig_sigmas(zs, 1.3)
        for x, y, a, b, n in zip(xs, ys, sx, sy, ns):
            x0, y0 = int(x) - 7, int(y) - 7
            gx = W_._int_gauss(np.array([x - x0]), np.array([a]), 15)[0]
            gy = W_._int_gauss(np.array([y - y0]), np.array([b]), 15)[0]
            lam[x0:x0 + 15, y0:y0 + 15] += n * gx[:, None] * gy[None, :]
        frames[f] = (rng.poisson(lam) / conversion + offset).astype(np.float32)
    return frames


def bench_frontend(dev, stream):
    """Frame -> ROI front end (difference-of-Gaussians filter, sigma 1, 13 px
    ROIs) on a 64-frame 512 x 512 movie, alone and followed by the 3D fit of the
    ROIs it finds (frames resident on the device); the numpy restatement of the
    front end on two frames for comparison."""
    import torch
    import bsfit
    from bsfit import workloads as W
    frames = synthetic_movie()
    fr = torch.from_numpy(frames).to(dev)
    h = bsfit.peak_kernel(1, 1.0)
    model = bsfit.Model(6, W.coeff3d())
    kw = dict(dog=True, cutoff=8.0, roi_size=13, stream=stream)
    with torch.cuda.stream(stream):
        rois, coords = bsfit.find_rois_torch(fr, 100.0, 0.5, h, **kw)
        model.fit_torch(rois.contiguous(), 30, stream=stream)
    stream.synchronize()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        with torch.cuda.stream(stream):
            rois, coords = bsfit.find_rois_torch(fr, 100.0, 0.5, h, capacity=len(coords), **kw)
        stream.synchronize()
    fe_s = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        with torch.cuda.stream(stream):
            rois, coords = bsfit.find_rois_torch(fr, 100.0, 0.5, h, capacity=len(coords), **kw)
            model.fit_torch(rois.contiguous(), 30, stream=stream)
        stream.synchronize()
    both_s = (time.perf_counter() - t0) / reps
    from oracle import frontend as FE  # CPU comparison leg only
    t0 = time.perf_counter()
    FE.find_rois(frames[:2], 100.0, 0.5, FE.peak_kernel(1, 1.0), True, 8.0, 13)
    cpu_per_frame = (time.perf_counter() - t0) / 2
    F = frames.shape[0]
    return {"movie": f"{F} frames 512x512, 150 emitters per frame, DoG sigma 1, 13 px ROIs",
            "rois_found": int(len(coords)), "frontend_frames_per_s": F / fe_s,
            "frames_to_fits_frames_per_s": F / both_s,
            "frames_to_fits_fits_per_s": len(coords) / both_s,
            "cpu_numpy_frames_per_s": 1.0 / cpu_per_frame}


def bench_gpu(args):
    import torch
    import bsfit
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    groups = make_workload()
    models = {id(g.coeff): bsfit.Model(6, g.coeff) for g in groups}
    stream = torch.cuda.Stream(dev)
    d_rois = [torch.from_numpy(g.rois).to(dev) for g in groups]
    n_step = sum(len(g.rois) for g in groups)

    # Autotuner: each size group's launch configuration (kernel variant,
    # warps per block) timed on a sample of the group and put in force; the
    # batched step runs with the configuration of its largest ROI size.
    tuned = {}
    if not args.no_tune:
        from bsfit import tuning as T
        for g, r in zip(groups, d_rois):
            ch = T.autotune(models[id(g.coeff)], r[:args.tune_rois], g.iterations, reps=2)
            tuned[str(g.roi_size)] = {k: ch[k] for k in ("variant", "warps_per_block",
                                                        "min_blocks", "rois_per_warp", "ms")}

    # Batched form: one persistent launch over all size groups per step (the
    # plain form, one call per size group, is timed beside it below).
    batch = bsfit.Batch([(models[id(g.coeff)], r, g.iterations) for g, r in zip(groups, d_rois)])
    outs = batch.outputs

    def step():
        batch.run(stream=stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 1)):
            step()
    stream.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    barrier()
    ms, value = aggregate_ranks(ev0.elapsed_time(ev1) / args.steps, n_step, world, dev)

    # Per-size kernel times of the plain form (one launch per size group, events
    # on the launch stream) and the roofline of the fitter kernel.
    iters = [o[0][5].float() for o in outs]
    flops = sum(float(((it + 2.0) * bsfit.eval_flops(6, g.roi_size)).sum().item())
                for it, g in zip(iters, groups))
    mean_iter = float(sum(it.sum().item() for it in iters) / n_step)
    per_launch = []
    for g, r, o in zip(groups, d_rois, outs):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            for _ in range(3):
                models[id(g.coeff)].fit_torch(r, g.iterations, out=o, stream=stream)
            b.record(stream)
        stream.synchronize()
        per_launch.append(a.elapsed_time(b) / 3)
    plain_ms = sum(per_launch)
    kernel_ms = ms  # the batched step is one kernel launch
    peak_scalar, peak_paired = bsfit.measure_fp32_peaks()
    peak = max(peak_scalar, peak_paired)
    achieved = flops / (kernel_ms * 1e-3) * 1e-12

    # End to end through the public call: host buffers (pinned), copies and the
    # per-call coefficient upload inside the timed region, as the mex does.
    pinned = [torch.from_numpy(g.rois).pin_memory().numpy() for g in groups]
    h2d = sum(p.nbytes for p in pinned) + sum(g.coeff.nbytes for g in groups)
    d2h = n_step * (6 + 5 + 1) * 4
    # the caller's output buffers (C ABI layout), allocated once and page-locked
    # like the inputs, as a host application streaming results would keep them
    # (pageable outputs measured 1.7% slower: the copies go through a staging
    # buffer)
    host_out = [tuple(torch.empty(shape, dtype=torch.float32).pin_memory().numpy()
                      for shape in ((6, len(g.rois)), (5, len(g.rois)), (len(g.rois),)))
                for g in groups]
    for _ in range(3):
        for g, p, o in zip(groups, pinned, host_out):
            bsfit.GPUmleFit_LM_multiD(p, 6, g.iterations, g.coeff, out=o)
    barrier()
    # three times the timed steps, up to 60 (about 1.8 s), so that a host-side
    # stall (a shared host: about one step in 20 to 30 takes 41-64 ms against
    # 29.2 ms) moves the mean little; each step's time is kept for the spread
    # reported beside it
    e2e_steps = max(1, min(3 * args.steps, 60))
    e2e_ms = []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ts = time.perf_counter()
        for g, p, o in zip(groups, pinned, host_out):
            bsfit.GPUmleFit_LM_multiD(p, 6, g.iterations, g.coeff, out=o)
        e2e_ms.append((time.perf_counter() - ts) * 1e3)
    torch.cuda.synchronize()
    barrier()
    _, e2e_value = aggregate_ranks((time.perf_counter() - t0) / e2e_steps * 1e3, n_step, world,
                                   dev)

    # The metric's per-model figures: 3D 13 px from the per-size timing above,
    # 5D 17 px (fit type 8, 60 iterations) on its own synthetic workload.
    fits_3d13 = None
    for g, t in zip(groups, per_launch):
        if g.roi_size == 13:
            fits_3d13 = len(g.rois) / (t * 1e-3)
    fits_5d17 = None
    tuned_models = {}
    if not args.no_5d:
        from bsfit import workloads as W
        w5 = W.workload_5d(args.rois_5d, s=17, stream=7)
        m5 = bsfit.Model(8, w5.coeff, coeff3=w5.coeff3, init_p=w5.init_p)
        r5 = torch.from_numpy(w5.rois).to(dev)
        o5 = (torch.empty((9, len(w5.rois)), device=dev), torch.empty((8, len(w5.rois)), device=dev),
              torch.empty((len(w5.rois),), device=dev))
        if not args.no_tune:
            # the tuner's choice for this model and size, on a sample of it
            from bsfit import tuning as T
            ch = T.autotune(m5, r5[:5000], w5.iterations, reps=2)
            tuned_models["5d_17"] = {k: ch[k] for k in ("variant", "warps_per_block",
                                                       "min_blocks", "ms")}
        with torch.cuda.stream(stream):
            m5.fit_torch(r5, w5.iterations, out=o5, stream=stream)
            a5, b5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a5.record(stream)
            for _ in range(2):
                m5.fit_torch(r5, w5.iterations, out=o5, stream=stream)
            b5.record(stream)
        stream.synchronize()
        fits_5d17 = len(w5.rois) / (a5.elapsed_time(b5) / 2 * 1e-3)
    # 4D colour (fit type 7, 13 px, 60 iterations): the serving stream's
    # largest share.
    fits_4d13 = None
    if not args.no_4d:
        from bsfit import workloads as W
        w7 = W.workload_4d(args.rois_4d, sizes=(13,), stream=6)[0]
        m7 = bsfit.Model(7, w7.coeff, init_p=w7.init_p)
        r7 = torch.from_numpy(w7.rois).to(dev)
        if not args.no_tune:
            from bsfit import tuning as T
            ch = T.autotune(m7, r7[:20000], w7.iterations, reps=2)
            tuned_models["4d_13"] = {k: ch[k] for k in ("variant", "warps_per_block",
                                                       "min_blocks", "ms")}
        with torch.cuda.stream(stream):
            m7.fit_torch(r7, w7.iterations, stream=stream)
            a7, b7 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a7.record(stream)
            for _ in range(2):
                m7.fit_torch(r7, w7.iterations, stream=stream)
            b7.record(stream)
        stream.synchronize()
        fits_4d13 = len(w7.rois) / (a7.elapsed_time(b7) / 2 * 1e-3)
    # 4Pi (four channels of 13 px, 100 iterations, one phase start), the
    # reference demo's fit on its own synthetic workload.
    fits_4pi = None
    if not args.no_4pi:
        from bsfit import workloads as W
        w4 = W.workload_4pi(args.rois_4pi, s=13, stream=8)
        m4 = bsfit.Model4Pi(w4.coeff, w4.extra["phase_shift"])
        cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        r4, z4, p4, d4 = (cu(w4.rois), cu(w4.extra["init_z"]), cu(w4.extra["init_phi"]),
                          cu(w4.extra["dT"]))
        with torch.cuda.stream(stream):
            m4.fit_torch(r4, w4.iterations, z4, p4, dT=d4, stream=stream)
            a4, b4 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a4.record(stream)
            for _ in range(2):
                m4.fit_torch(r4, w4.iterations, z4, p4, dT=d4, stream=stream)
            b4.record(stream)
        stream.synchronize()
        fits_4pi = w4.n_fits / (a4.elapsed_time(b4) / 2 * 1e-3)
    def timed(fn, reps=2):
        # mean ms of reps calls on the bench stream after one untimed call
        with torch.cuda.stream(stream):
            fn()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
        stream.synchronize()
        return a.elapsed_time(b) / reps

    # The colour configuration as stated: 500,000 ROIs of 13 and 15 px (half
    # each), fit type 7, 60 iterations, through the batched form (one
    # persistent launch over both sizes).
    c3_fig = None
    if not args.no_c3:
        from bsfit import workloads as W
        g7 = W.workload_4d(args.rois_c3, sizes=(13, 15), stream=9)
        m7c = bsfit.Model(7, g7[0].coeff, init_p=g7[0].init_p)
        b7 = bsfit.Batch([(m7c, torch.from_numpy(g.rois).to(dev), g.iterations) for g in g7])
        t7 = timed(lambda: b7.run(stream=stream))
        it7 = float(sum(o[0][6].float().sum().item() for o in b7.outputs) / args.rois_c3)
        c3_fig = {"fits_per_s": args.rois_c3 / (t7 * 1e-3), "ms": t7, "mean_iterations": it7,
                  "workload": f"{args.rois_c3} ROIs, 13x13 and 15x15 (half each), fit type 7, "
                              f"60 iterations, batched (one launch)"}
        del b7
    # The 4Pi configuration as stated: 250,000 ROIs of 4 x 16 x 16 px on a
    # 33 x 33 x 61 x 16 grid periodic in phase, per-channel offsets, 100
    # iterations, one launch.
    c4_fig = None
    if not args.no_c4:
        from bsfit import workloads as W
        w4c = W.workload_4pi_c4(args.rois_c4, s=16, stream=10)
        m4c = bsfit.Model4Pi(w4c.coeff, w4c.extra["phase_shift"])
        cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        r4c, z4c, p4c, d4c = (cu(w4c.rois), cu(w4c.extra["init_z"]), cu(w4c.extra["init_phi"]),
                              cu(w4c.extra["dT"]))
        o4c = m4c.fit_torch(r4c, w4c.iterations, z4c, p4c, dT=d4c, stream=stream)
        t4c = timed(lambda: m4c.fit_torch(r4c, w4c.iterations, z4c, p4c, dT=d4c, stream=stream))
        stream.synchronize()
        c4_fig = {"fits_per_s": w4c.n_fits / (t4c * 1e-3), "ms": t4c,
                  "mean_iterations": float(o4c[0][6].float().mean().item()),
                  "workload": f"{w4c.n_fits} ROIs of 4 x 16 x 16 px, coefficient grid "
                              f"{'x'.join(str(d) for d in reversed(w4c.coeff.shape))} (33 x 33 "
                              f"x 61 lateral / z samples, 16 phases per period, periodic), "
                              f"per-channel offsets, 100 iterations, one start, one launch"}
        del r4c
    # Parity-grade kernels (double-float): 3D 13 px ROIs of the step, the 4D
    # and 5D figures' workloads.
    parity_fig = None
    if not args.no_parity:
        g13 = next(g for g in groups if g.roi_size == 13)
        rp = d_rois[groups.index(g13)][:args.rois_parity]
        mp = models[id(g13.coeff)]
        tp = timed(lambda: mp.fit_torch(rp, g13.iterations, stream=stream, precision="parity"))
        parity_fig = {"3d_13px_fits_per_s": rp.shape[0] / (tp * 1e-3),
                      "3d_workload": f"{rp.shape[0]} ROIs 13x13 of the step, 30 iterations"}
        if not args.no_4d:
            n7 = min(args.rois_parity // 2, r7.shape[0])
            t = timed(lambda: m7.fit_torch(r7[:n7], w7.iterations, stream=stream,
                                           precision="parity"))
            parity_fig["4d_13px_fits_per_s"] = n7 / (t * 1e-3)
            parity_fig["4d_workload"] = f"{n7} ROIs of the 4D figure's workload"
        if not args.no_5d:
            n5 = min(args.rois_parity // 10, r5.shape[0])
            t = timed(lambda: m5.fit_torch(r5[:n5], w5.iterations, stream=stream,
                                           precision="parity"), reps=1)
            parity_fig["5d_17px_fits_per_s"] = n5 / (t * 1e-3)
            parity_fig["5d_workload"] = f"{n5} ROIs of the 5D figure's workload"
        parity_fig["kernel"] = ("fitdd_kernel<6|7|8>: the reference method in double-float on "
                                "the FP32 pipe, Fisher inverse in FP64")
    # FP64 reference-precision kernel (bit-identical to the FP64 oracle) on
    # 3D 13 px ROIs of the step's workload.
    fp64_fig = None
    if not args.no_fp64:
        g13 = next(g for g in groups if g.roi_size == 13)
        n64 = min(args.rois_fp64, len(g13.rois))
        r64 = d_rois[groups.index(g13)][:n64]
        m64 = models[id(g13.coeff)]
        with torch.cuda.stream(stream):
            m64.fit_f64_torch(r64, g13.iterations, stream=stream)
            a6, b6 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a6.record(stream)
            for _ in range(2):
                m64.fit_f64_torch(r64, g13.iterations, stream=stream)
            b6.record(stream)
        stream.synchronize()
        fp64_fig = {"3d_13px_fits_per_s": n64 / (a6.elapsed_time(b6) / 2 * 1e-3),
                    "workload": f"{n64} ROIs 13x13 of the step, fit type 6, "
                                f"{g13.iterations}-iteration cap",
                    "kernel": "fit64_kernel<6>: the reference method in double, bit-identical "
                              "to the FP64 oracle"}
    # Coefficient builder (bsarray, degree 3) on the 5D grid: GPU kernel
    # against the numpy restatement on the host.
    prefilter_fig = None
    if not args.no_prefilter:
        from bsfit import prefilter as PF
        grid = (9, 18, 41, 34, 34)  # (U, W, Z, X, Y) of the 5D figure's model
        smp = np.random.default_rng(3).random(grid)
        xs = torch.from_numpy(smp).to(dev)
        with torch.cuda.stream(stream):
            bsfit.bsarray_coeffs_torch(xs, stream=stream)
            ap, bp = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ap.record(stream)
            for _ in range(3):
                bsfit.bsarray_coeffs_torch(xs, stream=stream)
            bp.record(stream)
        stream.synchronize()
        t0 = time.perf_counter()
        PF.bsarray_coeffs(smp)
        cpu_s = time.perf_counter() - t0
        prefilter_fig = {"grid": "x".join(str(g) for g in reversed(grid)) + " (Y, X, Z, W, U) float64",
                         "gpu_ms": ap.elapsed_time(bp) / 3, "cpu_numpy_ms": cpu_s * 1e3}
    frontend_fig = None if args.no_frontend else bench_frontend(dev, stream)
    serving = None if args.no_serve else bench_serving(args, dev)
    if rank != 0:
        return 0
    cpu_n, cpu_t = run_cpu(groups, os.cpu_count() or 1, 0.016)
    # one core, as the reference's CPU mex runs (a loop over ROIs on one thread)
    cpu1_n, cpu1_t = run_cpu(groups, 1, 0.002)
    # DRAM traffic of the fitter per step: the ncu capture of the batched
    # kernel on 200k ROIs of the same size mix (summarised under profiles/)
    # measured its bytes against the algorithmic 4 s^2 + 48 B per ROI; the
    # step's traffic is that ratio times the step's algorithmic bytes.
    traffic = None
    issue = None
    tpath = os.path.join(ROOT, "profiles", "traffic_batch_kernel_3d.json")
    if os.path.exists(tpath):
        try:
            prof = json.load(open(tpath))
            ratio = float(prof["measured_over_algorithmic"])
            traffic = ratio * sum((4 * g.roi_size ** 2 + 48) * len(g.rois) for g in groups)
            # The binding limit of this kernel is instruction issue, not FMA
            # throughput: the fraction of the SM's issue rate it sustains.
            issue = {"ipc": prof["ipc"], "max_ipc": prof["max_ipc"],
                     "frac": prof["ipc"] / prof["max_ipc"],
                     "source": "ncu, profiles/batch_kernel_3d_200k.md"}
        except Exception:
            traffic = None
    line = {
        "metric": METRIC, "value": value, "unit": "fits/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded); inputs > L2, no flush",
        "config": {"workload": "3d_batched_1M_11-13-17", "rois": n_step, "fit_type": 6,
                   "iterations": ITERATIONS, "roi_sizes": list(SIZES), "size_ratio": [1, 2, 1],
                   "mean_iterations": mean_iter, "launches_per_step": 1, "form": "batched",
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": e2e_value, "unit": "fits/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                "step_ms_min": min(e2e_ms), "step_ms_median": float(np.median(e2e_ms)),
                "step_ms_max": max(e2e_ms),
                "host_buffers": "page-locked inputs and outputs, allocated once"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "measured FP32 FMA throughput on this device, the higher of "
                                    "scalar FFMA and paired FFMA2 chains (bsfit_measure_fp32_peaks); "
                                    "MEASURED_PEAKS.json has no FP32 figure",
                     "peak_scalar_tflops": peak_scalar, "peak_paired_tflops": peak_paired,
                     "peak_theoretical_tflops": 152 * 128 * 2 * 2.07e9 * 1e-12,
                     "flops_per_step": flops, "kernel_ms_per_step": kernel_ms,
                     "per": "launch (the batched step is one persistent launch over all sizes)",
                     "issue": issue},
        "plain_form": {"value": n_step / (plain_ms * 1e-3), "unit": "fits/s",
                       "launches_per_step": len(groups),
                       "kernel_ms_by_size": dict(zip([str(s) for s in SIZES], per_launch))},
        "cpu_baseline": {"value": cpu_n / cpu_t, "unit": "fits/s", "cores": os.cpu_count(),
                         "kind": "port",
                         "sample": f"{cpu_n} ROIs (1.6% of each size group), FP32 oracle port of "
                                   f"the reference CPU fitter, OpenMP over ROIs",
                         "single_core": {"value": cpu1_n / cpu1_t, "unit": "fits/s", "cores": 1,
                                         "sample": f"{cpu1_n} ROIs (0.2% of each size group)"}},
        "fits_per_s": {"3d_13px": fits_3d13, "4d_13px": fits_4d13,
                       "4d_workload": f"{args.rois_4d} ROIs 13x13, fit type 7, 60 iterations",
                       "5d_17px": fits_5d17,
                       "5d_workload": f"{args.rois_5d} ROIs 17x17, fit type 8, 60 iterations",
                       "4pi_13px": fits_4pi,
                       "4pi_workload": f"{args.rois_4pi} ROIs of 4 channels 13x13, 100 iterations"},
        "autotune": {"per_size": tuned,
                     "sample": f"{args.tune_rois} ROIs of each size group",
                     "batched_uses": str(max(SIZES)),
                     "per_model": tuned_models,
                     "per_model_sample": "20000 ROIs of the 4D figure, 5000 of the 5D figure"}
        if tuned else None,
        "config_3_colour": c3_fig,
        "config_4_4pi": c4_fig,
        "parity_precision": parity_fig,
        "reference_precision": fp64_fig,
        "prefilter": prefilter_fig,
        "frontend": frontend_fig,
        "serving": serving,
        "clocks": clk.summary(),
        "gpu_launches": args.steps,
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--kernel-only", action="store_true",
                    help="profiling case: only the fit launches of --rois ROIs of --sizes")
    ap.add_argument("--rois", type=int, default=N_ROIS)
    ap.add_argument("--batched", action="store_true", help="kernel-only: the batched form")
    ap.add_argument("--variant", type=int, default=None,
                    help="kernel-only, 3D: force this tuner variant (with --wpb warps per block)")
    ap.add_argument("--wpb", type=int, default=0, help="kernel-only: warps per block with --variant")
    ap.add_argument("--iterations", type=int, default=ITERATIONS,
                    help="kernel-only, 3D: the LM iteration cap (0: initial and CRLB passes only)")
    ap.add_argument("--eval", action="store_true",
                    help="kernel-only, 3D: the evaluation kernel at the fitted parameters")
    ap.add_argument("--model", default="3d", choices=["3d", "4d", "5d", "4pi", "3d64"],
                    help="kernel-only: model")
    ap.add_argument("--sizes", type=int, nargs="+", default=list(SIZES))
    ap.add_argument("--precision", default="f32", choices=["f32", "parity"],
                    help="kernel-only: the FP32 or the parity-grade (double-float) kernels")
    ap.add_argument("--rois-5d", type=int, default=50000, help="ROIs of the 5D 17 px figure")
    ap.add_argument("--no-5d", action="store_true")
    ap.add_argument("--rois-4d", type=int, default=50000, help="ROIs of the 4D 13 px figure")
    ap.add_argument("--no-4d", action="store_true")
    ap.add_argument("--rois-4pi", type=int, default=100000, help="ROIs of the 4Pi figure")
    ap.add_argument("--no-4pi", action="store_true")
    ap.add_argument("--rois-c3", type=int, default=500000, help="ROIs of the colour configuration")
    ap.add_argument("--no-c3", action="store_true")
    ap.add_argument("--rois-c4", type=int, default=250000, help="ROIs of the 4Pi configuration")
    ap.add_argument("--no-c4", action="store_true")
    ap.add_argument("--rois-parity", type=int, default=100000,
                    help="3D ROIs of the parity-grade figure (4D: half, 5D: a tenth)")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--tune-rois", type=int, default=100000)
    ap.add_argument("--no-prefilter", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="reference arm: skip the reference GPU kernel figure")
    ap.add_argument("--rois-fp64", type=int, default=100000, help="ROIs of the FP64 figure")
    ap.add_argument("--no-frontend", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-frames", type=int, default=80)
    args = ap.parse_args()
    if args.impl == "reference":
        return bench_reference(args)
    if args.kernel_only:
        return bench_kernel_only(args)
    return bench_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
