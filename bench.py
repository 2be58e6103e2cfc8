"""Benchmark: the large single bootstrap filter on GB300.

Workload: the 4D constant-velocity tracking model with Student-t (nu 10,
scale 0.5) position observations simulated from the model (seed 0), T = 200
steps, N = 2^24 particles, FP32 SoA state, FP64 block-level log-sum-exp, an
exact 64-bit fixed-point CDF, systematic resampling when ESS < N / 2.
One bench step = one complete filter run (initialize + 199 iterations) =
N * T particle-steps.  The metric is particle-steps per second.

    value  device-resident: observations already in HBM (vsmc_cuda_pf_run_device)
    e2e    through the C ABI with pinned host buffers (vsmc_cuda_pf_run):
           observations copied in, histories copied out, every step
    roofline  the fused move / likelihood / weight kernel, timed with CUDA
           events on the filter's stream, against the measured HBM copy peak
    cpu_baseline  the oracle's C restatement of the reference filter on the
           host cores (OpenMP), on a bounded sample of the workload

`--impl reference` times the reference arm: the oracle restatement of the
reference's CPU filter (the reference tree is not present on the GPU host),
rank 0 only.

Multi-GPU (torchrun): every rank runs an independent filter replica (the path
does not shard across filters); value = all ranks' particle-steps / max time.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_PARTICLES = 1 << 24
T_STEPS = 200
SCHEME = 2  # systematic
THRESHOLD = 0.5
L2_BYTES = 126 * 1024 * 1024
BYTES_PER_PARTICLE_STEP = 40  # 16 state read + 16 state write + 4 lw read + 4 lw write
METRIC = "particle-steps/sec (plain bootstrap filter)"
UNIT = "particle-steps/s"


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def measured_bf16_sustained():
    """Dense BF16 TFLOP/s of a seconds-long cuBLAS loop (the peak for a
    kernel timed inside a long run)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        if "bf16_tflops_sustained" in d:
            return float(d["bf16_tflops_sustained"]), "measured"
    return 1700.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}",
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"],
                    "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, nm in enumerate(names):
                if r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_setup(gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    """The largest x over all ranks (the slowest rank's time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank):
    """Each rank runs an independent filter replica with its own seed."""
    return 1 + rank


def aggregate_rate(units_per_rank, world, seconds_max):
    """Whole-job throughput: every rank's units over the slowest rank's time."""
    return world * units_per_rank / seconds_max


def simulate_obs(vc, T, seed=0):
    """Observations simulated on the device by the product simulator."""
    import torch
    truth = torch.zeros(4 * T, dtype=torch.float64, device="cuda")
    obs = torch.zeros(2 * T, dtype=torch.float64, device="cuda")
    m = vc.default_model()
    vc.call("vsmc_cuda_cv_simulate", seed, T, ctypes.byref(m),
            truth.data_ptr(), obs.data_ptr(),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return obs


def cpu_filter_rate(n, T, threads=0, seed=0):
    """Oracle restatement of the reference filter on host cores (FP32 state,
    systematic, ESS < N/2); returns (particle-steps/s, seconds, threads)."""
    from oracle import binding
    port = binding.port()
    m = binding.default_model()
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    port.vo_pf_simulate(seed, T, ctypes.byref(m), P(tr), P(ob))
    mean = np.zeros(2 * T)
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    logz = np.zeros(T)
    t0 = time.perf_counter()
    port.vo_pf_run(32, n, T, 1, SCHEME, THRESHOLD, ctypes.byref(m), P(ob),
                   threads, P(mean), P(ess), P(res), P(logz))
    dt = time.perf_counter() - t0
    nthreads = threads if threads > 0 else (os.cpu_count() or 1)
    return n * T / dt, dt, nthreads


def ref_filter_rate(n, T, seed=0):
    """The reference's own filter on host cores: its Sampler<T> with the
    OpenMP backend (StateOMP / MoveOMP / MonitorEvalOMP) from oracle/_ref,
    built from the reference's sources where they are present.  Returns
    (particle-steps/s, seconds, threads), or None without the build."""
    from oracle import binding
    if binding.build_ref() is None:
        return None
    ref = binding.ref()
    if ref is None:
        return None
    port = binding.port()
    m = binding.default_model()
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    port.vo_pf_simulate(seed, T, ctypes.byref(m), P(tr), P(ob))
    mean = np.zeros(2 * T)
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    logz = np.zeros(T)
    # the reference's OpenMP backend takes every host thread (OMP default)
    nthreads = int(os.environ.get("OMP_NUM_THREADS", "0")) or \
        (os.cpu_count() or 1)
    t0 = time.perf_counter()
    ref.ref_pf_run(32, n, T, 1, SCHEME, THRESHOLD, 0, m.dt, m.sigma_a,
                   m.obs_scale, m.nu, m.sd_pos0, m.sd_vel0, P(ob), P(mean),
                   P(ess), P(res), P(logz))
    dt = time.perf_counter() - t0
    return n * T / dt, dt, nthreads


def run_cpu_compare(args):
    """The reference itself (oracle/_ref) and the oracle's C restatement on
    the same sample and the same host threads: one JSON line with both
    rates and their ratio."""
    n, T = 1 << 20, 20
    ref_filter_rate(n, T)  # warm-up (and the build)
    cpu_filter_rate(n, T)
    r = ref_filter_rate(n, T)
    p = cpu_filter_rate(n, T)
    line = {"cpu_compare": "N=2^20 particles x T=20 steps, FP32 state, "
                           "systematic, ESS < N/2",
            "threads": p[2], "port": p[0],
            "reference": r[0] if r else None,
            "port_over_reference": (p[0] / r[0]) if r else None}
    print(json.dumps(line), flush=True)
    return 0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    n, T = 1 << 20, 50
    # the reference itself where it can be built here, else its C
    # restatement (the reference tree is absent on the GPU host)
    kind = "reference" if ref_filter_rate(1 << 12, 2) is not None else "port"
    rate = ref_filter_rate if kind == "reference" else cpu_filter_rate
    for _ in range(args.warmup):
        rate(n, T)
    total = 0.0
    rates = []
    for _ in range(args.steps):
        r, dt, threads = rate(n, T)
        total += dt
        rates.append(r)
    value = n * T * args.steps / total
    sample = (f"N=2^20 particles x T={T} steps per bench step (the "
              f"N=2^24, T=200 workload scaled down), FP32 state, systematic"
              + (", the reference's Sampler<T> with its OpenMP backend"
                 if kind == "reference" else
                 ", the oracle's C restatement of the reference filter"))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (observations simulated from the model, seed 0)",
        "config": {"workload": "large single bootstrap filter (CPU sample)",
                   "particles": n, "steps_T": T, "scheme": "systematic",
                   "threshold": THRESHOLD},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads,
                         "kind": kind, "sample": sample},
        "same_config": False,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def batched_spec(nf, seed):
    """Batched-filter workload: per filter acceleration sd ~ U(0.5, 2),
    observation scale ~ U(0.2, 1), particles log-uniform in [2^8, 2^16],
    horizon uniform in [50, 500]; seeded."""
    import vsmc_gb300 as vc
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(2.0 ** 8), np.log(2.0 ** 16), nf))
    n = np.minimum(np.round(n), 2 ** 16).astype(np.uint32)
    T = rng.integers(50, 501, nf).astype(np.uint32)
    models = []
    for _ in range(nf):
        m = vc.default_model()
        m.sigma_a = float(rng.uniform(0.5, 2.0))
        m.obs_scale = float(rng.uniform(0.2, 1.0))
        models.append(m)
    return n, T, models


def run_batched(args):
    """4096 independent filters stepped together (one persistent step kernel
    and one per-filter resampling kernel per step, the run as one graph)."""
    import torch
    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import vsmc_gb300 as vc
    vc.lib()
    nf = args.filters
    n, T, models = batched_spec(nf, 20261203 + rank)
    seeds = (np.arange(nf) + (rank << 20)).astype(np.uint32)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    b = vc.FilterBatch(n, T, seeds, models, scheme=vc.STRATIFIED,
                       stream=ctypes.c_void_p(stream.cuda_stream))
    obs = torch.zeros(b.obs_len(), dtype=torch.float64, device="cuda")
    b.simulate(obs.data_ptr())
    tune_ms = b.autotune(obs.data_ptr(), steps=args.tune_steps)
    shape = b.shape()
    for _ in range(args.warmup):
        b.run_device(obs.data_ptr())
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        b.run_device(obs.data_ptr())
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = ev0.elapsed_time(ev1)
    hist = b.history()
    # end to end: pinned host observations in, histories out, every run
    TT = b.total_steps
    obs_h = torch.empty(b.obs_len(), dtype=torch.float64, pin_memory=True)
    obs_h.copy_(obs.cpu())
    mean_h = torch.empty(2 * TT, dtype=torch.float64, pin_memory=True)
    ess_h = torch.empty(TT, dtype=torch.float64, pin_memory=True)
    res_h = torch.empty(TT, dtype=torch.int32, pin_memory=True)
    logz_h = torch.empty(TT, dtype=torch.float64, pin_memory=True)
    L = vc.lib()

    def e2e_run():
        vc.check(L.vsmc_cuda_batch_run(b.handle, obs_h.data_ptr(),
                                       mean_h.data_ptr(), ess_h.data_ptr(),
                                       res_h.data_ptr(), logz_h.data_ptr()),
                 "vsmc_cuda_batch_run")

    e2e_run()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(2, args.steps // 2)
    for _ in range(e2e_steps):
        e2e_run()
    e2e_s = time.perf_counter() - t0
    clocks.stop()
    psteps = float(b.particle_steps())
    b.close()
    ms_max = max_over_ranks(ms, world)
    e2e_max = max_over_ranks(e2e_s, world)
    value = aggregate_rate(psteps * args.steps, world, ms_max / 1000.0)
    peak, peak_kind = measured_peaks()
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import binding
        port = binding.port()
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        obs_np = obs_h.numpy().reshape(-1, 2)
        offs = np.concatenate([[0], np.cumsum(T.astype(np.int64))])
        done = 0.0
        t0 = time.perf_counter()
        k = 0
        while k < nf and time.perf_counter() - t0 < 10.0:
            Tk = int(T[k])
            om = binding.default_model()
            om.sigma_a = models[k].sigma_a
            om.obs_scale = models[k].obs_scale
            o = np.ascontiguousarray(obs_np[offs[k]:offs[k + 1]])
            z = np.zeros(2 * Tk)
            e = np.zeros(Tk)
            r = np.zeros(Tk, np.int32)
            lz = np.zeros(Tk)
            port.vo_pf_run(32, int(n[k]), Tk, int(seeds[k]), 1, 0.5,
                           ctypes.byref(om), P(o), 0, P(z), P(e), P(r), P(lz))
            done += float(n[k]) * Tk
            k += 1
        dt = time.perf_counter() - t0
        cpu = {"value": done / dt, "unit": UNIT,
               "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"the first {k} filters of the batch, one after "
                         "another, oracle restatement (OpenMP move)"}
    if rank == 0:
        line = {
            "metric": "particle-steps/sec (batched bootstrap filters)",
            "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (each filter's observations simulated from "
                    "its own model on the device)",
            "config": {"workload": f"{nf} batched filters: particles "
                                   "log-uniform [2^8, 2^16], horizons "
                                   "U[50, 500], sigma_a U(0.5, 2), obs scale "
                                   "U(0.2, 1), stratified, ESS < N/2",
                       "particle_steps_per_run": psteps,
                       "shape_ppt_block": list(shape),
                       "autotune_ms": [float(x) for x in tune_ms],
                       "resampled_fraction": float(np.mean(
                           [h["resampled"].mean() for h in hist])),
                       "l2": "state 2 x 4 x 4 B x sum N >> L2; no flush"},
            "e2e": {"value": aggregate_rate(psteps * e2e_steps, world,
                                            e2e_max),
                    "unit": UNIT, "h2d_bytes_per_step": 16 * TT,
                    "d2h_bytes_per_step": (16 + 8 + 4 + 8) * TT},
            "roofline": {"bound": "hbm",
                         "achieved": BYTES_PER_PARTICLE_STEP * psteps /
                         (ms_max / args.steps / 1000.0) / 1e9,
                         "peak": peak, "unit": "GB/s",
                         "peak_source": peak_kind,
                         "scope": "whole run (step + resampling kernels), "
                                  "40 B per particle-step"},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            # per run: the observation conversion and the reset, then per
            # global step the step kernel and the three resampling passes
            "gpu_launches": (2 + 4 * (int(T.max()) + 1)) * args.steps,
        }
        line["roofline"]["frac"] = line["roofline"]["achieved"] / peak
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_micro(args):
    """RNG and resampling microbenchmarks (the 2^30-word RNG and N = 2^24
    resampling workload): every call goes through the public C ABI, output
    in HBM; each item is the median of `steps` calls, each timed with CUDA
    events, after `warmup` calls.  Headline: raw Philox4x32-10 words/s."""
    import torch
    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import vsmc_gb300 as vc
    vc.lib()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    nw = 1 << args.rng_log2
    buf = torch.empty(8 * nw, dtype=torch.uint8, device="cuda")
    peak, peak_kind = measured_peaks()

    def timed(fn):
        """Median over `steps` calls, each between its own CUDA events (the
        resampling calls synchronize with the host, so one slow host-side
        call would otherwise weigh on the mean)."""
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True),
               torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        for e0, e1 in ev:
            e0.record(stream)
            fn()
            e1.record(stream)
        torch.cuda.synchronize()
        return float(np.median([e0.elapsed_time(e1) for e0, e1 in ev])) / 1000.0

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    items = {}
    # (name, engine kind, entry point, extra args, output bytes per value)
    rng_items = [
        ("philox4x32_u32", vc.PHILOX4X32, "vsmc_cuda_rng_rand", (), 4),
        ("threefry4x64_u64", vc.THREEFRY4X64, "vsmc_cuda_rng_rand", (), 8),
        ("u01_f64", vc.PHILOX4X32, "vsmc_cuda_rng_u01", (), 8),
        ("u01_f32", vc.PHILOX4X32, "vsmc_cuda_rng_u01_f32", (), 4),
        ("normal_f64", vc.PHILOX4X32, "vsmc_cuda_rng_normal",
         (ctypes.c_double(0.0), ctypes.c_double(1.0)), 8),
        ("normal_f32", vc.PHILOX4X32, "vsmc_cuda_rng_normal_f32",
         (ctypes.c_float(0.0), ctypes.c_float(1.0)), 4),
    ]
    wanted = set(args.items.split(",")) if args.items else None

    def keep(name):
        # the headline item always runs
        return wanted is None or name in wanted or name == "philox4x32_u32"

    for name, kind, fn, extra, vb in rng_items:
        if not keep(name):
            continue
        r = vc.rng(kind, seed=1)
        sec = timed(lambda: vc.call(fn, ctypes.byref(r), nw, buf.data_ptr(),
                                    *extra, sptr))
        items[name] = {"values": nw, "seconds": sec, "values_per_s": nw / sec,
                       "GB_per_s": vb * nw / sec / 1e9,
                       "frac_hbm": vb * nw / sec / 1e9 / peak}
    # resampling: normalised FP64 weights from log w ~ N(0, 3^2)
    n = 1 << args.rs_log2
    lw = np.random.default_rng(7).normal(0.0, 3.0, n)
    w = np.exp(lw - lw.max())
    w /= w.sum()
    w_dev = torch.from_numpy(w).cuda()
    rep = torch.empty(n, dtype=torch.int32, device="cuda")
    names = ["multinomial", "stratified", "systematic", "residual",
             "residual_stratified", "residual_systematic"]
    for scheme, name in enumerate(names):
        if not keep("resample_" + name):
            continue
        r = vc.rng(vc.PHILOX4X32, seed=1)
        sec = timed(lambda: vc.call("vsmc_cuda_resample", n, n,
                                    ctypes.byref(r), w_dev.data_ptr(),
                                    rep.data_ptr(), scheme, sptr))
        items["resample_" + name] = {
            "particles": n, "seconds": sec, "particles_per_s": n / sec,
            "GB_per_s": 12 * n / sec / 1e9,
            "frac_hbm": 12 * n / sec / 1e9 / peak}
    # the learned proposal's network on the tensor cores: loss + gradient
    # of a 65536-row minibatch (weight gradients on tcgen05), and the
    # forward pass over 2^20 rows in both forms (mma.sync per warp, tcgen05
    # per 128-row tile)
    mlp_items = [name for name in ("mlp_loss_grad", "mlp_forward",
                                   "mlp_forward_tc") if keep(name)]
    if mlp_items and wanted is not None:
        nparams = ctypes.c_size_t()
        npacked = ctypes.c_size_t()
        vc.call("vsmc_cuda_mlp_sizes", ctypes.byref(nparams),
                ctypes.byref(npacked))
        g = np.random.default_rng(5)
        params = torch.from_numpy(
            g.normal(0, 0.3, nparams.value).astype(np.float32)).cuda()
        packed = torch.empty(npacked.value, dtype=torch.int32, device="cuda")
        vc.call("vsmc_cuda_mlp_pack", params.data_ptr(), packed.data_ptr(),
                sptr)
        flops_row = 2.0 * (6 * 64 + 64 * 64 + 64 * 8)  # useful forward MACs
        for name in mlp_items:
            B = 1 << 16 if name == "mlp_loss_grad" else 1 << 20
            feat = torch.from_numpy(
                g.normal(0, 1, (B, 6)).astype(np.float32)).cuda()
            if name == "mlp_loss_grad":
                nu = torch.from_numpy(
                    g.normal(0, 1, (B, 4)).astype(np.float32)).cuda()
                loss = torch.zeros(1, dtype=torch.float64, device="cuda")
                grad = torch.zeros(nparams.value, dtype=torch.float32,
                                   device="cuda")
                fn = lambda: vc.call(  # noqa: E731
                    "vsmc_cuda_mlp_loss_grad", packed.data_ptr(), B,
                    feat.data_ptr(), nu.data_ptr(), loss.data_ptr(),
                    grad.data_ptr(), sptr)
            else:
                out = torch.empty((B, 8), dtype=torch.float32, device="cuda")
                entry = "vsmc_cuda_" + name
                fn = lambda: vc.call(  # noqa: E731
                    entry, packed.data_ptr(), B, feat.data_ptr(),
                    out.data_ptr(), sptr)
            sec = timed(fn)
            items[name] = {"rows": B, "seconds": sec, "rows_per_s": B / sec,
                           "forward_TFLOP_per_s": flops_row * B / sec / 1e12}
    clocks.stop()
    # end to end: Philox words into pinned host memory through the C ABI
    host = torch.empty(4 * nw, dtype=torch.uint8, pin_memory=True)
    r = vc.rng(vc.PHILOX4X32, seed=1)

    def e2e_call():
        vc.call("vsmc_cuda_rng_rand", ctypes.byref(r), nw, buf.data_ptr(),
                sptr)
        host.copy_(buf[:4 * nw], non_blocking=True)

    e2e_s = timed(e2e_call)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import binding
        port = binding.port()
        ns = 1 << 24
        out = np.zeros(ns, np.uint32)
        key = (ctypes.c_uint32 * 2)(1, 0)
        ctr = (ctypes.c_uint32 * 4)(0, 0, 0, 0)
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < 3.0:
            port.vo_philox4x32_words(key, ctr, ns, out.ctypes.data, 1)
            reps += 1
        dt = time.perf_counter() - t0
        cpu = {"value": ns * reps / dt, "unit": "words/s", "cores": 1,
               "kind": "port",
               "sample": f"{reps} x 2^24 Philox4x32-10 words, bulk path, "
                         "oracle restatement, one core"}
        nr = 1 << 22
        wr = w[:nr] / w[:nr].sum()
        repc = np.zeros(nr, np.int32)
        nxt = (ctypes.c_uint32 * 4)()
        t0 = time.perf_counter()
        port.vo_resample_words(1, nr, nr, key, ctr, wr.ctypes.data,
                               repc.ctypes.data, nxt)
        dt = time.perf_counter() - t0
        cpu["resample_stratified_particles_per_s"] = nr / dt
    ph = items["philox4x32_u32"]
    line = {
        "metric": "words/sec (Philox4x32-10 raw u32 through the engine's "
                  "bulk path)",
        "value": ph["values_per_s"], "unit": "words/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * ph["seconds"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (counter-based streams; weights from a seeded "
                "N(0, 3^2) log-weight draw)",
        "config": {"workload": f"RNG 2^{args.rng_log2} values per call; "
                               f"resampling N = 2^{args.rs_log2}, all six "
                               "schemes, FP64 weights",
                   "l2": "outputs 4-8 GiB >> L2; no flush",
                   "items": items},
        "e2e": {"value": nw / e2e_s, "unit": "words/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 4 * nw},
        "roofline": {"bound": "hbm", "achieved": ph["GB_per_s"],
                     "peak": peak, "unit": "GB/s", "peak_source": peak_kind,
                     "frac": ph["frac_hbm"],
                     "scope": "4 B written per word; the generator is "
                              "integer-pipe work (ncu pipe counters in "
                              "profiles)"},
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "gpu_launches": args.steps,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_learned(args):
    """Learned proposal vs bootstrap on the bearings-only model: R filters
    (independent seeds) on one simulated observation sequence; log-evidence
    SD over the R runs and the error of the posterior mean against an FP64
    oracle reference; the headline is the bootstrap-equivalent
    particle-step rate of the learned filter at equal log-evidence SD."""
    import torch
    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import vsmc_gb300 as vc
    vc.lib()
    m = vc.bearings_model()
    m.dt, m.q, m.sd_vel0 = args.bearings_dt, args.bearings_q, args.bearings_sdv
    T, R = 200, args.replicates
    obs = torch.zeros(T, dtype=torch.float64, device="cuda")
    truth = torch.zeros(4 * T, dtype=torch.float64, device="cuda")
    vc.call("vsmc_cuda_bearings_simulate", 0, T, ctypes.byref(m),
            truth.data_ptr(), obs.data_ptr(), None)
    obs_np = obs.cpu().numpy()
    # ---- training on simulated trajectories plus rows from the particle
    # clouds of bootstrap filters run on simulated tracks
    prop = vc.Proposal(seed=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rows = None
    if args.cloud_tracks > 0:
        rows = vc.cloud_rows(m, 12, args.cloud_tracks, args.cloud_particles,
                             T, args.cloud_candidates)
    losses = prop.train(m, seed=11, ntraj=args.train_traj, T=T,
                        batch=args.train_batch, steps=args.train_steps,
                        lr=args.lr, rows=rows)
    train_s = time.perf_counter() - t0
    cloud_rows_n = 0 if rows is None else int(rows[1].shape[0])
    del rows
    # ---- reference posterior mean (FP64 oracle bootstrap, host cores)
    ref_mean = None
    if not args.no_cpu_baseline:
        from oracle import binding
        port = binding.port()
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        Nref = args.ref_particles
        mean = np.zeros(2 * T)
        ess = np.zeros(T)
        res = np.zeros(T, np.int32)
        logz = np.zeros(T)
        t0 = time.perf_counter()
        om = binding.bearings_model()
        om.dt, om.q, om.sd_vel0 = m.dt, m.q, m.sd_vel0
        port.vo_bearings_pf_run(64, Nref, T, 123, 1, 0.5, ctypes.byref(om),
                                P(obs_np), None, 0, P(mean), P(ess), P(res),
                                P(logz))
        ref_s = time.perf_counter() - t0
        ref_mean = mean.reshape(T, 2)

    obs_all = torch.from_numpy(np.tile(obs_np, R)).cuda()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def measure(N, packed):
        b = vc.FilterBatch([N] * R, [T] * R, np.arange(R) + 1000,
                           models=[m] * R, bearings=True, packed=packed,
                           stream=ctypes.c_void_p(stream.cuda_stream))
        for _ in range(args.warmup):
            b.run_device(obs_all.data_ptr())
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            b.run_device(obs_all.data_ptr())
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / args.steps
        out = b.history()
        b.close()
        logz = np.array([o["logz"][-1] for o in out])
        # variance of the cumulative log-evidence over the R filters, by step
        lz_all = np.stack([o["logz"] for o in out])
        var_at = {str(t): float(lz_all[:, t].var())
                  for t in (0, 10, 30, 50, 100, T - 1)}
        ess_at = {str(t): float(np.mean([o["ess"][t] for o in out]) / N)
                  for t in (0, 10, 30, 50, 100, T - 1)}
        means = np.stack([o["mean"] for o in out])  # R x T x 2
        err = None
        if ref_mean is not None:
            err = float(np.sqrt(np.mean((means.mean(axis=0) - ref_mean) ** 2)))
        return {"N": N, "ms": ms, "rate": N * T * R / (ms / 1000.0),
                "logz_sd": float(logz.std()), "logz_mean": float(logz.mean()),
                "logz_var_by_step": var_at, "ess_frac_by_step": ess_at,
                "mean_rmse_vs_ref": err}

    clocks = ClockSampler(local)
    clocks.start()
    learned = measure(args.learned_particles, prop.packed.data_ptr())
    boot = [measure(N, None) for N in args.boot_particles]
    clocks.stop()
    # end to end: the learned filters through the C ABI, host observations
    # in and histories out every run
    NL = args.learned_particles
    b = vc.FilterBatch([NL] * R, [T] * R, np.arange(R) + 1000,
                       models=[m] * R, bearings=True,
                       packed=prop.packed.data_ptr(),
                       stream=ctypes.c_void_p(stream.cuda_stream))
    obs_h = torch.from_numpy(np.tile(obs_np, R)).pin_memory()
    hist_h = {k: torch.empty(R * T * w, dtype=dt, pin_memory=True)
              for k, w, dt in (("mean", 2, torch.float64),
                               ("ess", 1, torch.float64),
                               ("res", 1, torch.int32),
                               ("logz", 1, torch.float64))}
    L = vc.lib()

    def e2e_run():
        vc.check(L.vsmc_cuda_batch_run(
            b.handle, obs_h.data_ptr(), hist_h["mean"].data_ptr(),
            hist_h["ess"].data_ptr(), hist_h["res"].data_ptr(),
            hist_h["logz"].data_ptr()), "vsmc_cuda_batch_run")

    e2e_run()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(2, args.steps // 2)
    for _ in range(e2e_steps):
        e2e_run()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    b.close()
    h2d = obs_h.numel() * 8
    d2h = sum(v.numel() * v.element_size() for v in hist_h.values())
    # bootstrap N at the learned filter's log-evidence SD (log-log fit)
    lx = np.log([b["N"] for b in boot])
    ly = np.log([b["logz_sd"] for b in boot])
    slope, icpt = np.polyfit(lx, ly, 1)
    n_eq = float(np.exp((np.log(learned["logz_sd"]) - icpt) / slope))
    # bootstrap wall time at n_eq (linear in N between the measured points)
    ms_eq = float(np.interp(n_eq, [b["N"] for b in boot],
                            [b["ms"] for b in boot],
                            left=None, right=None))
    if n_eq > boot[-1]["N"]:
        ms_eq = boot[-1]["ms"] * n_eq / boot[-1]["N"]
    value = n_eq * T * R / (learned["ms"] / 1000.0)
    # the network's FLOPs per learned particle-step (t >= 1), unpadded:
    # 2 (6 x 64 + 64 x 64 + 64 x 8)
    flops = 2.0 * (6 * 64 + 64 * 64 + 64 * 8) * NL * (T - 1) * R
    achieved = flops / (learned["ms"] / 1000.0) / 1e12
    tpeak, tpeak_kind = measured_bf16_sustained()
    line = {
        "metric": "particle-steps/sec at fixed log-evidence SD "
                  "(learned proposal, bootstrap-equivalent)",
        "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": learned["ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 network (fp32 accumulate), fp32 state",
        "data": "synthetic bearings-only track (seed 0), T=200",
        "model": {"dt": m.dt, "q": m.q, "sigma_z": m.sigma_z,
                  "start": [m.x0, m.y0], "sd_pos0": m.sd_pos0,
                  "sd_vel0": m.sd_vel0},
        "config": {
            "workload": f"{R} filters x N={args.learned_particles} learned "
                        f"proposal vs bootstrap N in {args.boot_particles}",
            "train": {"trajectories": args.train_traj, "steps": T,
                      "cloud_tracks": args.cloud_tracks,
                      "cloud_particles": args.cloud_particles,
                      "cloud_candidates": args.cloud_candidates,
                      "cloud_rows": cloud_rows_n,
                      "batch": args.train_batch, "lr": args.lr,
                      "adam_steps": len(losses), "seconds": train_s,
                      "loss_first": float(losses[:50].mean()),
                      "loss_last": float(losses[-50:].mean())},
            "learned": learned, "bootstrap": boot,
            "bootstrap_n_at_equal_sd": n_eq,
            "bootstrap_ms_at_equal_sd": ms_eq,
            "speedup_at_equal_sd": ms_eq / learned["ms"],
            "reference": {"particles": args.ref_particles, "fp64": True,
                          "seconds": ref_s} if ref_mean is not None else None,
            "l2": "state 2 x 4 x 4 B x 2^22 particles = 128 MiB per learned "
                  "run's buffers, about L2; the network is in shared memory",
        },
        "e2e": {"value": n_eq * T * R / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "tensor", "achieved": achieved,
                     "peak": tpeak, "unit": "TFLOP/s",
                     "frac": achieved / tpeak, "peak_source": tpeak_kind,
                     "scope": "proposal network FLOPs of the learned run "
                              "over its wall time; the step kernel is "
                              "bound by the activations' ALU/SFU work and "
                              "latency, not the tensor pipe",
                     "traffic": None},
        "gpu_launches": (2 + 6 * (T + 1)) * args.steps,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def build_sampler_program(ref, out_dir):
    """nvcc build of tests/cpp/sampler_cuda.cu (vSMC's Sampler<T> on the
    fused FP32 backend, include/vsmc_cuda_sampler.cuh) against the reference
    tree `ref`; returns the binary's path."""
    from vsmc_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = os.path.join(out_dir, "sampler_cuda")
    cmd = [os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc"), "-std=c++17",
           "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ref, "include"),
           "-I", os.path.join(ROOT, "tests", "cpp", "shim"),
           "-I", os.path.join(ROOT, "include"),
           "-DVSMC_RNG_TYPE=::vsmc::Philox4x32", "-DVSMC_HAS_MKL=0",
           "-DVSMC_HAS_TBB=0", "-Xcompiler", "-w"]
    if os.uname().machine == "aarch64":
        cmd += ["-DVSMC_UTILITY_SIMD_HPP", "-DVSMC_HAS_SSE2=0",
                "-DVSMC_HAS_AVX2=0", "-DVSMC_HAS_AES_NI=0",
                "-DVSMC_HAS_RDRAND=0"]
    cmd += [os.path.join(ROOT, "tests", "cpp", "sampler_cuda.cu"), "-o", exe,
            "-L", libdir, "-lvsmc_cuda", f"-Xlinker=-rpath={libdir}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def run_sampler(args):
    """The large single filter driven by the reference's own Sampler<T>
    (initialize + iterate, Particle::resample, Monitor::eval) on the fused
    FP32 backend, with the model a user device functor: the plugin API a
    vSMC user switches to.  Each bench step is one whole run, timed on the
    host clock around initialize + T - 1 iterates (the Sampler API waits for
    every step's ESS, so the device work is inside it).  Needs the
    reference's headers (VSMC_REF_ROOT) to compile the program."""
    import tempfile
    import torch
    ref = os.environ.get("VSMC_REF_ROOT")
    if not ref or not os.path.isdir(os.path.join(ref, "include", "vsmc")):
        print(json.dumps({"metric": METRIC + " through vsmc::Sampler<T>",
                          "unavailable": "needs the reference's headers "
                                         "(VSMC_REF_ROOT) to compile the "
                                         "Sampler<T> program"}))
        return 0
    import vsmc_gb300 as vc
    vc.lib()
    n, T = args.n, args.T
    work = tempfile.mkdtemp(prefix="vsmc_sampler_")
    exe = build_sampler_program(ref, work)
    obs_dev = simulate_obs(vc, T, seed=0)
    obs = obs_dev.view(T, 2).cpu().numpy()
    obs_path = os.path.join(work, "obs.bin")
    out_path = os.path.join(work, "out.bin")
    np.ascontiguousarray(obs, dtype=np.float64).tofile(obs_path)
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    runs = args.warmup + args.steps
    r = subprocess.run([exe, str(n), str(T), "1", str(SCHEME),
                        repr(THRESHOLD), "1", obs_path, out_path, str(runs)],
                       capture_output=True, text=True, check=True)
    clocks.stop()
    ms_runs = json.loads(r.stdout.strip().splitlines()[-1])["ms"]
    timed = ms_runs[args.warmup:]
    v = np.fromfile(out_path, dtype=np.float64)
    resampled = int(v[3 * T:4 * T].sum())
    # the library's own device-resident run in this process, same workload
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    pf = vc.ParticleFilter(n, 32, SCHEME, THRESHOLD, seed=1, max_steps=T,
                           stream=ctypes.c_void_p(stream.cuda_stream))
    for _ in range(args.warmup):
        pf.run_device(T, obs_dev.data_ptr())
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        pf.run_device(T, obs_dev.data_ptr())
    ev1.record(stream)
    torch.cuda.synchronize()
    lib_ms = ev0.elapsed_time(ev1) / args.steps
    pf.close()
    psteps = float(n) * T
    ms = float(np.sum(timed))
    value = psteps * args.steps / (ms / 1000.0)
    line = {
        "metric": METRIC + " through vsmc::Sampler<T>", "value": value,
        "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (observations simulated from the model, seed 0)",
        "config": {
            "workload": "large single bootstrap filter through the reference's "
                        "Sampler<StateCUDA<4, float>> with InitializeCUDA / "
                        "MoveCUDA of a user device model and MonitorMeanCUDA",
            "particles": n, "steps_T": T, "scheme": "systematic",
            "threshold": THRESHOLD,
            "device_threshold": "the Sampler's (resampling queued right "
                                "after each step)",
            "timing": "host clock around initialize + iterate per run",
            "graph": "steps from t = 2 replayed as CUDA graphs",
            "resampled_steps_last_run": resampled,
            "ms_per_run_each": timed,
        },
        "library_run_ms": lib_ms,
        "sampler_over_library_time": (ms / args.steps) / lib_ms,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": (8 * 8 + 8) * T},
        "clocks": clocks.summary(),
        # per run: the reset, then per step the step kernel, the three
        # resampling passes and the scalars' copy to the host
        "gpu_launches": (1 + 5 * T) * args.steps,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_PARTICLES)
    ap.add_argument("--T", type=int, default=T_STEPS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="single",
                    choices=["single", "batched", "learned", "micro",
                             "sampler"])
    ap.add_argument("--replicates", type=int, default=1024)
    ap.add_argument("--learned-particles", type=int, default=1 << 12)
    ap.add_argument("--boot-particles", type=int, nargs="+",
                    default=[1 << 12, 1 << 14, 1 << 16])
    ap.add_argument("--train-traj", type=int, default=1 << 20)
    ap.add_argument("--train-batch", type=int, default=1 << 16)
    ap.add_argument("--train-steps", type=int, default=10000)
    ap.add_argument("--cloud-tracks", type=int, default=1024,
                    help="learned workload: bootstrap-filter tracks whose "
                         "particle clouds add training rows (0: none)")
    ap.add_argument("--cloud-particles", type=int, default=256)
    ap.add_argument("--cloud-candidates", type=int, default=256)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--ref-particles", type=int, default=1 << 18)
    ap.add_argument("--bearings-dt", type=float, default=1.0)
    ap.add_argument("--bearings-q", type=float, default=1.0)
    ap.add_argument("--bearings-sdv", type=float, default=0.5)
    ap.add_argument("--filters", type=int, default=4096)
    ap.add_argument("--rng-log2", type=int, default=30)
    ap.add_argument("--rs-log2", type=int, default=24)
    ap.add_argument("--items", default="",
                    help="micro workload: comma-separated item names to run "
                         "(default all; philox4x32_u32 always runs)")
    ap.add_argument("--tune-steps", type=int, default=60)
    ap.add_argument("--cpu-compare", action="store_true",
                    help="time the reference (oracle/_ref) beside the "
                         "oracle's C restatement on the host and exit")
    args = ap.parse_args()
    if args.cpu_compare:
        return run_cpu_compare(args)
    if args.impl == "reference":
        return run_reference(args)
    args.warmup = max(args.warmup, 3)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "learned":
        return run_learned(args)
    if args.workload == "micro":
        return run_micro(args)
    if args.workload == "sampler":
        return run_sampler(args)

    import torch
    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import vsmc_gb300 as vc
    vc.lib()
    n, T = args.n, args.T
    # a dedicated (non-legacy) stream: the filter captures its step in a graph
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    obs_dev = simulate_obs(vc, T, seed=0)
    pf = vc.ParticleFilter(n, 32, SCHEME, THRESHOLD, seed=replica_seed(rank),
                           max_steps=T, stream=sptr)

    # ---- device-resident timed region
    for _ in range(args.warmup):
        pf.run_device(T, obs_dev.data_ptr())
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        pf.run_device(T, obs_dev.data_ptr())
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = ev0.elapsed_time(ev1)
    hist = pf.history(T)

    # ---- fused step kernel alone (roofline), same stream, CUDA events
    nk = 50
    evk0 = torch.cuda.Event(enable_timing=True)
    evk1 = torch.cuda.Event(enable_timing=True)
    pf.run_device(T, obs_dev.data_ptr())
    for _ in range(5):
        pf.launch_step_kernel()
    evk0.record(stream)
    for _ in range(nk):
        pf.launch_step_kernel()
    evk1.record(stream)
    torch.cuda.synchronize()
    kernel_ms = evk0.elapsed_time(evk1) / nk

    # ---- end to end through the C ABI with pinned host buffers
    obs_host = torch.empty((T, 2), dtype=torch.float64, pin_memory=True)
    obs_host.copy_(obs_dev.view(T, 2).cpu())
    out_mean = torch.empty((T, 2), dtype=torch.float64, pin_memory=True)
    out_ess = torch.empty(T, dtype=torch.float64, pin_memory=True)
    out_res = torch.empty(T, dtype=torch.int32, pin_memory=True)
    out_logz = torch.empty(T, dtype=torch.float64, pin_memory=True)
    L = vc.lib()

    def e2e_run():
        vc.check(L.vsmc_cuda_pf_run(pf.handle, T, obs_host.data_ptr(),
                                    out_mean.data_ptr(), out_ess.data_ptr(),
                                    out_res.data_ptr(), out_logz.data_ptr()),
                 "vsmc_cuda_pf_run")

    for _ in range(2):
        e2e_run()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(2, args.steps // 2)
    for _ in range(e2e_steps):
        e2e_run()  # synchronizes: histories are in host memory on return
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    clocks.stop()
    pf.close()

    ms_max = max_over_ranks(ms, world)
    e2e_max = max_over_ranks(e2e_s, world)
    psteps = float(n) * T
    value = aggregate_rate(psteps * args.steps, world, ms_max / 1000.0)
    e2e_value = aggregate_rate(psteps * e2e_steps, world, e2e_max)
    peak, peak_kind = measured_peaks()
    achieved = BYTES_PER_PARTICLE_STEP * n / (kernel_ms / 1000.0) / 1e9
    # DRAM bytes per launch from the step kernel's ncu capture at the
    # bench's own size (N = 2^24); scaled by particles for another N
    traffic = None
    prof = os.path.join(ROOT, "profiles", "k_pf_step_N2e24.md")
    if os.path.exists(prof):
        import re
        with open(prof) as fh:
            mt = re.search(r"dram bytes per launch:\s*([0-9.]+)", fh.read())
        if mt:
            traffic = float(mt.group(1)) * n / float(1 << 24)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        r, dt, threads = cpu_filter_rate(1 << 20, 20)
        cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "N=2^20 particles x T=20 steps (one run), FP32 state, "
                         "systematic, oracle restatement of the reference "
                         "filter, OpenMP move / copy, sequential weights and "
                         "resampling as in the reference"}

    if rank == 0:
        # reset, T steps of 4 kernels (the fused step and 3 resampling
        # passes, which return at once on steps that do not resample),
        # final mean
        launches_per_run = 1 + 4 * T + 1
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (observations simulated from the model on the "
                    "device, seed 0)",
            "config": {
                "workload": "large single bootstrap filter: 4D constant "
                            "velocity, Student-t(10, 0.5) observations",
                "particles": n, "steps_T": T, "scheme": "systematic",
                "threshold": THRESHOLD, "state": "fp32 SoA",
                "reduction": "fp64 block-level log-sum-exp",
                "cdf": "exact 64-bit fixed point",
                "l2": "inputs larger than L2 (state 256 MiB + log-weights "
                      "64 MiB at N=2^24); no flush",
                "replicas": world,
                "resampled_steps_last_run": int(hist["resampled"].sum()),
                "final_log_evidence": float(hist["logz"][-1]),
            },
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": 16 * T,
                    "d2h_bytes_per_step": (16 + 8 + 4 + 8) * T},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_kind,
                         "kernel": "k_pf32_step (fused move / likelihood / "
                                   "log-weight / FP64 reduction)",
                         "kernel_ms": kernel_ms,
                         "bytes_per_launch": BYTES_PER_PARTICLE_STEP * n,
                         "traffic": traffic},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "gpu_launches": launches_per_run * args.steps,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
