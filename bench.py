#!/usr/bin/env python
"""DMC walker-steps/s of the GB300 walker path.

Workload: the unitary Fermi gas with N = 66 (33 up / 33 down), pair function
shells 0..6, cosh potential mu = 24 k_F, 4096 walkers, DMC with local
weights (idmc = 1), dt = 0.001 / E_FG, branching and population control
(target 4096).  Synthetic seeded inputs (no dataset is involved).

One step = one generation: the drift-diffusion move and full wavefunction /
local-energy evaluation of every walker, the DMC weight, estimators,
branching and population control (dmcbcs.f90:436-448).

Prints one JSON line.  Arms:
  (default)          the CUDA library through its C ABI
  --impl reference   the reference's CPU algorithm on the host cores: the
                     reference itself (Fortran + MPI + MKL) cannot be built
                     on these machines, so the CPU restatement (oracle/) runs
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DMC walker-steps/s @N=66: mixed/batched vs plain FP64 GPU, E_L rel err≤1e-6"
UNIT = "walker-steps/s"
WORKLOAD = "n66"

# DRAM bytes per walker-step (dram__bytes_read.sum + dram__bytes_write.sum of
# one step launch over 1024 walkers, one ncu capture of each walker kernel):
# FP64 walker kernel 4.14 MB, mixed walker kernel 4.20 MB.
NCU_TRAFFIC_BYTES_PER_WALKER = {"fp64": 4045.5, "mixed": 4102.5}

# FP32 flops (FFMA = 2, FADD/FMUL = 1) executed per walker-step by the mixed
# walker kernel, from the instruction counters of the same capture:
# 5.463e9 over 1024 walkers.  Reported beside the roofline, not in it: the
# double-float arithmetic executes ~4.7 FP32 flops per algorithmic flop.
MIXED_FP32_FLOPS_PER_WALKER = 5.335e6


def measured_peaks():
    """The machine's measured peaks (HBM copy GB/s, cuBLAS bf16 TFLOP/s), if the
    file is present next to this script."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def algorithmic_flops(nup, ndn, nd, K, npart):
    """FP64 flops of one walker-step of the reference algorithm: the five
    pair-orbital GEMMs, LU + inverse, inverse contractions, the Jastrow /
    potential pair loop (all pairs, upper bound), beta lookups and the O(N)
    step work."""
    P = npart * (npart - 1) // 2
    return 10 * nup * ndn * K + 2 * nd ** 3 + 8 * nd * (nup + ndn) + 60 * P + 40 * nup * ndn + 30 * npart


def executed_flops(nup, ndn, nd, K, npart, nk, npairs_active):
    """FP64 flops of one walker-step as this library computes it: S = U D^T,
    Gauss-Jordan inverse (nd^3 multiply-adds), the two contraction products
    G and H (2 nd^2 K multiply-adds each) and about 90 flops per active pair."""
    return 2 * nup * ndn * K + 2 * nd ** 3 + 4 * nup * ndn * K + 90 * npairs_active + 30 * npart * nk


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [t.strip() for t in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def fp64_peak_tflops(torch):
    """Measured FP64 peak: cuBLAS DGEMM 4096^3, best of 5 (CUDA events)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def cpu_reference_rate(nwalk, max_s, threads, gens_max=None):
    """The oracle (CPU restatement of the reference) on the host cores:
    walker-steps/s of full DMC generations of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from dmcbcs_project_gb300 import configs

    sysd, rund, _ = configs.workload(WORKLOAD, nwalk=nwalk)
    o = oracle.Oracle(sysd, rund, threads=threads)
    o.init_walkers()
    o.initial_eval()
    o.generation(False)                       # warm
    steps, t0 = 0, time.perf_counter()
    gens = 0
    while True:
        steps += o.num_walkers()
        o.generation(False)
        gens += 1
        el = time.perf_counter() - t0
        if el > max_s or (gens_max and gens >= gens_max):
            break
    return steps / el, steps, gens, el


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_seed(rank):
    """Random-number seed of the replica on one rank (independent walkers per GPU)."""
    return 17 + 1000003 * rank


def reduce_over_ranks(t, count, world):
    """The longest timed interval and the summed work over the ranks (each
    rank runs an independent replica); the identity on one rank.  Works on
    both backends: CUDA tensors for NCCL, CPU tensors for gloo."""
    if world <= 1:
        return t, count
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    tt = torch.tensor([float(t)], device=dev, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    ct = torch.tensor([float(count)], device=dev, dtype=torch.float64)
    dist.all_reduce(ct)
    return float(tt.item()), int(round(ct.item()))


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from dmcbcs_project_gb300 import configs

    nup, ndn, norb, nwalk, dt, _ = configs.WORKLOADS[WORKLOAD]
    nwalk = args.walkers or nwalk
    nsample = args.ref_walkers or nwalk
    # warm-up generations, then K timed generations of the sampled population
    rate_w, _, _, _ = cpu_reference_rate(nsample, 0.0, threads, gens_max=max(1, args.warmup))
    rate, steps, gens, el = cpu_reference_rate(nsample, 1e9, threads, gens_max=args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / max(gens, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "dmc_n66_33u33d", "walkers": nsample, "idmc": 1, "dt_efg": dt, "shells": norb,
                   "precision": "f64", "parallelism": "host threads"},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{gens} DMC generations of {nsample} walkers (N=66) on {threads} host threads; "
                                   "the reference Fortran/MPI/MKL build is not possible here, so the C "
                                   "restatement of its algorithm runs"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def time_path(ctx, args, world, local, barrier):
    """W warm-up and K timed generations on one context; device time from
    CUDA events around every generation (L2 flushed between them)."""
    import torch

    for _ in range(max(args.warmup, 3)):
        ctx.timed_generations(1, opcomp_last=False, flush_l2=True)
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    steps, dev_ms, kern_ms, launches = 0, 0.0, 0.0, 0
    for g in range(args.steps):
        s, ms, nl = ctx.timed_generations(1, opcomp_last=(g == args.steps - 1), flush_l2=True)
        steps += s
        dev_ms += ms
        launches += nl
        kern_ms += ctx.last_step_ms()
    barrier()
    clocks = sampler.stop()
    t_max, steps_all = reduce_over_ranks(dev_ms, steps, world)
    return {"value": steps_all / (t_max * 1e-3), "ms_per_step": t_max / max(args.steps, 1), "steps": steps,
            "kern_ms": kern_ms / max(args.steps, 1), "avg_n": steps / max(args.steps, 1), "launches": launches,
            "clocks": clocks}


def e2e_rate(ctx, info, args, world, barrier):
    """The same generations through the C ABI with the walker population in
    pinned host memory, as a host that keeps its own stacks holds it:
    dmc_generation_host every generation (the walker kernel reads each
    walker's state from the host arrays, one kernel writes the new
    population back) and the estimator sums."""
    import torch

    cap = info.capacity
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    host = {k: pin((cap, info.npart, 3), torch.float64) for k in ("x", "dpsi", "dpsig")}
    for k in ("psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0", "psigl0", "wt0"):
        host[k] = pin((cap,), torch.float64)
    host["is_"] = pin((cap,), torch.int32)
    host["irn"] = pin((cap,), torch.int64)
    host["cap"] = cap
    n_cur = ctx.get_walkers_into(host)
    n3b = 3 * info.npart * 8
    # read per walker: x, dpsig, 11 doubles, is, irn (dpsi only for rejected
    # moves: none with idmc = 1); written: every field
    per_in = 2 * n3b + 11 * 8 + 4 + 8
    per_out = 3 * n3b + 10 * 8 + 8 + 4 + 8
    nsteps = max(1, min(args.steps, args.e2e_steps))
    n_cur = ctx.generation_host(dict(host, n=n_cur), host, False)   # warm-up, untimed
    h2d = d2h = total = 0
    barrier()
    t0 = time.perf_counter()
    for g in range(nsteps):
        n_new = ctx.generation_host(dict(host, n=n_cur), host, g == nsteps - 1)
        total += n_cur
        h2d += n_cur * per_in + 4
        d2h += n_new * per_out + 16
        ctx.estimators()
        d2h += 3 * info.nest * 8
        n_cur = n_new
    barrier()
    t = time.perf_counter() - t0
    t_all, total_all = reduce_over_ranks(t, total, world)
    rate = total_all / t_all
    return {"value": rate, "unit": UNIT, "h2d_bytes_per_step": int(h2d / nsteps),
            "d2h_bytes_per_step": int(d2h / nsteps), "steps": nsteps,
            "path": "dmc_generation_host (population in pinned host arrays) + dmc_get_estimators"}


def accuracy_vs_fp64(ctx_mixed, ctx_fp64, hbar, nmax=512):
    """Per-configuration local-energy error of the mixed path against the
    FP64 path on the mixed run's current walkers."""
    w = ctx_mixed.walkers()
    x = w["x"][:nmax]
    a = ctx_mixed.hpsi(x)
    b = ctx_fp64.hpsi(x)
    ea = -hbar * a["d2psi"] + a["v"]
    eb = -hbar * b["d2psi"] + b["v"]
    rel = np.abs(ea - eb) / np.maximum(np.abs(eb), 1.0)
    dr = np.max(np.abs(a["dpsi"] - b["dpsi"]), axis=(1, 2)) / np.maximum(np.max(np.abs(b["dpsi"]), axis=(1, 2)), 1.0)
    return {"configs": int(x.shape[0]), "el_rel_err_max": float(rel.max()), "el_rel_err_median": float(np.median(rel)),
            "drift_rel_err_max": float(dr.max()), "log_psi_abs_err_max": float(np.max(np.abs(a["psil"] - b["psil"])))}


# The uneven batch: six systems (N up / N down) in one generation graph,
# 16384 walkers split over them by seeded weights, plain FP64
BATCH_SYSTEMS = ["n14", "n38", "n66", "p33_30", "p38_33", "n132"]
BATCH_WALKERS = 16384


def uneven_batch(args, rank, precision="fp64"):
    """Batched generations of the six systems with the tuned CTA split, then
    the same contexts one after another (dmc_timed_generations each), both
    with the L2 flushed before every generation."""
    from dmcbcs_project_gb300 import capi, configs

    rng = np.random.default_rng(2024)
    w = rng.uniform(0.5, 1.5, len(BATCH_SYSTEMS))
    nws = np.floor(BATCH_WALKERS * w / w.sum()).astype(int)
    nws[-1] += BATCH_WALKERS - int(nws.sum())
    ctxs, systems = [], []
    for i, (name, nw) in enumerate(zip(BATCH_SYSTEMS, nws)):
        s, r, meta = configs.workload(name, nwalk=int(nw), seed=1234 + i)
        r.seed = replica_seed(rank) + 7919 * i
        c = capi.Context(s, r, precision=precision)
        c.init_walkers()
        c.initial_eval()
        ctxs.append(c)
        systems.append(f"{meta['nup']}/{meta['ndn']}:{int(nw)}")
    gens = args.batch_steps
    with capi.Batch(ctxs) as b:
        initial = b.grids.tolist()
        grids, tune_ms = b.tune(3)
        b.generations(max(args.warmup, 3), opcomp_last=False, flush_l2=True)
        steps, ms, nl = b.generations(gens, opcomp_last=True, flush_l2=True)
    seq_steps, seq_ms, seq_flops = 0, 0.0, 0.0
    # algorithmic flops of one walker-step of each system (the reference
    # algorithm's count, as for the headline roofline)
    flops = [algorithmic_flops(c.info.nup, c.info.ndn, c.info.nd, c.info.ncol, c.info.npart) for c in ctxs]
    for c, f in zip(ctxs, flops):
        c.timed_generations(max(args.warmup, 3), opcomp_last=False, flush_l2=True)
        st, m, _ = c.timed_generations(gens, opcomp_last=True, flush_l2=True)
        seq_steps += st
        seq_ms += m
        seq_flops += f * st
    for c in ctxs:
        c.close()
    value = steps / (ms * 1e-3)
    seq = seq_steps / (seq_ms * 1e-3)
    # the batch's walker-steps split over the systems in proportion to their
    # target populations (population control holds each near its target)
    batch_flops = steps * float(np.dot(flops, nws)) / float(nws.sum())
    return {"workload": "uneven_batch_6_systems", "systems": systems, "walkers": BATCH_WALKERS, "precision": precision,
            "steps": gens, "unit": UNIT, "value": value, "ms_per_step": ms / max(gens, 1), "gpu_launches": nl,
            "grids_tuned": [int(g) for g in grids], "grids_initial": initial, "tune_pass_ms": tune_ms,
            "sequential": {"value": seq, "ms_per_step": seq_ms / max(gens, 1),
                           "algorithmic_tflops": seq_flops / (seq_ms * 1e-3) / 1e12},
            "speedup_vs_sequential": value / seq,
            "algorithmic_tflops": batch_flops / (ms * 1e-3) / 1e12,
            "algorithmic_tflops_note": "reference-algorithm flops per walker-step of each system x its walker-steps "
                                       "(batched: the measured total split by the systems' target populations)"}


def param_gradients(args, rank):
    """dmc_param_grad (adjoint d log Psi / d theta and d E_L / d theta for
    theta = vorb(1..7), bfact, b, d and the 16 knots of the up-down Jastrow
    spline: 26 parameters) on 8192 walkers of the N = 66 system, through the
    C ABI with host buffers; median of three calls after one warm-up."""
    from dmcbcs_project_gb300 import capi, configs

    s, r, _ = configs.workload(WORKLOAD, nwalk=args.pgrad_walkers, idmc=-1)
    r.seed = replica_seed(rank)
    knots = np.random.default_rng(2024).uniform(-0.3, 0.3, 16) * np.exp(-0.15 * np.arange(16))
    with capi.Context(s, r) as c:
        c.set_jastrow_spline(knots)
        c.init_walkers()
        x = c.walkers()["x"]
        c.param_grad(x[:64])
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            dl, de = c.param_grad(x)
            times.append(time.perf_counter() - t0)
        np_ = c.param_count()
    t = float(np.median(times))
    return {"workload": "param_grad_n66_33u33d", "walkers": int(x.shape[0]), "parameters": np_,
            "theta": "vorb(1..7), bfact, b, d, 16 Jastrow spline knots",
            "seconds_per_call": t, "walkers_per_s": x.shape[0] / t,
            "includes": "host-to-device copy of x, FP64 wavefunction and determinant evaluation, adjoint kernel, "
                        "device-to-host copy of both gradients"}


def sm_sweeps(args, rank):
    """Particle-by-particle VMC sweeps (dmc_sm_sweeps: FP32 ratios and
    Sherman-Morrison inverse updates, FP64 recompute of the inverse every 16
    sweeps, then the walkers re-evaluated by the mixed walker kernel) on the
    N = 66 workload's 4096 walkers, through the C ABI: one call of 16
    sweeps, median of three after one warm-up call."""
    from dmcbcs_project_gb300 import capi, configs

    s, r, _ = configs.workload(WORKLOAD, nwalk=args.walkers or configs.WORKLOADS[WORKLOAD][3], idmc=0)
    r.seed = replica_seed(rank)
    nsw = args.sweeps
    with capi.Context(s, r, precision="mixed") as c:
        c.init_walkers()
        c.initial_eval()
        c.sm_sweeps(2, 16)
        times, accs = [], []
        for _ in range(3):
            t0 = time.perf_counter()
            a, m = c.sm_sweeps(nsw, 16)
            times.append(time.perf_counter() - t0)
            accs.append(a / m)
        nw = c.num_walkers()
    t = float(np.median(times))
    return {"workload": "sm_sweeps_n66_33u33d", "walkers": nw, "sweeps_per_call": nsw, "recompute_every": 16,
            "move_scheme": "particle-by-particle Metropolis, Gaussian proposal of width sigma (no drift)",
            "unit": "walker-sweeps/s", "value": nw * nsw / t, "moves_per_s": nw * nsw * s.nbin[0] * 2 / t,
            "ms_per_call": 1e3 * t, "acceptance": float(np.mean(accs)),
            "includes": "FP64 inverse recompute every 16 sweeps, FP32 sweeps, final mixed re-evaluation of every "
                        "walker"}


def deck_system(name, nwalk, idmc=None, dt=None):
    """System and run descriptors of one of the reference's production decks
    (the committed parse in tests/golden/decks.json)."""
    from dmcbcs_project_gb300 import abi

    with open(os.path.join(ROOT, "tests", "golden", "decks.json")) as f:
        d = json.load(f)[name]
    r = dict(d["run"], nwalk=nwalk)
    if idmc is not None:
        r["idmc"] = idmc
    if dt is not None:
        r["dt"] = dt
    return abi.make_system(d["system"]), abi.make_run(r)


def energy_agreement(args, rank):
    """DMC energy of the mixed and the FP64 path on the reference's N = 66
    production deck (dmcbcs.dat: 10 fitted shells, beta b = 0.5, d = 5,
    dt = 5e-5).  Each precision runs R independent replicas (own seeds: no
    random stream is shared between replicas or precisions).  A replica:
    eq VMC generations at dt_eq from random walkers, eq_dmc DMC generations
    at the deck's dt, then nblocks blocks of nstep generations with the
    estimators on every generation; its energy is the mean of its block
    averages.  At dt = 5e-5 successive blocks are strongly correlated, so the
    error of a precision's energy is the standard error over its replicas
    (which also carries the spread of the starting walkers), not the block
    error."""
    from dmcbcs_project_gb300 import capi

    nw = args.energy_walkers
    out = {}
    for k, prec in enumerate(("mixed", "fp64")):
        reps = []
        for rep in range(args.energy_replicas):
            seed = replica_seed(rank) + 104729 * (1 + k * args.energy_replicas + rep)
            s, r = deck_system("dmcbcs.dat", nw, idmc=0, dt=args.energy_dt_eq)
            r.seed = seed
            with capi.Context(s, r, precision=prec) as v:
                v.init_walkers()
                v.initial_eval()
                for _ in range(args.energy_eq):
                    v.generation(False)
                w = v.walkers()
            s, r = deck_system("dmcbcs.dat", nw)
            r.seed = seed
            with capi.Context(s, r, precision=prec) as c:
                c.load_walkers(w["x"], w["irn"])
                c.initial_eval()
                for _ in range(args.energy_eq_dmc):
                    c.generation(False)
                c.zero_estimators()
                blocks = []
                for _ in range(args.energy_blocks):
                    for _ in range(args.energy_steps):
                        c.generation(True)
                    val, _ = c.block_update()
                    blocks.append(float(val[0]))
            reps.append(float(np.mean(blocks)))
        e = np.array(reps)
        out[prec] = {"energy": float(e.mean()), "error": float(e.std(ddof=1) / np.sqrt(len(e))),
                     "replicas": [round(v, 6) for v in reps]}
    d = out["mixed"]["energy"] - out["fp64"]["energy"]
    sig = float(np.hypot(out["mixed"]["error"], out["fp64"]["error"]))
    e = abs(out["fp64"]["energy"])
    return {"unit": "E / (N E_FG)", "system": "dmcbcs.dat (N = 66, 10 shells, dt = 5e-5)",
            "walkers_per_replica": nw, "replicas_per_precision": args.energy_replicas,
            "vmc_equilibration": {"generations": args.energy_eq, "dt": args.energy_dt_eq},
            "dmc_equilibration": args.energy_eq_dmc, "blocks": args.energy_blocks,
            "generations_per_block": args.energy_steps, "mixed": out["mixed"], "fp64": out["fp64"],
            "delta": d, "sigma": sig, "delta_over_sigma": abs(d) / sig if sig > 0 else None,
            "sigma_over_energy": sig / e if e > 0 else None,
            "note": "independent seeds for every replica of both precisions; errors from the spread over replicas"}


def run_gpu(args):
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from dmcbcs_project_gb300 import build as B

    B.build()
    from dmcbcs_project_gb300 import capi, configs

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    nup, ndn, norb, nwalk, dt, _ = configs.WORKLOADS[WORKLOAD]
    nwalk = args.walkers or nwalk
    sysd, rund, _ = configs.workload(WORKLOAD, nwalk=nwalk)
    rund.seed = replica_seed(rank)                      # independent replica per GPU
    precisions = ["mixed", "fp64"] if args.precision == "both" else [args.precision]
    ctxs, res = {}, {}
    for prec in precisions:
        ctx = capi.Context(sysd, rund, precision=prec)
        ctx.init_walkers()
        ctx.initial_eval()
        res[prec] = time_path(ctx, args, world, local, barrier)
        ctxs[prec] = ctx
    head = precisions[0]
    ctx = ctxs[head]
    info = ctx.info
    e2e = e2e_rate(ctx, info, args, world, barrier)

    flops_alg = algorithmic_flops(info.nup, info.ndn, info.nd, info.ncol, info.npart)
    flops_exe = executed_flops(info.nup, info.ndn, info.nd, info.ncol, info.npart, info.nk, info.nup * info.ndn)
    peak64 = capi.probe_peak("fp64") if rank == 0 else None
    peak32 = capi.probe_peak("fp32") if rank == 0 else None
    dgemm = fp64_peak_tflops(torch) if rank == 0 else None
    peaks = measured_peaks()

    def roofline(prec):
        r = res[prec]
        kms = r["kern_ms"]
        alg = flops_alg * r["avg_n"] / (kms * 1e-3) / 1e12
        if prec == "fp64":
            return {"bound": "fp64", "achieved": alg, "peak": dgemm, "unit": "TFLOP/s",
                    "frac": alg / dgemm if dgemm else None,
                    "traffic": NCU_TRAFFIC_BYTES_PER_WALKER["fp64"] * r["avg_n"],
                    "kernel": "walker_kernel<double>", "kernel_ms_per_launch": kms, "walkers_per_launch": r["avg_n"],
                    "algorithmic_flops_per_walker_step": flops_alg, "executed_flops_per_walker_step": flops_exe,
                    "executed_achieved": flops_exe * r["avg_n"] / (kms * 1e-3) / 1e12,
                    "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (no FP64 figure in the measured-peaks "
                                   "file); DFMA probe " + (f"{peak64:.3f}" if peak64 else "-") + " TFLOP/s"}
        # achieved = the reference algorithm's flops (not the double-float
        # instructions executed) per launch / the walker kernel's event time
        ex = MIXED_FP32_FLOPS_PER_WALKER
        bf16 = peaks.get("bf16_tflops")
        return {"bound": "fp32", "achieved": alg, "peak": peak32, "unit": "TFLOP/s",
                "frac": alg / peak32 if peak32 else None,
                "traffic": NCU_TRAFFIC_BYTES_PER_WALKER["mixed"] * r["avg_n"],
                "kernel": "walker_kernel<df>", "kernel_ms_per_launch": kms, "walkers_per_launch": r["avg_n"],
                "algorithmic_flops_per_walker_step": flops_alg,
                "peak_source": "FFMA throughput probe measured in this run (the measured-peaks file has no FP32 "
                               "figure)",
                "of_measured_bf16_tensor_peak": {"peak": bf16, "frac": alg / bf16 if bf16 else None,
                                                 "source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 burst)"},
                "of_measured_dgemm": {"peak": dgemm, "frac": alg / dgemm if dgemm else None},
                "executed": {"fp32_flops_per_walker_step": ex,
                             "achieved": ex * r["avg_n"] / (kms * 1e-3) / 1e12,
                             "frac_of_ffma_probe": (ex * r["avg_n"] / (kms * 1e-3) / 1e12 / peak32) if peak32
                             else None,
                             "note": "FP32 instructions of the double-float arithmetic (ncu counters); pipe "
                                     "busyness, not useful work"}}

    acc = accuracy_vs_fp64(ctxs["mixed"], ctxs["fp64"], sysd.hbar) if len(ctxs) == 2 and rank == 0 else None
    if acc is not None and args.energy_blocks > 0:
        acc["dmc_energy"] = energy_agreement(args, rank)

    # The mixed-precision benchmark configuration, 8192 walkers: N = 132 (66 up
    # / 66 down) and N = 66, both paths over a short run (not the headline;
    # reported beside it)
    def mixed_config(name, workload):
        s_, r_, _ = configs.workload(name, nwalk=8192)
        r_.seed = replica_seed(rank)
        sub, cs = {}, {}
        sub_args = argparse.Namespace(**vars(args))
        sub_args.steps = args.n132_steps
        for prec in ("mixed", "fp64"):
            cx = capi.Context(s_, r_, precision=prec)
            cx.init_walkers()
            cx.initial_eval()
            t = time_path(cx, sub_args, world, local, barrier)
            sub[prec] = {"value": t["value"], "ms_per_step": t["ms_per_step"], "avg_walkers": t["avg_n"],
                         "clocks": t["clocks"]}
            # the layout tuner on the same context (dmc_tune_layout), then the
            # same generations again with the layout it keeps
            kind, _ = cx.tune_layout(3)
            tt = time_path(cx, sub_args, world, local, barrier)
            sub[prec]["tuned_layout"] = {"kind": ["heuristic", "on-chip 256 threads", "union in global scratch"][kind],
                                         "value": tt["value"], "ms_per_step": tt["ms_per_step"]}
            cs[prec] = cx
        out = {"workload": workload, "walkers": 8192, "steps": args.n132_steps, "unit": UNIT,
               "mixed": sub["mixed"], "fp64": sub["fp64"], "speedup_vs_fp64": sub["mixed"]["value"] / sub["fp64"]["value"],
               "accuracy_vs_fp64": accuracy_vs_fp64(cs["mixed"], cs["fp64"], s_.hbar, nmax=256)
               if rank == 0 else None}
        for cx in cs.values():
            cx.close()
        return out

    # idmc = 10 (the driftless two-point move, two wavefunction evaluations
    # per walker-step) on the headline system, both paths (reported beside
    # the headline)
    def gf_move():
        s_, r_, _ = configs.workload(WORKLOAD, nwalk=nwalk, idmc=10)
        r_.seed = replica_seed(rank)
        sub_args = argparse.Namespace(**vars(args))
        sub_args.steps = args.gf_steps
        sub = {}
        for prec in ("mixed", "fp64"):
            cx = capi.Context(s_, r_, precision=prec)
            cx.init_walkers()
            cx.initial_eval()
            t = time_path(cx, sub_args, world, local, barrier)
            sub[prec] = {"value": t["value"], "ms_per_step": t["ms_per_step"], "avg_walkers": t["avg_n"],
                         "kernel_ms_per_launch": t["kern_ms"], "gpu_launches": t["launches"], "clocks": t["clocks"]}
            cx.close()
        return {"workload": "dmc_n66_33u33d_idmc10", "idmc": 10, "walkers": nwalk, "steps": args.gf_steps,
                "unit": UNIT, "wavefunction_evaluations_per_walker_step": 2, "mixed": sub["mixed"],
                "fp64": sub["fp64"], "speedup_vs_fp64": sub["mixed"]["value"] / sub["fp64"]["value"]}

    gf = gf_move() if len(ctxs) == 2 and args.gf_steps > 0 else None

    n132 = n66_8192 = None
    if len(ctxs) == 2 and args.n132_steps > 0:
        n132 = mixed_config("n132", "dmc_n132_66u66d")
        n66_8192 = mixed_config("n66", "dmc_n66_33u33d_8192")

    batch = None
    if args.batch_steps > 0:
        batch = uneven_batch(args, rank)
        mixed_batch = uneven_batch(args, rank, "mixed")
        batch["mixed"] = {k: mixed_batch[k] for k in ("value", "ms_per_step", "gpu_launches", "grids_tuned",
                                                      "sequential", "speedup_vs_sequential", "algorithmic_tflops")}
        batch["mixed"]["speedup_vs_fp64_batch"] = mixed_batch["value"] / batch["value"]
        if dgemm:
            # the FP64 batch against the FP64 roofline: what any split of the
            # SMs over the systems could still gain
            batch["frac_of_measured_dgemm"] = batch["algorithmic_tflops"] / dgemm
            batch["sequential"]["frac_of_measured_dgemm"] = batch["sequential"]["algorithmic_tflops"] / dgemm
    pgrad = param_gradients(args, rank) if args.pgrad_walkers > 0 else None
    sweeps = sm_sweeps(args, rank) if args.sweeps > 0 else None

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            rate, st, gens, el = cpu_reference_rate(args.cpu_walkers, args.cpu_seconds, threads)
            cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"{gens} DMC generations of {args.cpu_walkers} walkers of the same N=66 system "
                             f"({st} walker-steps, {el:.1f} s) on {threads} host threads"}
        r = res[head]
        line = {
            "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "df32+f32 (f64 move/weights)" if head == "mixed" else "f64", "data": "synthetic",
            "impl": f"gb300-{head}",
            "config": {"workload": "dmc_n66_33u33d", "walkers": nwalk, "avg_walkers": r["avg_n"], "idmc": 1,
                       "dt_efg": dt, "shells": norb, "ncol": info.ncol, "nd": info.nd, "precision": head,
                       "l2": "2xL2 buffer written between timed generations",
                       "parallelism": f"replicas{world}"},
            "e2e": e2e,
            "gpu_launches": r["launches"],
            "clocks": r["clocks"],
            "roofline": roofline(head),
            "cpu_baseline": cpu,
        }
        if "fp64" in res and head != "fp64":
            f = res["fp64"]
            line["fp64_path"] = {"value": f["value"], "ms_per_step": f["ms_per_step"], "gpu_launches": f["launches"],
                                 "clocks": f["clocks"], "roofline": roofline("fp64")}
            line["speedup_vs_fp64"] = r["value"] / f["value"]
            line["accuracy_vs_fp64"] = acc
        if n132:
            line["n132"] = n132
        if n66_8192:
            line["n66_8192"] = n66_8192
        if batch:
            line["uneven_batch"] = batch
        if pgrad:
            line["param_grad"] = pgrad
        if sweeps:
            line["sm_sweeps"] = sweeps
        if gf:
            line["idmc10"] = gf
        print(json.dumps(line), flush=True)
    for c in ctxs.values():
        c.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="both", choices=["both", "mixed", "fp64"],
                    help="both: the mixed path is the headline, the FP64 path is timed beside it")
    ap.add_argument("--walkers", type=int, default=None)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-walkers", type=int, default=512)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-walkers", type=int, default=None,
                    help="walkers of the reference arm (default: the GPU arm's workload, 4096)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n132-steps", type=int, default=20,
                    help="generations of the 8192-walker side measurements at N = 132 and N = 66 (0: skip)")
    ap.add_argument("--energy-blocks", type=int, default=10,
                    help="blocks of the mixed-vs-FP64 DMC energy comparison on the dmcbcs.dat deck (0: skip)")
    ap.add_argument("--energy-steps", type=int, default=20, help="generations per energy block")
    ap.add_argument("--energy-walkers", type=int, default=2048, help="walkers per energy replica")
    ap.add_argument("--energy-replicas", type=int, default=16, help="independent replicas per precision")
    ap.add_argument("--energy-eq", type=int, default=200, help="VMC equilibration generations")
    ap.add_argument("--energy-dt-eq", type=float, default=5e-3, help="VMC equilibration time step")
    ap.add_argument("--energy-eq-dmc", type=int, default=100, help="DMC equilibration generations")
    ap.add_argument("--pgrad-walkers", type=int, default=8192,
                    help="walkers of the adjoint parameter-gradient side measurement (0: skip)")
    ap.add_argument("--sweeps", type=int, default=16,
                    help="particle-by-particle sweeps per call of the Sherman-Morrison side measurement (0: skip)")
    ap.add_argument("--gf-steps", type=int, default=10,
                    help="generations of the idmc = 10 side measurement (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=20,
                    help="generations of the six-system uneven batch side measurement (0: skip)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
