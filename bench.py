#!/usr/bin/env python
"""Benchmark of the two-site effective-Hamiltonian matvec (src/apply.jl:93-105) at chi=2048.

Workload: XXZ chain (Delta = 0.5) two-site tensor with chi = 2048 on both bonds over 25 charges
with a binomial sector profile, d = 2, MPO bond 5, blocks N(0,1) from a seeded Philox stream
(synthetic: the reference publishes no dataset).  One step = one H_eff application
v -> envL . W1 . W2 . envR . v with every input resident in HBM.

Metric: H_eff GFLOP/s = planner-counted algorithmic flops (sum over the sector GEMMs of the four
contractions of 2*M*N*K) / seconds per step.  Every timed step is preceded by an L2 flush
(a 512 MiB write on the library's stream) outside the timed events.  The line also carries
"sweep": one 2-site DMRG sweep at maxdim = chi, FP64 drop-in vs the mixed configuration, with
the energy difference between the two.

    python bench.py [--steps K] [--warmup W] [--precision P] [--impl ours|reference]
                    [--no-sweep] [--sweep-chi X]

Multi-GPU (torchrun): one independent replica per rank (a DMRG chain does not shard), value =
all ranks' flops / max-over-ranks time, "scaling": "weak".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "H_eff matvec GFLOP/s at chi=2048 (2-site DMRG hot path)"
UNIT = "GFLOP/s"
# split precision of the headline H_eff: the Krylov setting of the mixed sweep, the fewest
# slices whose sweep energies stay within 1e-10 of the FP64 drop-in (0 = FP64)
DEFAULT_SLICES = 5


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--chi", type=int, default=2048)
    p.add_argument("--precision", type=int, default=None,
                   help="0 = FP64; s >= 2 = split bf16 with s slices (default: best available)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-sweep", action="store_true", help="skip the DMRG sweep measurement")
    p.add_argument("--gradient", action="store_true",
                   help="instead of the H_eff line: energy gradients of a converged L=64, "
                        "chi=512 XXZ chain (dE/dDelta and dE/dA by adjoint contractions)")
    p.add_argument("--cylinder", action="store_true",
                   help="instead of the H_eff line: mixed-precision 2-site DMRG sweeps of the "
                        "J1 Heisenberg 6 x 24 cylinder at maxdim --sweep-chi (default 1024)")
    p.add_argument("--sweeps", type=int, default=2, help="sweeps of the --cylinder run")
    p.add_argument("--compare-fp64", action="store_true",
                   help="--cylinder: run the last sweep also as the FP64 drop-in (FP64 "
                        "contractions, exact SVD) from the same state and report |dE| for every "
                        "energy of that sweep")
    p.add_argument("--mpo-shared-prefixes", action="store_true",
                   help="--cylinder with the MPO whose open terms share channels (w = 20 "
                        "instead of 26)")
    p.add_argument("--small-chain", action="store_true",
                   help="instead of the H_eff line: 4 FP64 sweeps of the L=32, maxdim 64 "
                        "Heisenberg chain, with the CPU oracle timed on the same sweeps")
    p.add_argument("--batched", type=int, default=0, metavar="N",
                   help="instead of the H_eff line: N independent XXZ chains (L in [32,128], "
                        "Delta in [0,1.5], maxdim in {128,256,512,1024}, seeded), one sweep "
                        "each, concurrently and one after the other")
    p.add_argument("--batched-concurrent-only", action="store_true",
                   help="--batched without the one-after-the-other comparison run")
    p.add_argument("--lockstep", action="store_true",
                   help="--batched: the chains in lock step on one context (one batched "
                        "eigensolve per step: every Krylov application one grouped launch per "
                        "phase for all chains, CUDA graph replay, tuned split-GEMM tiles), "
                        "timed beside the concurrent and one-by-one runs")
    p.add_argument("--dynamic", action="store_true",
                   help="--lockstep: the batcher takes the requests waiting when it is free "
                        "instead of waiting for every chain")
    p.add_argument("--fp64-check", type=int, default=0, metavar="K",
                   help="--batched: also run the first K chains one by one as the FP64 drop-in "
                        "and report |dE| of the batched energies against them")
    p.add_argument("--sweep-chi", type=int, default=None, help="maxdim of the sweep (default chi)")
    p.add_argument("--sweep-offload", type=int, default=0, metavar="W",
                   help="also run the mixed sweep with environments in a W-entry device window "
                        "(the rest in host memory; asynchronous copies with prefetch, and "
                        "blocking copies)")
    p.add_argument("--sweep-phases", action="store_true",
                   help="also report the sweep's eigensolve / truncation / environment times")
    p.add_argument("--tdvp", action="store_true",
                   help="instead: 1-site TDVP of an XXZ chain (complex symmetric MPS) and the "
                        "Delta derivative of a two-point function by central differences")
    p.add_argument("--tdvp-lx", type=int, default=32)
    p.add_argument("--tdvp-steps", type=int, default=10)
    p.add_argument("--dense-gemm", type=int, default=0, metavar="N",
                   help="instead: the split-precision GEMM on one dense N x N x N block "
                        "(--precision slices, default the headline's), kernel time by CUDA "
                        "events, algorithmic and executed TFLOP/s against the measured peak")
    p.add_argument("--tdvp-no-fd", action="store_true",
                   help="--tdvp: skip the finite-difference evolutions")
    p.add_argument("--tdvp-forward-only", action="store_true",
                   help="--tdvp: the plain sweeps alone (no derivative runs)")
    p.add_argument("--tdvp-kernel-times", action="store_true",
                   help="--tdvp: per-kernel device time of the plain sweeps (CUPTI activity "
                        "records through torch.profiler), against their wall time; diagnostic, "
                        "the sweep times of such a run are not reported as measurements")
    p.add_argument("--tdvp-adjoint", action="store_true",
                   help="--tdvp: also the reverse-mode gradient (every MPO tensor and initial "
                        "site tensor) over the same sweeps; its dC/dDelta and time")
    p.add_argument("--tdvp-precision", type=int, default=0,
                   help="block-GEMM arithmetic of the TDVP contractions (0 = FP64, S = slices)")
    return p.parse_args(argv)


# ---------------------------------------------------------------------------------------------
def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_rate(t_local, flops, ws, device=None):
    """Whole-job rate of ``ws`` independent replicas, one per rank, each timing the same step.

    The job's step time is the slowest rank's (all-reduce MAX over the default process group; any
    backend) and one job step does ``ws`` times the flops of one replica. Returns (step time in s,
    GFLOP/s)."""
    t = float(t_local)
    if ws > 1:
        import torch
        import torch.distributed as dist
        tt = torch.tensor([t], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    return t, ws * flops / t / 1e9


def clock_soak(run_batch, sync, seconds, per_batch):
    """Runs batches of the step, untimed, for at least ``seconds`` (synchronising after each
    batch), so that the clock sampler (one sample per 200 ms) sees the GPU under this step's load
    before the short timed region. Returns (seconds spent, steps run)."""
    t0 = time.perf_counter()
    n = 0
    while True:
        run_batch()
        sync()
        n += per_batch
        if time.perf_counter() - t0 >= seconds:
            return time.perf_counter() - t0, n


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def profile_traffic(kernel_key):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        return json.load(open(path)).get(kernel_key)
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------------------------
def workload_config(chi):
    """The ``config`` object of the H_eff line, identical in both arms."""
    return {"workload": f"H_eff matvec, XXZ Delta=0.5, chi={chi} on both bonds, 25 charges "
                        "binomial profile, d=2, MPO bond 5",
            "chi": chi,
            "l2": "GPU steps: L2 flushed before every timed step (512 MiB write); the CPU arm "
                  "has no device cache to flush"}


def oracle_inputs(chi):
    """(v, envL, envR, W, W) of the workload as oracle tensors: the same Philox draws the device
    path uploads, generated by the oracle itself (no library code involved)."""
    from oracle import mps as om
    return list(om.heff_workload(chi))


def cpu_heff_rate(chi, flops, budget_s=15.0, max_reps=40):
    """Oracle (NumPy/OpenBLAS restatement of the reference path) H_eff matvecs on the host
    cores: repeated until ~budget_s of CPU work."""
    from oracle import mps as om
    O = oracle_inputs(chi)
    om.applymps2site(*O)  # warm-up
    times = []
    t_all = time.perf_counter()
    while len(times) < max_reps and time.perf_counter() - t_all < budget_s:
        t0 = time.perf_counter()
        om.applymps2site(*O)
        times.append(time.perf_counter() - t0)
    cores = int(os.environ.get("OPENBLAS_NUM_THREADS", os.cpu_count() or 1))
    return flops / statistics.mean(times) / 1e9, len(times), statistics.mean(times), cores


def run_reference(args):
    """--impl reference: the reference algorithm's CPU path (the NumPy/OpenBLAS restatement;
    Julia is not available) timed on the host cores, same metric, unit and workload.  Nothing of
    the GPU library is imported or loaded here: the inputs come from the oracle's own Philox
    draws and the flop count from the oracle's own sector GEMMs."""
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    os.environ.setdefault("OPENBLAS_NUM_THREADS", str(os.cpu_count() or 1))
    from oracle import mps as om
    O = oracle_inputs(args.chi)
    flops = om.heff_flops(*O)  # counts the reference-order sector GEMMs of one application
    for _ in range(max(0, min(args.warmup, 2) - 1)):
        om.applymps2site(*O)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        om.applymps2site(*O)
        times.append(time.perf_counter() - t0)
    t = statistics.mean(times)
    value = flops / t / 1e9
    cores = int(os.environ["OPENBLAS_NUM_THREADS"])
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Philox N(0,1) blocks)",
        "config": workload_config(args.chi),
        "gflop_per_step": flops / 1e9,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full H_eff matvecs (NumPy/OpenBLAS oracle; "
                                   "Julia is absent)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------
# Krylov matvecs at 5 slices: with 4 (relative error 2e-8 per matvec) the Lanczos vectors of
# the first sweep's unconverged solves move the post-truncation energies by up to 5e-9
SWEEP_MIXED = dict(precision=5, energy_precision=7, env_precision=7, svd="gram")
# Truncation tie band (both sweeps): singular values within 1e-9 of the largest count as equal
# and the lowest sector keeps the state, so that SU(2) multiplets split by the maxdim cut are
# split the same way whatever the rounding of the two factorisations
SWEEP_TIEBAND = 1e-9
SWEEP_FP64 = dict(precision=0, energy_precision=0, env_precision=0, svd="exact")


def sweep_bench(ctx, chi, lx=32, seed=7, phases=False, offload=0):
    """One 2-site DMRG sweep (src/dmrg.jl:58-179) of the L=lx Heisenberg chain (J=1, OBC, Sz=0)
    at maxdim=chi from a random MPS whose bonds hold about chi states (binomial charge profile),
    canonicalised at site 1 with environments built (untimed). The sweep runs twice from copies
    of that state: the plain FP64 drop-in (FP64 contractions, exact per-sector SVD) and the mixed
    configuration (split-precision Krylov matvecs, FP64-class 7-slice energy and environment
    contractions, density-matrix truncation). Both are timed end to end on the host around a
    device synchronisation; |dE| compares every post-truncation energy of the two sweeps."""
    import mps_gb300 as mg
    from mps_gb300 import dmrg as gd
    Ws = gd.xxz_u1mpo(lx, 1.0, ctx=ctx)
    m0 = gd.mps_from_host(gd.binomial_mps_host(lx, lx // 2, chi, seed), ctx)
    gd.center_at(m0, 1, svd="gram")
    env0 = gd.initialenv(m0, Ws)
    kw = dict(maxdim=chi, tol=1e-10, lanczostol=1e-7, krylovdim=4, krylovmaxiter=8,
              tieband=SWEEP_TIEBAND)
    out = {}
    for name, cfg in (("fp64", SWEEP_FP64), ("mixed", SWEEP_MIXED)):
        mps = gd.MPState([mg.copy(A) for A in m0.As], center=1)
        env = [None if e is None else mg.copy(e) for e in env0]
        stats = []
        ctx.synchronize()
        t0 = time.perf_counter()
        es = gd.dmrg2sitesweep(mps, Ws, env, stats=stats, **kw, **cfg)
        ctx.synchronize()
        out[name] = (time.perf_counter() - t0, es, sum(i.numops for i in stats))
    t64, e64, n64 = out["fp64"]
    tmx, emx, nmx = out["mixed"]
    de = [abs(a - b) for a, b in zip(emx, e64)]
    breakdown = {}
    if phases:  # the same sweeps again, synchronised after every phase (not the timed numbers)
        for name, cfg in (("fp64", SWEEP_FP64), ("mixed", SWEEP_MIXED)):
            mps = gd.MPState([mg.copy(A) for A in m0.As], center=1)
            env = [None if e is None else mg.copy(e) for e in env0]
            pt = gd.PhaseTimer(ctx)
            gd.dmrg2sitesweep(mps, Ws, env, timing=pt, **kw, **cfg)
            breakdown[name] = {k: round(v, 3) for k, v in pt.s.items()}
    moved = {}
    if offload:  # the mixed sweep with environments kept off the device
        from mps_gb300.envstore import OffloadedEnvs
        for mode in ("async", "blocking"):
            mps = gd.MPState([mg.copy(A) for A in m0.As], center=1)
            env = [None if e is None else mg.copy(e) for e in env0]
            load = (lambda c, s, f: mg.from_flat(c, s, f, ctx)) if mode == "blocking" else None
            st = OffloadedEnvs(env, window=offload, ctx=ctx, load=load)
            del env
            ctx.synchronize()
            t0 = time.perf_counter()
            es = gd.dmrg2sitesweep(mps, Ws, st, **kw, **SWEEP_MIXED)
            ctx.synchronize()
            moved[mode] = {
                "sweep_s": time.perf_counter() - t0, "bit_identical": es == emx,
                "downloads": st.downloads, "uploads": st.uploads,
                "prefetches": st.prefetches, "prefetch_hits": st.prefetch_hits,
                "clean_evictions": st.clean_evictions,
                "GB_down": st.transfer.bytes_down / 1e9, "GB_up": st.transfer.bytes_up / 1e9}
    return {
        "workload": f"one 2-site DMRG sweep, Heisenberg chain L={lx} (J=1, OBC, Sz=0), "
                    f"maxdim={chi}, cutoff 1e-10, tie band {SWEEP_TIEBAND:g}, Krylov dim 4, "
                    f"maxiter 8, tol 1e-7; initial "
                    f"MPS: N(0,1) blocks (Philox seed {seed}), binomial bond profile ~{chi}",
        "fp64_s": t64, "mixed_s": tmx, "speedup_mixed_vs_fp64": t64 / tmx,
        "mixed_config": {k: v for k, v in SWEEP_MIXED.items()},
        "fp64_config": {k: v for k, v in SWEEP_FP64.items()},
        "energy_fp64": e64[-1], "energy_mixed": emx[-1],
        "dE_final": abs(emx[-1] - e64[-1]), "dE_max_over_sweep": max(de),
        "dE_rel_final": abs(emx[-1] - e64[-1]) / abs(e64[-1]),
        "matvecs_fp64": n64, "matvecs_mixed": nmx, "energies_per_sweep": len(e64),
        **({"phases_s": breakdown} if phases else {}),
        **({"offloaded_envs": {"window": offload, "resident_mixed_s": tmx, **moved}}
           if offload else {}),
    }


def run_ours(args):
    import numpy as np
    import torch

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import mps_gb300 as mg
    from mps_gb300 import dmrg as gd

    ctx = mg.get_context(local)
    stream = torch.cuda.ExternalStream(ctx.stream())
    prob = gd.heff_problem(args.chi, ctx=ctx)
    flops = mg.applymps2site_flops(*prob)
    S = DEFAULT_SLICES if args.precision is None else args.precision
    flush = torch.empty(512 * 2 ** 20 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    # prepared operators (built once per bond in a DMRG sweep); build time reported separately
    t0 = time.perf_counter()
    op = mg.Heff2(*prob, precision=S)
    ctx.synchronize()
    op_build_ms = (time.perf_counter() - t0) * 1e3
    op64 = mg.Heff2(*prob, precision=0) if S != 0 else op
    v = prob[0]

    def timed_steps(o, k, with_kernel_timing=False):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        ctx.set_timing(with_kernel_timing)
        with torch.cuda.stream(stream):
            for i in range(k):
                flush.zero_()
                starts[i].record(stream)
                out = o(v)
                ends[i].record(stream)
                del out
        torch.cuda.synchronize()
        return [s.elapsed_time(e) for s, e in zip(starts, ends)]

    for o in (op, op64):
        for _ in range(args.warmup):
            del_out = o(v)
            del del_out
    def soak_batch():
        with torch.cuda.stream(stream):
            for _ in range(20):
                flush.zero_()
                out = op(v)
                del out

    with ClockSampler(local) as cs:
        soak_s, soak_steps = clock_soak(soak_batch, torch.cuda.synchronize, 1.0, 20)
        barrier()
        launches0, _ = ctx.counters()
        ms = timed_steps(op, args.steps)
        launches = ctx.counters()[0] - launches0
    clocks = cs.summary()
    clocks["soak"] = f"{soak_steps} untimed steps ({soak_s:.2f} s) just before the timed ones"
    t, value = replica_rate(sum(ms) / len(ms) / 1e3, flops, ws, f"cuda:{local}")

    # the plain FP64 drop-in on the same inputs
    ms64 = timed_steps(op64, max(3, min(args.steps, 10))) if S != 0 else ms
    t64, value64 = replica_rate(sum(ms64) / len(ms64) / 1e3, flops, ws, f"cuda:{local}")

    # accuracy of this step against the FP64 drop-in
    y = op(v).to_flat()
    y64 = op64(v).to_flat()
    rel_err = float(np.linalg.norm(y - y64) / np.linalg.norm(y64))
    # the neighbouring slice counts on the same inputs (context for the headline's choice):
    # 3 slices (FP32-level accuracy, the fast kernel), 4 and 7 (the exact kernel)
    others = {}
    for S_alt in (3, 4, 7):
        if S_alt == S or S == 0:
            continue
        try:
            op_alt = mg.Heff2(*prob, precision=S_alt)
            for _ in range(args.warmup):
                op_alt(v)
            ms_alt = timed_steps(op_alt, max(3, min(args.steps, 10)))
            y_alt = op_alt(v).to_flat()
        except mg.MPSGError as e:  # reported, the headline stands without it
            others[str(S_alt)] = {"error": str(e)}
            continue
        t_alt = sum(ms_alt) / len(ms_alt)
        others[str(S_alt)] = {"ms_per_step": t_alt, "value": flops / (t_alt / 1e3) / 1e9,
                              "unit": UNIT,
                              "rel_err_vs_fp64": float(np.linalg.norm(y_alt - y64) /
                                                       np.linalg.norm(y64))}
        del op_alt

    # per-kernel CUDA-event times (second pass over the same steps)
    timed_steps(op, args.steps, with_kernel_timing=True)
    kinds = {k: ctx.kernel_time(k) for k in ("copy", "gemm_f64", "gemm_split", "pack",
                                             "pack_slices")}
    ctx.set_timing(False)

    # end to end through the C ABI with host buffers: H2D of all five inputs (overlapped with the
    # operator preparation), the reference-facing _applymps2site, D2H of v'
    host_in = [torch.from_numpy(x.to_flat()).pin_memory() for x in prob]
    host_out = torch.empty(prob[0].numel(), dtype=torch.float64).pin_memory()
    dev = [mg.zeros(x.charge, x.space, ctx) for x in prob]
    h2d = sum(h.numel() * 8 for h in host_in)
    d2h = host_out.numel() * 8
    e2e_t = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mg.applymps2site_host(*dev, host_in, host_out, precision=S)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_t.append(t1 - t0)
    e2e_out = host_out.numpy().copy()
    e2e_err = float(np.linalg.norm(e2e_out - y64) / np.linalg.norm(y64))
    _, e2e_value = replica_rate(statistics.mean(e2e_t), flops, ws, f"cuda:{local}")
    # the same reference-facing call in plain FP64 (the drop-in), fewer steps
    e2e64_t = []
    for i in range(2 + max(3, min(args.steps, 10))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mg.applymps2site_host(*dev, host_in, host_out, precision=0)
        t1 = time.perf_counter()
        if i >= 2:
            e2e64_t.append(t1 - t0)
    _, e2e64_value = replica_rate(statistics.mean(e2e64_t), flops, ws, f"cuda:{local}")
    e2e64_out = host_out.numpy().copy()

    # every result of this step against the oracle (the NumPy restatement of the reference's
    # contraction path, on the host cores) on the same inputs
    vs_oracle = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import mps as om
        from oracle import symtensors as ost
        want = ost.flatten(om.applymps2site(*oracle_inputs(args.chi)))
        nw = np.linalg.norm(want)
        rel = lambda y_: float(np.linalg.norm(y_ - want) / nw)
        vs_oracle = {"headline": rel(y), "fp64": rel(y64), "e2e": rel(e2e_out),
                     "e2e_fp64": rel(e2e64_out),
                     "oracle": "NumPy/OpenBLAS restatement of _applymps2site (apply.jl:93-105)"}

    peaks = measured_peaks()
    step_ms = sum(ms) / len(ms)
    if S == 0:
        gem_ms, gem_n, gem_f = kinds["gemm_f64"]
        a = torch.randn(8192, 8192, dtype=torch.float64, device=f"cuda:{local}")
        torch.matmul(a, a)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            torch.matmul(a, a)
        e1.record()
        torch.cuda.synchronize()
        peak = 3 * 2 * 8192 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12
        peak_src = "cuBLAS DGEMM 8192^3 measured in this run (no FP64 figure in MEASURED_PEAKS.json)"
        del a
        pipe, dtype = "fp64", "f64"
        achieved = gem_f / (gem_ms / 1e3) / 1e12 if gem_n else None
        kernel_desc = "grouped FP64 block GEMM (one launch per contraction)"
    else:
        gem_ms, gem_n, gem_f = kinds["gemm_split"]
        peak = peaks["bf16_tflops"] if peaks else 1900.0
        peak_src = "MEASURED_PEAKS.json bf16_tflops (burst)" if peaks else "fallback 1.9 PFLOP/s"
        pipe = "bf16-tensor (tcgen05)"
        dtype = f"f64 via {S} bf16 slices ({S * (S + 1) // 2} tcgen05 products, fp32 TMEM accumulate)"
        # achieved = the kernel's own algorithmic flops (sum of 2*M*N*K over the sector GEMMs of
        # the two W-folded contractions it runs) per second, not the executed slice products
        achieved = gem_f / (gem_ms / 1e3) / 1e12 if gem_n else None
        kernel_desc = ("split-precision grouped block GEMM (2 launches per H_eff application, "
                       "the W-folded contractions envLW.v and X.envRW; achieved = their sector "
                       "GEMM flops / summed GEMM time)")
    pairs = S * (S + 1) // 2 if S else 1
    roof = {"bound": "tensor", "pipe": pipe, "kernel": kernel_desc, "launches_timed": gem_n,
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved / peak) if achieved else None, "peak_source": peak_src + " (of measured)"
            if peaks else peak_src,
            # executed tensor work: every algorithmic flop costs `pairs` bf16 slice products
            "executed_tflops": achieved * pairs if achieved else None,
            "executed_frac": achieved * pairs / peak if achieved else None,
            "traffic": profile_traffic(f"gemm_p{S}_chi{args.chi}")}
    share = {k: round(v_[0] / args.steps / step_ms, 4) for k, v_ in kinds.items() if v_[1]}
    # HBM rooflines of the memory-bound kernels of one application: algorithmic bytes (copies:
    # 8 read + 8 written per element moved; packing: 8 + 8 read + 2 S written per element) over
    # their CUDA-event time, against the measured copy bandwidth
    hbm = peaks["hbm_gbs"] if peaks else 6800.0
    mem_roof = {}
    if S:
        copy_b, pack_b = op.traffic()
        for name, nbytes, ks in (("permute", copy_b, ("copy",)),
                                 ("pack", pack_b, ("pack", "pack_slices"))):
            ms_k = sum(kinds[k][0] for k in ks) / args.steps
            if ms_k > 0 and nbytes > 0:
                gbs = nbytes / (ms_k / 1e3) / 1e9
                mem_roof[name] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                                  "frac": gbs / hbm, "bytes_per_step": nbytes,
                                  "ms_per_step": ms_k}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype,
        "data": "synthetic (seeded Philox N(0,1) blocks)",
        "config": workload_config(args.chi),
        "run": {"precision_slices": S, "gflop_per_step": flops / 1e9,
                "op_build_ms": op_build_ms,
                "parallelism": "replicas" if ws > 1 else "single GPU"},
        "fp64": {"value": value64, "unit": UNIT, "ms_per_step": t64 * 1e3,
                 "speedup_mixed_vs_fp64": t64 / t,
                 "e2e": {"value": e2e64_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h,
                         "call": "mpsg_applymps2site_host, precision 0 (FP64 drop-in)"}},
        "rel_err_vs_fp64": rel_err,
        "rel_err_vs_oracle": vs_oracle,
        "other_slice_counts": others,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "rel_err_vs_fp64": e2e_err,
                "call": "mpsg_applymps2site_host (uploads on a copy stream overlapped with the "
                        "operator preparation)"},
        "gpu_launches": launches,
        "kernel_share_of_step": share,
        "roofline": roof,
        "memory_rooflines": mem_roof,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_sweep and ws == 1:
        line["sweep"] = sweep_bench(ctx, args.sweep_chi or args.chi, phases=args.sweep_phases,
                                    offload=args.sweep_offload)
    if rank == 0 and not args.no_cpu_baseline and ws == 1:
        os.environ.setdefault("OPENBLAS_NUM_THREADS", str(os.cpu_count() or 1))
        vv, n, tm, cores = cpu_heff_rate(args.chi, flops)
        line["cpu_baseline"] = {"value": vv, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{n} full H_eff matvecs of the same workload "
                                          f"({tm:.2f} s each), NumPy/OpenBLAS oracle"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_gradient(args):
    """Energy gradients by adjoint contractions on a DMRG-converged XXZ chain (L=64, Delta=0.5,
    maxdim 512): dE/dDelta (Hellmann-Feynman through the MPO cotangents) and dE/dA for every
    site tensor, from one forward and one backward sweep of FP64 contractions. Checked against
    central differences (h = 1e-5) of <psi|H(Delta)|psi> for the same state, and the gradient at
    the orthogonality center against 2 E A (stationarity)."""
    import numpy as np
    import mps_gb300 as mg
    from mps_gb300 import dmrg as gd
    from mps_gb300 import grad as gr
    lx, chi, delta = 64, 512, 0.5
    ctx = mg.get_context(0)
    Ws = gd.xxz_u1mpo(lx, delta, ctx=ctx)
    mps = gd.mps_from_host(gd.binomial_mps_host(lx, lx // 2, chi, 11), ctx)
    gd.center_at(mps, 1, svd="gram")
    env = gd.initialenv(mps, Ws)
    t0 = time.perf_counter()
    es = []
    for _ in range(4):
        es = gd.dmrg2sitesweep(mps, Ws, env, maxdim=chi, tol=1e-10, lanczostol=1e-9, krylovdim=4,
                               krylovmaxiter=8, precision=4, energy_precision=7,
                               env_precision=7, svd="gram")
    ctx.synchronize()
    t_dmrg = time.perf_counter() - t0
    t0 = time.perf_counter()
    E, g = gr.energy_gradients(mps.As, Ws)
    dEd = gr.xxz_delta_derivative(g, Ws, lx)
    grads = [g(A) for A in mps.As]
    ctx.synchronize()
    t_grad = time.perf_counter() - t0
    # the same gradients keeping only every ceil(sqrt(L))-th environment (recomputed per segment)
    import math
    t0 = time.perf_counter()
    Ec, gc = gr.energy_gradients_checkpointed(mps.As, Ws)
    dEd_c = gr.xxz_delta_derivative(gc, Ws, lx)
    ctx.synchronize()
    t_ckpt = time.perf_counter() - t0
    ckpt_rel = max(float(np.linalg.norm(gc(A).to_flat() - gA.to_flat())
                         / max(np.linalg.norm(gA.to_flat()), 1e-300))
                   for A, gA in zip(mps.As, grads))
    h = 1e-5
    ep = gr.energy_gradients(mps.As, gd.xxz_u1mpo(lx, delta + h, ctx=ctx))[0]
    em = gr.energy_gradients(mps.As, gd.xxz_u1mpo(lx, delta - h, ctx=ctx))[0]
    fd = (ep - em) / (2 * h)
    A1 = mps.As[0].to_flat()
    stat = float(np.linalg.norm(grads[0].to_flat() - 2 * E * A1) / np.linalg.norm(2 * E * A1))
    line = {
        "metric": "energy gradient s (dE/dDelta + dE/dA, adjoint contractions)",
        "value": t_grad, "unit": "s", "higher_is_better": False, "n_gpus": 1,
        "data": "synthetic (seeded Philox N(0,1) initial MPS)",
        "config": {"workload": f"XXZ chain L={lx}, Delta={delta}, maxdim {chi}, converged by 4 "
                               "mixed 2-site sweeps (Krylov 4 slices, energy/env 7 slices)",
                   "dtype": "f64"},
        "energy": E, "dE_dDelta": dEd, "dE_dDelta_fd": fd, "fd_abs_diff": abs(dEd - fd),
        "center_stationarity_relerr": stat, "dmrg_s": t_dmrg, "last_sweep_energy": es[-1],
        "checkpointed": {"s": t_ckpt, "every": math.ceil(math.sqrt(lx)),
                         "dE_dDelta": dEd_c, "max_rel_diff_dA": ckpt_rel,
                         "energy_abs_diff": abs(Ec - E)},
    }
    print(json.dumps(line), flush=True)


def run_cylinder(args):
    """2-site DMRG on the J1 Heisenberg cylinder (width 6, length 24, periodic around the
    circumference, column-major sites; MPO from the lattice generator, 20-26 channels) at
    maxdim chi from a random binomial-profile MPS: wall time of each mixed sweep (the sweep
    bench's mixed configuration) and the energies; a line per sweep goes to stderr as it ends.
    ``--compare-fp64`` repeats the last sweep as the FP64 drop-in from the same state."""
    import mps_gb300 as mg
    from mps_gb300 import dmrg as gd
    from mps_gb300 import lattice as lt
    width, length = 6, 24
    n = width * length
    chi = args.sweep_chi or 1024
    ctx = mg.get_context(0)
    Ws = lt.device_mpo(n, lt.cylinder_heisenberg_terms(width, length), ctx=ctx,
                       share_prefixes=args.mpo_shared_prefixes)
    mps = gd.mps_from_host(gd.binomial_mps_host(n, n // 2, chi, 13), ctx)
    t0 = time.perf_counter()
    gd.center_at(mps, 1, svd="gram", normalize=True)  # 144 random sites: keep the norm at 1
    env = gd.initialenv(mps, Ws)
    ctx.synchronize()
    t_init = time.perf_counter() - t0
    times, energies, matvecs = [], [], []
    kw = dict(maxdim=chi, tol=1e-10, lanczostol=1e-7, krylovdim=4, krylovmaxiter=8,
              tieband=SWEEP_TIEBAND)
    compare = None
    print(json.dumps({"init_s": t_init}), file=sys.stderr, flush=True)
    for k in range(args.sweeps):
        saved = None
        if args.compare_fp64 and k == args.sweeps - 1:  # the state the last sweep starts from
            saved = ([mg.copy(A) for A in mps.As], [None if e is None else mg.copy(e) for e in env])
        stats = []
        ctx.synchronize()
        t0 = time.perf_counter()
        es = gd.dmrg2sitesweep(mps, Ws, env, stats=stats, **kw, **SWEEP_MIXED)
        ctx.synchronize()
        times.append(time.perf_counter() - t0)
        energies.append(es[-1])
        matvecs.append(sum(i.numops for i in stats))
        print(json.dumps({"sweep": k + 1, "s": times[-1], "energy": es[-1],
                          "energy_per_site": es[-1] / n}), file=sys.stderr, flush=True)
        if saved is not None:
            m64 = gd.MPState(saved[0], center=1)
            e64_env = saved[1]
            del saved
            ctx.synchronize()
            t0 = time.perf_counter()
            e64 = gd.dmrg2sitesweep(m64, Ws, e64_env, **kw, **SWEEP_FP64)
            ctx.synchronize()
            t64 = time.perf_counter() - t0
            de = [abs(a - b) for a, b in zip(es, e64)]
            compare = {"fp64_sweep_s": t64, "mixed_sweep_s": times[-1],
                       "speedup_mixed_vs_fp64": t64 / times[-1],
                       "energy_fp64": e64[-1], "energy_mixed": es[-1],
                       "dE_final": de[-1], "dE_max_over_sweep": max(de),
                       "dE_rel_max_over_sweep": max(de) / abs(e64[-1]),
                       "energies_compared": len(de), "fp64_config": SWEEP_FP64}
            print(json.dumps({"fp64_sweep_s": t64, **{k_: v_ for k_, v_ in compare.items()
                                                      if k_ != "fp64_config"}}),
                  file=sys.stderr, flush=True)
            del m64, e64_env
    line = {
        "metric": "DMRG sweep s, J1 Heisenberg 6x24 cylinder", "value": times[-1], "unit": "s",
        "higher_is_better": False, "n_gpus": 1, "data": "synthetic (seeded Philox initial MPS)",
        "config": {"workload": f"6x24 cylinder (PBC around, OBC along), J1=1, Sz=0, maxdim {chi}, "
                               "cutoff 1e-10, Krylov dim 4, maxiter 8", "mixed": SWEEP_MIXED,
                   "mpo": "shared prefixes" if args.mpo_shared_prefixes else "one channel per term"},
        "sweep_s": times, "energy_per_sweep": energies, "energy_per_site": energies[-1] / n,
        "matvecs_per_sweep": matvecs, "init_s": t_init,
        "max_mpo_bond": max(W.space[2].dim() for W in Ws),
        **({"last_sweep_vs_fp64": compare} if compare else {}),
    }
    print(json.dumps(line), flush=True)


def run_small_chain(args):
    """The reference's CPU-sized DMRG case: Heisenberg chain L=32 (J=1, OBC, Sz=0), maxdim 64,
    cutoff 1e-10, Krylov dim 4, maxiter 8, four 2-site sweeps from a random MPS (seed 1911)
    canonicalised at site 1. The device runs the FP64 drop-in configuration; the CPU oracle
    (the reference's algorithm restated in NumPy) runs the same sweeps from the same tensors,
    timed beside it, and every post-truncation energy is compared."""
    import numpy as np

    import mps_gb300 as mg
    from mps_gb300 import dmrg as gd
    from oracle import mps as om
    from oracle import symtensors as st
    lx, chi, nsweeps = 32, 64, 4
    ctx = mg.get_context(0)
    sites = gd.random_mps_host(lx, lx // 2, chi, seed=1911)
    conv = lambda sp: tuple(st.VectorSpace(V.sectors, V.isdual) for V in sp)
    mo = om.MPState([st.from_flat(c, conv(sp), f) for c, sp, f in sites], 0)
    om.center_at(mo, 1)
    up = lambda T: mg.from_flat(T.charge, tuple(mg.VectorSpace(V.sectors, V.isdual)
                                                for V in T.space), st.flatten(T), ctx)
    md = gd.MPState([up(A) for A in mo.As], center=1)
    Wo, Wd = om.xxz_u1mpo(lx, 1.0), gd.xxz_u1mpo(lx, 1.0, ctx=ctx)
    eo, ed = om.initialenv(mo, Wo), gd.initialenv(md, Wd)
    kw = dict(maxdim=chi, tol=1e-10, lanczostol=1e-7, krylovdim=4, krylovmaxiter=8,
              tieband=1e-12)
    t_dev, t_cpu, e_dev, e_cpu, mv = [], [], [], [], []
    for _ in range(nsweeps):
        stats = []
        ctx.synchronize()
        t0 = time.perf_counter()
        es = gd.dmrg2sitesweep(md, Wd, ed, stats=stats, **kw)
        ctx.synchronize()
        t_dev.append(time.perf_counter() - t0)
        e_dev.append(es)
        mv.append(sum(i.numops for i in stats))
        t0 = time.perf_counter()
        e_cpu.append(om.dmrg2sitesweep(mo, Wo, eo, **kw))
        t_cpu.append(time.perf_counter() - t0)
    rel = max(float(np.max(np.abs(np.array(a) - np.array(b)) / np.abs(np.array(b))))
              for a, b in zip(e_dev, e_cpu))
    line = {
        "metric": "DMRG s for 4 sweeps, Heisenberg chain L=32, maxdim 64", "value": sum(t_dev),
        "unit": "s", "higher_is_better": False, "n_gpus": 1, "dtype": "f64",
        "data": "synthetic (seeded Philox initial MPS)",
        "config": {"workload": "Heisenberg chain L=32 (J=1, OBC, Sz=0), maxdim 64, cutoff 1e-10, "
                               "Krylov dim 4, maxiter 8, 4 sweeps, FP64 drop-in"},
        "sweep_s": t_dev, "matvecs_per_sweep": mv, "energy_final": e_dev[-1][-1],
        "max_rel_energy_diff_vs_oracle": rel,
        "cpu_baseline": {"value": sum(t_cpu), "unit": "s", "kind": "port",
                         "cores": int(os.environ.get("OPENBLAS_NUM_THREADS", os.cpu_count() or 1)),
                         "sample": "the same 4 sweeps from the same tensors (NumPy/OpenBLAS "
                                   "oracle)", "sweep_s": t_cpu},
    }
    print(json.dumps(line), flush=True)


def run_batched(args):
    """Many independent chains: one sweep of each of N seeded XXZ chains (mixed configuration).
    Timed (wall, setup included: random MPS, canonicalisation, environments): in lock step on
    one context with batched eigensolves (``--lockstep``), concurrently (one context / CUDA
    stream and one host thread per chain) and one after the other. ``--fp64-check K`` runs the
    first K chains as the FP64 drop-in and compares energies."""
    import mps_gb300 as mg
    from mps_gb300 import dmrg as gd
    specs = gd.chain_ensemble(args.batched)
    kw = dict(tol=1e-10, lanczostol=1e-7, krylovdim=4, krylovmaxiter=8, tieband=SWEEP_TIEBAND)
    o = gd.SweepOptions(**kw, **SWEEP_MIXED)
    ctx = mg.get_context(0)
    ctx.synchronize()
    res, stats, t_lock, launches = {}, {}, None, None
    if args.lockstep:
        k0, _ = ctx.counters()
        t0 = time.perf_counter()
        res["lockstep"] = gd.run_chains_lockstep(specs, 1, o, stats=stats,
                                                 wait_all=not args.dynamic)
        ctx.synchronize()
        t_lock = time.perf_counter() - t0
        launches = ctx.counters()[0] - k0
    t0 = time.perf_counter()
    res["concurrent"] = gd.run_chains(specs, 1, o, threads=len(specs))
    t_conc = time.perf_counter() - t0
    t_seq = None
    if not args.batched_concurrent_only:
        t0 = time.perf_counter()
        res["one_by_one"] = gd.run_chains(specs, 1, o, threads=1)
        t_seq = time.perf_counter() - t0
    fp64 = None
    if args.fp64_check:
        o64 = gd.SweepOptions(**kw, **SWEEP_FP64)
        fp64 = gd.run_chains(specs[:args.fp64_check], 1, o64, threads=1)

    def rel(a, b):
        return max(abs(x - y) / abs(y) for x, y in zip(a, b))

    main = "lockstep" if args.lockstep else "concurrent"
    t_main = t_lock if args.lockstep else t_conc
    line = {
        "metric": "independent DMRG chains, one sweep each: wall s", "value": t_main, "unit": "s",
        "higher_is_better": False, "n_gpus": 1, "data": "synthetic (seeded Philox)",
        "config": {"workload": f"{len(specs)} XXZ chains, L in [32,128], Delta in [0,1.5], maxdim "
                               "in {128,256,512,1024} (Philox seed 1911), one 2-site sweep each",
                   "mixed": SWEEP_MIXED, "sweep": kw, "chains": [list(s) for s in specs]},
        "mode": main, "lockstep_s": t_lock, "concurrent_s": t_conc, "one_by_one_s": t_seq,
        "speedup_vs_one_by_one": t_seq / t_main if t_seq else None,
        "speedup_vs_concurrent": t_conc / t_lock if args.lockstep else None,
        "max_rel_dE_vs_one_by_one": rel(res[main], res["one_by_one"]) if t_seq else None,
        "energies": res[main],
    }
    if args.lockstep:
        sizes = stats.pop("chains_per_batch")
        line["lockstep"] = {**stats, "kernel_launches": launches,
                            "mean_chains_per_batch": sum(sizes) / max(1, len(sizes))}
        line["max_rel_dE_lockstep_vs_concurrent"] = rel(res["lockstep"], res["concurrent"])
    if fp64 is not None:
        line["fp64_check"] = {"chains": args.fp64_check, "energies_fp64": fp64,
                              "rel_dE": [abs(a - b) / abs(b) for a, b in zip(res[main], fp64)]}
    print(json.dumps(line), flush=True)


def run_tdvp(args):
    """1-site TDVP (symmetric turning point: one sweep = exact-in-the-manifold step of 2 dt) of
    an XXZ chain (Delta = 0.5) from a seeded random U(1) MPS with a binomial bond profile of
    about chi states, on complex block-sparse tensors (two real parts, GPU contractions,
    per-sector complex SVD gauge moves). Reports seconds per sweep, norm and energy drift, and
    C(t) = <Sz_i Sz_{i+1}>(t) (i = L/2) with dC/dDelta twice: by forward-mode tangents through
    the sweeps (one evolution carrying derivatives, ``mps_gb300.tdvp_grad``) and by central
    differences (h = 1e-5: evolutions under H(Delta +- h) from the same state; off with
    --tdvp-no-fd); with --tdvp-adjoint also by reverse mode over the same sweeps (the gradient
    with respect to every MPO tensor and initial site tensor, contracted with dW/dDelta)."""
    import numpy as np
    import mps_gb300 as mg
    from mps_gb300 import ctensor as ct
    from mps_gb300 import dmrg as gd
    from mps_gb300 import tdvp as td
    lx, chi, delta, dt, h = args.tdvp_lx, args.sweep_chi or 64, 0.5, 0.05, 1e-5
    steps = args.tdvp_steps
    ctx = mg.get_context(0)
    ops = ct.gpu_ops(args.tdvp_precision, ctx)
    host = gd.binomial_mps_host(lx, lx // 2, chi, 17)
    i = lx // 2
    sz = td.site_operator(ops, mg.VectorSpace(gd.SITE), {0: -0.5, 1: 0.5})

    def evolve(d, timed):
        mps = gd.mps_from_host(host, ctx)
        gd.center_at(mps, 1)
        mg.rmul(mps.As[0], 1.0 / mg.norm(mps.As[0]))
        Ws = gd.xxz_u1mpo(lx, d, ctx=ctx)
        As = [ct.CTensor(A) for A in mps.As]
        env = td.initialenv(ops, As, Ws)
        e0 = td.energy(ops, As, Ws, env)
        stats = td.TDVPStats()
        times = []
        prof = None
        if timed and args.tdvp_kernel_times:
            import torch
            prof = torch.profiler.profile(activities=[torch.profiler.ProfilerActivity.CUDA])
            prof.__enter__()
        for _ in range(steps):
            ctx.synchronize()
            t0 = time.perf_counter()
            td.tdvp1sitesweep(ops, dt, As, Ws, env, turning="symmetric", stats=stats)
            ctx.synchronize()
            times.append(time.perf_counter() - t0)
        if prof is not None:
            prof.__exit__(None, None, None)
            kern = {}
            for ev in prof.key_averages():
                t = float(getattr(ev, "self_device_time_total",
                                  getattr(ev, "self_cuda_time_total", 0.0)) or 0.0)
                if t > 0:
                    kern[ev.key] = (kern.get(ev.key, (0, 0.0))[0] + int(ev.count),
                                    kern.get(ev.key, (0, 0.0))[1] + t)
            busy = sum(t for _, t in kern.values()) / 1e6
            top = sorted(kern.items(), key=lambda kv: -kv[1][1])[:25]
            print(json.dumps({"kernel_times": {
                "wall_s": sum(times), "device_busy_s": busy,
                "top": [{"kernel": k[:120], "launches": c, "s": t / 1e6, "share": t / 1e6 / busy}
                        for k, (c, t) in top]}}), file=sys.stderr, flush=True)
        c = td.expectation(ops, As, {i: sz, i + 1: sz}).real
        out = {"C": c, "sweep_s": times, "matvecs": stats.matvecs,
               "exponentials": stats.exponentials, "unconverged": stats.unconverged}
        if timed:
            out["norm_drift"] = abs(td.norm2(ops, As) - 1.0)
            out["energy_drift"] = abs(td.energy(ops, As, Ws, env) - e0)
        return out

    r0 = evolve(delta, True)
    print(json.dumps({"forward_s": sum(r0["sweep_s"]), "C": r0["C"]}), file=sys.stderr,
          flush=True)
    if args.tdvp_forward_only:
        print(json.dumps({
            "metric": "1-site TDVP sweep s (complex U(1) MPS)",
            "value": float(np.median(r0["sweep_s"])), "unit": "s", "higher_is_better": False,
            "n_gpus": 1, "data": "synthetic (seeded Philox N(0,1) initial MPS)",
            "config": {"workload": f"XXZ chain L={lx}, Delta={delta}, binomial bond profile "
                                   f"~{chi}, {steps} sweeps of dt={dt}, forward only"},
            "C_t": r0["C"], "sweep_s": r0["sweep_s"], "norm_drift": r0["norm_drift"],
            "energy_drift": r0["energy_drift"],
            "matvecs_per_sweep": r0["matvecs"] / steps}), flush=True)
        return
    # the derivative by tangents through the same sweeps
    from mps_gb300 import tdvp_grad as tg
    mps = gd.mps_from_host(host, ctx)
    gd.center_at(mps, 1)
    mg.rmul(mps.As[0], 1.0 / mg.norm(mps.As[0]))
    Ws = gd.xxz_u1mpo(lx, delta, ctx=ctx)
    dWs = [ops.lincomb([(1.0, a), (-1.0, b)])
           for a, b in zip(gd.xxz_u1mpo(lx, 1.0, ctx=ctx), gd.xxz_u1mpo(lx, 0.0, ctx=ctx))]
    As = [ct.CTensor(A) for A in mps.As]
    tstats = tg.TangentStats()
    ctx.synchronize()
    t0 = time.perf_counter()
    c_t, dc_t = tg.evolve_with_tangent(ops, As, Ws, dWs, dt, steps, {i: sz, i + 1: sz},
                                       stats=tstats)
    ctx.synchronize()
    tangent_s = time.perf_counter() - t0
    print(json.dumps({"tangent_s": tangent_s, "dC": dc_t.real}), file=sys.stderr, flush=True)
    del As, mps
    adj = {}
    if args.tdvp_adjoint:
        # reverse mode over the same sweeps: gradients of C with respect to every MPO tensor
        # and every initial site tensor; dC/dDelta = sum over sites of <grad W_l, dW_l>
        mps = gd.mps_from_host(host, ctx)
        gd.center_at(mps, 1)
        mg.rmul(mps.As[0], 1.0 / mg.norm(mps.As[0]))
        As = [ct.CTensor(A) for A in mps.As]
        astats = tg.TangentStats()
        ctx.synchronize()
        t0 = time.perf_counter()
        c_a, gW, gA = tg.evolve_with_adjoint(ops, As, Ws, dt, steps, {i: sz, i + 1: sz},
                                             quad=6, stats=astats)
        ctx.synchronize()
        adjoint_s = time.perf_counter() - t0
        dc_a = sum(ops.dot(g.re, dW) for g, dW in zip(gW, dWs))
        adj = {"dC_dDelta_adjoint": dc_a, "C_t_adjoint_run": c_a.real,
               "rel_diff_adjoint_vs_tangent": abs(dc_a - dc_t.real) / abs(dc_t.real),
               "adjoint_evolution_s": adjoint_s, "adjoint_quadrature_nodes": 6,
               "adjoint_matvecs": astats.matvecs, "adjoint_unconverged": astats.unconverged,
               "adjoint_gradients": f"{len(gW)} MPO tensors + {len(gA)} initial site tensors"}
        print(json.dumps({"adjoint_s": adjoint_s, "dC": dc_a}), file=sys.stderr, flush=True)
        del As, mps, gW, gA
    fd = None
    if not args.tdvp_no_fd:
        rp = evolve(delta + h, False)
        rm = evolve(delta - h, False)
        fd = (rp["C"] - rm["C"]) / (2 * h)
    line = {
        "metric": "1-site TDVP sweep s (complex U(1) MPS)", "value": float(np.median(r0["sweep_s"])),
        "unit": "s", "higher_is_better": False, "n_gpus": 1,
        "data": "synthetic (seeded Philox N(0,1) initial MPS)",
        "config": {"workload": f"XXZ chain L={lx}, Delta={delta}, binomial bond profile ~{chi}, "
                               f"{steps} sweeps of dt={dt} (each sweep evolves by 2 dt), "
                               "Krylov tol 1e-12, dim <= 30",
                   "dtype": "complex f64" + (f" via {args.tdvp_precision} bf16 slices"
                                             if args.tdvp_precision else "")},
        "t": 2 * dt * steps, "C_t": r0["C"],
        "dC_dDelta_tangent": dc_t.real, "dC_dDelta_fd": fd,
        "rel_diff_tangent_vs_fd": abs(dc_t.real - fd) / abs(fd) if fd else None,
        "C_t_tangent_run": c_t.real, "tangent_evolution_s": tangent_s,
        "forward_evolution_s": sum(r0["sweep_s"]),
        "tangent_matvecs": tstats.matvecs, "tangent_unconverged": tstats.unconverged,
        "norm_drift": r0["norm_drift"], "energy_drift": r0["energy_drift"],
        "matvecs_per_sweep": r0["matvecs"] / steps, "unconverged_exponentials": r0["unconverged"],
        "sweep_s": r0["sweep_s"],
    }
    line.update(adj)
    print(json.dumps(line), flush=True)


def run_dense_gemm(args):
    """The split-precision grouped GEMM on a single dense N x N x N problem (one sector): the
    per-tile pipeline without the ragged work distribution of the sector GEMMs."""
    import numpy as np
    import mps_gb300 as mg
    n = args.dense_gemm
    S = DEFAULT_SLICES if args.precision is None else args.precision
    ctx = mg.get_context(0)
    V = mg.VectorSpace([(0, n)])
    rng = np.random.default_rng(3)
    A = mg.from_flat(0, (V, mg.dual(V)), rng.standard_normal(n * n), ctx)
    B = mg.from_flat(0, (V, mg.dual(V)), rng.standard_normal(n * n), ctx)
    for _ in range(args.warmup):
        mg.matmul(A, B, precision=S)
    ctx.synchronize()
    ctx.set_timing(True)
    for _ in range(args.steps):
        mg.matmul(A, B, precision=S)
    ctx.synchronize()
    ms, nl, fl = ctx.kernel_time("gemm_split")
    ctx.set_timing(False)
    peaks = measured_peaks()
    peak = peaks["bf16_tflops"] if peaks else 1900.0
    tf = fl / (ms / 1e3) / 1e12
    pairs = S * (S + 1) // 2
    line = {"metric": "split-precision GEMM on a dense block: algorithmic TFLOP/s", "value": tf,
            "unit": "TFLOP/s", "higher_is_better": True, "n_gpus": 1,
            "data": "synthetic (N(0,1) blocks)",
            "config": {"workload": f"dense {n}^3 block GEMM, {S} bf16 slices"},
            "ms_per_gemm": ms / max(nl, 1), "launches": nl, "executed_tflops": tf * pairs,
            "executed_frac_of_measured_bf16_peak": tf * pairs / peak, "peak": peak}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.gradient:
        run_gradient(a)
    elif a.cylinder:
        run_cylinder(a)
    elif a.batched:
        run_batched(a)
    elif a.small_chain:
        run_small_chain(a)
    elif a.tdvp:
        run_tdvp(a)
    elif a.dense_gemm:
        run_dense_gemm(a)
    else:
        run_ours(a)
