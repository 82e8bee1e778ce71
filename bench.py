#!/usr/bin/env python
"""Benchmark: two-site finite DMRG sweep on one GB300.

Workload (the configuration the headline metric is quoted on): 1D Fermi-
Hubbard open chain, L=64, t=1, U=8, half filling (32 up, 32 down), total
Sz=0, U(1)xU(1) (N, Sz) quantum numbers, physical dimension 4 with
Jordan-Wigner fermion signs, MPO bond dimension 6; alternating up/down
product state; the bond dimension grows 1000 -> 1430 -> ... -> 4000 over 8
sweeps (untimed set-up), Lanczos tolerance 1e-10 (100 iterations at most).
Then ``--warmup`` sweeps and ``--steps`` timed sweeps run at D=4000 in the
split form (3xTF32 matvec on the tensor cores, FP64-accurate environments
and Rayleigh energies, FP64 Lanczos recurrence and SVD).

* ``value``: seconds per sweep at D=4000, device-resident state, CUDA events
  on the library's stream around the timed sweeps (lower is better).  The
  state (several GB) is far larger than L2, so no flush is needed.
* ``fp64``: ``--fp64-sweeps`` sweeps of the same state in the plain FP64 form
  (FP64 FMA end to end), timed the same way; ``split_speedup`` = FP64 sweep
  time / split sweep time, with both forms' energies and |dE/E| between them.
* ``e2e``: the same split sweep through the C ABI from host buffers: upload
  of the MPS, MPO and right environments, the sweep, download of the MPS
  and right environments -- the drop-in call's work.
* ``roofline``, ``kernels``, ``gpu_launches``: from one more split sweep run
  under the library's kernel profiler (CUDA events around every kernel
  family on the library stream; the Lanczos iteration then runs host-driven,
  one iteration at a time, instead of as a CUDA-graph while loop): the
  kernel family with the most device time, its algorithmic flops (2*m*n*k
  over the QN-allowed block products) or bytes / its event time, against
  the measured peak; with the host time spent planning contractions and
  waiting for the device.
* ``cpu_baseline``: the FP64 CPU restatement (numpy + the host BLAS, all
  host threads) on three real two-site updates of the same state (near
  both ends and at the centre); a sweep is estimated as 2(L-1) times their
  mean update time.  Its energy at the centre bond is compared with the
  GPU's.
* ``--impl reference``: the same CPU restatement on the same kind of updates
  (block structures at eight evenly spaced bonds recorded from a GPU run of
  this workload, ``--record-structure``; random data; Lanczos capped at the
  recorded iteration counts), the reference's own gqten+MKL path being
  unbuildable here; the same sweep estimate.

Other workloads (not the headline line): ``--model heisenberg`` (L=100
chain, D 500 -> 2000), ``--model j1j2`` (4x16 cylinder, D 2000 -> 6000) and
``--workload batched`` (64 seeded XXZ chains, L in [16, 64], Delta in
[0.5, 1.5], D in {64..512}, 4 sweeps each, run concurrently and one after
another; the metric is instances per second).

Multi-GPU: a sweep is a sequential chain of updates, so N>1 runs N
independent replicas (one per rank); value is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MODELS = {
    "hubbard": {"L": 64, "schedule": [1000, 1430, 1860, 2290, 2710, 3140, 3570, 4000],
                "workload": "hubbard_obc_L64_U8_half_filling_D1000to4000"},
    "heisenberg": {"L": 100, "schedule": [500, 800, 1100, 1400, 1700, 2000],
                   "workload": "heisenberg_obc_L100_Sz0_D500to2000"},
    "j1j2": {"L": 64, "Lx": 16, "Ly": 4, "J1": 1.0, "J2": 0.5,
             "schedule": [2000, 2570, 3140, 3710, 4290, 4860, 5430, 6000],
             "workload": "j1j2_cylinder_4x16_snake_J2_0.5_D2000to6000"},
}
L_SITES = MODELS["hubbard"]["L"]
WORKLOAD = MODELS["hubbard"]["workload"]
SCHEDULE = MODELS["hubbard"]["schedule"]
LANCZOS = (1e-10, 100)
FAMILIES = ("gemm_fp64", "gemm_tf32x3", "gemm_fp64tc", "permute", "vector", "skinny")
N_BONDS = 8   # bonds of the CPU sweep estimate, evenly spaced over the chain


def _structure_fixture(model):
    return os.path.join(ROOT, "tests", "golden", f"bench_bonds_{model}.json")


def _sample_bonds(L, n=N_BONDS):
    """n 'r'-update sites evenly spaced over the L-1 bonds (each stands for
    (L-1)/n of them); a sweep's 2(L-1) updates are estimated as 2(L-1)
    times the mean update time at these sites."""
    return [min(L - 3, max(1, int(round((k + 0.5) * (L - 1) / n)))) for k in range(n)]


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", choices=["fp64", "tf32x3", "fp64tc"], default="tf32x3")
    p.add_argument("--rayleigh", choices=["fp64", "fp64tc"], default="fp64tc",
                   help="arithmetic of the split form's Rayleigh-quotient energies")
    p.add_argument("--model", choices=sorted(MODELS), default="hubbard",
                   help="hubbard: L=64 chain, U=8, half filling, D 1000->4000 (headline); "
                        "heisenberg: L=100 chain, D 500->2000; j1j2: 4x16 open cylinder "
                        "(snake order), J1=1, J2=0.5, D 2000->6000")
    p.add_argument("--schedule", default=None,
                   help="comma-separated D per growth sweep; the last is the timed D")
    p.add_argument("--fp64-sweeps", type=int, default=1,
                   help="timed sweeps of the plain FP64 form after the split ones")
    p.add_argument("--autotune", action="store_true",
                   help="enable the tile-choice autotuner (gq_autotune_enable) for the run")
    p.add_argument("--profile-region", choices=["sweeps", "centre", "update"], default="sweeps",
                   help="what an external profiler started with --profile-from-start off "
                        "records: the timed sweeps, the centre bond's Lanczos solves in the "
                        "three forms, or the split form's two-site update at the centre bond")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--record-structure", action="store_true",
                   help="write the block structures of the sampled bonds (reference arm)")
    p.add_argument("--workload", choices=["sweep", "batched"], default="sweep",
                   help="sweep: the chain of --model; batched: 64 independent XXZ "
                        "chains, concurrent vs one after another")
    p.add_argument("--instances", type=int, default=64)
    p.add_argument("--threads", type=int, default=16)
    return p.parse_args()


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
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
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def _fp64_peak_tflops(torch):
    """cuBLAS DGEMM 8192^3 throughput on this GPU (FP64 peak reference)."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


def _select_model(args):
    """Module constants for the chosen model (hubbard: the headline chain,
    L=64, t=1, U=8, half filling, Sz=0, U(1)xU(1), Jordan-Wigner MPO of bond
    dimension 6, alternating up/down product state; heisenberg: the L=100
    chain, shuffled Neel product state; j1j2: the 4x16 open cylinder in snake
    order, J1=1, J2=0.5, Sz=0, shuffled Neel product state, MPO from the
    generator's compression, bond dimension <= 17)."""
    global L_SITES, WORKLOAD, SCHEDULE
    m = MODELS[args.model]
    L_SITES, WORKLOAD, SCHEDULE = m["L"], m["workload"], m["schedule"]
    if args.schedule is None:
        args.schedule = ",".join(map(str, SCHEDULE))


def _model(model="hubbard"):
    from mps2_gb300 import hamiltonians as H
    from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
    L = MODELS[model]["L"]
    if model == "hubbard":
        sv, mpo, qn0, gen = H.hubbard_chain(L, 1.0, 8.0)
        labels = [1 if i % 2 == 0 else 2 for i in range(L)]
    elif model == "j1j2":
        m = MODELS["j1j2"]
        pairs = H.j1j2_cylinder_pairs(m["Lx"], m["Ly"], m["J1"], m["J2"])
        sv, mpo, qn0, gen = H.heisenberg_pairs(L, pairs)
        labels = H.neel_shuffled_labels(L, 0)
    else:
        sv, mpo, qn0, gen = H.heisenberg_chain(L)
        labels = H.neel_shuffled_labels(L, 0)
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, labels, qn0)
    return mps, mpo


def _tensor_bytes(t):
    return 8 * t.size()


# ---------------------------------------------------------------------------
# CPU restatement timing (oracle) -- test infrastructure used as the baseline
# ---------------------------------------------------------------------------
def _oracle_update(mpsd, mpo, envs, c, D, iters_cap=None):
    """Time one 'r' two-site update at site c with the FP64 CPU restatement
    (the oracle).  mpsd: {site: tensor}, envs: {('l'|'r', len): tensor}
    (product tensors); iters_cap: Lanczos iterations at most (the GPU's
    count for this update)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle  # noqa: F401
    from oracle.lanczos import LanczosParams as OLP
    from oracle.vmps import SweepParams as OSP, two_site_update
    from _convert import to_oracle
    N = len(mpo)
    om = [None] * N
    for k, t in mpsd.items():
        om[k] = to_oracle(t)
    oo = [to_oracle(t) if t is not None else None for t in mpo]
    oe = {k: to_oracle(v) for k, v in envs.items()}
    lz = OLP(LANCZOS[0], iters_cap + 1 if iters_cap else LANCZOS[1])
    t0 = time.perf_counter()
    st = two_site_update(om, oo, oe, OSP(1, D, D, 0.0, lz), "r", c)
    return time.perf_counter() - t0, st


def _describe_index(ix):
    return {"dir": ix.dir, "sectors": [[list(q), d] for q, d in ix.sectors()]}


def _synthetic_bond(model, L, rec, seed):
    """Random tensors with a recorded bond's block structure."""
    import numpy as np
    from mps2_gb300.tensor import GQTensor, Index
    rng = np.random.default_rng(seed)
    c = rec["site"]
    _, mpo = _model(model)

    def idx(d):
        return Index([(tuple(q), n) for q, n in d["sectors"]], d["dir"])

    def rand(indices, div):
        t = GQTensor(indices, tuple(div))
        for cc in t.allowed_coords(tuple(div)):
            t.blocks[cc] = rng.standard_normal(t.block_shape(cc))
        return t

    A = rand([idx(d) for d in rec["A_c"]], rec["div_c"])
    B = rand([idx(d) for d in rec["A_c1"]], rec["div_c1"])
    Le = rand([idx(d) for d in rec["L_env"]], rec["div_l"])
    Re = rand([idx(d) for d in rec["R_env"]], rec["div_r"])
    return {c: A, c + 1: B}, mpo, {("l", c): Le, ("r", L - c - 2): Re}


def _cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count()


# ---------------------------------------------------------------------------
def run_reference(args):
    """CPU restatement on two-site updates with the recorded block
    structures of evenly spaced bonds, one bond per step (cycling)."""
    ws, rank = _dist()
    if rank != 0:
        return
    path = _structure_fixture(args.model)
    if not os.path.exists(path):
        print(json.dumps({"impl": "reference",
                          "unavailable": f"no recorded bond structures for the {args.model} "
                                         "workload (bench.py --record-structure)"}))
        return
    with open(path) as f:
        fix = json.load(f)
    D, L, recs = fix["D"], fix["L"], fix["bonds"]
    # untimed warm-up steps on the cheapest recorded bond
    cheap = min(recs, key=lambda r: r["theta_size"])
    for w in range(args.warmup):
        mpsd, mpo, envs = _synthetic_bond(args.model, L, cheap, 1000 + w)
        _oracle_update(mpsd, mpo, envs, cheap["site"], D, cheap["iters"])
    per_bond = {}
    for k in range(max(1, args.steps)):
        rec = recs[k % len(recs)]
        mpsd, mpo, envs = _synthetic_bond(args.model, L, rec, k)
        t, _ = _oracle_update(mpsd, mpo, envs, rec["site"], D, rec["iters"])
        per_bond.setdefault(rec["site"], []).append(t)
    means = [sum(v) / len(v) for v in per_bond.values()]
    per_update = sum(means) / len(means)
    sweep_s = per_update * 2 * (L - 1)
    sample = (f"{args.steps} two-site update(s), one per step, cycling over {len(per_bond)} of "
              f"the {len(recs)} recorded bonds (sites {sorted(per_bond)}), D={D}, random data "
              f"with the recorded block structures, Lanczos capped at the recorded iteration "
              f"counts; sweep = 2(L-1) x mean over bonds of the mean update time")
    line = {
        "metric": f"DMRG sweep time (s/sweep) at D={D}",
        "value": sweep_s, "unit": "s/sweep", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_update * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (random tensors with block structures recorded from a GPU run of "
                "this workload)",
        "config": {"workload": WORKLOAD, "D": D, "L": L, "cache": "inputs larger than L2"},
        "per_bond_seconds": {str(k): v for k, v in sorted(per_bond.items())},
        "cpu_baseline": {"value": sweep_s, "unit": "s/sweep", "cores": _cpu_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": sweep_s, "unit": "s/sweep", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def _stats_sum(stats, key):
    return sum(getattr(s, key) for s in stats)


def run_ours(args):
    import torch
    import torch.distributed as dist
    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from mps2_gb300 import _lib
    from mps2_gb300.vmps import (Contract, DMRGState, LanczosParams, LanczosSolver, SweepParams,
                                 library_stream, profile_enable, profile_read)
    _lib.check(_lib.load().gq_init(local))
    if args.autotune:
        from mps2_gb300.vmps import autotune_enable
        autotune_enable(True)
    sched = [int(x) for x in args.schedule.split(",")]
    D = sched[-1]
    lp = LanczosParams(*LANCZOS)

    def params(d, prec=args.precision):
        return SweepParams(1, d, d, 0.0, lp, precision=prec, rayleigh=args.rayleigh)

    mps, mpo = _model(args.model)
    st = DMRGState(mps.tens, mpo)
    t_setup = time.perf_counter()
    st.init_envs(args.precision)
    for d in sched:
        e0, stats = st.sweep(params(d))
        print(f"[setup] sweep at D={d}: E0={e0:.12f} max bond {max(x.D for x in stats)} "
              f"({_stats_sum(stats, 'update_seconds'):.1f}s)", file=sys.stderr)
    for w in range(args.warmup):
        e0, stats = st.sweep(params(D))
        print(f"[warmup {w}] D={D} E0={e0:.12f} {_stats_sum(stats, 'update_seconds'):.1f}s",
              file=sys.stderr)
    setup_s = time.perf_counter() - t_setup

    ext = torch.cuda.ExternalStream(library_stream())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)

    def timed_sweeps(n, prec):
        """n sweeps at D timed with CUDA events on the library stream."""
        out_stats, energies = [], []
        torch.cuda.synchronize()
        ev0.record(ext)
        for _ in range(n):
            e, s_ = st.sweep(params(D, prec))
            out_stats.extend(s_)
            energies.append(e)
        ev1.record(ext)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) * 1e-3, out_stats, energies

    # ---- timed sweeps (split form, the headline) ------------------------------
    clocks = ClockSampler(local)
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    # an external profiler started with --profile-from-start off records the
    # timed sweeps only (or the centre bond's solves, below)
    if args.profile_region == "sweeps":
        torch.cuda.profiler.start()
    t_split, timed_stats, energies = timed_sweeps(args.steps, args.precision)
    if args.profile_region == "sweeps":
        torch.cuda.profiler.stop()
    clk = clocks.stop()
    ms = t_split * 1e3
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    sweep_s = ms * 1e-3 / args.steps

    # ---- the plain FP64 form on the same state, timed the same way -----------
    fp64 = None
    if args.fp64_sweeps > 0 and args.precision != "fp64":
        t64, st64, e64 = timed_sweeps(args.fp64_sweeps, "fp64")
        s64 = t64 / args.fp64_sweeps
        fp64 = {"sweep_s": s64, "sweeps": args.fp64_sweeps, "energies": e64,
                "split_speedup": s64 / sweep_s,
                "delta_e_rel_split_vs_fp64": abs(energies[-1] - e64[-1]) / abs(e64[-1]),
                "time_split_s": {"lanczos": _stats_sum(st64, "lanczos_seconds"),
                                 "svd": _stats_sum(st64, "svd_seconds"),
                                 "env": _stats_sum(st64, "env_seconds")},
                "matvec_tflops": _stats_sum(st64, "matvec_flops") /
                max(_stats_sum(st64, "lanczos_seconds"), 1e-9) / 1e12}

    # ---- one more split sweep under the kernel profiler ------------------------
    profile_enable(True)
    torch.cuda.synchronize()
    ev0.record(ext)
    st.sweep(params(D))
    ev1.record(ext)
    torch.cuda.synchronize()
    prof_sweep_s = ev0.elapsed_time(ev1) * 1e-3
    prof = {k: profile_read(k) for k in FAMILIES}
    svd_span = {k: profile_read(k) for k in ("svd", "svd_eig", "svd_gather", "svd_factors",
                                              "svd_ortho", "svd_gram", "svd_reduce")}
    host_plan = profile_read("host_plan")
    host_sync = profile_read("host_sync")
    profile_enable(False)
    n_launch_ours = sum(v[0] for v in prof.values())

    # ---- end to end through the C ABI from host buffers ---------------------
    host_mps = [st.get_mps(i) for i in range(L_SITES)]
    host_renv = {n: st.get_env("r", n) for n in range(1, L_SITES - 1)}
    h2d = sum(_tensor_bytes(t) for t in host_mps) + sum(_tensor_bytes(t) for t in mpo) + \
        sum(_tensor_bytes(t) for t in host_renv.values())
    d2h = sum(_tensor_bytes(t) for t in host_mps) + sum(_tensor_bytes(t) for t in host_renv.values())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st2 = DMRGState(host_mps, mpo)
    for n, t in host_renv.items():
        st2.set_env("r", n, t)
    st2.sweep(params(D))
    out_mps = [st2.get_mps(i) for i in range(L_SITES)]
    out_env = [st2.get_env("r", n) for n in range(1, L_SITES - 1)]
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    del st2, out_mps, out_env, host_mps, host_renv

    # ---- bonds of the CPU estimate: a half sweep to the right, stopping at
    # the sampled sites (the state is converged, so this only moves the
    # centre); at the centre bond the Lanczos problem in all three forms ------
    bonds = _sample_bonds(L_SITES)
    centre = bonds[len(bonds) // 2]
    recs, cpu_times, solve, gpu_centre, cpu_centre = [], {}, {}, None, None
    cpu_bonds = [] if (rank != 0 or args.no_cpu_baseline) else [bonds[1], centre, bonds[-2]]
    i = 0
    for b in bonds:
        while i < b:
            st.update(params(D), "r", i)
            i += 1
        mpsd = {b: st.get_mps(b), b + 1: st.get_mps(b + 1)}
        envs = {("l", b): st.get_env("l", b),
                ("r", L_SITES - b - 2): st.get_env("r", L_SITES - b - 2)}
        if b == centre:
            theta = Contract(mpsd[b], mpsd[b + 1], ([2], [0]))
            eff = [envs[("l", b)], mpo[b], mpo[b + 1], envs[("r", L_SITES - b - 2)]]
            for prec in ("fp64", "tf32x3", "fp64tc"):
                profile_enable(True)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                if args.profile_region == "centre":
                    torch.cuda.profiler.start()
                r = LanczosSolver(eff, theta, lp, "cent", precision=prec, rayleigh=args.rayleigh)
                torch.cuda.synchronize()
                if args.profile_region == "centre":
                    torch.cuda.profiler.stop()
                dt = time.perf_counter() - t0
                pr = {k: profile_read(k) for k in FAMILIES}
                profile_enable(False)
                gemm = ("gemm_fp64", "gemm_tf32x3", "gemm_fp64tc", "skinny")
                gemm_ms = sum(pr[k][1] for k in gemm)
                gemm_fl = sum(pr[k][2] for k in gemm)
                solve[prec] = {"energy": r.gs_eng, "iters": r.iters, "seconds": dt,
                               "kernel_ms": {k: pr[k][1] for k in FAMILIES},
                               "matvec_gemm_tflops": gemm_fl / (gemm_ms * 1e-3) / 1e12
                               if gemm_ms else None}
        if b == centre and args.profile_region == "update":
            torch.cuda.synchronize()
            torch.cuda.profiler.start()
        g = st.update(params(D), "r", b)
        if b == centre and args.profile_region == "update":
            torch.cuda.synchronize()
            torch.cuda.profiler.stop()
        i = b + 1
        if b == centre:
            gpu_centre = g
        if args.record_structure and rank == 0:
            recs.append({
                "site": b, "iters": int(max(1, g.iters)), "theta_size": int(g.theta_size),
                "A_c": [_describe_index(ix) for ix in mpsd[b].indices],
                "A_c1": [_describe_index(ix) for ix in mpsd[b + 1].indices],
                "L_env": [_describe_index(ix) for ix in envs[("l", b)].indices],
                "R_env": [_describe_index(ix) for ix in envs[("r", L_SITES - b - 2)].indices],
                "div_c": list(mpsd[b].div), "div_c1": list(mpsd[b + 1].div),
                "div_l": list(envs[("l", b)].div),
                "div_r": list(envs[("r", L_SITES - b - 2)].div)})
        if b in cpu_bonds:
            t_cpu, ost = _oracle_update(mpsd, mpo, envs, b, D, int(max(1, g.iters)))
            cpu_times[b] = t_cpu
            if b == centre:
                cpu_centre = ost
        del mpsd, envs
    if args.record_structure and rank == 0:
        path = _structure_fixture(args.model)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump({"L": L_SITES, "D": D, "model": args.model, "bonds": recs}, f)
    cpu = None
    if cpu_times:
        mean_t = sum(cpu_times.values()) / len(cpu_times)
        cpu = {"value": mean_t * 2 * (L_SITES - 1), "unit": "s/sweep", "cores": _cpu_threads(),
               "kind": "port",
               "sample": (f"{len(cpu_times)} two-site updates of this run's converged D={D} "
                          f"state at sites {sorted(cpu_times)} (CPU seconds "
                          f"{[round(cpu_times[k], 2) for k in sorted(cpu_times)]}), Lanczos "
                          f"capped at the GPU's iteration count; sweep = 2(L-1) x mean "
                          f"update time"),
               "centre_energy_cpu": cpu_centre.e0 if cpu_centre else None,
               "centre_energy_gpu": gpu_centre.e0 if gpu_centre else None}
        if cpu_centre is not None and gpu_centre is not None:
            cpu["centre_delta_e_rel"] = abs(gpu_centre.e0 - cpu_centre.e0) / abs(cpu_centre.e0)

    # ---- roofline of the dominant kernel family ------------------------------
    peaks, peak_kind = _measured_peaks()
    fp64_peak = _fp64_peak_tflops(torch)
    fam = {"gemm_tf32x3": ("tensor", "TFLOP/s", 0.5 * peaks["bf16_tflops"],
                           f"half the {peak_kind} bf16 dense peak (the TF32 rate); useful flops"),
           "gemm_fp64": ("fp64", "TFLOP/s", fp64_peak, "cuBLAS DGEMM 8192^3 measured in this run"),
           "gemm_fp64tc": ("tensor", "TFLOP/s", peaks["bf16_tflops"] / 28.0,
                           f"the {peak_kind} bf16 dense peak / 28 (bf16 MMAs per FP64-accurate "
                           "product); useful flops"),
           "permute": ("hbm", "GB/s", peaks["hbm_gbs"], f"{peak_kind} HBM copy bandwidth"),
           "vector": ("hbm", "GB/s", peaks["hbm_gbs"], f"{peak_kind} HBM copy bandwidth"),
           "skinny": ("hbm", "GB/s", peaks["hbm_gbs"], f"{peak_kind} HBM copy bandwidth")}
    top = max(prof, key=lambda k: prof[k][1])
    n_l, t_ms, fl, by = prof[top]
    bound, unit, peak, note = fam[top]
    achieved = ((fl / 1e12) if unit == "TFLOP/s" else (by / 1e9)) / (t_ms * 1e-3) if t_ms else 0.0
    kernels = {k: {"launches": v[0], "ms": v[1],
                   "share_of_sweep": v[1] * 1e-3 / prof_sweep_s} for k, v in prof.items()}
    for k in ("vector", "skinny", "permute"):
        n_k, ms_k, _, by_k = prof[k]
        kernels[k]["gbs"] = by_k / 1e9 / (ms_k * 1e-3) if ms_k else None
    for k in ("gemm_fp64", "gemm_tf32x3", "gemm_fp64tc"):
        n_k, ms_k, fl_k, _ = prof[k]
        kernels[k]["tflops"] = fl_k / 1e12 / (ms_k * 1e-3) if ms_k else None
    line = {
        "metric": f"DMRG sweep time (s/sweep) at D={D}",
        "value": sweep_s, "unit": "s/sweep", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sweep_s * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else f"{args.precision} split products, f64 sums",
        "data": f"synthetic model ({args.model}), no dataset",
        "config": {"workload": WORKLOAD, "L": L_SITES, "D": D, "schedule": sched,
                   "precision": args.precision, "rayleigh": args.rayleigh,
                   "lanczos": list(LANCZOS), "autotune": bool(args.autotune),
                   "parallelism": f"replicas x{ws}",
                   "cache": "inputs larger than L2", "setup_seconds": setup_s},
        "energy_last_sweep": energies[-1],
        "energies": energies,
        "fp64": fp64,
        "gpu_launches": int(n_launch_ours),
        "profiled_sweep_s": prof_sweep_s,
        "time_split_s": {"lanczos": _stats_sum(timed_stats, "lanczos_seconds"),
                         "svd": _stats_sum(timed_stats, "svd_seconds"),
                         "env": _stats_sum(timed_stats, "env_seconds"),
                         "matvecs": _stats_sum(timed_stats, "matvecs"),
                         "svd_device_span": svd_span["svd"][1] * 1e-3,
                         "svd_decompositions": svd_span["svd_eig"][1] * 1e-3,
                         "svd_gram": svd_span["svd_gram"][1] * 1e-3,
                         "svd_reduction": svd_span["svd_reduce"][1] * 1e-3,
                         "svd_gather": svd_span["svd_gather"][1] * 1e-3,
                         "svd_factors": svd_span["svd_factors"][1] * 1e-3,
                         "svd_completion_qr": svd_span["svd_ortho"][1] * 1e-3,
                         "host_planning": host_plan[1] * 1e-3,
                         "host_plans": host_plan[0],
                         "host_sync_wait": host_sync[1] * 1e-3,
                         "host_syncs": host_sync[0]},
        "centre_problem": dict(solve, **({"delta_e_rel_split": abs(
            solve["tf32x3"]["energy"] - solve["fp64"]["energy"]) / abs(solve["fp64"]["energy"]),
            "delta_e_rel_fp64tc": abs(solve["fp64tc"]["energy"] - solve["fp64"]["energy"]) /
            abs(solve["fp64"]["energy"])} if solve else {})),
        "kernels": kernels,
        "roofline": {"bound": bound, "kernel": top, "achieved": achieved, "peak": peak,
                     "unit": unit, "frac": achieved / peak if peak else None, "traffic": None,
                     "peak_source": note, "launches": n_l, "kernel_ms": t_ms},
        "clocks": clk,
        "e2e": {"value": e2e_s, "unit": "s/sweep", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Batched independent instances
# ---------------------------------------------------------------------------
def batched_instances(n, seed=5):
    """n XXZ open chains, seeded: L uniform in [16, 64] (even, so the Neel
    state has Sz=0), Delta uniform in [0.5, 1.5], D in {64, 128, 256, 512}."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        L = int(rng.integers(8, 33)) * 2
        delta = float(rng.uniform(0.5, 1.5))
        D = int(rng.choice([64, 128, 256, 512]))
        out.append((L, delta, D))
    return out


def run_batched(args):
    """One step = every instance swept 4 times from its Neel product state,
    split form; timed one after another on one stream and concurrently
    (host threads with one stream each).  The metric is instances per
    second of the concurrent run; the serial run and the energy agreement
    between the two are reported beside it."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    from mps2_gb300 import _lib
    from mps2_gb300 import hamiltonians as H
    from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
    from mps2_gb300.vmps import DMRGState, LanczosParams, SweepParams, run_batch
    _lib.check(_lib.load().gq_init(0))
    cases = batched_instances(args.instances)
    built = []
    for L, delta, D in cases:
        sv, mpo, qn0, _ = H.heisenberg_chain(L, 1.0, delta)
        mps = FiniteMPS(sv)
        DirectStateInitMps(mps, H.neel_shuffled_labels(L, L), qn0)
        built.append((mps.tens, mpo))
    params = [SweepParams(4, D, D, 0.0, LanczosParams(1e-9, 100), precision=args.precision,
                          rayleigh=args.rayleigh) for _, _, D in cases]

    def serial():
        es = []
        for (tens, mpo), p in zip(built, params):
            st = DMRGState(tens, mpo)
            st.init_envs(p.precision)
            es.append(st.sweep(p)[0])
        return es

    def concurrent():
        states = [DMRGState(tens, mpo) for tens, mpo in built]
        return run_batch(states, params, init_envs=True, nthreads=args.threads)

    for _ in range(args.warmup):
        concurrent()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e_conc = concurrent()
    torch.cuda.synchronize()
    t_conc = (time.perf_counter() - t0) / args.steps
    t0 = time.perf_counter()
    e_ser = serial()
    torch.cuda.synchronize()
    t_ser = time.perf_counter() - t0
    dev = max(abs(a - b) / abs(b) for a, b in zip(e_conc, e_ser))
    line = {
        "metric": "batched XXZ instances, 4 sweeps each (instances/s)",
        "value": len(cases) / t_conc, "unit": "instances/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_conc * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else args.precision,
        "data": "synthetic models (seeded XXZ chains), no dataset",
        "config": {"workload": f"xxz_batch_{len(cases)}", "instances": len(cases),
                   "threads": args.threads, "precision": args.precision,
                   "L_range": [min(c[0] for c in cases), max(c[0] for c in cases)],
                   "D_set": sorted(set(c[2] for c in cases)), "sweeps": 4},
        "serial_seconds": t_ser, "concurrent_seconds": t_conc,
        "speedup_over_serial": t_ser / t_conc,
        "max_rel_energy_diff_concurrent_vs_serial": dev,
    }
    print(json.dumps(line))


def main():
    args = _args()
    _select_model(args)
    if args.workload == "batched":
        # one hardware queue per concurrent stream (must precede CUDA init)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
        run_batched(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
