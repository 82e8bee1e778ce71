#!/usr/bin/env python
"""Benchmark: two-site finite DMRG sweep on one GB300.

Workload (the configuration the headline metric is quoted on): spin-1/2
Heisenberg open chain, L=100, J=1, U(1) Sz, total Sz=0, Neel product state
with a seed-0 shuffled site order; the bond dimension grows
500 -> 800 -> 1100 -> 1400 -> 1700 -> 2000 (one sweep each), Lanczos tolerance
1e-10.  The growth sweeps up to 1700 prepare the state (untimed); then
``--warmup`` sweeps and ``--steps`` timed sweeps run at D=2000.

* ``value``: seconds per sweep at D=2000, device-resident state, CUDA events
  on the library's stream around the timed sweeps (lower is better).  The
  state (several GB) is far larger than L2, so no flush is needed.
* ``e2e``: the same sweep through the C ABI from host buffers: upload of the
  MPS, MPO and right environments, the sweep, download of the MPS and right
  environments -- the drop-in call's work.
* ``roofline``, ``kernels``, ``gpu_launches``: from one more sweep at D=2000
  run under the library's kernel profiler (CUDA events around every kernel
  family on the library stream; the Lanczos matvec then runs launch by
  launch instead of as a replayed CUDA graph): the kernel family with the
  most device time, its algorithmic flops (2*m*n*k over the QN-allowed
  block products) or bytes / its event time, against the measured peak.
* ``cpu_baseline``: the FP64 CPU restatement (numpy + the host BLAS) on one
  central two-site update of the same state, scaled to a sweep by the GPU's
  own ratio of sweep time to that update's time.
* ``--impl reference``: the same CPU restatement on the same kind of central
  update (block structure recorded from a GPU run), the reference's own
  gqten+MKL path being unbuildable here.

Other workloads (not the headline line): ``--model hubbard`` (L=64 Fermi-
Hubbard chain, t=1, U=8, half filling, D 1000 -> 4000 over 8 sweeps) and
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

SCHEDULE = [500, 800, 1100, 1400, 1700, 2000]
L_SITES = 100
LANCZOS = (1e-10, 100)
WORKLOAD = "heisenberg_obc_L100_Sz0_D500to2000"
FAMILIES = ("gemm_fp64", "gemm_tf32x3", "gemm_fp64tc", "permute", "vector", "skinny")
STRUCTURE_FIXTURE = os.path.join(ROOT, "tests", "golden", "bench_center_bond.json")


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", choices=["fp64", "tf32x3", "fp64tc"], default="tf32x3")
    p.add_argument("--rayleigh", choices=["fp64", "fp64tc"], default="fp64tc",
                   help="arithmetic of the split form's Rayleigh-quotient energies")
    p.add_argument("--model", choices=["heisenberg", "hubbard", "j1j2"], default="heisenberg",
                   help="heisenberg: L=100 chain, D 500->2000 (headline); hubbard: L=64 "
                        "chain, U=8, half filling, D 1000->4000; j1j2: 4x16 open cylinder "
                        "(snake order), J1=1, J2=0.5, D 2000->6000")
    p.add_argument("--schedule", default=None,
                   help="comma-separated D per growth sweep; the last is the timed D")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--record-structure", action="store_true",
                   help="write the central-bond block structure fixture")
    p.add_argument("--workload", choices=["sweep", "batched"], default="sweep",
                   help="sweep: the D=2000 chain (headline); batched: 64 independent XXZ "
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


HUBBARD = {"L": 64, "schedule": [1000, 1430, 1860, 2290, 2710, 3140, 3570, 4000],
           "workload": "hubbard_obc_L64_U8_half_filling_D1000to4000"}
J1J2 = {"L": 64, "Lx": 16, "Ly": 4, "J1": 1.0, "J2": 0.5,
        "schedule": [2000, 2570, 3140, 3710, 4290, 4860, 5430, 6000],
        "workload": "j1j2_cylinder_4x16_snake_J2_0.5_D2000to6000"}


def _select_model(args):
    """Module constants for the chosen model (heisenberg: the headline chain;
    hubbard: L=64, t=1, U=8, half filling, Sz=0, U(1)xU(1), Jordan-Wigner
    MPO of bond dimension 6, alternating up/down product state; j1j2: the
    4x16 open cylinder in snake order, J1=1, J2=0.5, Sz=0, shuffled Neel
    product state, MPO from the generator's compression, bond dimension <= 17)."""
    global L_SITES, WORKLOAD, SCHEDULE
    if args.model == "hubbard":
        L_SITES, WORKLOAD, SCHEDULE = HUBBARD["L"], HUBBARD["workload"], HUBBARD["schedule"]
    elif args.model == "j1j2":
        L_SITES, WORKLOAD, SCHEDULE = J1J2["L"], J1J2["workload"], J1J2["schedule"]
    if args.schedule is None:
        args.schedule = ",".join(map(str, SCHEDULE))


def _model(model="heisenberg"):
    from mps2_gb300 import hamiltonians as H
    from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
    if model == "hubbard":
        sv, mpo, qn0, gen = H.hubbard_chain(L_SITES, 1.0, 8.0)
        labels = [1 if i % 2 == 0 else 2 for i in range(L_SITES)]
    elif model == "j1j2":
        pairs = H.j1j2_cylinder_pairs(J1J2["Lx"], J1J2["Ly"], J1J2["J1"], J1J2["J2"])
        sv, mpo, qn0, gen = H.heisenberg_pairs(L_SITES, pairs)
        labels = H.neel_shuffled_labels(L_SITES, 0)
    else:
        sv, mpo, qn0, gen = H.heisenberg_chain(L_SITES)
        labels = H.neel_shuffled_labels(L_SITES, 0)
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, labels, qn0)
    return mps, mpo


def _tensor_bytes(t):
    return 8 * t.size()


# ---------------------------------------------------------------------------
# CPU restatement timing (oracle) -- test infrastructure used as the baseline
# ---------------------------------------------------------------------------
def _oracle_center_update(mpsd, mpo, envs, c, D, iters_cap=None):
    """Time one 'r' two-site update at site c with the FP64 CPU restatement.
    mpsd: {site: tensor}, envs: {('l'|'r', len): tensor} (product tensors)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
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


def _synthetic_center_state(fix, seed=0):
    """Random tensors with the recorded central-bond block structure."""
    import numpy as np
    from mps2_gb300.hamiltonians import heisenberg_chain
    from mps2_gb300.tensor import GQTensor, Index
    rng = np.random.default_rng(seed)
    N = fix["L"]
    c = fix["center"]
    sv, mpo, qn0, _ = heisenberg_chain(N)

    def idx(d):
        return Index([(tuple(q), n) for q, n in d["sectors"]], d["dir"])

    def rand(indices, div):
        t = GQTensor(indices, div)
        for cc in t.allowed_coords(div):
            t.blocks[cc] = rng.standard_normal(t.block_shape(cc))
        return t

    A = rand([idx(d) for d in fix["A_c"]], (0,))
    B = rand([idx(d) for d in fix["A_c1"]], (0,))
    Le = rand([idx(d) for d in fix["L"+"_env"]], (0,))
    Re = rand([idx(d) for d in fix["R_env"]], (0,))
    return {c: A, c + 1: B}, mpo, {("l", c): Le, ("r", N - c - 2): Re}


def _describe_index(ix):
    return {"dir": ix.dir, "sectors": [[list(q), d] for q, d in ix.sectors()]}


# ---------------------------------------------------------------------------
def run_reference(args):
    """CPU restatement on a central update with the recorded structure."""
    ws, rank = _dist()
    if rank != 0:
        return
    if args.model != "heisenberg":
        print(json.dumps({"impl": "reference",
                          "unavailable": "the recorded central-bond structure is the "
                                         "Heisenberg chain's only"}))
        return
    if not os.path.exists(STRUCTURE_FIXTURE):
        print(json.dumps({"impl": "reference",
                          "unavailable": "central-bond structure fixture missing"}))
        return
    with open(STRUCTURE_FIXTURE) as f:
        fix = json.load(f)
    D = fix["D"]
    c = fix["center"]
    mpsd, mpo, envs = _synthetic_center_state(fix)
    times = []
    for _ in range(args.warmup):
        _oracle_center_update(dict(mpsd), mpo, dict(envs), c, D, fix["center_iters"])
    for _ in range(max(1, args.steps)):
        t, st = _oracle_center_update(dict(mpsd), mpo, dict(envs), c, D, fix["center_iters"])
        times.append(t)
    per_update = sum(times) / len(times)
    sweep_s = per_update * fix["sweep_over_center"]
    cores = os.cpu_count()
    line = {
        "metric": f"DMRG sweep time (s/sweep) at D={D}",
        "value": sweep_s, "unit": "s/sweep", "impl": "reference", "n_gpus": args.gpus,
        "steps": len(times), "warmup": args.warmup, "ms_per_step": per_update * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (random tensors with the central-bond block structure recorded "
                "from a GPU run of this workload)",
        "config": {"workload": WORKLOAD, "D": D, "L": fix["L"],
                   "cache": "inputs larger than L2"},
        "cpu_baseline": {"value": sweep_s, "unit": "s/sweep", "cores": cores, "kind": "port",
                         "sample": f"{len(times)} central two-site update(s) at site {c}, "
                                   f"D={D}, Lanczos capped at {fix['center_iters']} iterations, "
                                   f"x{fix['sweep_over_center']:.1f} (GPU sweep/update time ratio)"},
        "e2e": {"value": sweep_s, "unit": "s/sweep", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


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
    sched = [int(x) for x in args.schedule.split(",")]
    D = sched[-1]
    lp = LanczosParams(*LANCZOS)

    def params(d, prec=args.precision):
        return SweepParams(1, d, d, 0.0, lp, precision=prec, rayleigh=args.rayleigh)

    mps, mpo = _model(args.model)
    st = DMRGState(mps.tens, mpo)
    t_setup = time.perf_counter()
    st.init_envs(args.precision)
    for d in sched[:-1]:
        e0, stats = st.sweep(params(d))
        print(f"[setup] sweep at D={d}: E0={e0:.12f} max bond {max(x.D for x in stats)} "
              f"({sum(x.update_seconds for x in stats):.1f}s)", file=sys.stderr)
    for w in range(args.warmup):
        e0, stats = st.sweep(params(D))
        print(f"[warmup {w}] D={D} E0={e0:.12f} {sum(x.update_seconds for x in stats):.1f}s",
              file=sys.stderr)
    setup_s = time.perf_counter() - t_setup

    # ---- timed sweeps -------------------------------------------------------
    ext = torch.cuda.ExternalStream(library_stream())
    clocks = ClockSampler(local)
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    # an external profiler started with --profile-from-start off records the
    # timed sweeps only
    torch.cuda.profiler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(ext)
    timed_stats, energies = [], []
    for k in range(args.steps):
        e0, stats = st.sweep(params(D))
        timed_stats.extend(stats)
        energies.append(e0)
    ev1.record(ext)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    sweep_s = ms * 1e-3 / args.steps

    # ---- one more sweep under the kernel profiler (CUDA events around every
    # kernel family; the Lanczos matvec then runs without graph replay): the
    # kernel shares, launch count and roofline come from it -------------------
    profile_enable(True)
    ev0.record(ext)
    st.sweep(params(D))
    ev1.record(ext)
    torch.cuda.synchronize()
    prof_sweep_s = ev0.elapsed_time(ev1) * 1e-3
    prof = {k: profile_read(k) for k in FAMILIES}
    svd_span = {k: profile_read(k) for k in ("svd", "svd_eig", "svd_gather", "svd_factors",
                                              "svd_ortho")}
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
    del st2, out_mps, out_env

    # ---- the central two-site problem: FP64 vs split, CPU restatement ------
    c = L_SITES // 2 - 1
    for i in range(0, c):
        st.update(params(D), "r", i)
    mpsd = {c: st.get_mps(c), c + 1: st.get_mps(c + 1)}
    envs = {("l", c): st.get_env("l", c), ("r", L_SITES - c - 2): st.get_env("r", L_SITES - c - 2)}
    theta = Contract(mpsd[c], mpsd[c + 1], ([2], [0]))
    eff = [envs[("l", c)], mpo[c], mpo[c + 1], envs[("r", L_SITES - c - 2)]]
    solve = {}
    for prec in ("fp64", "tf32x3", "fp64tc"):
        profile_enable(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = LanczosSolver(eff, theta, lp, "cent", precision=prec, rayleigh=args.rayleigh)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        pr = {k: profile_read(k) for k in FAMILIES}
        profile_enable(False)
        gemm_ms = sum(pr[k][1] for k in ("gemm_fp64", "gemm_tf32x3", "gemm_fp64tc", "skinny"))
        gemm_fl = sum(pr[k][2] for k in ("gemm_fp64", "gemm_tf32x3", "gemm_fp64tc", "skinny"))
        solve[prec] = {"energy": r.gs_eng, "iters": r.iters, "seconds": dt,
                       "kernel_ms": {k: pr[k][1] for k in FAMILIES},
                       "matvec_gemm_tflops": gemm_fl / (gemm_ms * 1e-3) / 1e12 if gemm_ms else None,
                       "tc_gemm_tflops": (pr["gemm_tf32x3"][2] / (pr["gemm_tf32x3"][1] * 1e-3) / 1e12
                                          if pr["gemm_tf32x3"][1] else None)}
    de = abs(solve["tf32x3"]["energy"] - solve["fp64"]["energy"]) / abs(solve["fp64"]["energy"])
    gpu_center = st.update(params(D), "r", c)
    if args.record_structure and rank == 0:
        center_struct = {
            "L": L_SITES, "center": c, "D": D, "center_iters": int(max(1, gpu_center.iters)),
            "sweep_over_center": sweep_s / gpu_center.update_seconds,
            "A_c": [_describe_index(ix) for ix in mpsd[c].indices],
            "A_c1": [_describe_index(ix) for ix in mpsd[c + 1].indices],
            "L_env": [_describe_index(ix) for ix in envs[("l", c)].indices],
            "R_env": [_describe_index(ix) for ix in envs[("r", L_SITES - c - 2)].indices],
        }
        os.makedirs(os.path.dirname(STRUCTURE_FIXTURE), exist_ok=True)
        with open(STRUCTURE_FIXTURE, "w") as f:
            json.dump(center_struct, f)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        t_cpu, ost = _oracle_center_update(mpsd, mpo, envs, c, D)
        cpu = {"value": sweep_s * t_cpu / gpu_center.update_seconds, "unit": "s/sweep",
               "cores": os.cpu_count(), "kind": "port",
               "sample": (f"1 central two-site update (site {c}, D={D}) of the same state: CPU "
                          f"{t_cpu:.2f}s vs GPU {gpu_center.update_seconds:.3f}s, scaled by the "
                          f"GPU sweep time; CPU E0={ost.e0:.12f} GPU E0={gpu_center.e0:.12f}")}

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
    tot = {k: sum(getattr(s, k) for s in timed_stats) for k in
           ("lanczos_seconds", "svd_seconds", "env_seconds", "update_seconds", "matvec_flops",
            "env_flops", "matvecs")}
    u64 = gpu_center.update_seconds - gpu_center.lanczos_seconds + solve["fp64"]["seconds"]
    line = {
        "metric": f"DMRG sweep time (s/sweep) at D={D}",
        "value": sweep_s, "unit": "s/sweep", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sweep_s * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "tf32x3 split products, f64 sums",
        "data": "synthetic model (Heisenberg chain), no dataset",
        "config": {"workload": WORKLOAD, "L": L_SITES, "D": D, "schedule": sched,
                   "precision": args.precision, "lanczos": list(LANCZOS),
                   "parallelism": f"replicas x{ws}", "cache": "inputs larger than L2",
                   "setup_seconds": setup_s},
        "energy_last_sweep": energies[-1],
        "gpu_launches": int(n_launch_ours),
        "profiled_sweep_s": prof_sweep_s,
        "time_split_s": {"lanczos": tot["lanczos_seconds"], "svd": tot["svd_seconds"],
                         "env": tot["env_seconds"], "matvecs": tot["matvecs"],
                         "svd_device_span": svd_span["svd"][1] * 1e-3,
                         "svd_decompositions": svd_span["svd_eig"][1] * 1e-3,
                         "svd_gather": svd_span["svd_gather"][1] * 1e-3,
                         "svd_factors": svd_span["svd_factors"][1] * 1e-3,
                         "svd_ortho": svd_span["svd_ortho"][1] * 1e-3,
                         "svd_ortho_calls": svd_span["svd_ortho"][0]},
        "central_problem": {"fp64": solve["fp64"], "tf32x3": solve["tf32x3"],
                            "fp64tc": solve["fp64tc"],
                            "delta_e_rel": de,
                            "delta_e_rel_fp64tc": abs(solve["fp64tc"]["energy"] -
                                                      solve["fp64"]["energy"]) /
                            abs(solve["fp64"]["energy"]),
                            "fp64_sweep_s_est": sweep_s * u64 / gpu_center.update_seconds},
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
