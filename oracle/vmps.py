"""FP64 CPU oracle: two-site finite variational MPS (DMRG) sweep.
TEST INFRASTRUCTURE ONLY (see ``oracle/bstensor.py``).

Restates ``include/gqmps2/algorithm/vmps/two_site_update_finite_vmps_impl.h``
of gqmps2 step by step: ``TwoSiteFiniteVMPS`` (77-101), ``InitEnvs``
(104-135), ``TwoSiteFiniteVMPSSweep`` (143-161), ``TwoSiteFiniteVMPSUpdate``
(164-340) and ``MeasureEE`` (43-52).  The per-update disk staging of
``LoadRelatedTens``/``DumpRelatedTens`` (343-494) is replaced by keeping the
environments in a dict keyed like the reference's env files
(``("l"|"r", length)``); which environment is used where is unchanged.
"""
from __future__ import annotations

import math
import time
from typing import Dict, List

import numpy as np

from .bstensor import BSTensor, contract, dag, svd
from .lanczos import LanczosParams, lanczos_solver


class SweepParams:
    """``SweepParams`` of ``two_site_update_finite_vmps.h:27-55``."""

    def __init__(self, sweeps, dmin, dmax, trunc_err, lancz_params=None):
        self.sweeps = int(sweeps)
        self.Dmin = int(dmin)
        self.Dmax = int(dmax)
        self.trunc_err = float(trunc_err)
        self.lancz_params = lancz_params or LanczosParams()


def measure_ee(svals) -> float:
    """``MeasureEE`` (43-52): sum of -p ln p with p = s^2 over kept values
    (values that are exactly zero contribute nothing)."""
    ee = 0.0
    for s in svals:
        p = float(s) ** 2
        if p > 0.0:
            ee += -p * math.log(p)
    return ee


class UpdateStats:
    __slots__ = ("site", "dir", "e0", "trunc_err", "D", "iters", "ee", "seconds")

    def __init__(self, **kw):
        for k, v in kw.items():
            setattr(self, k, v)

    def line(self) -> str:
        """The per-update log line of ``:329-338``."""
        return (f"Site {self.site:4d} E0 = {self.e0:20.16f} TruncErr = "
                f"{self.trunc_err:.2e} D = {self.D:5d} Iter = {self.iters:3d} "
                f"S = {self.ee:10.7f}")


def init_envs(mps: List[BSTensor], mpo: List[BSTensor], envs: Dict) -> None:
    """``InitEnvs`` (104-135): right environments R_1 .. R_{N-2}."""
    N = len(mps)
    renv = None
    for i in range(1, N - 1):
        A = mps[N - i]
        if i == 1:
            temp = contract(A, mpo[N - 1], [1], [0])
            renv = contract(temp, dag(A), [2], [1])
        else:
            t1 = contract(A, renv, [2], [0])
            t2 = contract(t1, mpo[N - i], [1, 2], [1, 3])
            renv = contract(t2, dag(A), [3, 1], [1, 2])
        envs[("r", i)] = renv


def _classify(N, dir, target):
    if dir == "r":
        ls, rs = target, target + 1
        lenv_len, renv_len = target, N - (target + 2)
        if target == 0:
            where, ldims, init_axes = "lend", 1, ([1], [0])
        elif target == N - 2:
            where, ldims, init_axes = "rend", 2, ([2], [0])
        else:
            where, ldims, init_axes = "cent", 2, ([2], [0])
        us_axes = None
    else:
        ls, rs = target - 1, target
        lenv_len, renv_len = target - 1, N - target - 1
        if target == N - 1:
            where, ldims, init_axes, us_axes = "rend", 2, ([2], [0]), ([2], [0])
        elif target == 1:
            where, ldims, init_axes, us_axes = "lend", 1, ([1], [0]), ([1], [0])
        else:
            where, ldims, init_axes, us_axes = "cent", 2, ([2], [0]), ([2], [0])
    return ls, rs, lenv_len, renv_len, where, ldims, init_axes, us_axes


def two_site_update(mps, mpo, envs, params: SweepParams, dir: str, target: int,
                    matvec_hook=None) -> UpdateStats:
    """``TwoSiteFiniteVMPSUpdate`` (164-340)."""
    t0 = time.perf_counter()
    N = len(mps)
    ls, rs, lenv_len, renv_len, where, ldims, init_axes, us_axes = _classify(N, dir, target)
    L = envs.get(("l", lenv_len)) if where != "lend" else None
    R = envs.get(("r", renv_len)) if where != "rend" else None
    eff_ham = [L, mpo[ls], mpo[rs], R]
    init = contract(mps[ls], mps[rs], *init_axes)
    res = lanczos_solver(eff_ham, init, params.lancz_params, where, matvec_hook)
    sv = svd(res.gs_vec, ldims, mps[ls].div, params.trunc_err, params.Dmin, params.Dmax)
    ee = measure_ee(sv.svals)
    if dir == "r":
        mps[ls] = sv.u
        mps[rs] = contract(sv.s, sv.vt, [1], [0])
    else:
        mps[ls] = contract(sv.u, sv.s, *us_axes)
        mps[rs] = sv.vt
    if dir == "r":
        if target != N - 2:
            A = mps[target]
            if target == 0:
                temp = contract(A, mpo[target], [0], [0])
                envs[("l", lenv_len + 1)] = contract(temp, dag(A), [2], [0])
            else:
                t1 = contract(envs[("l", lenv_len)], A, [0], [0])
                t2 = contract(t1, mpo[target], [0, 2], [0, 1])
                envs[("l", lenv_len + 1)] = contract(t2, dag(A), [0, 2], [0, 1])
    else:
        if target != 1:
            A = mps[target]
            if target == N - 1:
                temp = contract(A, mpo[target], [1], [0])
                envs[("r", renv_len + 1)] = contract(temp, dag(A), [2], [1])
            else:
                t1 = contract(A, eff_ham[3], [2], [0])
                t2 = contract(t1, mpo[target], [1, 2], [1, 3])
                envs[("r", renv_len + 1)] = contract(t2, dag(A), [3, 1], [1, 2])
    return UpdateStats(site=target, dir=dir, e0=res.gs_eng, trunc_err=sv.trunc_err,
                       D=sv.D, iters=res.iters, ee=ee,
                       seconds=time.perf_counter() - t0)


def two_site_sweep(mps, mpo, envs, params, stats=None, matvec_hook=None) -> float:
    """``TwoSiteFiniteVMPSSweep`` (143-161)."""
    N = len(mps)
    e0 = None
    for i in range(0, N - 1):
        st = two_site_update(mps, mpo, envs, params, "r", i, matvec_hook)
        e0 = st.e0
        if stats is not None:
            stats.append(st)
    for i in range(N - 1, 0, -1):
        st = two_site_update(mps, mpo, envs, params, "l", i, matvec_hook)
        e0 = st.e0
        if stats is not None:
            stats.append(st)
    return e0


def two_site_finite_vmps(mps, mpo, params: SweepParams, envs=None, stats=None,
                         sweep_energies=None, verbose=False) -> float:
    """``TwoSiteFiniteVMPS`` (77-101).  ``envs`` plays the role of the
    temp directory: pass ``None`` (or an empty dict) to build the right
    environments first, or the dict from a previous call to resume."""
    assert len(mps) == len(mpo)
    if envs is None:
        envs = {}
    if not envs:
        init_envs(mps, mpo, envs)
    e0 = None
    for sweep in range(1, params.sweeps + 1):
        st = [] if stats is None else stats
        e0 = two_site_sweep(mps, mpo, envs, params, st)
        if verbose:
            print(f"sweep {sweep}")
            for s in st[-2 * (len(mps) - 1):]:
                print(s.line())
        if sweep_energies is not None:
            sweep_energies.append(e0)
    return e0
