"""gqmps2's two-site DMRG entry points over the GPU library.

Mirrors the reference interface
(``include/gqmps2/algorithm/vmps/two_site_update_finite_vmps.h`` and
``include/gqmps2/algorithm/lanczos_solver.h``):

* ``SweepParams(sweeps, Dmin, Dmax, trunc_err, lancz_params, mps_path="mps",
  temp_path=".temp")`` plus the keywords ``precision`` ("fp64" | "tf32x3" |
  "fp64tc") and ``rayleigh`` ("fp64" | "fp64tc": arithmetic of the split
  form's Rayleigh-quotient energy);
* ``LanczosParams(error=1e-7, max_iterations=200)``;
* ``TwoSiteFiniteVMPS(mps, mpo, sweep_params) -> e0`` with the reference's
  file contract: the MPS is read from ``mps_path`` (``mps.Dump(path, True)``
  beforehand) and written back there; the right environments live in
  ``temp_path``; if ``temp_path`` exists the call resumes from it instead of
  building the environments (``two_site_update_finite_vmps_impl.h:86-89``);
  the ``FiniteMPS`` container is empty before and after;
* ``LanczosSolver(eff_ham, init_state, params, where) -> LanczosRes``.

Everything numeric runs in ``libgqmps2_gb300.so``; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import DeviceTensor, check, load
from .finite_mps import (FiniteMPS, GenEnvTenName, GenMPSTenName, kMpsPath, kRuntimeTempPath,
                         kUncentralizedCenterIdx,
                         read_tensor, write_tensor)
from .tensor import GQTensor, QN, Div

_PREC = {"fp64": _lib.PREC_FP64, "tf32x3": _lib.PREC_TF32X3, "fp64tc": _lib.PREC_FP64TC}


class LanczosParams:
    def __init__(self, error: float = 1.0e-7, max_iterations: int = 200):
        self.error = float(error)
        self.max_iterations = int(max_iterations)


class SweepParams:
    def __init__(self, sweeps, dmin, dmax, trunc_err, lancz_params=None,
                 mps_path: str = kMpsPath, temp_path: str = kRuntimeTempPath,
                 precision: str = "fp64", verbose: bool = False, rayleigh: str = "fp64"):
        self.sweeps = int(sweeps)
        self.Dmin = int(dmin)
        self.Dmax = int(dmax)
        self.trunc_err = float(trunc_err)
        self.lancz_params = lancz_params or LanczosParams()
        self.mps_path = mps_path
        self.temp_path = temp_path
        if precision not in _PREC:
            raise ValueError("precision must be 'fp64', 'tf32x3' or 'fp64tc'")
        if rayleigh not in ("fp64", "fp64tc"):
            raise ValueError("rayleigh must be 'fp64' or 'fp64tc'")
        self.precision = precision
        self.verbose = bool(verbose)
        self.rayleigh = rayleigh

    def to_c(self, sweeps: Optional[int] = None) -> _lib.SweepParamsC:
        return _lib.SweepParamsC(
            self.sweeps if sweeps is None else sweeps, self.Dmin, self.Dmax, self.trunc_err,
            _lib.LanczosParamsC(self.lancz_params.error, self.lancz_params.max_iterations,
                                _PREC[self.rayleigh]),
            _PREC[self.precision], 1 if self.verbose else 0)


class UpdateStats:
    __slots__ = tuple(f for f, _ in _lib.UpdateStatsC._fields_)

    def __init__(self, c: _lib.UpdateStatsC):
        for f in self.__slots__:
            setattr(self, f, getattr(c, f))
        self.dir = chr(self.dir)

    def line(self) -> str:
        """The reference's per-update log line (``:329-338``)."""
        return (f"Site {self.site:4d} E0 = {self.e0:20.16f} TruncErr = {self.trunc_err:.2e} "
                f"D = {self.D:5d} Iter = {self.iters:3d} LanczT = {self.lanczos_seconds:8.2f} "
                f"TotT = {self.update_seconds:8.2f} S = {self.ee:10.7f}")


def run_batch(states: Sequence["DMRGState"], params: Sequence[SweepParams],
              init_envs: bool = True, nthreads: int = 8) -> List[float]:
    """Sweep independent DMRG states concurrently (``gq_dmrg_run_batch``):
    host threads with one CUDA stream each take the states in order; each
    state builds its right environments (if ``init_envs``) and runs its own
    ``params[i].sweeps`` sweeps.  Returns each state's last energy."""
    n = len(states)
    if len(params) != n:
        raise ValueError("one SweepParams per state")
    hs = (C.c_void_p * max(n, 1))(*[s.h.value for s in states])
    ps = (_lib.SweepParamsC * max(n, 1))(*[p.to_c() for p in params])
    e0 = np.zeros(max(n, 1))
    check(load().gq_dmrg_run_batch(hs, n, ps, 1 if init_envs else 0, int(nthreads),
                                   e0.ctypes.data_as(_lib._DP)))
    return [float(x) for x in e0[:n]]


class DMRGState:
    """Device-resident MPS + MPO + environments (one ``gq_dmrg`` handle)."""

    def __init__(self, mps_tensors: Sequence[GQTensor], mpo: Sequence[GQTensor]):
        lib = load()
        n = len(mps_tensors)
        if n != len(mpo):
            raise ValueError("MPS and MPO lengths differ")
        self.N = n
        dm = [DeviceTensor.from_host(t) for t in mps_tensors]
        do = [DeviceTensor.from_host(t) for t in mpo]
        arr_m = (C.c_void_p * n)(*[t.h.value for t in dm])
        arr_o = (C.c_void_p * n)(*[t.h.value for t in do])
        h = C.c_void_p()
        check(lib.gq_dmrg_create(n, arr_m, arr_o, C.byref(h)))
        self.h = h

    def __del__(self):
        try:
            if self.h and self.h.value and _lib._lib is not None:
                _lib._lib.gq_dmrg_destroy(self.h)
        except Exception:
            pass
        self.h = None

    def init_envs(self, precision: str = "fp64"):
        check(load().gq_dmrg_init_envs(self.h, _PREC[precision]))

    def set_env(self, dir: str, length: int, t: GQTensor):
        d = DeviceTensor.from_host(t)
        check(load().gq_dmrg_set_env(self.h, ord(dir), int(length), d.h))

    def get_env(self, dir: str, length: int) -> GQTensor:
        out = C.c_void_p()
        check(load().gq_dmrg_get_env(self.h, ord(dir), int(length), C.byref(out)))
        return DeviceTensor(out.value).to_host()

    def sweep(self, params: SweepParams, sweeps: Optional[int] = None):
        ns = params.sweeps if sweeps is None else sweeps
        stats = (_lib.UpdateStatsC * max(1, 2 * (self.N - 1) * ns))()
        e0 = C.c_double()
        pc = params.to_c(ns)
        check(load().gq_dmrg_sweep(self.h, C.byref(pc), stats, C.byref(e0)))
        return e0.value, [UpdateStats(stats[i]) for i in range(2 * (self.N - 1) * ns)]

    def update(self, params: SweepParams, dir: str, target: int) -> UpdateStats:
        st = _lib.UpdateStatsC()
        pc = params.to_c(1)
        check(load().gq_dmrg_update(self.h, C.byref(pc), ord(dir), int(target), C.byref(st)))
        return UpdateStats(st)

    def get_mps(self, i: int) -> GQTensor:
        out = C.c_void_p()
        check(load().gq_dmrg_get_mps(self.h, int(i), C.byref(out)))
        return DeviceTensor(out.value).to_host()


def TwoSiteFiniteVMPS(mps: FiniteMPS, mpo: Sequence[GQTensor], sweep_params: SweepParams,
                      stats_out: Optional[list] = None) -> float:
    """``TwoSiteFiniteVMPS`` (``two_site_update_finite_vmps_impl.h:77-101``)."""
    N = mps.size()
    if N != len(mpo):
        raise ValueError("mps.size() != mpo.size()")
    sp = sweep_params
    tens = [read_tensor(GenMPSTenName(sp.mps_path, i)) for i in range(N)]
    st = DMRGState(tens, mpo)
    if not os.path.isdir(sp.temp_path):
        os.makedirs(sp.temp_path, exist_ok=True)
        st.init_envs(sp.precision)
    else:
        for length in range(1, N - 1):
            f = GenEnvTenName("r", length, sp.temp_path)
            if not os.path.exists(f):
                raise FileNotFoundError(f"cannot resume: {f} is missing")
            st.set_env("r", length, read_tensor(f))
    e0 = float("nan")
    for sweep in range(1, sp.sweeps + 1):
        if sp.verbose:
            print(f"sweep {sweep}")
        e0, stats = st.sweep(sp, sweeps=1)
        if stats_out is not None:
            stats_out.extend(stats)
    for i in range(N):
        write_tensor(st.get_mps(i), GenMPSTenName(sp.mps_path, i))
    for length in range(1, N - 1):
        write_tensor(st.get_env("r", length), GenEnvTenName("r", length, sp.temp_path))
    mps.clear()
    return e0


def autotune_enable(on: bool = True) -> None:
    """Tile-choice autotuner keyed on each contraction's block-size histogram
    (``gq_autotune_enable``); off by default."""
    check(load().gq_autotune_enable(1 if on else 0))


def profile_enable(on: bool = True) -> None:
    check(load().gq_profile_enable(1 if on else 0))


def profile_read(kernel: str):
    """(launches, total ms, flops, bytes) of one kernel family since the
    last :func:`profile_enable`."""
    n, ms, fl, by = C.c_int64(), C.c_double(), C.c_double(), C.c_double()
    check(load().gq_profile_read(_lib.PROF[kernel], C.byref(n), C.byref(ms), C.byref(fl),
                                 C.byref(by)))
    return n.value, ms.value, fl.value, by.value


def host_sync_count() -> int:
    """Host waits on the library's streams since it was loaded."""
    n = C.c_int64()
    check(load().gq_host_sync_count(C.byref(n)))
    return n.value


def library_stream() -> int:
    s = C.c_void_p()
    check(load().gq_get_stream(C.byref(s)))
    return s.value or 0


class LanczosRes:
    def __init__(self, iters, gs_eng, gs_vec):
        self.iters = iters
        self.gs_eng = gs_eng
        self.gs_vec = gs_vec


def _dev(t: Optional[GQTensor]):
    return None if t is None else DeviceTensor.from_host(t)


def LanczosSolver(eff_ham: Sequence[Optional[GQTensor]], init_state: GQTensor,
                  params: LanczosParams, where: str, precision: str = "fp64",
                  rayleigh: str = "fp64") -> LanczosRes:
    """``LanczosSolver`` (``lanczos_solver_impl.h:79-226``); ``eff_ham`` is
    ``[L, W_l, W_r, R]`` with ``L``/``R`` ``None`` at the chain ends.
    ``rayleigh`` ("fp64" | "fp64tc"): arithmetic of the split form's
    Rayleigh-quotient energy."""
    lib = load()
    L, Wl, Wr, R = [_dev(t) for t in eff_ham]
    x = DeviceTensor.from_host(init_state)
    it, e = C.c_int64(), C.c_double()
    out = C.c_void_p()
    lp = _lib.LanczosParamsC(params.error, params.max_iterations, _PREC[rayleigh])
    check(lib.gq_lanczos(L.h if L else None, Wl.h, Wr.h, R.h if R else None, _lib.WHERE[where],
                         x.h, C.byref(lp), _PREC[precision], C.byref(it), C.byref(e),
                         C.byref(out)))
    return LanczosRes(it.value, e.value, DeviceTensor(out.value).to_host())


def eff_ham_mul_state(eff_ham, state: GQTensor, where: str, precision: str = "fp64"):
    lib = load()
    L, Wl, Wr, R = [_dev(t) for t in eff_ham]
    x = DeviceTensor.from_host(state)
    out = C.c_void_p()
    fl = C.c_double()
    check(lib.gq_eff_ham_mul_state(L.h if L else None, Wl.h, Wr.h, R.h if R else None,
                                   _lib.WHERE[where], x.h, _PREC[precision], C.byref(out),
                                   C.byref(fl)))
    return DeviceTensor(out.value).to_host(), fl.value


def Contract(a: GQTensor, b: GQTensor, axes, precision: str = "fp64") -> GQTensor:
    lib = load()
    da, db = DeviceTensor.from_host(a), DeviceTensor.from_host(b)
    xa = np.ascontiguousarray(axes[0], dtype=np.int32)
    xb = np.ascontiguousarray(axes[1], dtype=np.int32)
    out = C.c_void_p()
    fl = C.c_double()
    check(lib.gq_contract(da.h, db.h, len(xa), xa.ctypes.data_as(_lib._IP),
                          xb.ctypes.data_as(_lib._IP), _PREC[precision], C.byref(out),
                          C.byref(fl)))
    return DeviceTensor(out.value).to_host()


def SVD(t: GQTensor, ldims: int, ldiv, trunc_err: float, dmin: int, dmax: int,
        scale_side: int = 0):
    """Returns (u, s, vt, actual_trunc_err, D)."""
    lib = load()
    d = DeviceTensor.from_host(t)
    ld = np.ascontiguousarray(list(ldiv), dtype=np.int32)
    cap = sum(ix.dim for ix in t.indices[:ldims]) * sum(ix.dim for ix in t.indices[ldims:]) + 1
    cap = max(cap, 1)
    s = np.zeros(min(cap, 1 << 24))
    u, vt = C.c_void_p(), C.c_void_p()
    err, D = C.c_double(), C.c_int64()
    check(lib.gq_svd(d.h, ldims, ld.ctypes.data_as(_lib._IP), trunc_err, dmin, dmax, scale_side,
                     C.byref(u), C.byref(vt), s.ctypes.data_as(_lib._DP), s.size, C.byref(err),
                     C.byref(D)))
    return (DeviceTensor(u.value).to_host(), s[:D.value].copy(), DeviceTensor(vt.value).to_host(),
            err.value, D.value)


# ---------------------------------------------------------------------------
# Finite-MPS canonicalisation and truncation (device)
# ---------------------------------------------------------------------------
def _mps_handles(mps: FiniteMPS):
    dev = [DeviceTensor.from_host(mps[i]) for i in range(mps.size())]
    arr = (C.c_void_p * len(dev))(*[t.h.value for t in dev])
    cano = (C.c_int * len(dev))(*mps.tens_cano_type)
    return dev, arr, cano


def mps_centralize(mps: FiniteMPS, center: int) -> None:
    """Backs ``FiniteMPS.Centralize`` (``gq_mps_centralize``)."""
    dev, arr, cano = _mps_handles(mps)
    check(load().gq_mps_centralize(arr, len(dev), int(center), cano))
    for i, t in enumerate(dev):
        mps[i] = t.to_host()
    mps.tens_cano_type = list(cano)


def TruncateMPS(mps: FiniteMPS, trunc_err: float, Dmin: int, Dmax: int):
    """``TruncateMPS`` (``finite_mps.h:251-300``) on the GPU.  Returns the
    (truncation error, D) of every bond, which the reference prints."""
    dev, arr, cano = _mps_handles(mps)
    n = len(dev)
    errs = np.zeros(max(n - 1, 1))
    Ds = np.zeros(max(n - 1, 1), dtype=np.int64)
    check(load().gq_mps_truncate(arr, n, cano, float(trunc_err), int(Dmin), int(Dmax),
                                 errs.ctypes.data_as(_lib._DP),
                                 Ds.ctypes.data_as(C.POINTER(C.c_int64))))
    for i, t in enumerate(dev):
        mps[i] = t.to_host()
    mps.tens_cano_type = list(cano)
    mps.center = kUncentralizedCenterIdx
    return [(float(e), int(d)) for e, d in zip(errs[:n - 1], Ds[:n - 1])]
