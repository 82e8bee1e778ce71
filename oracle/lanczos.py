"""FP64 CPU oracle: Lanczos ground-state solver of the two-site effective
Hamiltonian.  TEST INFRASTRUCTURE ONLY (see ``oracle/bstensor.py``).

Restates ``include/gqmps2/algorithm/lanczos_solver_impl.h`` of gqmps2:

* ``LanczosSolver`` (lines 79-226): no re-orthogonalisation, every Krylov
  vector kept, stop when ``E_old - E_new < error`` or ``m == eff_dim`` or
  ``m == max_iterations - 1``; breakdown (``|gamma| == 0``) handled as at
  lines 163-180.
* ``eff_ham_mul_state_{cent,lend,rend}`` (lines 228-256): the contraction
  chains that apply ``L . W_l . W_r . R`` to the two-site state.
* ``TridiagGsSolver`` (lines 259-313): ``LAPACKE_dstev``; scipy's ``dstev``
  (same LAPACK routine) stands in for MKL's.
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import lapack

from .bstensor import BSTensor, contract, dag, inner, linear_combine


class LanczosParams:
    """``LanczosParams`` of ``lanczos_solver.h:34-39``."""

    def __init__(self, error: float = 1e-7, max_iterations: int = 200):
        self.error = float(error)
        self.max_iterations = int(max_iterations)


class LanczosRes:
    def __init__(self, iters, gs_eng, gs_vec):
        self.iters = iters
        self.gs_eng = gs_eng
        self.gs_vec = gs_vec


def eff_ham_mul_state_cent(eff_ham, state: BSTensor) -> BSTensor:
    """``lanczos_solver_impl.h:228-236``."""
    res = contract(eff_ham[0], state, [0], [0])
    res = contract(res, eff_ham[1], [0, 2], [0, 1])
    res = contract(res, eff_ham[2], [4, 1], [0, 1])
    res = contract(res, eff_ham[3], [4, 1], [1, 0])
    return res


def eff_ham_mul_state_lend(eff_ham, state: BSTensor) -> BSTensor:
    """``lanczos_solver_impl.h:239-246``."""
    res = contract(state, eff_ham[1], [0], [0])
    res = contract(res, eff_ham[2], [0, 2], [1, 0])
    res = contract(res, eff_ham[3], [0, 3], [0, 1])
    return res


def eff_ham_mul_state_rend(eff_ham, state: BSTensor) -> BSTensor:
    """``lanczos_solver_impl.h:249-256``."""
    res = contract(state, eff_ham[0], [0], [0])
    res = contract(res, eff_ham[1], [2, 0], [0, 1])
    res = contract(res, eff_ham[2], [3, 0], [1, 0])
    return res


MATVEC = {"cent": eff_ham_mul_state_cent,
          "lend": eff_ham_mul_state_lend,
          "rend": eff_ham_mul_state_rend}


def tridiag_gs(a, b, n, want_vec: bool):
    """``TridiagGsSolver`` (``lanczos_solver_impl.h:259-313``): lowest
    eigenpair of the n x n symmetric tridiagonal matrix (diag a, offdiag b)."""
    d = np.array(a[:n], dtype=float)
    e = np.array(b[:n - 1], dtype=float)
    if n == 1:
        return float(d[0]), (np.ones(1) if want_vec else None)
    w, z, info = lapack.dstev(d, e, compute_v=1 if want_vec else 0)
    if info != 0:
        raise RuntimeError("?stev error.")
    if want_vec:
        # sign convention (a gauge choice; dstev's sign is arbitrary): the
        # largest-magnitude component, first on ties, is positive
        v = np.array(z[:, 0])
        if v[int(np.argmax(np.abs(v)))] < 0:
            v = -v
        return float(w[0]), v
    return float(w[0]), None


def eff_dim(eff_ham, where: str) -> int:
    """Product of the four (three) outer leg dimensions, ``:92-112``."""
    L, Wl, Wr, R = eff_ham
    if where == "cent":
        return L.indices[0].dim * Wl.indices[1].dim * Wr.indices[1].dim * R.indices[0].dim
    if where == "lend":
        return Wl.indices[0].dim * Wr.indices[1].dim * R.indices[0].dim
    return L.indices[0].dim * Wl.indices[1].dim * Wr.indices[0].dim


def lanczos_solver(eff_ham, init: BSTensor, params: LanczosParams, where: str,
                   matvec_hook=None) -> LanczosRes:
    """``LanczosSolver`` (``lanczos_solver_impl.h:79-226``).  ``init`` is
    consumed (normalised in place), as in the reference."""
    mv = MATVEC[where]
    if matvec_hook is not None:
        mv = matvec_hook
    dim = eff_dim(eff_ham, where)
    maxit = params.max_iterations
    bases = [None] * maxit
    a = [0.0] * maxit
    b = [0.0] * maxit
    N = [0.0] * maxit
    init.normalize()
    bases[0] = init
    last = mv(eff_ham, bases[0])
    a[0] = inner(bases[0], last)
    N[0] = 0.0
    m = 0
    energy0 = a[0]
    while True:
        m += 1
        if m == 1:
            gamma = linear_combine([1.0, -a[m - 1]], [last, bases[m - 1]])
        else:
            gamma = linear_combine([1.0, -a[m - 1], -np.sqrt(N[m - 1])],
                                   [last, bases[m - 1], bases[m - 2]])
        norm_gamma = gamma.normalize()
        if norm_gamma == 0.0:
            if m == 1:
                return LanczosRes(m, energy0, bases[0].copy())
            _, vec = tridiag_gs(a, b, m, True)
            gs = linear_combine(list(vec), bases[:m])
            return LanczosRes(m, energy0, gs)
        N[m] = norm_gamma ** 2
        b[m - 1] = norm_gamma
        bases[m] = gamma
        last = mv(eff_ham, bases[m])
        a[m] = inner(bases[m], last)
        e_new, _ = tridiag_gs(a, b, m + 1, False)
        if (energy0 - e_new) < params.error or m == dim or m == maxit - 1:
            _, vec = tridiag_gs(a, b, m + 1, True)
            gs = linear_combine(list(vec), bases[:m + 1])
            return LanczosRes(m, e_new, gs)
        energy0 = e_new
