"""Split-precision (3xTF32 on tcgen05) path against the FP64 oracle.

Tolerances: a 3xTF32 product carries about 2^-21 relative error and the
partial sums are merged in double-float, so contractions and matvecs are
checked at 1e-5 relative (2-norm over all blocks); energies of a Lanczos
solve at 1e-7 relative.  Each test also checks, through the kernel
profiler, that the tensor-core kernel really ran.
"""
import numpy as np
import pytest

import oracle
from oracle.lanczos import LanczosParams as OLP, MATVEC
from mps2_gb300 import hamiltonians as H
from mps2_gb300.tensor import GQTensor, IN, Index, OUT
from _convert import from_oracle, to_oracle
from _helpers import random_tensor, rel_err

pytestmark = pytest.mark.gpu

TC_TOL = 1e-5


@pytest.fixture(scope="module")
def lib():
    from mps2_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    return lib


def big_index(rng, qs, lo, hi, dir):
    return Index([((q,), int(rng.integers(lo, hi + 1))) for q in qs], dir)


def tc_launches(fn):
    from mps2_gb300.vmps import profile_enable, profile_read
    profile_enable(True)
    out = fn()
    n = profile_read("gemm_tf32x3")[0]
    profile_enable(False)
    return out, n


@pytest.mark.parametrize("axes", [([0], [0]), ([2], [0]), ([0, 2], [0, 1]), ([1, 2], [1, 3])])
def test_tc_contract_matches_oracle(lib, axes):
    from mps2_gb300.vmps import Contract
    xa, xb = axes
    rng = np.random.default_rng(21)
    ra = max(max(xa) + 1, 3)
    rb = max(max(xb) + 1, 3)
    ia = [big_index(rng, [-2, 0, 2], 60, 150, OUT if i % 2 else IN) for i in range(ra)]
    ib = [big_index(rng, [-2, 0, 2], 60, 150, OUT if i % 2 == 0 else IN) for i in range(rb)]
    for a_ax, b_ax in zip(xa, xb):
        ib[b_ax] = ia[a_ax].inverse()
    # large sectors on the contracted legs, the first free leg of a and the
    # last free leg of b; small ones elsewhere (keeps the operands moderate)
    free_a = [i for i in range(ra) if i not in xa]
    free_b = [i for i in range(rb) if i not in xb]
    for i in free_a[1:]:
        ia[i] = Index([((0,), 2), ((2,), 1)], ia[i].dir)
    for i in free_b[:-1]:
        ib[i] = Index([((0,), 2), ((-2,), 1)], ib[i].dir)
    a = random_tensor(rng, ia, GQTensor(ia).block_div(tuple(0 for _ in ia)))
    b = random_tensor(rng, ib, GQTensor(ib).block_div(tuple(0 for _ in ib)))
    ref = oracle.contract(to_oracle(a), to_oracle(b), xa, xb)
    got, n = tc_launches(lambda: Contract(a, b, (xa, xb), precision="tf32x3"))
    assert n > 0, "the tensor-core kernel did not run"
    assert rel_err(got, ref) <= TC_TOL


def _random_env_case(rng, where, D_lo=60, D_hi=140):
    """Random environments with large sectors around a Heisenberg MPO."""
    sv, mpo, qn0, _ = H.heisenberg_chain(8)
    Wl, Wr = (mpo[0], mpo[1]) if where == "lend" else ((mpo[6], mpo[7]) if where == "rend"
                                                        else (mpo[3], mpo[4]))
    qs = [-4, -2, 0, 2, 4]
    lbond = big_index(rng, qs, D_lo, D_hi, IN)    # Theta's left leg
    rbond = big_index(rng, qs, D_lo, D_hi, OUT)   # Theta's right leg
    L = R = None
    legs = []
    if where != "lend":
        L = random_tensor(rng, [lbond.inverse(), Wl.indices[0].inverse(), lbond], (0,))
        legs.append(lbond)
    legs += [Wl.indices[2], Wr.indices[2]]
    if where != "rend":
        R = random_tensor(rng, [rbond.inverse(), Wr.indices[3].inverse(), rbond], (0,))
        legs.append(rbond)
    st = random_tensor(rng, legs, (0,))
    return [L, Wl, Wr, R], st


@pytest.mark.parametrize("where", ["cent", "lend", "rend"])
def test_tc_matvec_matches_oracle(lib, where):
    from mps2_gb300.vmps import eff_ham_mul_state
    rng = np.random.default_rng(31)
    eff, st = _random_env_case(rng, where)
    ref = MATVEC[where]([to_oracle(t) if t is not None else None for t in eff], to_oracle(st))
    (got, flops), n = tc_launches(lambda: eff_ham_mul_state(eff, st, where, "tf32x3"))
    if where == "cent":
        # at the chain ends the state has only d*d rows or columns, so those
        # skinny products stay on the FP64 kernel by design
        assert n > 0, "the tensor-core kernel did not run"
    assert rel_err(got, ref) <= TC_TOL


def test_tc_lanczos_energy_matches_fp64_same_problem(lib):
    """Heisenberg L=20, D=200 (the reference's CPU-runnable case): take the
    central effective Hamiltonian mid-sweep from an FP64 run and solve it in
    both forms from the same start vector.  With the FP64 Rayleigh-quotient
    correction the split form's energy agrees to 1e-9 relative."""
    from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
    from mps2_gb300.vmps import (Contract, DMRGState, LanczosParams, LanczosSolver,
                                 SweepParams)
    N, D = 20, 200
    sv, mpo, qn0, _ = H.heisenberg_chain(N)
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, H.neel_shuffled_labels(N, 0), qn0)
    st = DMRGState(mps.tens, mpo)
    st.init_envs("fp64")
    sp = SweepParams(3, D, D, 0.0, LanczosParams(1e-10, 100), precision="fp64")
    st.sweep(sp)
    c = N // 2 - 1
    for i in range(c):
        st.update(sp, "r", i)
    L = st.get_env("l", c)
    R = st.get_env("r", N - c - 2)
    theta = Contract(st.get_mps(c), st.get_mps(c + 1), ([2], [0]))
    eff = [L, mpo[c], mpo[c + 1], R]
    lp = LanczosParams(1e-12, 100)
    e64 = LanczosSolver(eff, theta, lp, "cent", precision="fp64").gs_eng
    (res, n) = tc_launches(lambda: LanczosSolver(eff, theta, lp, "cent", precision="tf32x3"))
    assert n > 0, "the tensor-core kernel did not run"
    rel = abs(res.gs_eng - e64) / abs(e64)
    print(f"E fp64 {e64:.14f} tf32x3 {res.gs_eng:.14f} rel {rel:.2e}")
    assert rel <= 1e-9
