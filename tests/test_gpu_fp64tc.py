"""FP64-accurate tensor-core form (exact bf16 digits, exact FP32 partial
sums) against the FP64 oracle.

Tolerances: the form's error is about 2^-55 of max|a_i.| * max|b_.j| per
product term, so contractions and matvecs are checked at 1e-13 relative
(2-norm over all blocks), at 1e-12 (the per-matvec bar of the plain form)
when the operands' entries spread over twelve decades, and integer operands
must come out bit-exact.  Each test
checks through the kernel profiler that the tensor-core kernel ran.
"""
import numpy as np
import pytest

import oracle
from oracle.lanczos import MATVEC
from mps2_gb300.tensor import GQTensor, IN, Index, OUT
from _convert import from_oracle, to_oracle
from _helpers import random_tensor, rel_err
from test_gpu_tf32 import _random_env_case, big_index

pytestmark = pytest.mark.gpu

TOL = 1e-13
TOL_SPREAD = 1e-12


@pytest.fixture(scope="module")
def lib():
    from mps2_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    return lib


class Launches(int):
    """Tensor-core launch count that prints every family's count."""

    def __new__(cls, counts):
        obj = super().__new__(cls, counts["gemm_fp64tc"])
        obj.counts = counts
        return obj

    def __repr__(self):
        return f"{int(self)} (all families: {self.counts})"


def oz_launches(fn):
    from mps2_gb300 import _lib
    from mps2_gb300.vmps import profile_enable, profile_read
    profile_enable(True)
    out = fn()
    counts = {k: profile_read(k)[0] for k in _lib.PROF}
    profile_enable(False)
    return out, Launches(counts)


def _operands(rng, xa, xb, lo=60, hi=150):
    ra = max(max(xa) + 1, 3)
    rb = max(max(xb) + 1, 3)
    ia = [big_index(rng, [-2, 0, 2], lo, hi, OUT if i % 2 else IN) for i in range(ra)]
    ib = [big_index(rng, [-2, 0, 2], lo, hi, OUT if i % 2 == 0 else IN) for i in range(rb)]
    for a_ax, b_ax in zip(xa, xb):
        ib[b_ax] = ia[a_ax].inverse()
    free_a = [i for i in range(ra) if i not in xa]
    free_b = [i for i in range(rb) if i not in xb]
    for i in free_a[1:]:
        ia[i] = Index([((0,), 2), ((2,), 1)], ia[i].dir)
    for i in free_b[:-1]:
        ib[i] = Index([((0,), 2), ((-2,), 1)], ib[i].dir)
    a = random_tensor(rng, ia, GQTensor(ia).block_div(tuple(0 for _ in ia)))
    b = random_tensor(rng, ib, GQTensor(ib).block_div(tuple(0 for _ in ib)))
    return a, b


def _map_blocks(t, fn):
    for k in list(t.blocks):
        t.blocks[k] = fn(t.blocks[k])
    return t


@pytest.mark.parametrize("axes", [([0], [0]), ([2], [0]), ([0, 2], [0, 1]), ([1, 2], [1, 3])])
@pytest.mark.parametrize("spread", [0, 12])
def test_fp64tc_contract_matches_oracle(lib, axes, spread):
    from mps2_gb300.vmps import Contract
    xa, xb = axes
    rng = np.random.default_rng(41 + spread)
    a, b = _operands(rng, xa, xb)
    if spread:
        sc = lambda x: x * 10.0 ** rng.uniform(-spread, 0, x.shape)
        _map_blocks(a, sc)
        _map_blocks(b, sc)
    ref = oracle.contract(to_oracle(a), to_oracle(b), xa, xb)
    got, n = oz_launches(lambda: Contract(a, b, (xa, xb), precision="fp64tc"))
    assert n > 0, "the tensor-core kernel did not run"
    assert rel_err(got, ref) <= (TOL_SPREAD if spread else TOL)


def test_fp64tc_integer_operands_are_exact(lib):
    """Integer entries in [-127, 127] (rows and columns long enough that each
    has a maximum of at least 64): every entry is its own leading digit, so
    the result is the FP32 tensor-core sums of integer products below 2^14,
    256 at a time, added in FP64 -- exact only if the tensor cores add those
    integers exactly.  The result must match FP64 bit for bit."""
    from mps2_gb300.vmps import Contract
    rng = np.random.default_rng(7)
    a, b = _operands(rng, [1], [0], lo=300, hi=700)
    ints = lambda x: rng.integers(-127, 128, x.shape).astype(np.float64)
    _map_blocks(a, ints)
    _map_blocks(b, ints)
    ref = oracle.contract(to_oracle(a), to_oracle(b), [1], [0])
    got, n = oz_launches(lambda: Contract(a, b, ([1], [0]), precision="fp64tc"))
    assert n > 0, "the tensor-core kernel did not run"
    assert rel_err(got, ref) == 0.0


def test_fp64tc_long_k_beyond_two_to_the_sixteen(lib):
    """A thin block pair with k = 70000 > 2^16 (as the J1-J2 cylinder's
    environment contractions have): runs on the FP64-accurate kernel, within
    the tolerance of the others."""
    from mps2_gb300.vmps import Contract
    rng = np.random.default_rng(12)
    r = Index([((0,), 9)], OUT)
    k = Index([((0,), 70000)], OUT)
    c = Index([((0,), 7)], OUT)
    a = GQTensor([r, k], (0,), {(0, 0): rng.standard_normal((9, 70000))})
    b = GQTensor([k.inverse(), c], (0,), {(0, 0): rng.standard_normal((70000, 7))})
    ref = oracle.contract(to_oracle(a), to_oracle(b), [1], [0])
    got, n = oz_launches(lambda: Contract(a, b, ([1], [0]), precision="fp64tc"))
    assert n > 0, "the tensor-core kernel did not run"
    assert rel_err(got, ref) <= TOL


@pytest.mark.parametrize("where", ["cent", "lend", "rend"])
def test_fp64tc_matvec_matches_oracle(lib, where):
    from mps2_gb300.vmps import eff_ham_mul_state
    rng = np.random.default_rng(51)
    eff, st = _random_env_case(rng, where)
    ref = MATVEC[where]([to_oracle(t) if t is not None else None for t in eff], to_oracle(st))
    (got, flops), n = oz_launches(lambda: eff_ham_mul_state(eff, st, where, "fp64tc"))
    if where == "cent":
        assert n > 0, "the tensor-core kernel did not run"
    assert rel_err(got, ref) <= TOL


def test_sweeps_in_fp64tc_and_split_forms_match_fp64(lib):
    """Heisenberg L=20, D=200, 4 sweeps, Lanczos 1e-9 (the reference's
    CPU-runnable configuration): the FP64-accurate tensor-core form tracks
    the FP64 form's per-sweep energies to 1e-10 relative; the split form
    (3xTF32 matvec, FP64-accurate environments, energies taken as
    FP64-accurate tensor-core Rayleigh quotients) ends within 1e-9.

    The run is still converging (the energy drops by ~2e-3 per sweep), so
    each sweep's energy carries the Lanczos stopping tolerance (1e-9
    absolute, ~1e-10 relative here): rounding-level differences between two
    arithmetic forms move where the solves stop.  The first sweeps agree to
    1e-13 or better; the products themselves are checked bit-exactly and to
    1e-13 by the contraction and matvec tests above."""
    from mps2_gb300 import hamiltonians as H
    from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
    from mps2_gb300.vmps import DMRGState, LanczosParams, SweepParams, profile_enable, profile_read
    N, D = 20, 200
    sv, mpo, qn0, _ = H.heisenberg_chain(N)
    energies = {}
    for prec, ray in (("fp64", "fp64"), ("fp64tc", "fp64"), ("tf32x3", "fp64tc")):
        mps = FiniteMPS(sv)
        DirectStateInitMps(mps, H.neel_shuffled_labels(N, 0), qn0)
        st = DMRGState(mps.tens, mpo)
        profile_enable(True)
        st.init_envs(prec)
        sp = SweepParams(1, D, D, 0.0, LanczosParams(1e-9, 100), precision=prec, rayleigh=ray)
        energies[prec] = [st.sweep(sp)[0] for _ in range(4)]
        if prec != "fp64":
            assert profile_read("gemm_fp64tc")[0] > 0, "the tensor-core kernel did not run"
        profile_enable(False)
    print(energies)
    for e64, e in zip(energies["fp64"], energies["fp64tc"]):
        assert abs(e - e64) / abs(e64) <= 1e-10
    assert abs(energies["tf32x3"][-1] - energies["fp64"][-1]) / abs(energies["fp64"][-1]) <= 1e-9


def test_fp64tc_matvec_on_symmetric_single_sector_problem(lib):
    """The reference's Lanczos set-up (one sector per leg, D=256: dense
    256 x 512 blocks, k up to 512): the FP64-accurate tensor-core matvec
    against the FP64 one and the oracle."""
    from mps2_gb300.vmps import eff_ham_mul_state
    from test_oracle_golden import _random_sym_env
    rng = np.random.default_rng(3)
    eff, theta = _random_sym_env(rng, 256, 2, 2)
    ref = MATVEC["cent"](eff, theta)
    effg = [from_oracle(t) for t in eff]
    th = from_oracle(theta)
    (got64, _), _ = oz_launches(lambda: eff_ham_mul_state(effg, th, "cent", "fp64"))
    (gottc, _), n = oz_launches(lambda: eff_ham_mul_state(effg, th, "cent", "fp64tc"))
    assert n > 0, "the tensor-core kernel did not run"
    e64, etc = rel_err(got64, ref), rel_err(gottc, ref)
    print(f"fp64 {e64:.2e} fp64tc {etc:.2e}")
    assert e64 <= 1e-13
    assert etc <= TOL, (e64, etc)


def test_fp64tc_lanczos_energy_matches_fp64_same_problem(lib):
    """The reference's Lanczos set-up (``test_lanczos_solver.cc:121-153``:
    symmetric environments, one sector per leg) at D=256, 7 Lanczos steps:
    the FP64-accurate tensor-core Lanczos tracks the FP64 one's energy to
    1e-9 relative.  The matvecs themselves agree to ~5e-16 (the test
    above); this random operator's unconverged Krylov recurrence amplifies
    that difference to ~5e-11 in the Ritz value, as it would any other
    FP64 summation order."""
    from mps2_gb300.vmps import LanczosParams, LanczosSolver
    from test_oracle_golden import _random_sym_env
    rng = np.random.default_rng(3)
    eff, theta = _random_sym_env(rng, 256, 2, 2)
    eff = [from_oracle(t) for t in eff]
    theta = from_oracle(theta)
    lp = LanczosParams(1e-15, 8)
    e64 = LanczosSolver(eff, theta, lp, "cent", precision="fp64").gs_eng
    res, n = oz_launches(lambda: LanczosSolver(eff, theta, lp, "cent", precision="fp64tc"))
    assert n > 0, "the tensor-core kernel did not run"
    assert abs(res.gs_eng - e64) / abs(e64) <= 1e-9, (res.gs_eng, e64)
