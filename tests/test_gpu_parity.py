"""GPU parity tests: the CUDA path through the C ABI against the FP64 oracle.

Tolerances (FP64 form): per contraction / per matvec relative error
<= 1e-12 (2-norm over all blocks); Lanczos energy within 1e-10 relative;
per-sweep DMRG energies within 1e-10 relative; golden energies within the
reference's own tolerances.
"""
import numpy as np
import pytest

import oracle
from oracle.lanczos import LanczosParams as OLP, MATVEC
from oracle.vmps import SweepParams as OSP
from mps2_gb300 import hamiltonians as H
from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
from mps2_gb300.tensor import GQTensor, IN, Index, OUT
from _convert import from_oracle, to_oracle
from _helpers import first_allowed_div, oracle_state, random_index, random_tensor, rel_err
from golden_cases import cases

pytestmark = pytest.mark.gpu

MATVEC_TOL = 1e-12


@pytest.fixture(scope="module")
def lib():
    from mps2_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    return lib


# --------------------------------------------------------------------------
# contraction engine
# --------------------------------------------------------------------------
CONTRACT_CASES = [
    # (rank a, rank b, axes_a, axes_b) covering in-place NN / TN / NT and
    # permuted operands, as used by the matvec and environment growth
    ([0], [0]),
    ([0, 2], [0, 1]),
    ([4, 1], [0, 1]),
    ([4, 1], [1, 0]),
    ([2], [0]),
    ([1, 2], [1, 3]),
    ([3, 1], [1, 2]),
    ([0, 2], [1, 0]),
]


@pytest.mark.parametrize("case", range(len(CONTRACT_CASES)))
def test_contract_matches_oracle(lib, case):
    from mps2_gb300.vmps import Contract
    rng = np.random.default_rng(100 + case)
    xa, xb = CONTRACT_CASES[case]
    ra = max(max(xa) + 1, 3)
    rb = max(max(xb) + 1, 3)
    ia = [random_index(rng, 3, 2, 5, OUT if rng.random() < 0.5 else IN) for _ in range(ra)]
    ib = [random_index(rng, 3, 2, 5, OUT if rng.random() < 0.5 else IN) for _ in range(rb)]
    for a_ax, b_ax in zip(xa, xb):
        ib[b_ax] = ia[a_ax].inverse()
    a = random_tensor(rng, ia, first_allowed_div(ia), fill=0.8)
    b = random_tensor(rng, ib, first_allowed_div(ib), fill=0.8)
    assert a.blocks and b.blocks
    ref = oracle.contract(to_oracle(a), to_oracle(b), xa, xb)
    got = Contract(a, b, (xa, xb))
    assert [ix.sectors() for ix in got.indices] == [ix.sectors() for ix in ref.indices]
    assert rel_err(got, ref) <= MATVEC_TOL


# --------------------------------------------------------------------------
# effective-Hamiltonian matvec
# --------------------------------------------------------------------------
def _eff_ham_case(where, build, N, labels, D, seed):
    om, oo, envs = oracle_state(build, labels, 1, D)
    rng = np.random.default_rng(seed)
    i = N // 2 - 1 if where == "cent" else (0 if where == "lend" else N - 2)
    L = envs.get(("l", i)) if where != "lend" else None
    R = envs.get(("r", N - i - 2)) if where != "rend" else None
    Wl, Wr = oo[i], oo[i + 1]
    legs = []
    if where != "lend":
        legs.append(L.indices[0].inverse())
    legs += [Wl.indices[2], Wr.indices[2]]
    if where != "rend":
        legs.append(R.indices[0].inverse())
    div = om[0].div if where == "lend" else tuple(0 for _ in om[0].div)
    from mps2_gb300.tensor import Index
    st = random_tensor(rng, [Index(ix.sectors(), ix.dir) for ix in legs], div)
    eff = [L, Wl, Wr, R]
    return eff, st


@pytest.mark.parametrize("where", ["lend", "cent", "rend"])
@pytest.mark.parametrize("model", ["heisenberg", "hubbard"])
def test_matvec_matches_oracle(lib, where, model):
    from mps2_gb300.vmps import eff_ham_mul_state
    if model == "heisenberg":
        N = 12
        build = lambda: H.heisenberg_chain(N)
        labels = [i % 2 for i in range(N)]
        D = 24
    else:
        N = 8
        build = lambda: H.hubbard_chain(N, 1.0, 8.0)
        labels = [1 if i % 2 == 0 else 2 for i in range(N)]
        D = 32
    eff, st = _eff_ham_case(where, build, N, labels, D, seed=7)
    ref = MATVEC[where](eff, to_oracle(st))
    got, flops = eff_ham_mul_state([from_oracle(t) if t is not None else None for t in eff], st,
                                   where)
    assert flops > 0
    assert rel_err(got, ref) <= MATVEC_TOL


# --------------------------------------------------------------------------
# Lanczos
# --------------------------------------------------------------------------
@pytest.mark.parametrize("where", ["lend", "cent", "rend"])
def test_lanczos_matches_oracle(lib, where):
    from mps2_gb300.vmps import LanczosParams, LanczosSolver
    N = 10
    eff, st = _eff_ham_case(where, lambda: H.heisenberg_chain(N), N, [i % 2 for i in range(N)],
                            16, seed=3)
    ref = oracle.lanczos_solver(eff, to_oracle(st), OLP(1e-10, 60), where)
    got = LanczosSolver([from_oracle(t) if t is not None else None for t in eff], st,
                        LanczosParams(1e-10, 60), where)
    assert abs(got.gs_eng - ref.gs_eng) <= 1e-10 * abs(ref.gs_eng)
    # ground states agree up to sign
    a = got.gs_vec
    s = np.sign(sum(float(np.sum(a.blocks[k] * ref.gs_vec.blocks[k]))
                    for k in ref.gs_vec.blocks if k in a.blocks))
    assert rel_err(a * s, ref.gs_vec) <= 1e-6


@pytest.mark.parametrize("prec", ["fp64", "tf32x3", "fp64tc"])
def test_lanczos_device_loop_matches_host_driven_loop(lib, prec):
    """The Lanczos iteration run as a CUDA-graph while loop on the device
    (default) and driven from the host one iteration at a time (what the
    kernel profiler forces) launch the same kernels in the same order:
    bitwise identical energies, iteration counts and ground states.  The
    device loop waits on the host once per solve, the host-driven one once
    more per iteration."""
    from mps2_gb300.vmps import LanczosParams, LanczosSolver, host_sync_count, profile_enable
    from test_oracle_golden import _random_sym_env
    rng = np.random.default_rng(8)
    eff, theta = _random_sym_env(rng, 160, 2, 2)
    eff = [from_oracle(t) for t in eff]
    theta = from_oracle(theta)
    lp = LanczosParams(1e-12, 40)
    c0 = host_sync_count()
    a = LanczosSolver(eff, theta, lp, "cent", precision=prec)
    c1 = host_sync_count()
    profile_enable(True)
    b = LanczosSolver(eff, theta, lp, "cent", precision=prec)
    c2 = host_sync_count()
    profile_enable(False)
    assert a.iters == b.iters and a.iters >= 10
    assert a.gs_eng == b.gs_eng
    assert rel_err(a.gs_vec, to_oracle(b.gs_vec)) == 0.0
    # the device loop saves one host wait per iteration; what remains does
    # not grow with the iterations (one for the solve, the rest the API's
    # tensor transfers)
    assert (c2 - c1) - (c1 - c0) == a.iters
    assert c1 - c0 < a.iters


def test_lanczos_device_loop_stops_at_max_iterations(lib):
    """A solve that cannot meet its tolerance stops after max_iterations - 1
    iterations (``lanczos_solver_impl.h:205-219``), in the device loop as on
    the oracle."""
    from mps2_gb300.vmps import LanczosParams, LanczosSolver
    from test_oracle_golden import _random_sym_env
    rng = np.random.default_rng(9)
    eff, theta = _random_sym_env(rng, 120, 2, 2)
    ref = oracle.lanczos_solver(eff, theta, OLP(0.0, 7), "cent")
    got = LanczosSolver([from_oracle(t) for t in eff], from_oracle(theta),
                        LanczosParams(0.0, 7), "cent")
    assert got.iters == ref.iters == 6
    assert abs(got.gs_eng - ref.gs_eng) <= 1e-10 * abs(ref.gs_eng)


def test_lanczos_vs_dense_diagonalisation(lib):
    """The reference's Lanczos unit test (``test_lanczos_solver.cc:111``)
    through the GPU solver."""
    from mps2_gb300.vmps import LanczosParams, LanczosSolver
    from test_oracle_golden import _random_sym_env, dense_eff_ham
    rng = np.random.default_rng(0)
    eff, theta = _random_sym_env(rng, 20, 2, 2)
    e_dense = np.linalg.eigvalsh(dense_eff_ham(eff))[0]
    for prm in [(1e-9, 200), (1e-16, 20)]:
        got = LanczosSolver([from_oracle(t) for t in eff], from_oracle(theta),
                            LanczosParams(*prm), "cent")
        assert abs(got.gs_eng - e_dense) <= 1e-8


# --------------------------------------------------------------------------
# truncating SVD
# --------------------------------------------------------------------------
@pytest.mark.parametrize("dmax,trunc", [(6, 0.0), (12, 1e-3), (1000, 0.0)])
def test_svd_matches_oracle(lib, dmax, trunc):
    from mps2_gb300.vmps import SVD
    rng = np.random.default_rng(5)
    l = random_index(rng, 4, 2, 4, IN)
    s1 = random_index(rng, 2, 1, 1, OUT)
    s2 = random_index(rng, 2, 1, 1, OUT)
    r = random_index(rng, 4, 2, 4, OUT)
    t = random_tensor(rng, [l, s1, s2, r], (0,))
    ref = oracle.svd(to_oracle(t), 2, (0,), trunc, 1, dmax)
    u, s, vt, err, D = SVD(t, 2, (0,), trunc, 1, dmax)
    assert D == ref.D
    assert abs(err - ref.trunc_err) <= 1e-12
    np.testing.assert_allclose(s, ref.svals, rtol=1e-12, atol=1e-14)
    assert [ix.sectors() for ix in u.indices] == [ix.sectors() for ix in ref.u.indices]
    assert rel_err(u, ref.u) <= 1e-9
    assert rel_err(vt, ref.vt) <= 1e-9


def test_svd_zero_completion_matches_oracle(lib):
    """Rank-deficient groups: kept zero singular values take the canonical
    Householder completion on both sides."""
    from mps2_gb300.vmps import SVD
    rng = np.random.default_rng(11)
    l = random_index(rng, 3, 1, 3, IN)
    s1 = random_index(rng, 2, 1, 1, OUT)
    s2 = random_index(rng, 2, 1, 1, OUT)
    r = random_index(rng, 3, 1, 3, OUT)
    t = random_tensor(rng, [l, s1, s2, r], (0,), fill=0.3)
    ref = oracle.svd(to_oracle(t), 2, (0,), 0.0, 64, 64)
    u, s, vt, err, D = SVD(t, 2, (0,), 0.0, 64, 64)
    assert D == ref.D
    np.testing.assert_allclose(s, ref.svals, rtol=1e-12, atol=1e-14)
    assert rel_err(u, ref.u) <= 1e-9
    assert rel_err(vt, ref.vt) <= 1e-9


def _scale_leg(t, leg, s):
    """t with its slices along `leg` (sectors in index order, flattened)
    multiplied by the values s."""
    out = t.copy()
    offs = np.cumsum([0] + [d for _, d in t.indices[leg].sectors()])
    for k in out.blocks:
        sh = [1] * out.blocks[k].ndim
        sh[leg] = -1
        out.blocks[k] = out.blocks[k] * s[offs[k[leg]]:offs[k[leg] + 1]].reshape(sh)
    return out


@pytest.mark.parametrize("scale_side", [1, 2])
@pytest.mark.parametrize("big_side", ["l", "r"])
@pytest.mark.parametrize("size", ["mid", "large"])
def test_svd_gram_routes_match_oracle(lib, scale_side, big_side, size):
    """Groups of a few hundred rows on one side: the sweep's Gram routes
    ('r': U orthonormal, S.Vt returned; 'l': V orthonormal, U.S returned),
    on the canonical side's Gram matrix or -- when the other side is much
    smaller -- on the other side's, against the oracle's SVD.  The large
    case (groups up to 1350 x 580) takes the Gram matrices and projections
    through the FP64-accurate tensor-core contraction."""
    from mps2_gb300.vmps import SVD
    rng = np.random.default_rng(17 + scale_side)
    if size == "mid":
        big = Index([((-1,), 300), ((1,), 280)], IN)
        small = Index([((-1,), 60), ((1,), 70)], IN)
    else:
        big = Index([((-1,), 700), ((1,), 650)], IN)
        small = Index([((-1,), 300), ((1,), 280)], IN)
    l = big if big_side == "l" else small
    r = (small if big_side == "l" else big).inverse()
    s1 = Index([((1,), 1), ((-1,), 1)], OUT)
    s2 = Index([((1,), 1), ((-1,), 1)], OUT)
    t = random_tensor(rng, [l, s1, s2, r], (0,))
    ref = oracle.svd(to_oracle(t), 2, (0,), 0.0, 1, 150)
    u, s, vt, err, D = SVD(t, 2, (0,), 0.0, 1, 150, scale_side=scale_side)
    assert D == ref.D
    np.testing.assert_allclose(s, ref.svals, rtol=1e-10)
    ru, rvt = from_oracle(ref.u), from_oracle(ref.vt)
    if scale_side == 2:
        rvt = _scale_leg(rvt, 0, np.asarray(ref.svals))
    else:
        ru = _scale_leg(ru, 2, np.asarray(ref.svals))
    assert rel_err(u, to_oracle(ru)) <= 1e-9
    assert rel_err(vt, to_oracle(rvt)) <= 1e-9


# --------------------------------------------------------------------------
# full sweeps
# --------------------------------------------------------------------------
GOLDEN = cases()


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_dmrg_golden_energy_gpu(lib, name):
    from mps2_gb300.vmps import DMRGState, LanczosParams, SweepParams
    build, labs, p, golden, tol, line = GOLDEN[name]
    sv, mpo, qn0, _ = build()
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, labs, qn0)
    st = DMRGState(mps.tens, mpo)
    st.init_envs("fp64")
    e0, stats = st.sweep(SweepParams(p[0], p[1], p[2], p[3], LanczosParams(p[4], p[5])))
    assert abs(e0 - golden) <= tol, (name, e0, golden)


def test_dmrg_per_sweep_energies_match_oracle(lib):
    from mps2_gb300.vmps import DMRGState, LanczosParams, SweepParams
    N = 16
    sv, mpo, qn0, _ = H.heisenberg_chain(N)
    mps = FiniteMPS(sv)
    labels = H.neel_shuffled_labels(N, 0)
    DirectStateInitMps(mps, labels, qn0)
    st = DMRGState(mps.tens, mpo)
    st.init_envs("fp64")
    sp = SweepParams(1, 24, 24, 0.0, LanczosParams(1e-10, 60))
    om = [to_oracle(t) for t in mps.tens]
    oo = [to_oracle(t) for t in mpo]
    envs = {}
    oracle.init_envs(om, oo, envs)
    for sweep in range(3):
        e_gpu, stats = st.sweep(sp)
        ost = []
        from oracle.vmps import two_site_sweep
        e_cpu = two_site_sweep(om, oo, envs, OSP(1, 24, 24, 0.0, OLP(1e-10, 60)), ost)
        assert abs(e_gpu - e_cpu) <= 1e-10 * abs(e_cpu), (sweep, e_gpu, e_cpu)
        assert [s.D for s in stats] == [s.D for s in ost]


def test_two_site_finite_vmps_file_contract(lib, tmp_path):
    """Drop-in call with the reference's file contract and resume
    (``test_two_site_update_finite_vmps.cc:192-220``)."""
    from mps2_gb300.vmps import LanczosParams, SweepParams, TwoSiteFiniteVMPS
    import os
    build, labs, p, golden, tol, _ = GOLDEN["1DHeisenberg"]
    sv, mpo, qn0, _ = build()
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, labs, qn0)
    sp = SweepParams(p[0], p[1], p[2], p[3], LanczosParams(p[4], p[5]),
                     mps_path=str(tmp_path / "mps"), temp_path=str(tmp_path / ".temp"))
    mps.Dump(sp.mps_path, True)
    assert mps.empty()
    e0 = TwoSiteFiniteVMPS(mps, mpo, sp)
    assert abs(e0 - golden) <= tol and mps.empty()
    assert os.path.exists(os.path.join(sp.temp_path, "renv1.gqten"))
    e1 = TwoSiteFiniteVMPS(mps, mpo, sp)   # resumes from temp_path
    assert abs(e1 - golden) <= tol and mps.empty()


def test_dmrg_kitaev_extend_direct_random_init_gpu(lib):
    """``2DKitaevSimpleCase`` (``test_two_site_update_finite_vmps.cc:311-345``)
    through the product's ``ExtendDirectRandomInitMps`` (random sum of the two
    Neel states, centralised on the GPU): golden energy -1.0 within 1e-12."""
    from mps2_gb300.finite_mps import ExtendDirectRandomInitMps
    from mps2_gb300.vmps import DMRGState, LanczosParams, SweepParams
    from test_oracle_golden import kitaev_case
    sv, mpo, qn0, labs, p, golden, tol = kitaev_case()
    mps = FiniteMPS(sv)
    ExtendDirectRandomInitMps(mps, labs, qn0, 2, seed=0)
    assert mps.GetCenter() != 0 and mps.GetTenCanoType(0) == FiniteMPS.NONE
    assert all(mps.GetTenCanoType(i) == FiniteMPS.RIGHT for i in range(1, len(mps)))
    st = DMRGState(mps.tens, mpo)
    st.init_envs("fp64")
    e0, _ = st.sweep(SweepParams(p[0], p[1], p[2], p[3], LanczosParams(p[4], p[5])))
    assert abs(e0 - golden) <= tol, e0
