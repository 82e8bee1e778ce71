"""Pin the FP64 oracle against the reference's golden energies (CPU)."""
import numpy as np
import pytest

import oracle
from oracle.lanczos import LanczosParams
from oracle.vmps import SweepParams
from mps2_gb300.finite_mps import FiniteMPS, DirectStateInitMps
from golden_cases import cases
from _convert import to_oracle

CASES = cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_golden_energy(name):
    build, labs, p, golden, tol, line = CASES[name]
    sv, mpo, qn0, _ = build()
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, labs, qn0)
    sp = SweepParams(p[0], p[1], p[2], p[3], LanczosParams(p[4], p[5]))
    e0 = oracle.two_site_finite_vmps([to_oracle(t) for t in mps.tens],
                                     [to_oracle(t) for t in mpo], sp)
    assert abs(e0 - golden) <= tol, (name, e0, golden)


def test_oracle_resume_keeps_energy():
    """Second call on the same state and environments (the reference's
    continue-simulation test, ``test_two_site_update_finite_vmps.cc:215-220``)."""
    build, labs, p, golden, tol, _ = CASES["1DHeisenberg"]
    sv, mpo, qn0, _ = build()
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, labs, qn0)
    om = [to_oracle(t) for t in mps.tens]
    oo = [to_oracle(t) for t in mpo]
    envs = {}
    sp = SweepParams(p[0], p[1], p[2], p[3], LanczosParams(p[4], p[5]))
    e1 = oracle.two_site_finite_vmps(om, oo, sp, envs=envs)
    e2 = oracle.two_site_finite_vmps(om, oo, sp, envs=envs)
    assert abs(e1 - golden) <= tol and abs(e2 - golden) <= tol


def _rand_sym(rng, n):
    """``RandRealSymMat`` (``tests/testing_utils.h:28-45``): A + A^T with
    uniform [0, 1) entries (numpy's generator stands in for ``rand()``)."""
    a = rng.random((n, n))
    return a + a.T


def _random_sym_env(rng, D, w, d):
    """The set-up of ``test_lanczos_solver.cc:121-153``: one QN sector per
    leg, L[i,k,j] = R[j,k,i] = M[i,j], W[k,i,j,k] = m[i,j]."""
    q0 = (0,)
    din = oracle.Index([(q0, d)], oracle.IN)
    Din = oracle.Index([(q0, D)], oracle.IN)
    vin = oracle.Index([(q0, w)], oracle.IN)
    dout, Dout, vout = din.inverse(), Din.inverse(), vin.inverse()
    M = _rand_sym(rng, D)
    m = _rand_sym(rng, d)
    Lb = np.repeat(M[:, None, :], w, axis=1)
    Rb = np.repeat(M.T[:, None, :], w, axis=1)
    Wb = np.zeros((w, d, d, w))
    for k in range(w):
        Wb[k, :, :, k] = m
    L = oracle.BSTensor([Dout, vout, Din], q0, {(0, 0, 0): Lb})
    Wl = oracle.BSTensor([vin, din, dout, vout], q0, {(0, 0, 0, 0): Wb})
    Wr = oracle.BSTensor([vin, din, dout, vout], q0, {(0, 0, 0, 0): Wb.copy()})
    R = oracle.BSTensor([Din, vin, Dout], q0, {(0, 0, 0): Rb})
    theta = oracle.BSTensor([Din, dout, dout, Dout], q0,
                            {(0, 0, 0, 0): rng.random((D, d, d, D))})
    return [L, Wl, Wr, R], theta


def dense_eff_ham(eff_ham):
    L, Wl, Wr, R = [t.to_dense() for t in eff_ham]
    D, d = L.shape[0], Wl.shape[1]
    h = np.einsum("awb,wstv,vxyc,dce->btyeasxd", L, Wl, Wr, R)
    return h.reshape(D * d * d * D, -1)


@pytest.mark.parametrize("params", [(1e-9, 200), (1e-16, 20)])
def test_oracle_lanczos_vs_dense(params):
    """``test_lanczos_solver.cc:111``: |E_lanczos - E_dense| <= 1e-8."""
    rng = np.random.default_rng(0)
    D, w, d = 20, 2, 2
    eff_ham, theta = _random_sym_env(rng, D, w, d)
    res = oracle.lanczos_solver(eff_ham, theta, LanczosParams(*params), "cent")
    Hd = dense_eff_ham(eff_ham)
    assert np.allclose(Hd, Hd.T)
    e_dense = np.linalg.eigvalsh(Hd)[0]
    assert abs(res.gs_eng - e_dense) <= 1e-8


def kitaev_case():
    """``2DKitaevSimpleCase`` (``test_two_site_update_finite_vmps.cc:311-345``):
    the honeycomb zz model on 4 x 2 sites from the random sum of the two Neel
    product states (``ExtendDirectRandomInitMps`` with enlarged dimension 2),
    4 sweeps, D=8, truncation error 1e-4, Lanczos tolerance 1e-10; golden
    energy -1.0 (tolerance 1e-12)."""
    from mps2_gb300 import hamiltonians as H
    N = 8
    sv, mpo, qn0, _ = H.heisenberg_pairs(N, H.kitaev_simple_pairs(4, 2), ising_only=True)
    labs = [[i % 2 for i in range(N)], [(i + 1) % 2 for i in range(N)]]
    return sv, mpo, qn0, labs, (4, 8, 8, 1e-4, 1e-10, 200), -1.0, 1e-12


def test_oracle_kitaev_extend_direct_random_init():
    import oracle.finite_mps as ofm
    from mps2_gb300.finite_mps import extend_direct_random_tensors
    sv, mpo, qn0, labs, p, golden, tol = kitaev_case()
    mps = FiniteMPS(sv)
    tens = [to_oracle(t) for t in extend_direct_random_tensors(mps, labs, qn0, 2, seed=0)]
    cano = [0] * len(tens)
    ofm.centralize(tens, cano, 0)
    nrm = np.sqrt(sum(float(np.sum(b * b)) for b in tens[0].blocks.values()))
    for k in tens[0].blocks:
        tens[0].blocks[k] = tens[0].blocks[k] / nrm
    sp = SweepParams(p[0], p[1], p[2], p[3], LanczosParams(p[4], p[5]))
    e0 = oracle.two_site_finite_vmps(tens, [to_oracle(t) for t in mpo], sp)
    assert abs(e0 - golden) <= tol, e0


def test_extend_direct_random_tensors_structure():
    """Each bond carries one sector of the enlarged dimension per product
    state, with that product state's bond charge (as DirectStateInitMps
    computes it); every tensor has the reference's divergences."""
    from mps2_gb300.finite_mps import extend_direct_random_tensors
    sv, mpo, qn0, labs, *_ = kitaev_case()
    mps = FiniteMPS(sv)
    tens = extend_direct_random_tensors(mps, labs, qn0, 2, seed=3)
    for j, lab in enumerate(labs):
        d = FiniteMPS(sv)
        DirectStateInitMps(d, lab, qn0)
        for i in range(len(tens) - 1):
            rvb = tens[i].indices[-1]
            assert rvb.dims[j] == 2
            assert rvb.qns[j] == d.tens[i].indices[-1].qns[0]
    assert all(t.div == qn0 for t in tens[1:])
    assert all(t.blocks for t in tens)
