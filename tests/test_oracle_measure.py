"""The oracle's finite-MPS measurements (``finite_mps_measu.h``) against
exact diagonalisation: an 8-site Heisenberg chain's DMRG ground state,
<Sz_i> and <Sz_i Sz_j> (identity inserts) and <S+_i S-_j>."""
import numpy as np

import oracle
from oracle.finite_mps import NONE
from oracle.lanczos import LanczosParams as OLP
from oracle.measure import measure_one_site, measure_two_site
from oracle.vmps import SweepParams as OSP
from mps2_gb300 import hamiltonians as H
from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
from _convert import to_oracle

N = 8


def _ground_state_mps():
    sv, mpo, qn0, _ = H.heisenberg_chain(N)
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, H.neel_shuffled_labels(N, 0), qn0)
    om = [to_oracle(t) for t in mps.tens]
    oo = [to_oracle(t) for t in mpo]
    oracle.two_site_finite_vmps(om, oo, OSP(6, 16, 16, 0.0, OLP(1e-12, 100)))
    _, ops = H.spin_half_ops()
    return om, {k: to_oracle(v) for k, v in ops.items()}


def _exact():
    sz = np.diag([0.5, -0.5])
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])   # basis (up, down): S+ |down> = |up>
    sm = sp.T
    eye = np.eye(2)

    def site_op(o, i):
        m = np.array([[1.0]])
        for k in range(N):
            m = np.kron(m, o if k == i else eye)
        return m
    h = np.zeros((2 ** N, 2 ** N))
    for i in range(N - 1):
        h += site_op(sz, i) @ site_op(sz, i + 1)
        h += 0.5 * (site_op(sp, i) @ site_op(sm, i + 1) + site_op(sm, i) @ site_op(sp, i + 1))
    w, v = np.linalg.eigh(h)
    g = v[:, 0]
    return g, site_op, sz, sp, sm


def test_oracle_measurements_match_exact_diagonalisation():
    om, ops = _ground_state_mps()
    g, site_op, sz, sp, sm = _exact()
    cano = [NONE] * N
    got = measure_one_site(om, cano, ops["sz"])
    ref = [g @ site_op(sz, i) @ g for i in range(N)]
    np.testing.assert_allclose(got, ref, atol=1e-8)
    pairs = [(0, 1), (0, 5), (2, 7), (3, 4)]
    got = measure_two_site(om, cano, ops["sz"], ops["sz"], ops["id"], pairs)
    ref = [g @ site_op(sz, i) @ site_op(sz, j) @ g for i, j in pairs]
    np.testing.assert_allclose(got, ref, atol=1e-8)
    got = measure_two_site(om, cano, ops["sp"], ops["sm"], ops["id"], pairs)
    ref = [g @ site_op(sp, i) @ site_op(sm, j) @ g for i, j in pairs]
    np.testing.assert_allclose(got, ref, atol=1e-8)
