"""The oracle's Centralize / TruncateMPS against the reference's own checks
(``test_finite_mps.cc:66-160, 247-252``): after ``Centralize(c)`` every
site left of c is left-canonical and every site right of it
right-canonical (A^dag A = identity, diagonal within 1e-15, the
reference's bound), the canonical types follow, and the state itself is
unchanged."""
import numpy as np

import oracle
from oracle.finite_mps import LEFT, NONE, RIGHT, centralize, truncate_mps
from _convert import to_oracle
from _mps_case import reference_mps_tensors


def _state(mps):
    """Dense wavefunction of a small MPS (site order)."""
    psi = mps[0].to_dense()
    for t in mps[1:]:
        psi = np.tensordot(psi, t.to_dense(), axes=([psi.ndim - 1], [0]))
    return psi


def _check_center(mps, cano, center):
    n = len(mps)
    for i in range(n):
        if i == center:
            assert cano[i] == NONE
            continue
        t = mps[i]
        if i < center:
            assert cano[i] == LEFT
            axes = [0] if i == 0 else [0, 1]
        else:
            assert cano[i] == RIGHT
            axes = [1] if i == n - 1 else [1, 2]
        g = oracle.contract(t, oracle.dag(t), axes, axes).to_dense()
        assert g.shape[0] == g.shape[1]
        np.testing.assert_allclose(np.diag(g), 1.0, atol=1e-15)


def test_oracle_centralize_matches_reference_checks():
    rng = np.random.default_rng(2)
    tens, _ = reference_mps_tensors(rng)
    mps = [to_oracle(t) for t in tens]
    cano = [NONE] * 5
    psi0 = _state(mps)
    for c in [0, 2, 4, 0, 1, 2, 3, 4]:
        centralize(mps, cano, c)
        _check_center(mps, cano, c)
        np.testing.assert_allclose(_state(mps), psi0, atol=1e-12)


def test_oracle_truncate_mps_runs_the_reference_cases():
    rng = np.random.default_rng(4)
    tens, _ = reference_mps_tensors(rng)
    mps = [to_oracle(t) for t in tens]
    cano = [NONE] * 5
    res = truncate_mps(mps, cano, 0.0, 1, 3)
    assert all(D <= 3 for _, D in res)
    res = truncate_mps(mps, cano, 0.0, 2, 2)
    assert all(D <= 2 for _, D in res)
    assert cano == [NONE] * 5
    nrm = np.linalg.norm(_state(mps))
    assert abs(nrm - 1.0) <= 1e-12
