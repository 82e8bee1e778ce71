"""Device ``Centralize`` / ``TruncateMPS`` against the oracle and the
reference's canonical-identity checks (``test_finite_mps.cc:66-160,
247-252``)."""
import numpy as np
import pytest

import oracle
from oracle.finite_mps import NONE, centralize, truncate_mps
from mps2_gb300.finite_mps import FiniteMPS
from mps2_gb300.site_vec import SiteVec
from _convert import to_oracle
from _helpers import rel_err
from _mps_case import reference_mps_tensors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from mps2_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    return lib


def _mps(seed):
    rng = np.random.default_rng(seed)
    tens, pb = reference_mps_tensors(rng)
    mps = FiniteMPS(SiteVec(5, pb))
    for i, t in enumerate(tens):
        mps[i] = t
    return mps, [to_oracle(t) for t in tens]


def test_device_centralize_matches_oracle(lib):
    mps, om = _mps(2)
    ocano = [NONE] * 5
    for c in [0, 2, 4, 0, 1, 2, 3, 4]:
        mps.Centralize(c)
        centralize(om, ocano, c)
        assert mps.GetTensCanoType() == ocano
        assert mps.GetCenter() == c
        for i in range(5):
            assert rel_err(mps[i], om[i]) <= 1e-10, (c, i)
        n = 5
        for i in range(n):
            if i == c:
                continue
            t = to_oracle(mps[i])
            axes = ([0] if i == 0 else [0, 1]) if i < c else ([1] if i == n - 1 else [1, 2])
            g = oracle.contract(t, oracle.dag(t), axes, axes).to_dense()
            np.testing.assert_allclose(np.diag(g), 1.0, atol=1e-14)


def test_device_truncate_mps_matches_oracle(lib):
    from mps2_gb300.vmps import TruncateMPS
    mps, om = _mps(4)
    ocano = [NONE] * 5
    for trunc, dmin, dmax in [(0.0, 1, 3), (0.0, 2, 2)]:
        got = TruncateMPS(mps, trunc, dmin, dmax)
        ref = truncate_mps(om, ocano, trunc, dmin, dmax)
        assert [d for _, d in got] == [d for _, d in ref]
        np.testing.assert_allclose([e for e, _ in got], [e for e, _ in ref], atol=1e-12)
        assert mps.GetTensCanoType() == ocano
        for i in range(5):
            assert rel_err(mps[i], om[i]) <= 1e-10, i
