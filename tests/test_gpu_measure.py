"""Device finite-MPS measurements (``mps2_gb300.measure``) against the
oracle's on the same DMRG ground state (10-site Heisenberg chain, D=16),
and the reference's result-file format."""
import json

import numpy as np
import pytest

import oracle
from oracle.finite_mps import NONE
from oracle.lanczos import LanczosParams as OLP
from oracle.measure import measure_one_site, measure_two_site
from oracle.vmps import SweepParams as OSP
from mps2_gb300 import hamiltonians as H
from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
from _convert import from_oracle, to_oracle

pytestmark = pytest.mark.gpu

N = 10


@pytest.fixture(scope="module")
def lib():
    from mps2_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    return lib


def _state():
    sv, mpo, qn0, _ = H.heisenberg_chain(N)
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, H.neel_shuffled_labels(N, 0), qn0)
    om = [to_oracle(t) for t in mps.tens]
    oo = [to_oracle(t) for t in mpo]
    oracle.two_site_finite_vmps(om, oo, OSP(4, 16, 16, 0.0, OLP(1e-12, 100)))
    dev = FiniteMPS(sv)
    for i, t in enumerate(om):
        dev[i] = from_oracle(t)
    dev.tens_cano_type = [NONE] * N
    _, ops = H.spin_half_ops()
    return dev, om, ops


def test_measure_one_site_matches_oracle(lib, tmp_path):
    from mps2_gb300.measure import MeasureOneSiteOp
    dev, om, ops = _state()
    res = MeasureOneSiteOp(dev, ops["sz"], str(tmp_path / "sz"))
    ref = measure_one_site(om, [NONE] * N, to_oracle(ops["sz"]))
    np.testing.assert_allclose([r.avg for r in res], ref, atol=1e-12)
    assert [r.sites for r in res] == [[i] for i in range(N)]
    assert dev.GetCenter() == N - 1
    data = json.load(open(tmp_path / "sz.json"))
    assert [d[0] for d in data] == [[i] for i in range(N)]
    np.testing.assert_allclose([d[1] for d in data], ref, atol=1e-11)


def test_measure_two_site_matches_oracle(lib, tmp_path):
    from mps2_gb300.measure import MeasureOneSiteOp, MeasureTwoSiteOp
    dev, om, ops = _state()
    pairs = [[0, 1], [0, 6], [2, 9], [4, 5], [3, 8]]
    res = MeasureTwoSiteOp(dev, [ops["sp"], ops["sm"]], ops["id"], pairs,
                           str(tmp_path / "spsm"))
    ref = measure_two_site(om, [NONE] * N, to_oracle(ops["sp"]), to_oracle(ops["sm"]),
                           to_oracle(ops["id"]), [tuple(p) for p in pairs])
    np.testing.assert_allclose([r.avg for r in res], ref, atol=1e-12)
    # the per-event insert-operator overload gives the same numbers
    inst = [[ops["id"]] * (j - i - 1) for i, j in pairs]
    res2 = MeasureTwoSiteOp(dev, [ops["sp"], ops["sm"]], inst, pairs, str(tmp_path / "spsm2"))
    np.testing.assert_allclose([r.avg for r in res2], ref, atol=1e-12)
    # a list of one-site operators
    sets = MeasureOneSiteOp(dev, [ops["sz"], ops["id"]], [str(tmp_path / "a"),
                                                         str(tmp_path / "b")])
    np.testing.assert_allclose([r.avg for r in sets[1]], 1.0, atol=1e-12)
