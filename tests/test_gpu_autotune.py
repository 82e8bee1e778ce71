"""Tile-choice autotuner: with it on, every new block-size histogram of a
matvec contraction times the candidate tensor-core thresholds once; the
results must not depend on the choice beyond the form's own accuracy
(FP64-accurate form: per-sweep energies equal to 1e-11)."""
import pytest

from mps2_gb300 import hamiltonians as H
from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from mps2_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    return lib


def _sweeps(prec, tuned):
    from mps2_gb300.vmps import DMRGState, LanczosParams, SweepParams, autotune_enable
    N, D = 20, 300
    sv, mpo, qn0, _ = H.heisenberg_chain(N)
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, H.neel_shuffled_labels(N, 0), qn0)
    autotune_enable(tuned)
    try:
        st = DMRGState(mps.tens, mpo)
        st.init_envs(prec)
        sp = SweepParams(1, D, D, 0.0, LanczosParams(1e-10, 100), precision=prec)
        return [st.sweep(sp)[0] for _ in range(3)]
    finally:
        autotune_enable(False)


def test_autotuned_sweeps_match_fixed_thresholds(lib):
    fixed = _sweeps("fp64tc", False)
    tuned = _sweeps("fp64tc", True)
    tuned_again = _sweeps("fp64tc", True)   # second run: every signature cached
    for a, b, c in zip(fixed, tuned, tuned_again):
        assert abs(a - b) <= 1e-11 * abs(a)
        assert abs(a - c) <= 1e-11 * abs(a)
