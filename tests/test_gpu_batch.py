"""Batched independent instances (``gq_dmrg_run_batch``): several XXZ chains
of different lengths, anisotropies and bond dimensions swept concurrently,
one host thread and CUDA stream per instance at a time.

Each instance's energy must equal the one from running it alone on the
main stream (same kernels, same order: 1e-13 relative), and the FP64 oracle
pins two of them (1e-10 relative, the per-sweep bar of the plain form).
"""
import numpy as np
import pytest

import oracle
from oracle.lanczos import LanczosParams as OLP
from oracle.vmps import SweepParams as OSP
from mps2_gb300 import hamiltonians as H
from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
from _convert import to_oracle

pytestmark = pytest.mark.gpu

# (L, Delta, D)
CASES = [(8, 0.7, 16), (10, 1.3, 32), (12, 0.55, 16), (14, 1.05, 32), (16, 0.9, 24),
         (10, 1.45, 16)]
SWEEPS = 2
LANCZOS = (1e-10, 60)


@pytest.fixture(scope="module")
def lib():
    from mps2_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    return lib


def _instance(L, delta):
    sv, mpo, qn0, _ = H.heisenberg_chain(L, 1.0, delta)
    mps = FiniteMPS(sv)
    labels = H.neel_shuffled_labels(L, L)
    DirectStateInitMps(mps, labels, qn0)
    return mps, mpo


def _params(D, prec="fp64", sweeps=SWEEPS):
    from mps2_gb300.vmps import LanczosParams, SweepParams
    return SweepParams(sweeps, D, D, 0.0, LanczosParams(*LANCZOS), precision=prec)


@pytest.mark.parametrize("prec", ["fp64", "tf32x3"])
def test_batch_matches_single_instance_runs(lib, prec):
    from mps2_gb300.vmps import DMRGState, run_batch
    single = []
    for L, delta, D in CASES:
        mps, mpo = _instance(L, delta)
        st = DMRGState(mps.tens, mpo)
        st.init_envs(prec)
        e, _ = st.sweep(_params(D, prec))
        single.append(e)
    states, params = [], []
    for L, delta, D in CASES:
        mps, mpo = _instance(L, delta)
        states.append(DMRGState(mps.tens, mpo))
        params.append(_params(D, prec))
    batch = run_batch(states, params, init_envs=True, nthreads=3)
    for (L, delta, D), e1, eb in zip(CASES, single, batch):
        assert abs(eb - e1) <= 1e-13 * abs(e1), (L, delta, D, e1, eb)


def test_batch_energies_match_oracle(lib):
    from mps2_gb300.vmps import DMRGState, run_batch
    picked = [CASES[0], CASES[2]]
    states = []
    for L, delta, D in picked:
        mps, mpo = _instance(L, delta)
        states.append(DMRGState(mps.tens, mpo))
    batch = run_batch(states, [_params(D) for _, _, D in picked], init_envs=True, nthreads=2)
    for (L, delta, D), eb in zip(picked, batch):
        mps, mpo = _instance(L, delta)
        om = [to_oracle(t) for t in mps.tens]
        oo = [to_oracle(t) for t in mpo]
        e_cpu = oracle.two_site_finite_vmps(om, oo, OSP(SWEEPS, D, D, 0.0, OLP(*LANCZOS)))
        assert abs(eb - e_cpu) <= 1e-10 * abs(e_cpu), (L, delta, D, eb, e_cpu)
