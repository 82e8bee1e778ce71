"""Per-update parity with the FP64 oracle at the benchmark's workload sizes.

The oracle's traces (``tests/golden/trace_*.json``, written by
``tests/golden/make_traces.py``) hold every two-site update's energy E0,
truncation error, kept bond dimension D and entanglement entropy S -- the
fields of the reference's per-update log line
(``two_site_update_finite_vmps_impl.h:329-338``) -- for:

* the Heisenberg chain L=20, D=200, 4 sweeps, Lanczos (1e-9, 100): the
  reference's CPU-runnable configuration;
* a reduced U(1)xU(1) Fermi-Hubbard chain, L=16, U=8, half filling, D=128,
  4 sweeps (the model of the D=4000 benchmark at a size the oracle runs in
  seconds).

The plain FP64 form must reproduce each update: identical D, E0 within
1e-10 relative, and S and the truncation error within the bounds below.
The split form (3xTF32 matvec, FP64-accurate environments and Rayleigh
energies) must reach every sweep's energy within 1e-9 relative with
identical D.  Also here: split-form batched chains against FP64
single-instance runs, and a graded-spectrum SVD with groups of several
hundred rows (the Gram routes) against the oracle's SVD.
"""
import json
import os

import numpy as np
import pytest

import oracle
from mps2_gb300 import hamiltonians as H
from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
from mps2_gb300.tensor import IN, OUT, Index
from _convert import from_oracle, to_oracle
from _helpers import random_tensor, rel_err

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Bounds of the plain form against the oracle, per update.  E0: the
# per-sweep energy bar.  S and the truncation error come from the kept and
# discarded singular values; the GPU's Gram-matrix routes resolve a singular
# value s to about 1e-16 s_max^2 / s absolute, so values near the truncation
# cut (~1e-5 s_max here) carry ~1e-11 relative error and values below
# ~1e-7 s_max count as zero (their weight, < 1e-14 each, is what the
# absolute term of the truncation-error bound allows for).
E0_RTOL = 1e-10
EE_ATOL = 1e-8
TE_RTOL, TE_ATOL = 1e-3, 1e-11
SPLIT_E_RTOL = 1e-9


@pytest.fixture(scope="module")
def lib():
    from mps2_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    return lib


def _load(name):
    with open(os.path.join(GOLDEN, f"trace_{name}.json")) as f:
        return json.load(f)


def _model(name):
    tr = _load(name)
    if name.startswith("heisenberg"):
        sv, mpo, qn0, _ = H.heisenberg_chain(tr["L"])
    else:
        sv, mpo, qn0, _ = H.hubbard_chain(tr["L"], 1.0, 8.0)
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, tr["labels"], qn0)
    return tr, mps, mpo


def _gpu_trace(name, prec, rayleigh="fp64"):
    from mps2_gb300.vmps import DMRGState, LanczosParams, SweepParams
    tr, mps, mpo = _model(name)
    st = DMRGState(mps.tens, mpo)
    st.init_envs(prec)
    sp = SweepParams(1, tr["D"], tr["D"], 0.0, LanczosParams(*tr["lanczos"]), precision=prec,
                     rayleigh=rayleigh)
    stats, sweep_e = [], []
    for _ in range(tr["sweeps"]):
        e0, s = st.sweep(sp)
        stats.extend(s)
        sweep_e.append(e0)
    return tr, stats, sweep_e


@pytest.mark.parametrize("name", ["heisenberg_L20_D200", "hubbard_L16_D128"])
def test_fp64_per_update_trace_matches_oracle(lib, name):
    tr, stats, sweep_e = _gpu_trace(name, "fp64")
    ref = tr["updates"]
    assert len(stats) == len(ref)
    worst = {"e0": 0.0, "ee": 0.0, "te": 0.0}
    for k, (g, o) in enumerate(zip(stats, ref)):
        where = (k, o["site"], o["dir"])
        assert (g.site, g.dir) == (o["site"], o["dir"]), where
        assert g.D == o["D"], (where, g.D, o["D"])
        de = abs(g.e0 - o["e0"]) / abs(o["e0"])
        dee = abs(g.ee - o["ee"])
        dte = abs(g.trunc_err - o["trunc_err"])
        worst["e0"] = max(worst["e0"], de)
        worst["ee"] = max(worst["ee"], dee)
        worst["te"] = max(worst["te"], dte / (TE_RTOL * o["trunc_err"] + TE_ATOL))
        assert de <= E0_RTOL, (where, g.e0, o["e0"])
        assert dee <= EE_ATOL, (where, g.ee, o["ee"])
        assert dte <= TE_RTOL * o["trunc_err"] + TE_ATOL, (where, g.trunc_err, o["trunc_err"])
    for e, o in zip(sweep_e, tr["sweep_energies"]):
        assert abs(e - o) <= E0_RTOL * abs(o)
    print(name, "worst relative E0 / absolute S / truncation-error bound fraction:", worst)


@pytest.mark.parametrize("name", ["heisenberg_L20_D200", "hubbard_L16_D128"])
def test_split_form_every_sweep_matches_oracle(lib, name):
    tr, stats, sweep_e = _gpu_trace(name, "tf32x3", rayleigh="fp64tc")
    ref = tr["updates"]
    assert [s.D for s in stats] == [o["D"] for o in ref]
    dev = [abs(e - o) / abs(o) for e, o in zip(sweep_e, tr["sweep_energies"])]
    print(name, "split form per-sweep |dE/E|:", dev)
    assert max(dev) <= SPLIT_E_RTOL, dev
    # S and the truncation error of the split form's ground states
    dee = max(abs(g.ee - o["ee"]) for g, o in zip(stats, ref))
    print(name, "split form max |dS|:", dee)
    assert dee <= 1e-5


def test_split_form_batched_chains_match_fp64_single_runs(lib):
    """Batched XXZ chains in the split form (FP32-split products with FP64
    Lanczos and FP64-accurate Rayleigh energies), run concurrently, against
    the same chains run one at a time in the plain FP64 form."""
    from mps2_gb300.vmps import DMRGState, LanczosParams, SweepParams, run_batch
    cases = [(16, 0.6, 64), (20, 1.2, 64), (24, 0.9, 128), (18, 1.45, 32), (22, 0.75, 96),
             (16, 1.1, 48)]
    lp = LanczosParams(1e-10, 100)

    def chain(L, delta):
        sv, mpo, qn0, _ = H.heisenberg_chain(L, 1.0, delta)
        mps = FiniteMPS(sv)
        DirectStateInitMps(mps, H.neel_shuffled_labels(L, L), qn0)
        return mps, mpo

    fp64 = []
    for L, delta, D in cases:
        mps, mpo = chain(L, delta)
        st = DMRGState(mps.tens, mpo)
        st.init_envs("fp64")
        fp64.append(st.sweep(SweepParams(4, D, D, 0.0, lp, precision="fp64"))[0])
    states, params = [], []
    for L, delta, D in cases:
        mps, mpo = chain(L, delta)
        states.append(DMRGState(mps.tens, mpo))
        params.append(SweepParams(4, D, D, 0.0, lp, precision="tf32x3", rayleigh="fp64tc"))
    split = run_batch(states, params, init_envs=True, nthreads=3)
    dev = [abs(s - e) / abs(e) for s, e in zip(split, fp64)]
    print("batched split vs FP64 single |dE/E|:", dev)
    assert max(dev) <= SPLIT_E_RTOL, dev


def _scale_leg(t, leg, s):
    out = t.copy()
    offs = np.cumsum([0] + [d for _, d in t.indices[leg].sectors()])
    for k in out.blocks:
        sh = [1] * out.blocks[k].ndim
        sh[leg] = -1
        out.blocks[k] = out.blocks[k] * s[offs[k[leg]]:offs[k[leg] + 1]].reshape(sh)
    return out


@pytest.mark.parametrize("dmax", [1000, 1600])
@pytest.mark.parametrize("scale_side", [1, 2])
def test_graded_spectrum_large_groups_svd_matches_oracle(lib, scale_side, dmax):
    """Groups of ~1150 x ~1150 (every one on a Gram route, with FP64-accurate
    tensor-core Gram products) whose singular values are graded over about
    twelve decades, as a converged two-site state's are: D, the truncation
    error and the kept singular values against the oracle's SVD, and the
    truncated product U.S.Vt against the oracle's.  With D=1000 the cut lies
    near 1e-5 s_max; with D=1600 near 1e-8 s_max, so that about 150 kept
    values lie below the Gram routes' floor (~1e-7 of the group's largest),
    where the GPU keeps them as zeros with orthonormal completion vectors
    instead of the oracle's singular vectors: the product then differs by
    the weight of those values, which the bound below allows for and the
    test prints."""
    from mps2_gb300.vmps import SVD
    rng = np.random.default_rng(33)
    l = Index([((-1,), 600), ((1,), 560)], IN)
    r = Index([((-1,), 590), ((1,), 570)], OUT)
    s1 = Index([((1,), 1), ((-1,), 1)], OUT)
    s2 = Index([((1,), 1), ((-1,), 1)], OUT)
    t = random_tensor(rng, [l, s1, s2, r], (0,))
    gl = 10.0 ** (-6.0 * rng.permutation(l.dim) / l.dim)
    gr = 10.0 ** (-6.0 * rng.permutation(r.dim) / r.dim)
    t = _scale_leg(_scale_leg(t, 0, gl), 3, gr)
    ref = oracle.svd(to_oracle(t), 2, (0,), 0.0, 1, dmax)
    u, s, vt, err, D = SVD(t, 2, (0,), 0.0, 1, dmax, scale_side=scale_side)
    assert D == ref.D
    rs = np.asarray(ref.svals)
    smax = rs.max()
    # a value s is resolved to ~1e-16 s_max^2 / s by the Gram routes
    atol = 1e-13 * smax ** 2 / np.maximum(rs, 1e-300)
    big = rs > 1e-6 * smax
    assert np.all(np.abs(np.asarray(s)[big] - rs[big]) <= atol[big] + 1e-12 * rs[big])
    assert abs(err - ref.trunc_err) <= TE_RTOL * ref.trunc_err + TE_ATOL, (err, ref.trunc_err)
    ru, rvt = from_oracle(ref.u), from_oracle(ref.vt)
    if scale_side == 2:
        rvt = _scale_leg(rvt, 0, rs)
    else:
        ru = _scale_leg(ru, 2, rs)
    prod = oracle.contract(to_oracle(u), to_oracle(vt), [2], [0])
    prod_ref = oracle.contract(to_oracle(ru), to_oracle(rvt), [2], [0])
    below = np.sqrt(np.sum(rs[rs <= 2e-7 * smax] ** 2) / np.sum(rs ** 2))
    dev = rel_err(from_oracle(prod), prod_ref)
    print(f"D={dmax} side={scale_side}: |U.S.Vt - oracle| / |oracle| = {dev:.2e}, weight of "
          f"kept values below the floor {below:.2e}")
    assert dev <= 1e-9 + 2.0 * below
