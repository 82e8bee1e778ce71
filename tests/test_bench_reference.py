"""The CPU legs of ``bench.py`` (host only): the reference arm's per-bond
CPU update on random tensors with a recorded block structure, and the
estimate of a sweep from evenly spaced bonds."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_sample_bonds_cover_the_chain():
    import bench
    b = bench._sample_bonds(64)
    assert b == sorted(b) and len(set(b)) == len(b) == bench.N_BONDS
    assert 1 <= b[0] <= 8 and 55 <= b[-1] <= 61
    gaps = np.diff(b)
    assert gaps.max() - gaps.min() <= 1


def test_reference_update_on_recorded_structure(tmp_path, capsys):
    """A bond structure taken from a small oracle state (Hubbard, bulk sites
    of the 64-site model's MPO) runs through the reference arm's synthetic
    update and sweep estimate."""
    import bench
    import oracle
    from _convert import from_oracle, to_oracle
    from mps2_gb300 import hamiltonians as H
    from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
    from oracle.lanczos import LanczosParams as OLP
    from oracle.vmps import SweepParams as OSP, two_site_update
    sv, mpo, qn0, _ = H.hubbard_chain(8, 1.0, 8.0)
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, [1 if i % 2 == 0 else 2 for i in range(8)], qn0)
    om = [to_oracle(t) for t in mps.tens]
    oo = [to_oracle(t) for t in mpo]
    sp = OSP(1, 16, 16, 0.0, OLP(1e-8, 20))
    envs = {}
    oracle.two_site_finite_vmps(om, oo, sp, envs=envs)
    b, L = 3, 64
    # a consistent state at bond b: the 'r' half sweep up to it
    for i in range(b):
        two_site_update(om, oo, envs, sp, "r", i)
    A, B = from_oracle(om[b]), from_oracle(om[b + 1])
    Le, Re = from_oracle(envs[("l", b)]), from_oracle(envs[("r", 8 - b - 2)])
    rec = {"site": b, "iters": 2, "theta_size": 0,
           "A_c": [bench._describe_index(ix) for ix in A.indices],
           "A_c1": [bench._describe_index(ix) for ix in B.indices],
           "L_env": [bench._describe_index(ix) for ix in Le.indices],
           "R_env": [bench._describe_index(ix) for ix in Re.indices],
           "div_c": list(A.div), "div_c1": list(B.div), "div_l": list(Le.div),
           "div_r": list(Re.div)}
    mpsd, mpo64, env = bench._synthetic_bond("hubbard", L, rec, seed=1)
    assert len(mpo64) == L
    t, st = bench._oracle_update(mpsd, mpo64, env, b, 16, rec["iters"])
    assert t > 0 and np.isfinite(st.e0) and 1 <= st.D <= 16
    fix = tmp_path / "bench_bonds_hubbard.json"
    fix.write_text(json.dumps({"L": L, "D": 16, "model": "hubbard", "bonds": [rec]}))

    class Args:
        model, steps, warmup, gpus = "hubbard", 2, 1, 1
    old = bench._structure_fixture
    bench._structure_fixture = lambda model: str(fix)
    try:
        bench.run_reference(Args())
    finally:
        bench._structure_fixture = old
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "s/sweep"
    assert line["value"] == pytest.approx(2 * (L - 1) * line["ms_per_step"] * 1e-3)
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "s/sweep", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["higher_is_better"] is False and line["steps"] == 2 and line["warmup"] == 1
