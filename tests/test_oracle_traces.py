"""The committed per-update oracle traces (``tests/golden/trace_*.json``) are
what the oracle computes, and the Heisenberg L=20, D=200 trace ends at the
exact ground-state energy of that chain (sparse exact diagonalisation of the
Sz=0 sector, 184756 states) to the accuracy D=200 allows."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, f"trace_{name}.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("name", ["heisenberg_L20_D200", "hubbard_L16_D128"])
def test_trace_fixture_is_the_oracles(name):
    from golden.make_traces import trace
    ref = _load(name)
    got = trace(name)
    assert len(got["updates"]) == len(ref["updates"])
    for g, o in zip(got["updates"], ref["updates"]):
        assert (g["site"], g["dir"], g["D"]) == (o["site"], o["dir"], o["D"])
        assert abs(g["e0"] - o["e0"]) <= 1e-12 * abs(o["e0"])
        assert abs(g["ee"] - o["ee"]) <= 1e-10
        assert abs(g["trunc_err"] - o["trunc_err"]) <= 1e-9 * o["trunc_err"] + 1e-15


def _heisenberg_obc_ground_energy(L):
    """Lowest eigenvalue of sum_i S_i.S_{i+1} (open chain) in the Sz=0 sector."""
    import itertools
    import scipy.sparse as sp
    from scipy.sparse.linalg import eigsh
    states = np.array([sum(1 << i for i in c) for c in itertools.combinations(range(L), L // 2)],
                      dtype=np.int64)
    states.sort()
    n = len(states)
    diag = np.zeros(n)
    rows, cols = [], []
    for i in range(L - 1):
        bi = (states >> i) & 1
        bj = (states >> (i + 1)) & 1
        diag += np.where(bi == bj, 0.25, -0.25)
        flip = np.nonzero(bi != bj)[0]
        partner = states[flip] ^ ((1 << i) | (1 << (i + 1)))
        rows.append(flip)
        cols.append(np.searchsorted(states, partner))
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    h = sp.csr_matrix((np.full(len(r), 0.5), (r, c)), shape=(n, n)) + sp.diags(diag)
    return float(eigsh(h, k=1, which="SA", tol=1e-12)[0][0])


def test_heisenberg_trace_reaches_exact_ground_energy():
    tr = _load("heisenberg_L20_D200")
    e_ed = _heisenberg_obc_ground_energy(tr["L"])
    e_dmrg = tr["sweep_energies"][-1]
    assert e_dmrg >= e_ed - 1e-10          # variational
    assert (e_dmrg - e_ed) / abs(e_ed) <= 1e-8, (e_dmrg, e_ed)
