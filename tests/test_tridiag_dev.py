"""The Lanczos tridiagonal solver of the device loop
(``mps2_gb300/csrc/tridiag_dev.cuh``: multisection on Sturm counts for the
lowest eigenvalue, inverse iteration for its vector) run on the host against
``scipy.linalg.eigh_tridiagonal``: Lanczos matrices of random symmetric
operators, random and graded tridiagonals, split (zero off-diagonal) and
nearly split matrices, sizes 1 to 300."""
import os
import subprocess

import numpy as np
import pytest
import scipy.linalg as sl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "tridiag_test.cpp")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("tridiag") / "tridiag_test")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", SRC, "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _lanczos_matrix(n, m, seed):
    """a, b of m Lanczos steps (no re-orthogonalisation, as the solver) on a
    random symmetric n x n operator."""
    rng = np.random.default_rng(seed)
    H = rng.standard_normal((n, n))
    H = H + H.T
    v = rng.standard_normal(n)
    v /= np.linalg.norm(v)
    a, b, vp, beta = [], [], np.zeros(n), 0.0
    for _ in range(m):
        w = H @ v - beta * vp
        al = v @ w
        w -= al * v
        a.append(al)
        beta = np.linalg.norm(w)
        if len(a) < m:
            b.append(beta)
        vp, v = v, w / beta
    return np.array(a), np.array(b)


def _cases():
    rng = np.random.default_rng(3)
    out = [(np.array([-1.5]), np.zeros(0)), (np.array([1.0, 2.0]), np.array([0.5])),
           (np.array([0.0, 0.0]), np.array([1.0]))]
    for n, m, s in [(200, 2, 1), (200, 3, 2), (400, 20, 3), (400, 60, 4), (600, 100, 5)]:
        out.append(_lanczos_matrix(n, m, s))
    for n in (5, 17, 64, 300):
        out.append((rng.standard_normal(n), rng.standard_normal(n - 1)))
    a = rng.standard_normal(30) * 10.0 ** rng.uniform(-8, 8, 30)
    out.append((a, rng.standard_normal(29) * 10.0 ** rng.uniform(-8, 8, 29)))
    b = rng.standard_normal(39)
    b[[5, 20]] = 0.0                                         # split matrix
    out.append((rng.standard_normal(40), b))
    b = rng.standard_normal(39)
    b[[7, 30]] = 1e-13                                       # nearly split
    out.append((rng.standard_normal(40), b))
    out.append((np.full(12, 2.0), np.full(11, 1e-9)))        # tight cluster
    out.append((np.array([-20.7551371, -20.7551370]), np.array([3e-6])))  # converged Lanczos
    return out


def test_lowest_eigenpair_matches_eigh_tridiagonal(exe, tmp_path):
    cases = _cases()
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        for a, b in cases:
            f.write(np.int32(a.size).tobytes() + a.astype(np.float64).tobytes()
                    + b.astype(np.float64).tobytes())
    r = subprocess.run([exe, str(inp), str(tmp_path / "out.bin")], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    buf = np.frombuffer(open(tmp_path / "out.bin", "rb").read(), dtype=np.float64)
    off = 0
    for a, b in cases:
        n = a.size
        lam, vec = buf[off], buf[off + 1:off + 1 + n]
        off += 1 + n
        w, V = sl.eigh_tridiagonal(a, b) if n > 1 else (a.copy(), np.ones((1, 1)))
        tn = np.abs(a).max() + 2 * (np.abs(b).max() if n > 1 else 0.0)
        # eigenvalue: a few units of the matrix scale
        assert abs(lam - w[0]) <= 8 * 2.2e-16 * tn, (n, lam, w[0])
        # vector: unit length, float64 residual, largest component positive
        T = np.diag(a) + (np.diag(b, 1) + np.diag(b, -1) if n > 1 else 0.0)
        assert abs(np.linalg.norm(vec) - 1.0) <= 1e-14
        assert np.linalg.norm(T @ vec - lam * vec) <= 1e-13 * tn, n
        assert vec[np.argmax(np.abs(vec))] > 0
        # and the same vector as LAPACK's wherever the lowest value is isolated
        gap = (w[1] - w[0]) if n > 1 else np.inf
        if gap > 1e-6 * tn:
            ref = V[:, 0] * np.sign(V[np.argmax(np.abs(V[:, 0])), 0])
            assert np.abs(vec - ref).max() <= 1e-12 * tn / gap + 1e-14, n
