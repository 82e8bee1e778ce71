"""The MRRR building block of the eigensolver (``mps2_gb300/csrc/mrrr.cuh``)
on the host: tridiagonal matrices from LAPACK's ``dsytrd`` of graded positive
semi-definite matrices shaped like DMRG Gram matrices (spectra over 16
decades).  For the eigenvalues above 1e-14 of the largest: the values match
``eigh_tridiagonal``; every vector has a float64 residual; vectors of
eigenvalues with relative gaps above 1e-2 and above T's noise level are
orthogonal without any re-orthogonalisation; after the small clusters are
orthonormalised and one CholeskyQR2 pass, the whole set is orthonormal to
float64 precision."""
import os
import subprocess

import numpy as np
import pytest
import scipy.linalg as sl
from scipy.linalg import lapack

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "mrrr_test.cpp")
FLOOR = 1e-14


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("mrrr") / "mrrr_test")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", SRC, "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _graded(n, decades, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) * (10.0 ** (-decades / 2 * np.arange(n) / n))[None, :]
    return B @ B.T


def _tridiag(A):
    c, d, e, tau, info = lapack.dsytrd(A, lower=1)
    assert info == 0
    return d, e


def test_mrrr_eigenpairs_above_the_floor(exe, tmp_path):
    cases = [(_graded(n, dec, s), n) for n, dec, s in
             [(40, 16, 1), (120, 16, 2), (257, 16, 3), (300, 10, 4), (200, 20, 5)]]
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        for A, n in cases:
            d, e = _tridiag(A)
            f.write(np.int32(n).tobytes() + d.tobytes() + e.tobytes())
    r = subprocess.run([exe, str(inp), str(tmp_path / "out.bin"), str(FLOOR)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    buf = open(tmp_path / "out.bin", "rb").read()
    off = 0
    for A, n in cases:
        d, e = _tridiag(A)
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        tn = np.abs(d).max() + 2 * np.abs(e).max()
        k = int(np.frombuffer(buf, np.int32, 1, off)[0]); off += 4
        sigma = float(np.frombuffer(buf, np.float64, 1, off)[0]); off += 8
        lam = np.frombuffer(buf, np.float64, k, off).copy(); off += 8 * k
        Z = np.frombuffer(buf, np.float64, n * k, off).reshape(k, n).T.copy(); off += 8 * n * k
        ref = sl.eigh_tridiagonal(d, e, eigvals_only=True)
        lmax = ref[-1]
        assert k >= 1 and np.all(np.diff(lam) >= 0)
        kk = min(k, int((ref > FLOOR * lmax).sum()))
        assert np.abs(lam[-kk:] - ref[-kk:]).max() <= 8e-15 * lmax
        res = np.linalg.norm(T @ Z - Z * lam[None, :], axis=0) / tn
        assert res.max() <= 1e-14
        # well separated (relative gap > 1e-2 on both sides, above the noise
        # level) -> orthogonal as computed
        mu = lam - sigma
        gap = np.minimum(np.r_[np.inf, np.diff(mu)], np.r_[np.diff(mu), np.inf]) / mu
        sep = (gap > 1e-2) & (mu > 8 * abs(sigma))
        Zs = Z[:, sep]
        assert np.abs(Zs.T @ Zs - np.eye(Zs.shape[1])).max() <= 1e-10
        # small clusters and the noise-level block orthonormalised, then CholeskyQR2
        start = 0
        for i in range(1, k + 1):
            if i == k or (mu[i] > 8 * abs(sigma) and mu[i] - mu[i - 1] > 1e-3 * mu[i]):
                if i - start > 1:
                    Z[:, start:i] = np.linalg.qr(Z[:, start:i])[0]
                start = i
        for _ in range(2):
            R = np.linalg.cholesky(Z.T @ Z).T
            Z = sl.solve_triangular(R, Z.T, trans="T", lower=False).T
        assert np.abs(Z.T @ Z - np.eye(k)).max() <= 1e-14
        assert (np.linalg.norm(T @ Z - Z * lam[None, :], axis=0) / tn).max() <= 1e-14
