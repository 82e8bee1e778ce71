"""The header-only C++ front end (``include/gqmps2_gb300.hpp``) compiled with
g++ against the library: its host parts on the CPU (tensor files shared with
the Python side, ``DirectStateInitMps``, ``SiteVec``, ``TenVec``), and on the
GPU the reference's 1DHeisenberg DMRG case restated in C++
(``test_two_site_update_finite_vmps.cc:186-220``: golden energy
-2.493577133888 to 1e-12, then a resumed call), a ``LanczosSolver``,
``FiniteMPS::Centralize``, ``TruncateMPS`` and the measurements through the
same header (against the Python API on the same state)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "shim_test.cpp")
GOLDEN_1D_HEISENBERG = -2.493577133888


@pytest.fixture(scope="module")
def shim_exe(tmp_path_factory):
    from mps2_gb300 import build
    so = build.build()
    libdir = os.path.dirname(os.path.abspath(so))
    exe = str(tmp_path_factory.mktemp("shim") / "shim_test")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", f"-I{os.path.join(ROOT, 'include')}", SRC,
           "-o", exe, f"-L{libdir}", "-lgqmps2_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run(exe, mode, d, timeout):
    r = subprocess.run([exe, mode, str(d)], capture_output=True, text=True, timeout=timeout)
    return r.returncode, r.stdout, r.stderr


def test_cpp_shim_host(shim_exe, tmp_path):
    from _helpers import random_index, random_tensor
    from mps2_gb300 import hamiltonians as H
    from mps2_gb300.finite_mps import (DirectStateInitMps, FiniteMPS, GenMPSTenName,
                                       read_tensor, write_tensor)
    from mps2_gb300.tensor import IN, OUT
    rng = np.random.default_rng(5)
    t = random_tensor(rng, [random_index(rng, 3, 2, 4, IN, nq=2),
                            random_index(rng, 2, 1, 3, OUT, nq=2),
                            random_index(rng, 4, 2, 4, OUT, nq=2)], (0, 0))
    write_tensor(t, str(tmp_path / "in.gqten"))
    rc, out, err = _run(shim_exe, "host", tmp_path, 60)
    assert rc == 0, out + err
    assert "host ok" in out
    # DumpMeasuRes writes what the Python DumpMeasuRes writes
    from mps2_gb300.measure import DumpMeasuRes, MeasuResElem
    DumpMeasuRes([MeasuResElem([0], 0.25), MeasuResElem([1, 4], -0.125)], str(tmp_path / "py"))
    assert (tmp_path / "measu.json").read_text() == (tmp_path / "py.json").read_text()
    # the C++ writer reproduces the Python file byte for byte
    assert (tmp_path / "out.gqten").read_bytes() == (tmp_path / "in.gqten").read_bytes()
    # DirectStateInitMps agrees with the Python one
    sv, _, qn0, _ = H.heisenberg_chain(6)
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, [i % 2 for i in range(6)], qn0)
    for i in range(6):
        c = read_tensor(GenMPSTenName(str(tmp_path / "mps"), i))
        assert c.indices == mps[i].indices and tuple(c.div) == tuple(mps[i].div)
        assert c.dense_equal(mps[i])


@pytest.mark.gpu
def test_cpp_shim_dmrg(shim_exe, tmp_path):
    from mps2_gb300 import hamiltonians as H
    from mps2_gb300.finite_mps import write_tensor
    _, mpo, _, _ = H.heisenberg_chain(6)
    os.makedirs(tmp_path / "mpo")
    for i, w in enumerate(mpo):
        write_tensor(w, str(tmp_path / "mpo" / f"mpo_ten{i}.gqten"))
    rc, out, err = _run(shim_exe, "dmrg", tmp_path, 300)
    assert rc == 0, out + err
    vals = {}
    for line in out.splitlines():
        k, _, v = line.partition(" ")
        vals[k] = v
    assert vals["failures"] == "0", out
    assert abs(float(vals["e0"]) - GOLDEN_1D_HEISENBERG) <= 1e-12
    assert abs(float(vals["e0_resume"]) - GOLDEN_1D_HEISENBERG) <= 1e-12
    assert int(vals["updates"]) == 4 * 2 * 5
    assert abs(float(vals["lanczos_e"]) - GOLDEN_1D_HEISENBERG) <= 1e-10
    assert vals["center"] == "3"
    assert vals["cano"].split() == ["1", "1", "1", "0", "2", "2"]
    assert float(vals["left_canonical_err"]) <= 1e-13
    # TruncateMPS to D = 2 (test_finite_mps.cc: every bond within Dmax, the
    # state normalised)
    assert int(vals["truncate_bonds"]) == 5
    assert int(vals["truncate_dmax"]) == 2
    assert abs(float(vals["truncate_norm"]) - 1.0) <= 1e-12
    # measurements through the C++ header against the Python API on the same
    # MPS (finite_mps_measu.h); the singlet ground state has <Sz_i> = 0
    import json
    from mps2_gb300.finite_mps import FiniteMPS
    from mps2_gb300.measure import MeasureOneSiteOp, MeasureTwoSiteOp
    sv, _, _, _ = H.heisenberg_chain(6)
    _, ops = H.spin_half_ops()
    pm = FiniteMPS(sv)
    pm.Load(str(tmp_path / "mps_meas"))
    py1 = MeasureOneSiteOp(pm, ops["sz"], str(tmp_path / "py_sz"))
    pairs = [[0, 1], [0, 3], [2, 5], [1, 4]]
    py2 = MeasureTwoSiteOp(pm, [ops["sz"], ops["sz"]], ops["id"], pairs, str(tmp_path / "py_szsz"))
    c1 = json.load(open(tmp_path / "sz.json"))
    c2 = json.load(open(tmp_path / "szsz.json"))
    assert int(vals["meas_one"]) == 6 and int(vals["meas_two"]) == 4
    assert vals["meas_center"] == "1"   # the last event started at site 1
    assert [e[0] for e in c1] == [[i] for i in range(6)] and [e[0] for e in c2] == pairs
    for (sites, v), e in zip(c1, py1):
        assert abs(v - e.avg) <= 1e-11 and abs(v) <= 1e-10
    for (sites, v), e in zip(c2, py2):
        assert abs(v - e.avg) <= 1e-11
    assert c2[0][1] < -0.1   # nearest neighbours anti-aligned
    # split form: 3xTF32 products, FP64-accurate energy; 1e-9 relative
    assert abs(float(vals["e0_split"]) - GOLDEN_1D_HEISENBERG) <= 1e-9 * abs(GOLDEN_1D_HEISENBERG)
