"""Host-side logic that needs no GPU: parameter validation of the Python
API, the measurement result-file format, the batched-instance workload
definition and the C ABI's struct layouts."""
import ctypes as C
import json

import pytest

from mps2_gb300 import _lib
from mps2_gb300.measure import DumpMeasuRes, MeasuResElem
from mps2_gb300.vmps import LanczosParams, SweepParams


def test_sweep_params_validate_precision_names():
    sp = SweepParams(1, 8, 8, 0.0, LanczosParams(1e-8), precision="tf32x3", rayleigh="fp64tc")
    c = sp.to_c()
    assert c.precision == _lib.PREC_TF32X3
    assert c.lanczos.rayleigh == _lib.PREC_FP64TC
    for bad in ("fp32", "tf32"):
        with pytest.raises(ValueError):
            SweepParams(1, 8, 8, 0.0, precision=bad)
    with pytest.raises(ValueError):
        SweepParams(1, 8, 8, 0.0, rayleigh="tf32x3")


def test_ctypes_structs_match_the_c_layout():
    # gq_lanczos_params {double, int64, int} and gq_sweep_params as declared
    assert C.sizeof(_lib.LanczosParamsC) == 24
    assert _lib.SweepParamsC.lanczos.offset == 32
    assert C.sizeof(_lib.SweepParamsC) == 64


def test_measurement_file_format(tmp_path):
    res = [MeasuResElem([0], 0.25), MeasuResElem([1, 4], -0.125)]
    DumpMeasuRes(res, str(tmp_path / "m"))
    text = open(tmp_path / "m.json").read()
    assert text.startswith("[\n  [[0], ") and text.endswith("]")
    data = json.loads(text)
    assert data == [[[0], 0.25], [[1, 4], -0.125]]


def test_batched_workload_definition():
    import bench
    cases = bench.batched_instances(64)
    assert len(cases) == 64
    assert all(16 <= L <= 64 and L % 2 == 0 for L, _, _ in cases)
    assert all(0.5 <= d <= 1.5 for _, d, _ in cases)
    assert {D for _, _, D in cases} <= {64, 128, 256, 512}
    assert cases == bench.batched_instances(64)   # seeded


def _is_id_op(t):
    """``test_site_vec.cc:22-39``: rank 2, square, (IN, OUT) legs that are
    each other's inverse, identity elements."""
    import numpy as np
    from mps2_gb300.tensor import IN
    assert len(t.indices) == 2 and t.indices[0].dim == t.indices[1].dim
    assert t.indices[0].dir == IN and t.indices[0].inverse() == t.indices[1]
    assert np.array_equal(t.to_dense(), np.eye(t.indices[0].dim))


def test_site_vec_basic_features():
    """``test_site_vec.cc:78-101``: the same local spaces, uniform and mixed."""
    from mps2_gb300.site_vec import SiteVec
    from mps2_gb300.tensor import Index, OUT
    pb_out1 = Index([((0,), 1), ((1,), 1)], OUT)
    pb_out2 = Index([((1,), 3)], OUT)
    pb_in1, pb_in2 = pb_out1.inverse(), pb_out2.inverse()
    for n, pb in ((1, pb_out1), (1, pb_in1), (3, pb_out1), (3, pb_in1)):
        sv = SiteVec(n, pb)
        assert sv.size == n and sv.sites == [pb_out1] * n
        for op in sv.id_ops:
            _is_id_op(op)
    for spaces in ([pb_out1], [pb_out2, pb_out2], [pb_out1, pb_out2, pb_out1],
                   [pb_in2, pb_out1, pb_out1, pb_in1, pb_out2]):
        sv = SiteVec(spaces)
        assert sv.size == len(spaces)
        for s, ix in zip(sv.sites, spaces):
            assert s == (ix if ix.dir == OUT else ix.inverse())
        for op in sv.id_ops:
            _is_id_op(op)


def test_ten_vec_io(tmp_path):
    """``test_ten_vec.cc:27-60`` on the MPS container: dump three tensors
    (one with release), deallocate, load them back permuted."""
    import numpy as np
    from mps2_gb300.finite_mps import FiniteMPS
    from mps2_gb300.site_vec import SiteVec
    from mps2_gb300.tensor import GQTensor, Index, OUT
    rng = np.random.default_rng(2)
    idx_out = Index([((0,), 2), ((1,), 2)], OUT)
    idx_in = idx_out.inverse()

    def rand(div):
        t = GQTensor([idx_in, idx_out], (div,))
        for c in t.allowed_coords((div,)):
            t.blocks[c] = rng.standard_normal(t.block_shape(c))
        return t
    tens = [rand(0), rand(1), rand(-1)]
    v = FiniteMPS(SiteVec(3, idx_out))
    for i, t in enumerate(tens):
        v[i] = t
    names = [str(tmp_path / f"ten{i}.gqten") for i in range(3)]
    v.DumpTen(0, names[0])
    v.DumpTen(1, names[1], True)
    v.DumpTen(2, names[2], False)
    v.dealloc(0)
    v.dealloc(2)
    assert v.empty()
    v.LoadTen(0, names[2])
    v.LoadTen(1, names[0])
    v.LoadTen(2, names[1])
    for got, want in zip((v[0], v[1], v[2]), (tens[2], tens[0], tens[1])):
        assert got.indices == want.indices and got.dense_equal(want)


def test_finite_mps_write_access_resets_canonical_types():
    """``finite_mps.h:67-75``: writing a site marks it non-canonical and the
    MPS uncentralised; reading does not."""
    from mps2_gb300 import hamiltonians as H
    from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS, kUncentralizedCenterIdx
    sv, _, qn0, _ = H.heisenberg_chain(6)
    mps = FiniteMPS(sv)
    assert mps.GetCenter() == kUncentralizedCenterIdx
    DirectStateInitMps(mps, [i % 2 for i in range(6)], qn0)
    assert mps.GetCenter() == 0 and mps.GetTenCanoType(3) == FiniteMPS.RIGHT
    t = mps[3]
    assert mps.GetTenCanoType(3) == FiniteMPS.RIGHT
    mps[3] = t
    assert mps.GetTenCanoType(3) == FiniteMPS.NONE
    assert mps.GetCenter() == kUncentralizedCenterIdx


def test_j1j2_cylinder_workload_definition():
    """The J1-J2 4x16 cylinder workload: 64 sites, D 2000 -> 6000 over eight
    calls, an Sz = 0 product state, the generator's MPO (bulk bond dimension
    at most 17 after compression)."""
    import argparse
    import bench
    args = argparse.Namespace(model="j1j2", schedule=None)
    saved = (bench.L_SITES, bench.WORKLOAD, bench.SCHEDULE)
    try:
        bench._select_model(args)
        assert bench.L_SITES == 64 and args.schedule.split(",")[0] == "2000"
        assert args.schedule.split(",")[-1] == "6000" and len(args.schedule.split(",")) == 8
        mps, mpo = bench._model("j1j2")
        assert mps.size() == 64 and len(mpo) == 64
        assert max(w.indices[-1].dim for w in mpo[1:-1]) <= 17
        # total Sz = 0: the head tensor's right bond carries the charge of sites 1..N-1
        # and the head site's own charge cancels it
        q_head = tuple(mps[0].div)
        assert q_head == (0,)
    finally:
        bench.L_SITES, bench.WORKLOAD, bench.SCHEDULE = saved


def test_update_log_line_format():
    """The per-update line of ``two_site_update_finite_vmps_impl.h:330-338``:
    fixed notation, E0 with 16 decimals, TruncErr in scientific with 2, the
    two timings with 2, S with 7."""
    from mps2_gb300 import _lib
    from mps2_gb300.vmps import UpdateStats
    c = _lib.UpdateStatsC()
    c.site, c.dir, c.e0, c.trunc_err, c.D, c.iters = 7, ord("r"), -2.4935771338879276, 1.25e-9, 8, 12
    c.ee, c.lanczos_seconds, c.update_seconds = 0.6931471805599453, 0.0123, 1.5
    line = UpdateStats(c).line()
    assert line == ("Site    7 E0 =  -2.4935771338879276 TruncErr = 1.25e-09 D =     8 Iter =  12 "
                    "LanczT =     0.01 TotT =     1.50 S =  0.6931472")
