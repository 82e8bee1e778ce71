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
