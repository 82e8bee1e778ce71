"""The no-allocation contraction entry point against the regular one.

``gq_contract_noalloc`` serves callers that own all device memory and cannot
let the library allocate while they work (it keeps its scratch in arrays
reserved when the library is loaded).  Its result must equal
``gq_contract``'s FP64 result, call after call, within the tolerance the
FP64 parity tests use.  This file is collected last so that a failure here
comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from _helpers import first_allowed_div, random_index, random_tensor, rel_err
from mps2_gb300.tensor import GQTensor, IN, OUT

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the FP64 per-contraction tolerance of test_gpu_parity.py


def _contract_noalloc(lib, a, b, axes, out_structure):
    from mps2_gb300 import _lib
    da = _lib.DeviceTensor.from_host(a)
    db = _lib.DeviceTensor.from_host(b)
    dout = _lib.DeviceTensor.from_host(out_structure)   # created up front by the caller
    xa = np.ascontiguousarray(axes[0], dtype=np.int32)
    xb = np.ascontiguousarray(axes[1], dtype=np.int32)
    _lib.check(lib.gq_contract_noalloc(da.h, db.h, len(xa), xa.ctypes.data_as(_lib._IP),
                                       xb.ctypes.data_as(_lib._IP), dout.h))
    return dout.to_host()


def test_noalloc_contract_matches_gq_contract_twice():
    from mps2_gb300 import _lib
    from mps2_gb300.vmps import Contract
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    rng = np.random.default_rng(77)
    cases = [([0, 2], [0, 1]), ([4, 1], [1, 0])]
    for xa, xb in cases:
        ra = max(max(xa) + 1, 3)
        rb = max(max(xb) + 1, 3)
        ia = [random_index(rng, 3, 2, 5, OUT if rng.random() < 0.5 else IN) for _ in range(ra)]
        ib = [random_index(rng, 3, 2, 5, OUT if rng.random() < 0.5 else IN) for _ in range(rb)]
        for a_ax, b_ax in zip(xa, xb):
            ib[b_ax] = ia[a_ax].inverse()
        a = random_tensor(rng, ia, first_allowed_div(ia), fill=0.8)
        b = random_tensor(rng, ib, first_allowed_div(ib), fill=0.8)
        ref = Contract(a, b, (xa, xb), precision="fp64")
        # the caller's output: the regular result's structure, filled with
        # garbage so that a block the entry point fails to write shows up
        out = GQTensor(ref.indices, ref.div,
                       {k: np.full(v.shape, 1e300) for k, v in ref.blocks.items()})
        for call in range(2):
            got = _contract_noalloc(lib, a, b, (xa, xb), out)
            assert sorted(got.blocks) == sorted(ref.blocks)
            assert rel_err(got, ref) <= TOL, (xa, xb, call)


def test_noalloc_rejects_oversized_operands():
    from mps2_gb300 import _lib
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    from mps2_gb300.tensor import Index
    # a and b of 2^20 + 1 elements each exceed the 2^21-element scratch
    ix = Index([((0,), 1025)], OUT)
    jx = Index([((0,), 1024)], OUT)
    a = GQTensor([ix.inverse(), jx], (0,), {(0, 0): np.zeros((1025, 1024))})
    b = GQTensor([jx.inverse(), ix], (0,), {(0, 0): np.zeros((1024, 1025))})
    out = GQTensor([ix.inverse(), ix], (0,), {(0, 0): np.zeros((1025, 1025))})
    da = _lib.DeviceTensor.from_host(a)
    db = _lib.DeviceTensor.from_host(b)
    do = _lib.DeviceTensor.from_host(out)
    xa = np.array([1], dtype=np.int32)
    xb = np.array([0], dtype=np.int32)
    rc = lib.gq_contract_noalloc(da.h, db.h, 1, xa.ctypes.data_as(_lib._IP),
                                 xb.ctypes.data_as(_lib._IP), do.h)
    assert rc == 1
    assert b"no-allocation scratch" in lib.gq_last_error()


def test_noalloc_large_blocks_and_unreached_block_against_oracle():
    """Sector dimensions of 60 to 150, so that output blocks span several 64 x 64
    tiles and operand blocks exceed one 16384-element permute chunk; the
    contracted leg comes first in a, so a is permuted; the caller's output
    holds every block its legs allow, some of which no block pair reaches:
    those must come back as exact zeros.  Checked against the FP64 oracle
    and against gq_contract, on two calls in a row."""
    import oracle
    from _convert import to_oracle
    from mps2_gb300 import _lib
    from mps2_gb300.tensor import Index
    from mps2_gb300.vmps import Contract
    lib = _lib.load()
    _lib.check(lib.gq_init(0))
    rng = np.random.default_rng(2024)
    c = Index([((-1,), 90), ((0,), 120), ((1,), 140)], IN)
    l0 = Index([((-1,), 110), ((0,), 130), ((1,), 75)], OUT)
    l1 = Index([((0,), 2), ((1,), 2)], OUT)
    e = Index([((-1,), 80), ((0,), 100), ((2,), 60)], IN)
    a = random_tensor(rng, [c, l0, l1], (0,), fill=1.0)
    b = random_tensor(rng, [c.inverse(), e], (0,), fill=1.0)
    assert a.size() + b.size() < 2 ** 21
    assert max(v.size for v in a.blocks.values()) > 16384
    ref = oracle.contract(to_oracle(a), to_oracle(b), [0], [0])
    reg = Contract(a, b, ([0], [0]), precision="fp64")
    full = GQTensor([l0, l1, e], (0,))
    unreached = [k for k in full.allowed_coords((0,)) if k not in ref.blocks]
    assert unreached, "the case must hold an output block that no pair reaches"
    out = GQTensor(full.indices, full.div,
                   {k: np.full(full.block_shape(k), 1e300) for k in full.allowed_coords((0,))})
    assert any(v.shape[0] * v.shape[1] > 64 and v.shape[2] > 64 for v in ref.blocks.values())
    for call in range(2):
        got = _contract_noalloc(lib, a, b, ([0], [0]), out)
        for k in unreached:
            assert np.all(got.blocks[k] == 0.0), (k, call)
        assert rel_err(got, ref) <= TOL, call
        assert rel_err(got, reg) <= TOL, call
