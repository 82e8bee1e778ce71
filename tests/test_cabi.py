"""CPU checks of the C ABI library: it builds, loads without a GPU, and
exports every entry point that ``include/gqmps2_gb300.h`` declares."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gqmps2_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gq_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from mps2_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ["gq_tensor_create", "gq_contract", "gq_eff_ham_mul_state", "gq_lanczos", "gq_svd",
              "gq_dmrg_sweep", "gq_last_error"]:
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    from mps2_gb300 import _lib
    for s in declared_symbols():
        assert hasattr(lib, s), s
        assert s in _lib.EXPORTS, f"{s} has no Python binding"


def test_last_error_starts_empty(lib):
    assert lib.gq_last_error() == b""


def test_host_tensor_file_roundtrip(tmp_path):
    """The documented tensor file layout round-trips bit-exactly
    (``tests/test_one_dim_tn/test_ten_vec.cc:27-60`` checks dump/load)."""
    import numpy as np
    from mps2_gb300.finite_mps import read_tensor, write_tensor
    from _helpers import random_index, random_tensor
    from mps2_gb300.tensor import IN, OUT
    rng = np.random.default_rng(1)
    t = random_tensor(rng, [random_index(rng, 3, 2, 4, IN, nq=2), random_index(rng, 2, 1, 3, OUT, nq=2),
                            random_index(rng, 4, 2, 4, OUT, nq=2)], (0, 0))
    f = str(tmp_path / "t.gqten")
    write_tensor(t, f)
    u = read_tensor(f)
    assert u.indices == t.indices and tuple(u.div) == tuple(t.div)
    assert sorted(u.blocks) == sorted(t.blocks)
    for k in t.blocks:
        assert np.array_equal(u.blocks[k], t.blocks[k])


def test_product_raises_without_library(tmp_path, monkeypatch):
    """No silent CPU fallback: a missing library is an error."""
    from mps2_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(_lib.LibraryUnavailable):
        _lib.load(str(tmp_path / "missing.so"))
