"""ctypes binding of ``libgqmps2_gb300.so`` (C ABI: ``include/gqmps2_gb300.h``).

The product has no CPU path: if the library is missing or cannot load, every
entry point raises :class:`LibraryUnavailable`.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .tensor import GQTensor, Index, QN

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgqmps2_gb300.so")

GQ_OK = 0
PREC_FP64 = 0
PREC_TF32X3 = 1
PREC_FP64TC = 2
WHERE = {"lend": 0, "cent": 1, "rend": 2}


class LibraryUnavailable(RuntimeError):
    pass


class GQError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[gq status {code}] {msg}")
        self.code = code


class LanczosParamsC(C.Structure):
    _fields_ = [("error", C.c_double), ("max_iterations", C.c_int64), ("rayleigh", C.c_int)]


class SweepParamsC(C.Structure):
    _fields_ = [("sweeps", C.c_int64), ("dmin", C.c_int64), ("dmax", C.c_int64),
                ("trunc_err", C.c_double), ("lanczos", LanczosParamsC),
                ("precision", C.c_int), ("verbose", C.c_int)]


class UpdateStatsC(C.Structure):
    _fields_ = [("site", C.c_int32), ("dir", C.c_int32), ("e0", C.c_double),
                ("trunc_err", C.c_double), ("D", C.c_int64), ("iters", C.c_int64),
                ("ee", C.c_double), ("lanczos_seconds", C.c_double),
                ("update_seconds", C.c_double), ("svd_seconds", C.c_double),
                ("env_seconds", C.c_double), ("matvecs", C.c_int64),
                ("matvec_flops", C.c_double), ("env_flops", C.c_double),
                ("theta_size", C.c_int64)]


_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
_I = C.c_int
_I64 = C.c_int64
_D = C.c_double
_IP = C.POINTER(C.c_int)
_I64P = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)

EXPORTS = {
    "gq_init": (_I, [_I]),
    "gq_last_error": (C.c_char_p, []),
    "gq_synchronize": (_I, []),
    "gq_tensor_create": (_I, [_I, _I, _IP, _IP, _IP, _I64P, _IP, _I64, _IP, _DP, _PP]),
    "gq_tensor_describe": (_I, [_P, _IP, _IP, _I64P, _I64P, _I64P]),
    "gq_tensor_export": (_I, [_P, _IP, _IP, _IP, _I64P, _IP, _IP, _DP]),
    "gq_tensor_destroy": (_I, [_P]),
    "gq_contract": (_I, [_P, _P, _I, _IP, _IP, _I, _PP, _DP]),
    "gq_contract_noalloc": (_I, [_P, _P, _I, _IP, _IP, _P]),
    "gq_eff_ham_mul_state": (_I, [_P, _P, _P, _P, _I, _P, _I, _PP, _DP]),
    "gq_lanczos": (_I, [_P, _P, _P, _P, _I, _P, C.POINTER(LanczosParamsC), _I, _I64P, _DP, _PP]),
    "gq_svd": (_I, [_P, _I, _IP, _D, _I64, _I64, _I, _PP, _PP, _DP, _I64, _DP, _I64P]),
    "gq_dmrg_create": (_I, [_I, _PP, _PP, _PP]),
    "gq_dmrg_init_envs": (_I, [_P, _I]),
    "gq_dmrg_set_env": (_I, [_P, _I, _I, _P]),
    "gq_dmrg_get_env": (_I, [_P, _I, _I, _PP]),
    "gq_dmrg_sweep": (_I, [_P, C.POINTER(SweepParamsC), C.POINTER(UpdateStatsC), _DP]),
    "gq_dmrg_update": (_I, [_P, C.POINTER(SweepParamsC), _I, _I, C.POINTER(UpdateStatsC)]),
    "gq_dmrg_run_batch": (_I, [C.POINTER(_P), _I, C.POINTER(SweepParamsC), _I, _I, _DP]),
    "gq_tensor_dag": (_I, [_P, C.POINTER(_P)]),
    "gq_autotune_enable": (_I, [_I]),
    "gq_mps_centralize": (_I, [C.POINTER(_P), _I, _I, _IP]),
    "gq_mps_truncate": (_I, [C.POINTER(_P), _I, _IP, C.c_double, C.c_int64, C.c_int64, _DP,
                             C.POINTER(C.c_int64)]),
    "gq_dmrg_get_mps": (_I, [_P, _I, _PP]),
    "gq_dmrg_destroy": (_I, [_P]),
    "gq_profile_enable": (_I, [_I]),
    "gq_profile_read": (_I, [_I, _I64P, _DP, _DP, _DP]),
    "gq_get_stream": (_I, [_PP]),
    "gq_tensor_create_blocks": (_I, [_I, _I, _IP, _IP, _IP, _I64P, _IP, _I64, _IP,
                                     C.POINTER(_DP), _PP]),
    "gq_host_sync_count": (_I, [_I64P]),
}

PROF = {"gemm_fp64": 0, "gemm_tf32x3": 1, "permute": 2, "vector": 3, "skinny": 4,
        "gemm_fp64tc": 5, "svd": 6, "svd_eig": 7, "svd_gather": 8, "svd_factors": 9,
        "svd_ortho": 10, "svd_gram": 11, "svd_reduce": 12, "host_plan": 13, "host_sync": 14}

_lib: Optional[C.CDLL] = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the library and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise LibraryUnavailable(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    try:
        lib = C.CDLL(path)
    except OSError as e:
        raise LibraryUnavailable(f"cannot load {path}: {e}") from e
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != GQ_OK:
        raise GQError(code, load().gq_last_error().decode())


def _iarr(vals):
    a = np.ascontiguousarray(np.asarray(vals, dtype=np.int32))
    return a, a.ctypes.data_as(_IP)


def _i64arr(vals):
    a = np.ascontiguousarray(np.asarray(vals, dtype=np.int64))
    return a, a.ctypes.data_as(_I64P)


class DeviceTensor:
    """Owning handle to a block-sparse tensor in GPU memory."""

    def __init__(self, handle: int):
        self.h = C.c_void_p(handle)

    def __del__(self):
        try:
            if self.h and self.h.value and _lib is not None:
                _lib.gq_tensor_destroy(self.h)
        except Exception:
            pass
        self.h = None

    @classmethod
    def from_host(cls, t: GQTensor) -> "DeviceTensor":
        lib = load()
        rank, nq = t.rank, t.nq
        dirs, pdirs = _iarr([ix.dir for ix in t.indices])
        nsecs, pnsecs = _iarr([ix.nsec for ix in t.indices])
        qns, pqns = _iarr([v for ix in t.indices for q in ix.qns for v in q])
        dims, pdims = _i64arr([d for ix in t.indices for d in ix.dims])
        div = t.div if t.div is not None else QN((0,) * nq)
        dv, pdv = _iarr(list(div))
        coords = t.sorted_block_coords()
        cd, pcd = _iarr([c for cc in coords for c in cc] or [0])
        out = C.c_void_p()
        if not coords:
            data = np.zeros(1)
            check(lib.gq_tensor_create(rank, nq, pdirs, pnsecs, pqns, pdims, pdv, 0, pcd,
                                       data.ctypes.data_as(_DP), C.byref(out)))
            return cls(out.value)
        # each block from its own buffer: no host-side gather into one array
        blocks = [np.ascontiguousarray(t.blocks[c], dtype=np.float64) for c in coords]
        ptrs = (_DP * len(blocks))(*[b.ctypes.data_as(_DP) for b in blocks])
        check(lib.gq_tensor_create_blocks(rank, nq, pdirs, pnsecs, pqns, pdims, pdv, len(coords),
                                          pcd, ptrs, C.byref(out)))
        return cls(out.value)

    def describe(self):
        r, nq = C.c_int(), C.c_int()
        ns, nb, ne = C.c_int64(), C.c_int64(), C.c_int64()
        check(load().gq_tensor_describe(self.h, C.byref(r), C.byref(nq), C.byref(ns),
                                        C.byref(nb), C.byref(ne)))
        return r.value, nq.value, ns.value, nb.value, ne.value

    def size(self) -> int:
        return self.describe()[4]

    def to_host(self, with_data: bool = True) -> GQTensor:
        rank, nq, ns, nb, ne = self.describe()
        dirs = np.zeros(rank, np.int32)
        nsecs = np.zeros(rank, np.int32)
        qns = np.zeros(max(ns * nq, 1), np.int32)
        dims = np.zeros(max(ns, 1), np.int64)
        div = np.zeros(nq, np.int32)
        coords = np.zeros(max(nb * rank, 1), np.int32)
        data = np.empty(max(ne, 1), np.float64)
        check(load().gq_tensor_export(
            self.h, dirs.ctypes.data_as(_IP), nsecs.ctypes.data_as(_IP), qns.ctypes.data_as(_IP),
            dims.ctypes.data_as(_I64P), div.ctypes.data_as(_IP), coords.ctypes.data_as(_IP),
            data.ctypes.data_as(_DP) if with_data else None))
        indices = []
        so = 0
        for l in range(rank):
            secs = []
            for s in range(nsecs[l]):
                q = tuple(int(v) for v in qns[(so + s) * nq:(so + s + 1) * nq])
                secs.append((q, int(dims[so + s])))
            so += nsecs[l]
            indices.append(Index(secs, int(dirs[l])))
        t = GQTensor(indices, tuple(int(v) for v in div))
        off = 0
        for b in range(nb):
            c = tuple(int(v) for v in coords[b * rank:(b + 1) * rank])
            shape = t.block_shape(c)
            n = int(np.prod(shape))
            # views of the one exported buffer (no second host copy)
            t.blocks[c] = data[off:off + n].reshape(shape) if with_data else np.zeros(shape)
            off += n
        return t
