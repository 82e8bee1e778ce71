"""Observables of a finite MPS over the GPU library.

Restates ``one_dim_tn/mps/finite_mps/finite_mps_measu.h``:
``MeasureOneSiteOp`` (:150-214), ``MeasureTwoSiteOp`` (:216-298),
``MeasureMultiSiteOp`` (:300-364), the averages ``OneSiteOpAvg``
(:366-402), ``MultiSiteOpAvg`` (:404-460), ``OpsVecAvg`` (:462-526),
``CtrctMidTen`` (:528-554) and ``DumpMeasuRes`` (:556-584, the
``<basename>.json`` text format).

The MPS is uploaded once; every ``Centralize`` (device SVDs) and every
contraction of the transfer-matrix chain runs on the GPU.  Only the last
full contraction of each measure event -- two tensors the size of one site
tensor, reduced to one number -- is formed on the host.  Like the
reference, the measurement leaves the MPS centralised at the last site it
visited.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence, Union

import numpy as np

from . import _lib
from ._lib import DeviceTensor, check, load
from .finite_mps import FiniteMPS
from .tensor import GQTensor


class MeasuResElem:
    """``MeasuResElem``: the sites of the operators and the average."""

    def __init__(self, sites: Sequence[int], avg: float):
        self.sites = [int(s) for s in sites]
        self.avg = float(avg)

    def __repr__(self):
        return f"MeasuResElem({self.sites}, {self.avg!r})"


def DumpMeasuRes(res: Sequence[MeasuResElem], basename: str) -> None:
    """``DumpMeasuRes``: ``[\\n  [[i, j], avg],\\n ...]`` in ``basename.json``
    (averages printed with 12 significant digits in a 14-wide field)."""
    with open(basename + ".json", "w") as f:
        f.write("[\n")
        for n, e in enumerate(res):
            f.write("  [[" + ", ".join(str(s) for s in e.sites) + "], ")
            f.write(f"{e.avg:14.12g}")
            f.write("]\n" if n == len(res) - 1 else "],\n")
        f.write("]")


# ---------------------------------------------------------------------------
# device helpers
# ---------------------------------------------------------------------------
def _contract(a: DeviceTensor, b: DeviceTensor, xa, xb) -> DeviceTensor:
    ia = np.ascontiguousarray(xa, dtype=np.int32)
    ib = np.ascontiguousarray(xb, dtype=np.int32)
    out = C.c_void_p()
    fl = C.c_double()
    check(load().gq_contract(a.h, b.h, len(ia), ia.ctypes.data_as(_lib._IP),
                             ib.ctypes.data_as(_lib._IP), _lib.PREC_FP64, C.byref(out),
                             C.byref(fl)))
    return DeviceTensor(out.value)


def _dag(a: DeviceTensor) -> DeviceTensor:
    out = C.c_void_p()
    check(load().gq_tensor_dag(a.h, C.byref(out)))
    return DeviceTensor(out.value)


def _full(a: GQTensor, b: GQTensor, xa, xb) -> float:
    """Contraction of every leg of a with every leg of b (real tensors)."""
    acc = 0.0
    bmap = {}
    for kb, vb in b.blocks.items():
        key = tuple(kb[j] for j in xb)
        bmap[key] = vb
    for ka, va in a.blocks.items():
        key = tuple(ka[j] for j in xa)
        vb = bmap.get(key)
        if vb is not None:
            acc += float(np.tensordot(va, vb, axes=(list(xa), list(xb))))
    return acc


class _DeviceMPS:
    """The MPS on the device, with the reference's canonical-type bookkeeping."""

    def __init__(self, mps: FiniteMPS):
        self.host = mps
        self.n = mps.size()
        self.t = [DeviceTensor.from_host(mps[i]) for i in range(self.n)]
        self.cano = list(mps.tens_cano_type)
        self.center = mps.center

    def centralize(self, c: int) -> None:
        arr = (C.c_void_p * self.n)(*[t.h.value for t in self.t])
        cano = (C.c_int * self.n)(*self.cano)
        check(load().gq_mps_centralize(arr, self.n, int(c), cano))
        self.cano = list(cano)
        self.center = c

    def write_back(self) -> None:
        for i, t in enumerate(self.t):
            self.host[i] = t.to_host()
        self.host.tens_cano_type = list(self.cano)
        self.host.center = self.center


def _one_site_avg(cent: DeviceTensor, op: DeviceTensor, site: int, n: int) -> float:
    """``OneSiteOpAvg`` (:366-402)."""
    if site == 0:
        x1, y1, x2, y2 = [0], [0], [0, 1], [1, 0]
    elif site == n - 1:
        x1, y1, x2, y2 = [1], [0], [0, 1], [0, 1]
    else:
        x1, y1, x2, y2 = [1], [0], [0, 2, 1], [0, 1, 2]
    temp = _contract(cent, op, x1, y1)
    return _full(temp.to_host(), _dag(cent).to_host(), x2, y2)


def _ctrct_mid_ten(dm: _DeviceMPS, site: int, op: GQTensor, id_op: GQTensor,
                   t: DeviceTensor) -> DeviceTensor:
    """``CtrctMidTen`` (:528-554)."""
    a = dm.t[site]
    if _same_tensor(op, id_op):
        temp = _contract(a, t, [0], [0])
        return _contract(temp, _dag(a), [0, 2], [1, 0])
    temp1 = _contract(a, t, [0], [0])
    temp2 = _contract(temp1, DeviceTensor.from_host(op), [0], [0])
    return _contract(temp2, _dag(a), [1, 2], [0, 1])


def _same_tensor(a: GQTensor, b: GQTensor) -> bool:
    if a.indices != b.indices or set(a.blocks) != set(b.blocks):
        return False
    return all(np.array_equal(a.blocks[k], b.blocks[k]) for k in a.blocks)


def _ops_vec_avg(dm: _DeviceMPS, ops: Sequence[GQTensor], head: int, tail: int) -> float:
    """``OpsVecAvg`` (:462-526): the MPS is centralised at ``head``."""
    id_ops = dm.host.GetSitesInfo().id_ops
    if head == 0:
        a1, a2, a3 = [0], [1], [0]
    else:
        a1, a2, a3 = [1], [0, 2], [0, 1]
    h = dm.t[head]
    temp0 = _contract(h, DeviceTensor.from_host(ops[0]), a1, [0])
    t = _contract(temp0, _dag(h), a2, a3)
    assert len(ops) == tail - head + 1
    for i in range(head + 1, tail):
        t = _ctrct_mid_ten(dm, i, ops[i - head], id_ops[i], t)
    if tail == dm.n - 1:
        b1, b2 = [0, 1], [0, 1]
    else:
        b1, b2 = [0, 1, 2], [2, 0, 1]
    tl = dm.t[tail]
    temp2 = _contract(tl, t, [0], [0])
    temp3 = _contract(temp2, DeviceTensor.from_host(ops[-1]), [0], [0])
    return _full(temp3.to_host(), _dag(tl).to_host(), b1, b2)


def _multi_site_avg(dm: _DeviceMPS, phys_ops, inst_ops_set, sites) -> MeasuResElem:
    """``MultiSiteOpAvg`` (:404-437): ops = A, inserts, B, inserts, ...,
    optionally a tail string after the last physical operator."""
    n_inst, n_phys = len(inst_ops_set), len(phys_ops)
    assert n_phys in (n_inst + 1, n_inst)
    ops: List[GQTensor] = []
    for i in range(n_phys - 1):
        ops.append(phys_ops[i])
        ops.extend(inst_ops_set[i])
    ops.append(phys_ops[-1])
    if n_inst == n_phys:
        ops.extend(inst_ops_set[-1])
    head = sites[0]
    tail = head + len(ops) - 1
    return MeasuResElem(sites, _ops_vec_avg(dm, ops, head, tail))


# ---------------------------------------------------------------------------
# public entry points
# ---------------------------------------------------------------------------
def MeasureOneSiteOp(mps: FiniteMPS, ops: Union[GQTensor, Sequence[GQTensor]],
                     res_file_basenames: Union[str, Sequence[str]]):
    """One operator (returns a list of ``MeasuResElem``) or a list of
    operators (returns one list per operator), measured on every site."""
    single = isinstance(ops, GQTensor)
    op_list = [ops] if single else list(ops)
    names = [res_file_basenames] if single else list(res_file_basenames)
    assert len(op_list) == len(names)
    dm = _DeviceMPS(mps)
    n = dm.n
    dops = [DeviceTensor.from_host(o) for o in op_list]
    res = [[None] * n for _ in op_list]
    for i in range(n):
        dm.centralize(i)
        for j, d in enumerate(dops):
            res[j][i] = MeasuResElem([i], _one_site_avg(dm.t[i], d, i, n))
    dm.write_back()
    for r, name in zip(res, names):
        DumpMeasuRes(r, name)
    return res[0] if single else res


def _is_ordered(sites):
    return list(sites) == sorted(sites)


def MeasureMultiSiteOp(mps: FiniteMPS, phys_ops_set, inst_ops_set, sites_set,
                       res_file_basename: str) -> List[MeasuResElem]:
    """Both reference overloads: ``inst_ops_set[i]`` is either a list of
    lists of insert operators (one list per gap, :300-340) or a list of
    single insert operators repeated across each gap (:342-364)."""
    dm = _DeviceMPS(mps)
    res = []
    for phys_ops, inst, sites in zip(phys_ops_set, inst_ops_set, sites_set):
        assert len(sites) > 1 and _is_ordered(sites)
        dm.centralize(sites[0])
        if inst and isinstance(inst[0], GQTensor):
            # same insert operator across each gap (:439-460)
            assert len(phys_ops) == len(inst) + 1
            inst = [[inst[i]] * (sites[i + 1] - sites[i] - 1) for i in range(len(inst))]
        res.append(_multi_site_avg(dm, phys_ops, inst, sites))
    dm.write_back()
    DumpMeasuRes(res, res_file_basename)
    return res


def MeasureTwoSiteOp(mps: FiniteMPS, phys_ops: Sequence[GQTensor], inst_ops, sites_set,
                     res_file_basename: str) -> List[MeasuResElem]:
    """``<A_i O ... O B_j>`` for each pair in ``sites_set``; ``inst_ops`` is
    one insert operator for every gap (:261-298) or one list of insert
    operators per measure event (:216-259)."""
    assert len(phys_ops) == 2
    n_ev = len(sites_set)
    phys_set = [list(phys_ops)] * n_ev
    if isinstance(inst_ops, GQTensor):
        inst_set = [[inst_ops]] * n_ev
    else:
        assert len(inst_ops) == n_ev
        inst_set = []
        for i in range(n_ev):
            assert sites_set[i][1] - sites_set[i][0] - 1 == len(inst_ops[i])
            inst_set.append([list(inst_ops[i])])
    return MeasureMultiSiteOp(mps, phys_set, inst_set, sites_set, res_file_basename)
