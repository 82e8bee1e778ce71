"""Finite-state machine of the MPO generator.

Restates gqmps2's ``one_dim_tn/mpo/mpogen/fsm.h`` (same names and results):

* a term becomes an ``FSMPath`` over the N+1 FSM sites (the bonds, with the
  two chain ends): the ready state before its first operator, a fresh middle
  state on every inner bond, the final state after its last operator
  (``FSM::AddPath``, ``fsm.h:109-151``);
* ``GenMatRepr`` (``:154-168``, ``:171-240``) lays the paths out as one
  symbolic operator matrix per site.  Rows/columns of an FSM site are
  [ready, middle states in order of creation, final], each present only when
  used.  A path's operator is added to an occupied element unless it equals
  the element already there -- so an identical single-site term added twice
  counts once, as in the reference;
* ``GenCompressedMatRepr`` (``:243-252``) compresses columns left to right,
  then rows right to left, with the compressers of ``symb_alg``;
* ``LabelConvertor`` (``:261-281``) hands out labels for coefficients and
  operators in order of first appearance.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, List, Optional, Sequence

from .symb_alg import (OpRepr, SparOpReprMat, SparOpReprMatColCompresser,
                       SparOpReprMatRowCompresser, kIdOpLabel, kNullOpRepr)

kFSMReadyStatIdx = 0
kFSMFinalStatIdx = -1


@dataclass
class FSMNode:
    fsm_site_idx: int = 0
    fsm_stat_idx: int = 0


class FSMPath:
    def __init__(self, phys_site_num: int, fsm_site_num: int):
        self.fsm_nodes: List[FSMNode] = [FSMNode() for _ in range(fsm_site_num)]
        self.op_reprs: List[OpRepr] = [kNullOpRepr] * phys_site_num


class FSM:
    def __init__(self, phys_site_num: int = 0):
        n = int(phys_site_num)
        self.phys_site_num_ = n
        self.fsm_site_num_ = n + 1
        self.mid_stat_nums_ = [0] * (n + 1)
        self.has_readys_ = [False] * (n + 1)
        self.has_finals_ = [False] * (n + 1)
        self.fsm_paths_: List[FSMPath] = []
        self.id_op_labels_ = [kIdOpLabel] * n

    def phys_size(self) -> int:
        return self.phys_site_num_

    def fsm_size(self) -> int:
        return self.fsm_site_num_

    def ReplaceIdOpLabels(self, labels: Sequence[int]) -> None:
        if len(labels) != len(self.id_op_labels_):
            raise ValueError("one identity label per site")
        self.id_op_labels_ = [int(l) for l in labels]

    def GetFSMPaths(self) -> List[FSMPath]:
        return list(self.fsm_paths_)

    def AddPath(self, head: int, tail: int, ntrvl_ops: Sequence[OpRepr]) -> None:
        """Operators ``ntrvl_ops`` on sites head..tail, identities elsewhere."""
        n = self.phys_site_num_
        if not (0 <= head <= tail < n) or len(ntrvl_ops) != tail - head + 1:
            raise ValueError("AddPath: the operators do not span head..tail inside the chain")
        path = FSMPath(n, self.fsm_site_num_)
        for i in range(n):
            if head <= i <= tail:
                path.op_reprs[i] = ntrvl_ops[i - head]
            else:
                path.op_reprs[i] = OpRepr(self.id_op_labels_[i])
        path.fsm_nodes[0] = FSMNode(0, kFSMReadyStatIdx)
        self.has_readys_[0] = True
        for i in range(n):
            s = i + 1
            if i < head:
                path.fsm_nodes[s] = FSMNode(s, kFSMReadyStatIdx)
                self.has_readys_[s] = True
            elif i >= tail:
                path.fsm_nodes[s] = FSMNode(s, kFSMFinalStatIdx)
                self.has_finals_[s] = True
            else:
                self.mid_stat_nums_[s] += 1
                path.fsm_nodes[s] = FSMNode(s, self.mid_stat_nums_[s])
        self.fsm_paths_.append(path)

    # ------------------------------------------------------------------
    def _site_dims(self) -> List[int]:
        return [self.mid_stat_nums_[i] + int(self.has_readys_[i]) + int(self.has_finals_[i])
                for i in range(self.fsm_site_num_)]

    def _final_idxs(self, dims: Sequence[int]) -> List[int]:
        out = [-1] * self.fsm_site_num_
        for i in range(self.fsm_site_num_):
            if self.has_finals_[i]:
                out[i] = dims[i] - 1 if self.has_readys_[i] else 0
        return out

    def _coor(self, node: FSMNode, site: int, final_idxs: Sequence[int]) -> int:
        if node.fsm_stat_idx == kFSMFinalStatIdx:
            return final_idxs[site]
        if not self.has_readys_[site] and not self.has_finals_[site]:
            return node.fsm_stat_idx - 1
        return node.fsm_stat_idx

    def GenMatRepr(self) -> List[SparOpReprMat]:
        dims = self._site_dims()
        finals = self._final_idxs(dims)
        mats = [SparOpReprMat(dims[i], dims[i + 1]) for i in range(self.phys_site_num_)]
        for path in self.fsm_paths_:
            for i in range(self.phys_site_num_):
                x = self._coor(path.fsm_nodes[i], i, finals)
                y = self._coor(path.fsm_nodes[i + 1], i + 1, finals)
                op = path.op_reprs[i]
                cur = mats[i](x, y)
                if cur == kNullOpRepr:
                    mats[i].SetElem(x, y, op)
                elif cur != op:
                    mats[i].SetElem(x, y, cur + op)
        return mats

    def GenCompressedMatRepr(self) -> List[SparOpReprMat]:
        mats = self.GenMatRepr()
        n = self.phys_site_num_
        for i in range(n - 1):
            SparOpReprMatColCompresser(mats[i], mats[i + 1])
        for i in range(n - 1, 0, -1):
            SparOpReprMatRowCompresser(mats[i], mats[i - 1])
        return mats


class LabelConvertor:
    """Label of an object = its position among the distinct objects seen so
    far (``fsm.h:261-281``).  Two objects are the same when their ``key``
    values are equal (default: the object itself)."""

    def __init__(self, first=None, key: Optional[Callable] = None):
        self._key = key or (lambda o: o)
        self._hub: list = []
        self._lut: dict = {}
        if first is not None:
            self.Convert(first)

    def Convert(self, obj) -> int:
        k = self._key(obj)
        label = self._lut.get(k)
        if label is None:
            label = len(self._hub)
            self._lut[k] = label
            self._hub.append(obj)
        return label

    def GetLabelObjMapping(self) -> list:
        return list(self._hub)
