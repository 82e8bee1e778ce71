"""Matrix-product-operator generator (gqmps2 ``MPOGenerator``).

API mirrors ``include/gqmps2/one_dim_tn/mpo/mpogen/mpogen.h:40-121``:
``AddTerm`` in its three overloads (generic operator string at
``mpogen_impl.h:86-121``; physical operators with insertion operators such as
a Jordan-Wigner string at ``:143-197``; one- or two-body shorthand at
``:213-243``), ``GetFSM`` and ``Gen`` (``:246-285``).

The construction is the reference's, step for step, so the MPO tensors come
out element for element as gqmps2 builds them:

* every term becomes a path of the finite-state machine (``fsm.FSM``), with
  the term's coefficient label on its first operator (``:97-115``);
  coefficients and operators are labelled in order of first appearance,
  coefficient 1 and the first site's identity taking label 0
  (``:64-72``); two operators are the same when their legs and elements are
  equal;
* the machine's symbolic matrices are compressed (``FSM::GenCompressedMatRepr``,
  columns left to right, rows right to left);
* the columns of each site's matrix are grouped by the quantum number of the
  bond state, groups in order of first appearance, and within a group the
  later column first (``SortSparOpReprMatColsByQN_``, ``:300-349``); the QN
  of a column reached through operator ``O`` from a row with QN ``q`` is
  ``q - Div(O)`` (``CalcTgtRvbQN_``, ``:288-297``); the next site's rows
  follow the same permutation (``:269, :275``);
* each symbolic element is realised as ``sum_i c_i * O_i`` and written into
  the MPO tensor where it is nonzero (``:352-451``): head ``(p_in, r, p_out)``,
  bulk ``(l, p_in, p_out, r)``, tail ``(p_in, l, p_out)``, l IN and r OUT.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np

from .fsm import FSM, LabelConvertor
from .site_vec import SiteVec
from .symb_alg import OpRepr, SparOpReprMat, kNullOpRepr
from .tensor import GQTensor, Index, OUT, QN, Div


def _op_key(op: GQTensor):
    """Equality of operators: same legs, same elements (0.0 == -0.0)."""
    dense = op.to_dense() + 0.0
    return (tuple(op.indices), dense.shape, dense.tobytes())


def _coef_key(c):
    return float(c)


class MPOGenerator:
    def __init__(self, site_vec: SiteVec, zero_div):
        self.site_vec = site_vec
        self.N = site_vec.size
        self.zero_div = QN(zero_div)
        self.pb_out = list(site_vec.sites)
        self.pb_in = [ix.inverse() for ix in self.pb_out]
        self.id_ops = list(site_vec.id_ops)
        self.fsm_ = FSM(self.N)
        self.op_label_convertor_ = LabelConvertor(self.id_ops[0], key=_op_key)
        self.fsm_.ReplaceIdOpLabels([self.op_label_convertor_.Convert(o) for o in self.id_ops])
        self.coef_label_convertor_ = LabelConvertor(1.0, key=_coef_key)
        self.bond_dims: List[int] = []

    def GetFSM(self) -> FSM:
        return self.fsm_

    # ------------------------------------------------------------------
    def AddTerm(self, coef, *args, **kw):
        """Overloads (same meaning as the reference):

        * ``AddTerm(coef, [ops], [sites])``
        * ``AddTerm(coef, [phys_ops], [sites], [inst_ops], inst_ops_idxs_set=None)``
        * ``AddTerm(coef, op1, site1, op2=None, site2=0, inst_op=None, inst_op_idxs=None)``
        """
        if args and isinstance(args[0], (list, tuple)):
            ops, idxs = list(args[0]), list(args[1])
            if len(args) >= 3 or "inst_ops" in kw:
                inst_ops = list(args[2]) if len(args) >= 3 else list(kw["inst_ops"])
                inst_set = args[3] if len(args) >= 4 else kw.get("inst_ops_idxs_set")
                self._add_with_inst(coef, ops, idxs, inst_ops, inst_set)
            else:
                self._add_generic(coef, ops, idxs)
            return
        op1, i1 = args[0], args[1]
        op2 = args[2] if len(args) > 2 else kw.get("op2")
        i2 = args[3] if len(args) > 3 else kw.get("op2_idx", 0)
        inst = args[4] if len(args) > 4 else kw.get("inst_op")
        inst_idxs = args[5] if len(args) > 5 else kw.get("inst_op_idxs")
        if op2 is None or (isinstance(op2, GQTensor) and op2.is_default()):
            self._add_generic(coef, [op1], [i1])
        elif inst is None or inst.is_default():
            self._add_generic(coef, [op1, op2], [i1, i2])
        elif not inst_idxs:
            self._add_with_inst(coef, [op1, op2], [i1, i2], [inst], None)
        else:
            self._add_with_inst(coef, [op1, op2], [i1, i2], [inst], [list(inst_idxs)])

    def _add_with_inst(self, coef, phys_ops, phys_idxs, inst_ops, inst_set):
        """``mpogen_impl.h:143-197``: insertion operators between the
        physical ones (and optionally a tail string to the chain end)."""
        if len(phys_ops) < 2 or len(phys_ops) != len(phys_idxs):
            raise ValueError("need at least two physical operators")
        if len(inst_ops) not in (len(phys_ops) - 1, len(phys_ops)):
            raise ValueError("wrong number of insertion operators")
        ops, idxs = [], []
        for i in range(len(phys_ops) - 1):
            ops.append(phys_ops[i])
            idxs.append(phys_idxs[i])
            rng = (range(phys_idxs[i] + 1, phys_idxs[i + 1]) if not inst_set
                   else inst_set[i])
            for j in rng:
                ops.append(inst_ops[i])
                idxs.append(j)
        ops.append(phys_ops[-1])
        idxs.append(phys_idxs[-1])
        if len(inst_ops) == len(phys_ops):
            rng = range(phys_idxs[-1], self.N) if not inst_set else inst_set[-1]
            for j in rng:
                ops.append(inst_ops[-1])
                idxs.append(j)
        self._add_generic(coef, ops, idxs)

    def _add_generic(self, coef, ops, idxs):
        """``mpogen_impl.h:86-121``.  When a site index repeats, the first
        operator given for it is used, as the reference's ``std::find``
        lookup at ``:102`` does (this is what happens to the tail string's
        entry on the last physical site)."""
        if len(ops) != len(idxs) or not ops:
            raise ValueError("operators and site indexes differ in length")
        if list(idxs) != sorted(idxs):
            raise ValueError("site indexes must be ascending")
        if idxs[-1] >= self.N:
            raise ValueError("site index out of range")
        if coef == 0:
            return
        coef_label = self.coef_label_convertor_.Convert(coef)
        head, tail = idxs[0], idxs[-1]
        reprs = []
        for s in range(head, tail + 1):
            if s in idxs:
                loc = idxs.index(s)
                label = self.op_label_convertor_.Convert(ops[loc])
                reprs.append(OpRepr(coef_label, label) if loc == 0 else OpRepr(label))
            else:
                reprs.append(OpRepr(self.op_label_convertor_.Convert(self.id_ops[s])))
        self.fsm_.AddPath(head, tail, reprs)

    # ------------------------------------------------------------------
    def _sort_cols_by_qn(self, m: SparOpReprMat, lvb: Index, ops: Sequence[GQTensor]):
        """``SortSparOpReprMatColsByQN_``: permutes m's columns in place and
        returns (permutation, right bond index)."""
        groups: List[list] = []          # [qn, count]
        order: List[int] = []
        for y in range(m.cols):
            col_qn = None
            for x, elem in m.col_items(y):
                q = self.zero_div - Div(ops[elem.ops[0]]) + lvb.qn_of_coor(x)
                if col_qn is None:
                    col_qn = q
                    offset = 0
                    for g in groups:
                        if g[0] == q:
                            g[1] += 1
                            break
                        offset += g[1]
                    else:
                        groups.append([q, 1])
                    order.insert(offset, y)
                elif q != col_qn:
                    raise ValueError("operator breaks the quantum-number conservation "
                                     f"(bond state {y} reached with two quantum numbers)")
            if col_qn is None:
                raise ValueError(f"bond state {y} has no incoming operator")
        m.TransposeCols(order)
        return order, Index([(q, n) for q, n in groups], OUT)

    def Gen(self) -> List[GQTensor]:
        N = self.N
        if N < 2:
            raise ValueError("an MPO needs at least two sites")
        mats = self.fsm_.GenCompressedMatRepr()
        coefs = self.coef_label_convertor_.GetLabelObjMapping()
        ops = self.op_label_convertor_.GetLabelObjMapping()
        dense_ops = [o.to_dense() for o in ops]
        self.bond_dims = [m.cols for m in mats[:-1]]
        zero = self.zero_div
        vb = Index([(zero, 1)], OUT)
        order: List[int] = []
        mpo: List[GQTensor] = []
        for s in range(N):
            m = mats[s]
            if s > 0:
                m.TransposeRows(order)
            lvb = vb
            if s < N - 1:
                order, vb = self._sort_cols_by_qn(m, lvb, ops)
            d_in, d_out = self.pb_in[s].dim, self.pb_out[s].dim
            dense = np.zeros((m.rows, d_in, d_out, m.cols))
            for x in range(m.rows):
                for y, elem in m.row_items(x):
                    op = elem.Realize(coefs, dense_ops)
                    nz = op != 0.0
                    dense[x, :, :, y][nz] = op[nz]
            if s == 0:
                idx = [self.pb_in[0], vb, self.pb_out[0]]
                arr = dense[0].transpose(0, 2, 1)            # (p_in, r, p_out)
            elif s == N - 1:
                idx = [self.pb_in[s], lvb.inverse(), self.pb_out[s]]
                arr = dense[:, :, :, 0].transpose(1, 0, 2)    # (p_in, l, p_out)
            else:
                idx = [lvb.inverse(), self.pb_in[s], self.pb_out[s], vb]
                arr = dense
            mpo.append(_dense_to_blocks(arr, idx, zero))
        return mpo


def _dense_to_blocks(arr: np.ndarray, indices: Sequence[Index], div) -> GQTensor:
    t = GQTensor(indices, div)
    offs = [np.concatenate([[0], np.cumsum(ix.dims)]).astype(int) for ix in indices]
    for coords in t.allowed_coords(div):
        sl = tuple(slice(o[c], o[c + 1]) for o, c in zip(offs, coords))
        blk = arr[sl]
        if np.any(blk != 0.0):
            t.blocks[coords] = np.ascontiguousarray(blk)
    # anything nonzero outside the allowed blocks means a QN-violating operator
    check = np.zeros_like(arr)
    for coords, blk in t.blocks.items():
        sl = tuple(slice(o[c], o[c + 1]) for o, c in zip(offs, coords))
        check[sl] = blk
    if not np.array_equal(check, arr):
        raise ValueError("operator breaks the quantum-number conservation")
    return t
