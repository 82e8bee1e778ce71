"""Matrix-product-operator generator (gqmps2 ``MPOGenerator``).

API mirrors ``include/gqmps2/one_dim_tn/mpo/mpogen/mpogen.h:40-121``:
``AddTerm`` in its three overloads (generic operator string at
``mpogen_impl.h:86-121``; physical operators with insertion operators such as
a Jordan-Wigner string at ``:143-197``; one- or two-body shorthand at
``:213-243``) and ``Gen`` (``:246-285``).

Construction (this project's own): every term becomes a path through a
finite-state automaton whose states live on the bonds.  Paths share a state
while they have applied the same operators starting from the same head
site (prefix sharing), so e.g. a nearest-neighbour Heisenberg chain gets the
familiar 5 states per bond (ready, S^z, S^+, S^-, final) and a Hubbard chain
with four hopping channels gets 6.  The term's coefficient is folded into
the operator on its last site so that prefixes stay shareable; transitions
into the final state add up.  The MPO matrices that come out have the
reference's layout:

* bond states ordered [ready, intermediate states in creation order, final],
  then grouped by quantum number in order of first appearance, one sector
  per distinct QN (as ``SortSparOpReprMatColsByQN_``, ``mpogen_impl.h:300-349``);
* the QN of the state reached through operator ``O`` from a state with QN
  ``q`` is ``q - Div(O)`` (``CalcTgtRvbQN_``, ``:288-297``);
* leg orders head ``(p_in, r, p_out)``, bulk ``(l, p_in, p_out, r)``, tail
  ``(p_in, l, p_out)`` (``:359, :377, :398``), l IN and r OUT.

The bond dimensions can differ from the reference's symbolic compression
(``fsm.h:232-241`` plus ``symb_alg/coef_op_alg.h``) for long-range terms;
the Hamiltonian represented is the same.
"""
from __future__ import annotations

from typing import Dict, List, Sequence

import numpy as np

from .site_vec import SiteVec
from .tensor import GQTensor, Index, OUT, QN, Div


class _OpTable:
    """Interns dense operator matrices so equal operators share an id."""

    def __init__(self):
        self.mats: List[np.ndarray] = []
        self.divs: List[QN] = []
        self._lut: Dict[tuple, int] = {}

    def add(self, op: GQTensor) -> int:
        dense = op.to_dense()
        key = (dense.shape, dense.tobytes())
        i = self._lut.get(key)
        if i is None:
            i = len(self.mats)
            self._lut[key] = i
            self.mats.append(dense)
            self.divs.append(Div(op))
        return i


class MPOGenerator:
    def __init__(self, site_vec: SiteVec, zero_div):
        self.site_vec = site_vec
        self.N = site_vec.size
        self.zero_div = QN(zero_div)
        self.pb_out = list(site_vec.sites)
        self.pb_in = [ix.inverse() for ix in self.pb_out]
        self.ops = _OpTable()
        self.id_ids = [self.ops.add(op) for op in site_vec.id_ops]
        # (coef, head, [op id per site head..tail])
        self.terms: List[tuple] = []

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
        if coef == 0:
            return
        if len(ops) != len(idxs) or not ops:
            raise ValueError("operators and site indexes differ in length")
        if list(idxs) != sorted(idxs):
            raise ValueError("site indexes must be ascending")
        if idxs[-1] >= self.N:
            raise ValueError("site index out of range")
        head, tail = idxs[0], idxs[-1]
        per_site: Dict[int, GQTensor] = {}
        for op, s in zip(ops, idxs):
            if s not in per_site:
                per_site[s] = op
        chain = []
        for s in range(head, tail + 1):
            chain.append(self.ops.add(per_site[s]) if s in per_site else self.id_ids[s])
        self.terms.append((float(coef), head, chain))

    # ------------------------------------------------------------------
    def Gen(self) -> List[GQTensor]:
        N = self.N
        if N < 2:
            raise ValueError("an MPO needs at least two sites")
        # states per bond b = 0..N-2 (bond b sits between site b and b+1)
        mids: List[Dict[tuple, int]] = [dict() for _ in range(N - 1)]
        mid_qn: List[List[QN]] = [[] for _ in range(N - 1)]
        has_ready = [False] * (N - 1)
        has_final = [False] * (N - 1)
        zero = self.zero_div
        # transitions[site] : dict (row_key, col_key) -> (op_id or dense, accumulate?)
        trans: List[Dict[tuple, np.ndarray]] = [dict() for _ in range(N)]
        set_once: List[Dict[tuple, int]] = [dict() for _ in range(N)]

        def mid_key(head, chain, b):
            return ("m", head, tuple(chain[: b - head + 1]))

        for coef, head, chain in self.terms:
            tail = head + len(chain) - 1
            for b in range(0, head):
                has_ready[b] = True
            for b in range(tail, N - 1):
                has_final[b] = True
            q = zero
            for s in range(head, tail + 1):
                op_id = chain[s - head]
                q = q - self.ops.divs[op_id]
                row = ("ready",) if s == head else mid_key(head, chain, s - 1)
                if s == tail:
                    if q != zero:
                        raise ValueError("term does not conserve the quantum number")
                    key = (row, ("final",))
                    mat = coef * self.ops.mats[op_id]
                    if key in trans[s]:
                        trans[s][key] = trans[s][key] + mat
                    else:
                        trans[s][key] = mat
                else:
                    col = mid_key(head, chain, s)
                    if col not in mids[s]:
                        mids[s][col] = len(mids[s])
                        mid_qn[s].append(q)
                    elif mid_qn[s][mids[s][col]] != q:
                        raise ValueError("inconsistent intermediate quantum number")
                    set_once[s][(row, col)] = op_id

        # bond state lists: [ready, mids..., final], then grouped by QN
        bond_states: List[List[tuple]] = []
        bond_index: List[Index] = []
        for b in range(N - 1):
            states = []
            if has_ready[b]:
                states.append((("ready",), zero))
            for key, pos in sorted(mids[b].items(), key=lambda kv: kv[1]):
                states.append((key, mid_qn[b][pos]))
            if has_final[b]:
                states.append((("final",), zero))
            order_qn: List[QN] = []
            groups: Dict[QN, list] = {}
            for key, q in states:
                if q not in groups:
                    groups[q] = []
                    order_qn.append(q)
                groups[q].append(key)
            ordered = [k for q in order_qn for k in groups[q]]
            bond_states.append(ordered)
            bond_index.append(Index([(q, len(groups[q])) for q in order_qn], OUT))

        # ready->ready and final->final identities
        for s in range(N):
            lrows = [("ready",)] if s == 0 else bond_states[s - 1]
            rcols = [("final",)] if s == N - 1 else bond_states[s]
            idm = self.ops.mats[self.id_ids[s]]
            if ("ready",) in lrows and ("ready",) in rcols:
                set_once[s][(("ready",), ("ready",))] = self.id_ids[s]
            if ("final",) in lrows and ("final",) in rcols:
                key = (("final",), ("final",))
                trans[s][key] = trans[s].get(key, 0) + idm

        mpo: List[GQTensor] = []
        for s in range(N):
            lrows = [("ready",)] if s == 0 else bond_states[s - 1]
            rcols = [("final",)] if s == N - 1 else bond_states[s]
            rpos = {k: i for i, k in enumerate(lrows)}
            cpos = {k: i for i, k in enumerate(rcols)}
            d = self.pb_out[s].dim
            dense = np.zeros((len(lrows), d, d, len(rcols)))
            for (r, c), op_id in set_once[s].items():
                dense[rpos[r], :, :, cpos[c]] = self.ops.mats[op_id]
            for (r, c), mat in trans[s].items():
                dense[rpos[r], :, :, cpos[c]] += mat
            if s == 0:
                idx = [self.pb_in[0], bond_index[0], self.pb_out[0]]
                arr = dense[0].transpose(0, 2, 1)          # (p_in, r, p_out)
            elif s == N - 1:
                idx = [self.pb_in[s], bond_index[s - 1].inverse(), self.pb_out[s]]
                arr = dense[:, :, :, 0].transpose(1, 0, 2)  # (p_in, l, p_out)
            else:
                idx = [bond_index[s - 1].inverse(), self.pb_in[s], self.pb_out[s], bond_index[s]]
                arr = dense
            mpo.append(_dense_to_blocks(arr, idx, zero))
        self.bond_dims = [ix.dim for ix in bond_index]
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
