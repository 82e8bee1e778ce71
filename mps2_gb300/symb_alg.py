"""Symbolic algebra of MPO coefficients and operators (host side of the MPO
generator).

Restates gqmps2's ``one_dim_tn/mpo/mpogen/symb_alg/coef_op_alg.h`` and
``symb_alg/sparse_mat.h`` with the same meaning, names and results:

* ``CoefRepr`` (``coef_op_alg.h:34-99``): a coefficient written as a sum of
  coefficient labels; equality compares the labels as a multiset, ``+``
  concatenates, ``Realize`` sums the labelled values in list order.
* ``OpRepr`` (``:112-259``): an operator written as a sum of labelled base
  operators, each with a ``CoefRepr``; a base label occurs at most once (its
  coefficients are merged), equality ignores the order of the terms.
* ``SeparateCoefAndBase`` (``:267-284``), ``GetOpReprCoef`` (``:287-289``).
* ``SparMat`` (``sparse_mat.h:17-200``): a rows x cols matrix whose unset
  elements read as the null element; setting the null element is a no-op, and
  removing the only row or column leaves a 0 x 0 matrix, as the reference's
  does.
* ``SparOpReprMat`` (``coef_op_alg.h:300-515``): row/column sorting by fill,
  common row/column coefficients, linear-combination detection.
* the incomplete products of a coefficient matrix and an operator matrix
  (``:520-603``), row/column linear combinations (``:606-676``), the
  delinearisers (``:679-740``) and the row/column compressers (``:743-804``).

The data structure is this project's own: a matrix is a list of per-row
dictionaries (column -> element), so the compressers walk only the set
elements.  Two deliberate differences, neither of which changes a result:
the delinearisers resume the scan at the removed row instead of restarting
from row 1 (rows before it cannot change: their test reads only rows above
them, which a removal leaves alone), and the reference's ``exit(1)`` on an
unsupported coefficient product becomes a ``ValueError``.
"""
from __future__ import annotations

from typing import Dict, Iterable, List, Sequence, Tuple

# ---------------------------------------------------------------------------
# coefficients
# ---------------------------------------------------------------------------
CoefLabel = int
kIdCoefLabel: CoefLabel = 0


class CoefRepr:
    """Sum of coefficient labels (``coef_op_alg.h:34-99``)."""

    __slots__ = ("labels", "_key")

    def __init__(self, labels: Iterable[int] | int = ()):
        if isinstance(labels, CoefRepr):
            labels = labels.labels
        elif isinstance(labels, int):
            labels = (labels,)
        self.labels: Tuple[int, ...] = tuple(int(x) for x in labels)
        self._key = tuple(sorted(self.labels))

    def GetCoefLabelList(self) -> List[int]:
        return list(self.labels)

    def __eq__(self, other) -> bool:
        return isinstance(other, CoefRepr) and self._key == other._key

    def __ne__(self, other) -> bool:
        return not self == other

    def __hash__(self) -> int:
        return hash(self._key)

    def __add__(self, other: "CoefRepr") -> "CoefRepr":
        return CoefRepr(self.labels + _as_coef(other).labels)

    def Realize(self, label_coef_mapping: Sequence):
        coef = 0
        for label in self.labels:
            coef += label_coef_mapping[label]
        return coef

    def __repr__(self) -> str:
        return f"CoefRepr({list(self.labels)})"


kNullCoefRepr = CoefRepr(())
kIdCoefRepr = CoefRepr((kIdCoefLabel,))


def _as_coef(c) -> CoefRepr:
    return c if isinstance(c, CoefRepr) else CoefRepr(c)


# ---------------------------------------------------------------------------
# operators
# ---------------------------------------------------------------------------
OpLabel = int
kIdOpLabel: OpLabel = 0


class OpRepr:
    """Sum of labelled base operators with symbolic coefficients
    (``coef_op_alg.h:112-259``).

    ``OpRepr()`` is the null operator; ``OpRepr(label)``;
    ``OpRepr(coef, label)``; ``OpRepr([coefs], [labels])`` (repeated labels
    merge their coefficients); ``OpRepr([labels])`` (identity coefficients).
    """

    __slots__ = ("coefs", "ops", "_key")

    def __init__(self, *args):
        if not args:
            coefs, labels = [], []
        elif len(args) == 1:
            a = args[0]
            if isinstance(a, (list, tuple)):
                labels = list(a)
                coefs = [kIdCoefRepr] * len(labels)
            else:
                coefs, labels = [kIdCoefRepr], [a]
        elif len(args) == 2:
            c, l = args
            if isinstance(l, (list, tuple)):
                coefs, labels = [_as_coef(x) for x in c], list(l)
                if len(coefs) != len(labels):
                    raise ValueError("OpRepr: coefficient and label lists differ in length")
            else:
                coefs, labels = [_as_coef(c)], [l]
        else:
            raise TypeError("OpRepr takes at most two arguments")
        out_c: List[CoefRepr] = []
        out_l: List[int] = []
        for c, l in zip(coefs, labels):
            l = int(l)
            try:
                k = out_l.index(l)
            except ValueError:
                out_c.append(c)
                out_l.append(l)
            else:
                out_c[k] = out_c[k] + c
        self.coefs: Tuple[CoefRepr, ...] = tuple(out_c)
        self.ops: Tuple[int, ...] = tuple(out_l)
        self._key = frozenset((l, c._key) for l, c in zip(out_l, out_c))

    @classmethod
    def _raw(cls, coefs: Sequence[CoefRepr], ops: Sequence[int]) -> "OpRepr":
        """Build from term lists already free of repeated labels."""
        o = cls.__new__(cls)
        o.coefs = tuple(coefs)
        o.ops = tuple(ops)
        o._key = frozenset((l, c._key) for l, c in zip(o.ops, o.coefs))
        return o

    def GetCoefReprList(self) -> List[CoefRepr]:
        return list(self.coefs)

    def GetOpLabelList(self) -> List[int]:
        return list(self.ops)

    def __len__(self) -> int:
        return len(self.ops)

    def __eq__(self, other) -> bool:
        return isinstance(other, OpRepr) and self._key == other._key

    def __ne__(self, other) -> bool:
        return not self == other

    def __hash__(self) -> int:
        return hash(self._key)

    def __add__(self, other: "OpRepr") -> "OpRepr":
        if not other.ops:
            return self
        coefs = list(self.coefs)
        ops = list(self.ops)
        for c, l in zip(other.coefs, other.ops):
            try:
                k = ops.index(l)
            except ValueError:
                coefs.append(c)
                ops.append(l)
            else:
                coefs[k] = coefs[k] + c
        return OpRepr._raw(coefs, ops)

    def Realize(self, label_coef_mapping: Sequence, label_op_mapping: Sequence):
        """``sum_i coef_i * op_i`` in term order (``:225-246``)."""
        if not self.ops:
            return None
        op = self.coefs[0].Realize(label_coef_mapping) * label_op_mapping[self.ops[0]]
        for c, l in zip(self.coefs[1:], self.ops[1:]):
            op = op + c.Realize(label_coef_mapping) * label_op_mapping[l]
        return op

    def __repr__(self) -> str:
        if not self.ops:
            return "OpRepr()"
        return "OpRepr(" + " + ".join(f"{list(c.labels)}*{l}"
                                      for c, l in zip(self.coefs, self.ops)) + ")"


kNullOpRepr = OpRepr()
kIdOpRepr = OpRepr(kIdOpLabel)


def SeparateCoefAndBase(op: OpRepr) -> Tuple[CoefRepr, OpRepr]:
    """``coef_op_alg.h:267-284``: a coefficient common to every term and the
    operator without it; a mixed operator gives (identity, itself)."""
    n = len(op.ops)
    if n == 0:
        return kNullCoefRepr, kNullOpRepr
    if n == 1:
        return op.coefs[0], OpRepr._raw((kIdCoefRepr,), op.ops)
    c0 = op.coefs[0]
    for c in op.coefs[1:]:
        if c != c0:
            return kIdCoefRepr, op
    return c0, OpRepr._raw((kIdCoefRepr,) * n, op.ops)


def GetOpReprCoef(op: OpRepr) -> CoefRepr:
    return SeparateCoefAndBase(op)[0]


# ---------------------------------------------------------------------------
# sparse matrices
# ---------------------------------------------------------------------------
class SparMat:
    """Matrix of symbolic elements; unset elements read as ``null``."""

    null = None

    def __init__(self, rows: int = 0, cols: int = 0):
        self.rows = int(rows)
        self.cols = int(cols)
        self._r: List[Dict[int, object]] = [dict() for _ in range(self.rows)]

    def copy(self):
        m = type(self).__new__(type(self))
        m.rows, m.cols = self.rows, self.cols
        m._r = [dict(r) for r in self._r]
        return m

    # element access ---------------------------------------------------------
    def __call__(self, x: int, y: int):
        return self._r[x].get(y, self.null)

    def SetElem(self, x: int, y: int, elem) -> None:
        if elem == self.null:
            return
        if not (0 <= x < self.rows and 0 <= y < self.cols):
            raise IndexError(f"element ({x}, {y}) outside a {self.rows} x {self.cols} matrix")
        self._r[x][y] = elem

    def is_set(self, x: int, y: int) -> bool:
        return y in self._r[x]

    def row_items(self, x: int):
        """The set elements of row x, by ascending column."""
        return sorted(self._r[x].items())

    def col_items(self, y: int):
        return [(x, r[y]) for x, r in enumerate(self._r) if y in r]

    def GetRow(self, x: int) -> list:
        r = self._r[x]
        return [r.get(y, self.null) for y in range(self.cols)]

    def GetCol(self, y: int) -> list:
        return [r.get(y, self.null) for r in self._r]

    def __eq__(self, other) -> bool:
        if not isinstance(other, SparMat):
            return NotImplemented
        if self.rows != other.rows or self.cols != other.cols:
            return False
        for a, b in zip(self._r, other._r):
            for y in set(a) | set(b):
                if a.get(y, self.null) != b.get(y, other.null):
                    return False
        return True

    def __ne__(self, other) -> bool:
        return not self == other

    # structure --------------------------------------------------------------
    def RemoveRow(self, x: int) -> None:
        if not 0 <= x < self.rows:
            raise IndexError("row out of range")
        if self.rows == 1:
            self.rows, self.cols, self._r = 0, 0, []
            return
        del self._r[x]
        self.rows -= 1

    def RemoveCol(self, y: int) -> None:
        if not 0 <= y < self.cols:
            raise IndexError("column out of range")
        if self.cols == 1:
            self.rows, self.cols, self._r = 0, 0, []
            return
        self._r = [{(c if c < y else c - 1): e for c, e in r.items() if c != y} for r in self._r]
        self.cols -= 1

    def SwapTwoRows(self, a: int, b: int) -> None:
        self._r[a], self._r[b] = self._r[b], self._r[a]

    def SwapTwoCols(self, a: int, b: int) -> None:
        if a == b:
            return
        swap = {a: b, b: a}
        self._r = [{swap.get(c, c): e for c, e in r.items()} for r in self._r]

    def TransposeRows(self, order: Sequence[int]) -> None:
        """Row i becomes the old row ``order[i]``."""
        if len(order) != self.rows:
            raise ValueError("TransposeRows: permutation length differs from the row count")
        self._r = [self._r[i] for i in order]

    def TransposeCols(self, order: Sequence[int]) -> None:
        """Column i becomes the old column ``order[i]``."""
        if len(order) != self.cols:
            raise ValueError("TransposeCols: permutation length differs from the column count")
        new_of_old = {old: new for new, old in enumerate(order)}
        self._r = [{new_of_old[c]: e for c, e in r.items()} for r in self._r]

    def nnz_row(self, x: int) -> int:
        return len(self._r[x])

    def nnz_col(self, y: int) -> int:
        return sum(1 for r in self._r if y in r)

    def __repr__(self) -> str:
        lines = [f"{type(self).__name__}({self.rows}, {self.cols})"]
        for x in range(self.rows):
            for y, e in self.row_items(x):
                lines.append(f"  ({x}, {y}) = {e!r}")
        return "\n".join(lines)


class SparCoefReprMat(SparMat):
    null = kNullCoefRepr


class SparOpReprMat(SparMat):
    """``coef_op_alg.h:300-515``."""

    null = kNullOpRepr

    def SortRows(self) -> List[int]:
        """Rows by ascending number of set elements (ties keep their
        order); returns the permutation applied."""
        order = [x for _, x in sorted((self.nnz_row(x), x) for x in range(self.rows))]
        self.TransposeRows(order)
        return order

    def SortCols(self) -> List[int]:
        order = [y for _, y in sorted((self.nnz_col(y), y) for y in range(self.cols))]
        self.TransposeCols(order)
        return order

    def _common_coef(self, elems) -> CoefRepr:
        coefs = [GetOpReprCoef(e) for e in elems]
        if not coefs:
            return kNullCoefRepr
        c0 = coefs[0]
        for c in coefs:
            if c != c0:
                return kIdCoefRepr
        return c0

    def CalcRowCoef(self, x: int) -> CoefRepr:
        return self._common_coef(e for _, e in self.row_items(x))

    def CalcColCoef(self, y: int) -> CoefRepr:
        return self._common_coef(e for _, e in self.col_items(y))

    def RemoveRowCoef(self, x: int) -> None:
        r = self._r[x]
        for y in list(r):
            r[y] = SeparateCoefAndBase(r[y])[1]

    def RemoveColCoef(self, y: int) -> None:
        for r in self._r:
            if y in r:
                r[y] = SeparateCoefAndBase(r[y])[1]

    @staticmethod
    def _overlap(tgt: Dict[int, OpRepr], base_items) -> CoefRepr:
        """``CalcRowOverlap_``/``CalcColOverlap_`` (``:468-512``): the
        coefficient c with tgt = c * base on every set element of base."""
        poss: List[CoefRepr] = []
        for k, base in base_items:
            t = tgt.get(k, kNullOpRepr)
            if t == base:
                poss.append(kIdCoefRepr)
            else:
                c, b = SeparateCoefAndBase(t)
                if b == base:
                    poss.append(c)
                else:
                    return kNullCoefRepr
        if not poss:
            return kNullCoefRepr
        for c in poss:
            if c != poss[0]:
                return kNullCoefRepr
        return poss[0]

    def CalcRowLinCmb(self, x: int) -> List[CoefRepr]:
        tgt = self._r[x]
        return [self._overlap(tgt, self.row_items(i)) for i in range(x)]

    def CalcColLinCmb(self, y: int) -> List[CoefRepr]:
        tgt = {x: r[y] for x, r in enumerate(self._r) if y in r}
        return [self._overlap(tgt, self.col_items(j)) for j in range(y)]


SparOpReprMatVec = List[SparOpReprMat]


# ---------------------------------------------------------------------------
# incomplete products
# ---------------------------------------------------------------------------
def CoefReprOpReprIncompleteMulti(coef: CoefRepr, op: OpRepr) -> OpRepr:
    """``coef_op_alg.h:520-532``: only an operator whose coefficients are all
    identity can take a non-identity coefficient."""
    if op == kNullOpRepr:
        return kNullOpRepr
    if coef == kIdCoefRepr:
        return op
    for c in op.coefs:
        if c != kIdCoefRepr:
            raise ValueError("CoefReprOpReprIncompleteMulti: operator already carries a "
                             "coefficient")
    return OpRepr._raw((coef,) * len(op.ops), op.ops)


def SparCoefReprMatSparOpReprMatIncompleteMulti(coef_mat: SparCoefReprMat,
                                                op_mat: SparOpReprMat) -> SparOpReprMat:
    """``res(x, y) = sum_k coef(x, k) * op(k, y)``, terms added by ascending k
    (``coef_op_alg.h:535-582``)."""
    if coef_mat.cols != op_mat.rows:
        raise ValueError("incomplete product: inner dimensions differ")
    res = SparOpReprMat(coef_mat.rows, op_mat.cols)
    for x in range(coef_mat.rows):
        acc: Dict[int, OpRepr] = {}
        for k, c in coef_mat.row_items(x):
            for y, o in op_mat.row_items(k):
                acc[y] = acc.get(y, kNullOpRepr) + CoefReprOpReprIncompleteMulti(c, o)
        for y, e in acc.items():
            res.SetElem(x, y, e)
    return res


def SparOpReprMatSparCoefReprMatIncompleteMulti(op_mat: SparOpReprMat,
                                                coef_mat: SparCoefReprMat) -> SparOpReprMat:
    """``res(x, y) = sum_k op(x, k) * coef(k, y)``, terms added by ascending k
    (``coef_op_alg.h:556-603``)."""
    if op_mat.cols != coef_mat.rows:
        raise ValueError("incomplete product: inner dimensions differ")
    res = SparOpReprMat(op_mat.rows, coef_mat.cols)
    for x in range(op_mat.rows):
        acc: Dict[int, OpRepr] = {}
        for k, o in op_mat.row_items(x):
            for y, c in coef_mat.row_items(k):
                acc[y] = acc.get(y, kNullOpRepr) + CoefReprOpReprIncompleteMulti(c, o)
        for y, e in acc.items():
            res.SetElem(x, y, e)
    return res


# ---------------------------------------------------------------------------
# linear combinations, delinearisation, compression
# ---------------------------------------------------------------------------
def _scaled(elem: OpRepr, coef: CoefRepr) -> OpRepr:
    cs = []
    for c in elem.coefs:
        if c != kIdCoefRepr:
            raise ValueError("linear combination of rows that carry coefficients")
        cs.append(coef)
    return OpRepr._raw(cs, elem.ops)


def _lin_cmb(lines, cmb: Sequence[CoefRepr]) -> Dict[int, OpRepr]:
    """``CalcSparOpReprMatRowLinCmb``/``ColLinCmb`` (``:606-676``) over the
    set elements; ``lines[i]`` yields line i's (position, element) pairs."""
    if not cmb:
        raise ValueError("empty linear combination")
    res: Dict[int, OpRepr] = {}
    for i, c in enumerate(cmb):
        if c == kNullCoefRepr:
            continue
        ident = c == kIdCoefRepr
        for j, e in lines(i):
            res[j] = res.get(j, kNullOpRepr) + (e if ident else _scaled(e, c))
    return res


def _as_vec(d: Dict[int, OpRepr], n: int) -> List[OpRepr]:
    return [d.get(j, kNullOpRepr) for j in range(n)]


def CalcSparOpReprMatRowLinCmb(m: SparOpReprMat, cmb: Sequence[CoefRepr]) -> List[OpRepr]:
    return _as_vec(_lin_cmb(m.row_items, cmb), m.cols)


def CalcSparOpReprMatColLinCmb(m: SparOpReprMat, cmb: Sequence[CoefRepr]) -> List[OpRepr]:
    return _as_vec(_lin_cmb(m.col_items, cmb), m.rows)


def _same_line(res: Dict[int, OpRepr], items) -> bool:
    line = dict(items)
    for j in set(res) | set(line):
        if res.get(j, kNullOpRepr) != line.get(j, kNullOpRepr):
            return False
    return True


def _take(dst: SparMat, src: SparMat) -> None:
    """Make ``dst`` hold ``src`` (the reference's by-reference follower)."""
    dst.rows, dst.cols, dst._r = src.rows, src.cols, src._r


def SparOpReprMatRowDelinearize(target: SparOpReprMat, follower: SparOpReprMat) -> None:
    """Remove every row of ``target`` that is a combination of the rows
    above it and fold the combination into ``follower``'s columns
    (``coef_op_alg.h:679-708``).  Both matrices change in place."""
    i = 1
    while i < target.rows:
        cmb = target.CalcRowLinCmb(i)
        if _same_line(_lin_cmb(target.row_items, cmb), target.row_items(i)):
            n = target.rows
            target.RemoveRow(i)
            trans = SparCoefReprMat(n, n - 1)
            for j in range(i):
                trans.SetElem(j, j, kIdCoefRepr)
                trans.SetElem(i, j, cmb[j])
            for j in range(i + 1, n):
                trans.SetElem(j, j - 1, kIdCoefRepr)
            _take(follower, SparOpReprMatSparCoefReprMatIncompleteMulti(follower, trans))
        else:
            i += 1


def SparOpReprMatColDelinearize(target: SparOpReprMat, follower: SparOpReprMat) -> None:
    """Column version of the above (``coef_op_alg.h:711-740``)."""
    i = 1
    while i < target.cols:
        cmb = target.CalcColLinCmb(i)
        if _same_line(_lin_cmb(target.col_items, cmb), target.col_items(i)):
            n = target.cols
            target.RemoveCol(i)
            trans = SparCoefReprMat(n - 1, n)
            for j in range(i):
                trans.SetElem(j, j, kIdCoefRepr)
                trans.SetElem(j, i, cmb[j])
            for j in range(i + 1, n):
                trans.SetElem(j - 1, j, kIdCoefRepr)
            _take(follower, SparCoefReprMatSparOpReprMatIncompleteMulti(trans, follower))
        else:
            i += 1


def SparOpReprMatRowCompresser(target: SparOpReprMat, follower: SparOpReprMat) -> None:
    """``coef_op_alg.h:743-772``: sort target's rows, move common row
    coefficients into follower's columns, then delinearise.  Both matrices
    change in place."""
    if target.rows != follower.cols:
        raise ValueError("row compresser: target rows differ from follower columns")
    n = target.rows
    if n == 1:
        return
    order = target.SortRows()
    follower.TransposeCols(order)
    diag = SparCoefReprMat(n, n)
    separate = False
    for x in range(n):
        c = target.CalcRowCoef(x)
        diag.SetElem(x, x, c if c != kNullCoefRepr else kIdCoefRepr)
        if c != kNullCoefRepr and c != kIdCoefRepr:
            separate = True
            target.RemoveRowCoef(x)
    if separate:
        _take(follower, SparOpReprMatSparCoefReprMatIncompleteMulti(follower, diag))
    SparOpReprMatRowDelinearize(target, follower)


def SparOpReprMatColCompresser(target: SparOpReprMat, follower: SparOpReprMat) -> None:
    """``coef_op_alg.h:775-804``: the column version."""
    if target.cols != follower.rows:
        raise ValueError("column compresser: target columns differ from follower rows")
    n = target.cols
    if n == 1:
        return
    order = target.SortCols()
    follower.TransposeRows(order)
    diag = SparCoefReprMat(n, n)
    separate = False
    for y in range(n):
        c = target.CalcColCoef(y)
        diag.SetElem(y, y, c if c != kNullCoefRepr else kIdCoefRepr)
        if c != kNullCoefRepr and c != kIdCoefRepr:
            separate = True
            target.RemoveColCoef(y)
    if separate:
        _take(follower, SparCoefReprMatSparOpReprMatIncompleteMulti(diag, follower))
    SparOpReprMatColDelinearize(target, follower)
