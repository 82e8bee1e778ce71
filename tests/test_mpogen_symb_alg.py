"""Symbolic algebra of the MPO generator against the reference's unit tests
(``tests/test_one_dim_tn/test_mpogen/test_mpogen_coef_op_alg.cc``): the same
cases and benchmark matrices, random cases seeded."""
import random

import pytest

from mps2_gb300.symb_alg import (
    CalcSparOpReprMatColLinCmb, CalcSparOpReprMatRowLinCmb, CoefRepr, OpRepr,
    SparCoefReprMat, SparCoefReprMatSparOpReprMatIncompleteMulti, SparOpReprMat,
    SparOpReprMatColCompresser, SparOpReprMatRowCompresser,
    SparOpReprMatSparCoefReprMatIncompleteMulti, kIdCoefLabel, kIdCoefRepr, kIdOpLabel,
    kIdOpRepr, kNullCoefRepr, kNullOpRepr)

RNG = random.Random(20191029)
K_MAX_TERMS = 5


def rand_coef():
    return CoefRepr([RNG.randrange(1 << 30) for _ in range(RNG.randrange(K_MAX_TERMS) + 1)])


def rand_op():
    n = RNG.randrange(K_MAX_TERMS) + 1
    return OpRepr([rand_coef() for _ in range(n)], [RNG.randrange(1 << 30) for _ in range(n)])


def rand_fill(m, filling, gen):
    for _ in range(max(1, (m.rows * m.cols) // filling)):
        m.SetElem(RNG.randrange(m.rows), RNG.randrange(m.cols), gen())


# --- CoefRepr (:106-170) ------------------------------------------------------
def test_coef_repr_init_equal_add():
    assert CoefRepr().GetCoefLabelList() == []
    assert CoefRepr(kIdCoefLabel).GetCoefLabelList() == [kIdCoefLabel]
    for size in (1, 2, 5, 10):
        labels = [RNG.randrange(1 << 30) for _ in range(size)]
        assert CoefRepr(labels) == CoefRepr(list(reversed(labels)))
        assert CoefRepr(labels) != CoefRepr(labels + [7])
    for ls, rs in ((0, 0), (1, 0), (0, 1), (2, 3), (5, 5)):
        a = [RNG.randrange(99) for _ in range(ls)]
        b = [RNG.randrange(99) for _ in range(rs)]
        assert (CoefRepr(a) + CoefRepr(b)).GetCoefLabelList() == a + b


# --- OpRepr (:176-305) --------------------------------------------------------
def test_op_repr_init():
    assert OpRepr().GetCoefReprList() == [] and OpRepr().GetOpLabelList() == []
    op = OpRepr(3)
    assert op.GetCoefReprList() == [kIdCoefRepr] and op.GetOpLabelList() == [3]
    op = OpRepr(CoefRepr(2), 3)
    assert op.GetCoefReprList() == [CoefRepr(2)] and op.GetOpLabelList() == [3]
    # repeated labels merge their coefficients
    op = OpRepr([1, 2, 3], [5, 6, 5])
    assert op.GetOpLabelList() == [5, 6]
    assert op.GetCoefReprList() == [CoefRepr([1, 3]), CoefRepr(2)]
    assert OpRepr([4, 5]) == OpRepr([kIdCoefRepr, kIdCoefRepr], [4, 5])


def test_op_repr_equal_and_add():
    for size in (1, 2, 5, 10):
        coefs = [rand_coef() for _ in range(size)]
        labels = RNG.sample(range(1 << 20), size)
        a = OpRepr(coefs, labels)
        assert a == OpRepr(list(reversed(coefs)), list(reversed(labels)))
        assert a != OpRepr(coefs[:-1], labels[:-1])
    for ls, rs in ((1, 1), (2, 3), (5, 5)):
        ca, la = [rand_coef() for _ in range(ls)], RNG.sample(range(1000), ls)
        cb, lb = [rand_coef() for _ in range(rs)], RNG.sample(range(1000, 2000), rs)
        assert OpRepr(ca, la) + OpRepr(cb, lb) == OpRepr(ca + cb, la + lb)
    a, b = OpRepr(1, 1), OpRepr(2, 1)
    assert a + b == OpRepr(CoefRepr([1, 2]), 1)


# --- SparMat (:312-556) -------------------------------------------------------
@pytest.mark.parametrize("rows,cols", [(1, 1), (1, 5), (5, 3), (3, 5), (5, 5)])
def test_spar_mat_getters_remove_swap_transpose(rows, cols):
    m = SparCoefReprMat(rows, cols)
    assert (m.rows, m.cols) == (rows, cols)
    assert all(m(x, y) == kNullCoefRepr for x in range(rows) for y in range(cols))
    dense = [[kNullCoefRepr] * cols for _ in range(rows)]
    for _ in range(rows * cols):
        x, y, c = RNG.randrange(rows), RNG.randrange(cols), rand_coef()
        m.SetElem(x, y, c)
        dense[x][y] = c
    m.SetElem(0, 0, kNullCoefRepr)          # setting null changes nothing
    assert m(0, 0) == dense[0][0]
    for x in range(rows):
        assert m.GetRow(x) == dense[x]
    for y in range(cols):
        assert m.GetCol(y) == [dense[x][y] for x in range(rows)]
    if rows > 1:
        m2 = m.copy()
        m2.RemoveRow(1)
        assert [m2.GetRow(x) for x in range(rows - 1)] == dense[:1] + dense[2:]
        m2 = m.copy()
        m2.SwapTwoRows(0, rows - 1)
        assert m2.GetRow(0) == dense[rows - 1] and m2.GetRow(rows - 1) == dense[0]
    if cols > 1:
        m2 = m.copy()
        m2.RemoveCol(1)
        assert [m2.GetRow(x) for x in range(rows)] == [r[:1] + r[2:] for r in dense]
        m2 = m.copy()
        m2.SwapTwoCols(0, cols - 1)
        assert m2.GetCol(0) == [r[cols - 1] for r in dense]
    perm = list(range(rows))
    RNG.shuffle(perm)
    m2 = m.copy()
    m2.TransposeRows(perm)
    assert [m2.GetRow(i) for i in range(rows)] == [dense[p] for p in perm]
    perm = list(range(cols))
    RNG.shuffle(perm)
    m2 = m.copy()
    m2.TransposeCols(perm)
    assert [m2.GetCol(i) for i in range(cols)] == [[r[p] for r in dense] for p in perm]
    one = SparCoefReprMat(1, cols)
    one.RemoveRow(0)
    assert (one.rows, one.cols) == (0, 0)


# --- SparOpReprMat (:559-827) -------------------------------------------------
@pytest.mark.parametrize("rows,cols", [(1, 1), (1, 5), (5, 1), (3, 5), (5, 3), (5, 5), (20, 20)])
def test_sort_rows_and_cols(rows, cols):
    m = SparOpReprMat(rows, cols)
    rand_fill(m, 3, rand_op)
    m.SortRows()
    nnz = [sum(e != kNullOpRepr for e in m.GetRow(x)) for x in range(rows)]
    assert nnz == sorted(nnz)
    m.SortCols()
    nnz = [sum(e != kNullOpRepr for e in m.GetCol(y)) for y in range(cols)]
    assert nnz == sorted(nnz)


def test_calc_row_and_col_coefs():
    c1, c2, c3 = rand_coef(), rand_coef(), rand_coef()
    m = SparOpReprMat(5, 5)
    m.SetElem(0, 4, OpRepr(1))
    m.SetElem(1, 1, OpRepr([c1, c1], [2, 3]))
    m.SetElem(1, 3, OpRepr(c2, 4))
    m.SetElem(3, 1, OpRepr(c1, 5))
    m.SetElem(3, 3, OpRepr(c1, 6))
    m.SetElem(4, 2, OpRepr(c3, 7))
    assert [m.CalcRowCoef(i) for i in range(5)] == [kIdCoefRepr, kIdCoefRepr, kNullCoefRepr,
                                                    c1, c3]
    assert [m.CalcColCoef(i) for i in range(5)] == [kNullCoefRepr, c1, c3, kIdCoefRepr,
                                                    kIdCoefRepr]


def _lin_cmb_cases(transpose):
    """Row cases (:661-738); ``transpose`` gives the column cases (:740-817)."""
    def mat(r, c):
        return SparOpReprMat(c, r) if transpose else SparOpReprMat(r, c)

    def put(m, x, y, e):
        m.SetElem(y, x, e) if transpose else m.SetElem(x, y, e)

    def cmb(m, i):
        return m.CalcColLinCmb(i) if transpose else m.CalcRowLinCmb(i)

    m = mat(1, 1)
    assert cmb(m, 0) == []
    put(m, 0, 0, rand_op())
    assert cmb(m, 0) == []

    m = mat(2, 2)
    assert cmb(m, 0) == [] and cmb(m, 1) == [kNullCoefRepr]
    put(m, 0, 0, OpRepr(1))
    assert cmb(m, 1) == [kNullCoefRepr]
    put(m, 1, 0, OpRepr(1))
    assert cmb(m, 1) == [kIdCoefRepr]
    put(m, 1, 0, OpRepr(1, 1))
    assert cmb(m, 1) == [CoefRepr(1)]
    put(m, 0, 1, OpRepr(2))
    assert cmb(m, 1) == [kNullCoefRepr]
    put(m, 1, 1, OpRepr(1, 2))
    assert cmb(m, 1) == [CoefRepr(1)]
    put(m, 1, 1, OpRepr(2, 2))
    assert cmb(m, 1) == [kNullCoefRepr]

    m = mat(3, 2)
    assert cmb(m, 2) == [kNullCoefRepr, kNullCoefRepr]
    put(m, 0, 0, OpRepr(1))
    put(m, 1, 1, OpRepr(2))
    assert cmb(m, 2) == [kNullCoefRepr, kNullCoefRepr]
    put(m, 2, 0, OpRepr(1))
    assert cmb(m, 2) == [kIdCoefRepr, kNullCoefRepr]
    put(m, 2, 1, OpRepr(2))
    assert cmb(m, 2) == [kIdCoefRepr, kIdCoefRepr]
    put(m, 2, 0, OpRepr(1, 1))
    assert cmb(m, 2) == [CoefRepr(1), kIdCoefRepr]
    put(m, 2, 1, OpRepr(2, 2))
    assert cmb(m, 2) == [CoefRepr(1), CoefRepr(2)]
    # the combination itself reproduces the row (or column)
    lc = (CalcSparOpReprMatColLinCmb if transpose else CalcSparOpReprMatRowLinCmb)(
        m, cmb(m, 2))
    assert lc == (m.GetCol(2) if transpose else m.GetRow(2))


def test_row_lin_cmb():
    _lin_cmb_cases(False)


def test_col_lin_cmb():
    _lin_cmb_cases(True)


# --- incomplete products (:829-1068) --------------------------------------------
def test_coef_op_incomplete_multi():
    res = SparCoefReprMatSparOpReprMatIncompleteMulti(SparCoefReprMat(), SparOpReprMat())
    assert res == SparOpReprMat()
    cm, om = SparCoefReprMat(1, 1), SparOpReprMat(1, 1)
    assert SparCoefReprMatSparOpReprMatIncompleteMulti(cm, om) == SparOpReprMat(1, 1)
    cm.SetElem(0, 0, CoefRepr(1))
    om.SetElem(0, 0, OpRepr(1))
    b = SparOpReprMat(1, 1)
    b.SetElem(0, 0, OpRepr(1, 1))
    assert SparCoefReprMatSparOpReprMatIncompleteMulti(cm, om) == b

    j, jp, s = CoefRepr(1), CoefRepr(2), 1
    cm, om, b = SparCoefReprMat(2, 4), SparOpReprMat(4, 6), SparOpReprMat(2, 6)
    cm.SetElem(0, 0, kIdCoefRepr); cm.SetElem(1, 1, j); cm.SetElem(1, 2, j); cm.SetElem(1, 3, jp)
    om.SetElem(0, 0, kIdOpRepr); om.SetElem(2, 1, kIdOpRepr); om.SetElem(3, 2, kIdOpRepr)
    om.SetElem(0, 3, OpRepr(j, s)); om.SetElem(0, 4, OpRepr(jp, s)); om.SetElem(1, 5, OpRepr(s))
    b.SetElem(0, 0, kIdOpRepr); b.SetElem(1, 1, OpRepr(j, kIdOpLabel))
    b.SetElem(1, 2, OpRepr(jp, kIdOpLabel)); b.SetElem(0, 3, OpRepr(j, s))
    b.SetElem(0, 4, OpRepr(jp, s)); b.SetElem(1, 5, OpRepr(j, s))
    assert SparCoefReprMatSparOpReprMatIncompleteMulti(cm, om) == b

    cm, om, b = SparCoefReprMat(4, 6), SparOpReprMat(6, 4), SparOpReprMat(4, 4)
    cm.SetElem(0, 0, kIdCoefRepr); cm.SetElem(1, 1, j); cm.SetElem(1, 2, jp)
    cm.SetElem(2, 3, j); cm.SetElem(2, 4, jp); cm.SetElem(3, 5, j)
    om.SetElem(2, 0, kIdOpRepr); om.SetElem(3, 1, kIdOpRepr); om.SetElem(0, 2, OpRepr(j, s))
    om.SetElem(1, 3, OpRepr(s)); om.SetElem(4, 3, OpRepr(s)); om.SetElem(5, 3, kIdOpRepr)
    b.SetElem(1, 0, OpRepr(jp, kIdOpLabel)); b.SetElem(2, 1, OpRepr(j, kIdOpLabel))
    b.SetElem(0, 2, OpRepr(j, s)); b.SetElem(1, 3, OpRepr(j, s)); b.SetElem(2, 3, OpRepr(jp, s))
    b.SetElem(3, 3, OpRepr(j, kIdOpLabel))
    assert SparCoefReprMatSparOpReprMatIncompleteMulti(cm, om) == b

    k, sx, sy, sz = CoefRepr(2), 1, 2, 3
    cm, om, b = SparCoefReprMat(4, 5), SparOpReprMat(5, 6), SparOpReprMat(4, 6)
    cm.SetElem(0, 0, kIdCoefRepr); cm.SetElem(1, 1, j); cm.SetElem(2, 2, j)
    cm.SetElem(3, 3, j); cm.SetElem(1, 4, k)
    om.SetElem(0, 0, OpRepr(j, sx)); om.SetElem(0, 1, OpRepr(j, sy)); om.SetElem(0, 2, OpRepr(j, sz))
    om.SetElem(4, 3, OpRepr(sx)); om.SetElem(0, 4, OpRepr(k, sz)); om.SetElem(1, 5, OpRepr(sx))
    om.SetElem(2, 5, OpRepr(sy)); om.SetElem(3, 5, OpRepr(sz))
    b.SetElem(0, 0, OpRepr(j, sx)); b.SetElem(0, 1, OpRepr(j, sy)); b.SetElem(0, 2, OpRepr(j, sz))
    b.SetElem(1, 3, OpRepr(k, sx)); b.SetElem(0, 4, OpRepr(k, sz)); b.SetElem(1, 5, OpRepr(j, sx))
    b.SetElem(2, 5, OpRepr(j, sy)); b.SetElem(3, 5, OpRepr(j, sz))
    assert SparCoefReprMatSparOpReprMatIncompleteMulti(cm, om) == b

    cm, om, b = SparCoefReprMat(5, 6), SparOpReprMat(6, 1), SparOpReprMat(5, 1)
    cm.SetElem(0, 0, j); cm.SetElem(1, 1, j); cm.SetElem(2, 2, j); cm.SetElem(3, 3, k)
    cm.SetElem(2, 4, k); cm.SetElem(4, 5, j)
    for x, e in enumerate([OpRepr(sx), OpRepr(sy), OpRepr(sz), kIdOpRepr, OpRepr(sz), kIdOpRepr]):
        om.SetElem(x, 0, e)
    b.SetElem(0, 0, OpRepr(j, sx)); b.SetElem(1, 0, OpRepr(j, sy)); b.SetElem(2, 0, OpRepr(j + k, sz))
    b.SetElem(3, 0, OpRepr(k, kIdOpLabel)); b.SetElem(4, 0, OpRepr(j, kIdOpLabel))
    assert SparCoefReprMatSparOpReprMatIncompleteMulti(cm, om) == b


def test_op_coef_incomplete_multi():
    assert SparOpReprMatSparCoefReprMatIncompleteMulti(SparOpReprMat(), SparCoefReprMat()) \
        == SparOpReprMat()
    cm, om = SparCoefReprMat(1, 1), SparOpReprMat(1, 1)
    assert SparOpReprMatSparCoefReprMatIncompleteMulti(om, cm) == SparOpReprMat(1, 1)
    cm.SetElem(0, 0, CoefRepr(1))
    om.SetElem(0, 0, OpRepr(1))
    b = SparOpReprMat(1, 1)
    b.SetElem(0, 0, OpRepr(1, 1))
    assert SparOpReprMatSparCoefReprMatIncompleteMulti(om, cm) == b

    j, jp, s = CoefRepr(1), CoefRepr(2), 1
    om, cm, b = SparOpReprMat(4, 4), SparCoefReprMat(4, 2), SparOpReprMat(4, 2)
    om.SetElem(0, 2, OpRepr(s)); om.SetElem(1, 0, kIdOpRepr); om.SetElem(1, 3, OpRepr(j, s))
    om.SetElem(2, 1, kIdOpRepr); om.SetElem(2, 3, OpRepr(jp, s)); om.SetElem(3, 3, OpRepr(j, kIdOpLabel))
    cm.SetElem(0, 0, jp); cm.SetElem(1, 0, j); cm.SetElem(2, 0, j); cm.SetElem(3, 1, kIdCoefRepr)
    b.SetElem(0, 0, OpRepr(j, s)); b.SetElem(1, 0, OpRepr(jp, kIdOpLabel)); b.SetElem(1, 1, OpRepr(j, s))
    b.SetElem(2, 0, OpRepr(j, kIdOpLabel)); b.SetElem(2, 1, OpRepr(jp, s))
    b.SetElem(3, 1, OpRepr(j, kIdOpLabel))
    assert SparOpReprMatSparCoefReprMatIncompleteMulti(om, cm) == b

    k, sx, sy, sz = CoefRepr(2), 1, 2, 3
    om, cm, b = SparOpReprMat(4, 5), SparCoefReprMat(5, 4), SparOpReprMat(4, 4)
    om.SetElem(0, 0, OpRepr(sx)); om.SetElem(0, 1, OpRepr(sy)); om.SetElem(0, 2, OpRepr(sz))
    om.SetElem(1, 3, OpRepr(sx)); om.SetElem(1, 4, OpRepr(sx)); om.SetElem(2, 4, OpRepr(sy))
    om.SetElem(3, 4, OpRepr(sz))
    cm.SetElem(0, 0, j); cm.SetElem(1, 1, j); cm.SetElem(2, 2, j + k); cm.SetElem(3, 3, k)
    cm.SetElem(4, 3, j)
    b.SetElem(0, 0, OpRepr(j, sx)); b.SetElem(0, 1, OpRepr(j, sy)); b.SetElem(0, 2, OpRepr(j + k, sz))
    b.SetElem(1, 3, OpRepr(k + j, sx)); b.SetElem(2, 3, OpRepr(j, sy)); b.SetElem(3, 3, OpRepr(j, sz))
    assert SparOpReprMatSparCoefReprMatIncompleteMulti(om, cm) == b


# --- compressers (:1071-1574) ---------------------------------------------------
def _mats(spec):
    """spec: (rows, cols, {(x, y): elem})."""
    r, c, elems = spec
    m = SparOpReprMat(r, c)
    for (x, y), e in elems.items():
        m.SetElem(x, y, e)
    return m


A, B, C, D, E = (OpRepr(i) for i in range(1, 6))
I = kIdOpRepr

ROW_CASES = [
    # (m1, m2) -> (bchmk_m1, bchmk_m2); row compresser on m1, follower m2
    ((1, 1, {}), (1, 1, {}), (1, 1, {}), (1, 1, {})),
    ((1, 1, {(0, 0): A}), (1, 1, {(0, 0): B}), (1, 1, {(0, 0): A}), (1, 1, {(0, 0): B})),
    ((2, 1, {(0, 0): C, (1, 0): D}), (1, 2, {(0, 0): A, (0, 1): B}),
     (2, 1, {(0, 0): C, (1, 0): D}), (1, 2, {(0, 0): A, (0, 1): B})),
    ((2, 1, {(0, 0): I, (1, 0): I}), (1, 2, {(0, 0): A, (0, 1): B}),
     (1, 1, {(0, 0): I}), (1, 1, {(0, 0): A + B})),
    ((2, 1, {(0, 0): C, (1, 0): C}), (1, 2, {(0, 0): A, (0, 1): B}),
     (1, 1, {(0, 0): C}), (1, 1, {(0, 0): A + B})),
    ((3, 1, {(0, 0): D, (1, 0): D, (2, 0): E}), (1, 3, {(0, 0): A, (0, 1): B, (0, 2): C}),
     (2, 1, {(0, 0): D, (1, 0): E}), (1, 2, {(0, 0): A + B, (0, 1): C})),
    ((3, 1, {(0, 0): D, (1, 0): E, (2, 0): E}), (1, 3, {(0, 0): A, (0, 1): B, (0, 2): C}),
     (2, 1, {(0, 0): D, (1, 0): E}), (1, 2, {(0, 0): A, (0, 1): B + C})),
    ((3, 1, {(0, 0): D, (1, 0): E, (2, 0): D}), (1, 3, {(0, 0): A, (0, 1): B, (0, 2): C}),
     (2, 1, {(0, 0): D, (1, 0): E}), (1, 2, {(0, 0): A + C, (0, 1): B})),
    ((3, 2, {(0, 0): D, (1, 1): E, (2, 0): D, (2, 1): E}),
     (1, 3, {(0, 0): A, (0, 1): B, (0, 2): C}),
     (2, 2, {(0, 0): D, (1, 1): E}), (1, 2, {(0, 0): A + C, (0, 1): B + C})),
    ((3, 2, {(0, 0): D, (0, 1): E, (1, 0): D, (2, 1): E}),
     (1, 3, {(0, 0): A, (0, 1): B, (0, 2): C}),
     (2, 2, {(0, 0): D, (1, 1): E}), (1, 2, {(0, 0): A + B, (0, 1): A + C})),
    ((3, 2, {(0, 0): OpRepr(1, 4), (0, 1): OpRepr(2, 5), (1, 0): D, (2, 1): E}),
     (1, 3, {(0, 0): A, (0, 1): B, (0, 2): C}),
     (2, 2, {(0, 0): D, (1, 1): E}),
     (1, 2, {(0, 0): OpRepr(1, 1) + B, (0, 1): OpRepr(2, 1) + C})),
]


def _row_case_11():
    j, k, sx, sy, sz = CoefRepr(1), CoefRepr(2), 1, 2, 3
    m1 = (5, 1, {(0, 0): OpRepr(j, sx), (1, 0): OpRepr(j, sy), (2, 0): OpRepr(j + k, sz),
                 (3, 0): OpRepr(k, kIdOpLabel), (4, 0): OpRepr(j, kIdOpLabel)})
    m2 = (4, 5, {(0, 0): OpRepr(sx), (0, 1): OpRepr(sy), (0, 2): OpRepr(sz), (1, 3): OpRepr(sx),
                 (1, 4): OpRepr(sx), (2, 4): OpRepr(sy), (3, 4): OpRepr(sz)})
    b1 = (4, 1, {(0, 0): OpRepr(sx), (1, 0): OpRepr(sy), (2, 0): OpRepr(sz), (3, 0): I})
    b2 = (4, 4, {(0, 0): OpRepr(j, sx), (0, 1): OpRepr(j, sy), (0, 2): OpRepr(j + k, sz),
                 (1, 3): OpRepr(j + k, sx), (2, 3): OpRepr(j, sy), (3, 3): OpRepr(j, sz)})
    return m1, m2, b1, b2


def _row_case_12():
    s = OpRepr(1)
    m1 = (2, 2, {(0, 1): I, (1, 0): s, (1, 1): I})
    m2 = (2, 2, {(0, 0): I, (1, 1): s})
    return m1, m2, m1, m2


@pytest.mark.parametrize("case", ROW_CASES + [_row_case_11(), _row_case_12()])
def test_row_compresser(case):
    m1, m2, b1, b2 = (_mats(c) for c in case)
    SparOpReprMatRowCompresser(m1, m2)
    assert m1 == b1
    assert m2 == b2


def _col_cases():
    cases = [
        ((1, 1, {}), (1, 1, {}), (1, 1, {}), (1, 1, {})),
        ((1, 1, {(0, 0): A}), (1, 1, {(0, 0): I}), (1, 1, {(0, 0): A}), (1, 1, {(0, 0): I})),
        ((1, 2, {(0, 0): A, (0, 1): B}), (2, 1, {(0, 0): C, (1, 0): D}),
         (1, 2, {(0, 0): A, (0, 1): B}), (2, 1, {(0, 0): C, (1, 0): D})),
        ((1, 2, {(0, 0): I, (0, 1): I}), (2, 1, {(0, 0): A, (1, 0): B}),
         (1, 1, {(0, 0): I}), (1, 1, {(0, 0): A + B})),
        ((1, 2, {(0, 0): A, (0, 1): A}), (2, 1, {(0, 0): B, (1, 0): C}),
         (1, 1, {(0, 0): A}), (1, 1, {(0, 0): B + C})),
        ((1, 3, {(0, 0): A, (0, 1): A, (0, 2): B}), (3, 1, {(0, 0): C, (1, 0): D, (2, 0): E}),
         (1, 2, {(0, 0): A, (0, 1): B}), (2, 1, {(0, 0): C + D, (1, 0): E})),
        ((1, 3, {(0, 0): A, (0, 1): B, (0, 2): A}), (3, 1, {(0, 0): C, (1, 0): D, (2, 0): E}),
         (1, 2, {(0, 0): A, (0, 1): B}), (2, 1, {(0, 0): C + E, (1, 0): D})),
    ]
    alp, bet, a, b, c, d, e = 1, 2, 1, 2, 3, 4, 5
    cases.append((
        (2, 3, {(0, 0): OpRepr(alp, a), (0, 1): OpRepr(a), (1, 0): OpRepr(bet, b),
                (1, 2): OpRepr(b)}),
        (3, 1, {(0, 0): OpRepr(c), (1, 0): OpRepr(d), (2, 0): OpRepr(e)}),
        (2, 2, {(0, 0): OpRepr(a), (1, 1): OpRepr(b)}),
        (2, 1, {(0, 0): OpRepr(d) + OpRepr(alp, c), (1, 0): OpRepr(e) + OpRepr(bet, c)})))
    s = OpRepr(1)
    cases.append((
        (2, 6, {(0, 0): I, (1, 1): I, (0, 2): s, (1, 3): I, (0, 4): s, (1, 5): s}),
        (6, 4, {(0, 2): s, (1, 0): s, (2, 1): I, (3, 3): I, (4, 0): s, (5, 0): I}),
        (2, 4, {(0, 0): I, (0, 2): s, (1, 1): I, (1, 3): s}),
        (4, 4, {(0, 2): s, (1, 0): s, (1, 3): I, (2, 0): s, (2, 1): I, (3, 0): I})))
    j1, j2, sl = 1, 2, 1
    cases.append((
        (1, 3, {(0, 0): I, (0, 1): OpRepr(j1, sl), (0, 2): OpRepr(j2, sl)}),
        (3, 6, {(0, 0): I, (0, 2): OpRepr(j1, sl), (0, 4): OpRepr(j2, sl), (1, 1): I,
                (1, 5): OpRepr(sl), (2, 3): I}),
        (1, 2, {(0, 0): I, (0, 1): OpRepr(sl)}),
        (2, 6, {(0, 0): I, (0, 2): OpRepr(j1, sl), (0, 4): OpRepr(j2, sl),
                (1, 1): OpRepr(j1, kIdOpLabel), (1, 3): OpRepr(j2, kIdOpLabel),
                (1, 5): OpRepr(j1, sl)})))
    j, k, sx, sy, sz = 1, 2, 1, 2, 3
    cases.append((
        (1, 5, {(0, 0): I, (0, 1): OpRepr(j, sx), (0, 2): OpRepr(j, sy), (0, 3): OpRepr(j, sz),
                (0, 4): OpRepr(k, sx)}),
        (5, 6, {(0, 0): OpRepr(j, sx), (0, 1): OpRepr(j, sy), (0, 2): OpRepr(j, sz),
                (0, 4): OpRepr(k, sz), (1, 5): OpRepr(sx), (2, 5): OpRepr(sy),
                (3, 5): OpRepr(sz), (4, 3): OpRepr(sx)}),
        (1, 4, {(0, 0): I, (0, 1): OpRepr(sx), (0, 2): OpRepr(sy), (0, 3): OpRepr(sz)}),
        (4, 6, {(0, 0): OpRepr(j, sx), (0, 1): OpRepr(j, sy), (0, 2): OpRepr(j, sz),
                (0, 4): OpRepr(k, sz), (1, 3): OpRepr(k, sx), (1, 5): OpRepr(j, sx),
                (2, 5): OpRepr(j, sy), (3, 5): OpRepr(j, sz)})))
    cases.append((
        (2, 2, {(0, 1): s, (1, 0): I, (1, 1): I}), (2, 2, {(0, 0): I, (1, 1): s}),
        (2, 2, {(0, 1): s, (1, 0): I, (1, 1): I}), (2, 2, {(0, 0): I, (1, 1): s})))
    return cases


@pytest.mark.parametrize("case", _col_cases())
def test_col_compresser(case):
    m1, m2, b1, b2 = (_mats(c) for c in case)
    SparOpReprMatColCompresser(m1, m2)
    assert m1 == b1
    assert m2 == b2
