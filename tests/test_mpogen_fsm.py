"""The MPO generator's finite-state machine and its compressed matrices
against the reference's benchmark matrices
(``tests/test_one_dim_tn/test_mpogen/test_mpogen_fsm.cc`` and
``test_mpogen.cc``: the same cases, the same expected matrices)."""
import numpy as np
import pytest

from mps2_gb300.fsm import FSM, FSMNode, LabelConvertor, kFSMFinalStatIdx, kFSMReadyStatIdx
from mps2_gb300.mpogen import MPOGenerator
from mps2_gb300.site_vec import SiteVec
from mps2_gb300.symb_alg import CoefRepr, OpRepr, SparOpReprMat, kIdOpLabel, kIdOpRepr
from mps2_gb300.tensor import GQTensor, Index, IN, OUT

S = OpRepr(1)
I = kIdOpRepr


def mat(r, c, elems):
    m = SparOpReprMat(r, c)
    for (x, y), e in elems.items():
        m.SetElem(x, y, e)
    return m


def nodes(*pairs):
    return [FSMNode(a, b) for a, b in pairs]


# --- FSM construction and paths (fsm.cc:13-206) -------------------------------
@pytest.mark.parametrize("n", [0, 1, 5, 20])
def test_fsm_initialization(n):
    f = FSM(n)
    assert f.phys_size() == n and f.fsm_size() == n + 1
    assert FSM().phys_size() == 0 and FSM().fsm_size() == 1


def test_add_path():
    assert FSM(1).GetFSMPaths() == []
    f = FSM(1)
    f.AddPath(0, 0, [I])
    p = f.GetFSMPaths()
    assert len(p) == 1 and p[0].fsm_nodes == nodes((0, 0), (1, -1)) and p[0].op_reprs == [I]

    f = FSM(2)
    f.AddPath(0, 0, [S])
    f.AddPath(1, 1, [S])
    p = f.GetFSMPaths()
    assert p[0].fsm_nodes == nodes((0, 0), (1, -1), (2, -1)) and p[0].op_reprs == [S, I]
    assert p[1].fsm_nodes == nodes((0, 0), (1, 0), (2, -1)) and p[1].op_reprs == [I, S]

    f = FSM(2)
    f.AddPath(0, 1, [S, S])
    f.AddPath(0, 1, [S, S])
    p = f.GetFSMPaths()
    assert p[0].fsm_nodes == nodes((0, 0), (1, 1), (2, -1))
    assert p[1].fsm_nodes == nodes((0, 0), (1, 2), (2, -1))

    f = FSM(4)
    f.AddPath(0, 1, [S, S])
    f.AddPath(1, 2, [S, S])
    f.AddPath(2, 3, [S, S])
    p = f.GetFSMPaths()
    assert p[0].op_reprs == [S, S, I, I]
    assert p[0].fsm_nodes == nodes((0, 0), (1, 1), (2, -1), (3, -1), (4, -1))
    assert p[1].op_reprs == [I, S, S, I]
    assert p[1].fsm_nodes == nodes((0, 0), (1, 0), (2, 1), (3, -1), (4, -1))
    assert p[2].op_reprs == [I, I, S, S]
    assert p[2].fsm_nodes == nodes((0, 0), (1, 0), (2, 0), (3, 1), (4, -1))

    f = FSM(5)
    f.AddPath(0, 4, [S, I, I, I, S])
    f.AddPath(1, 4, [S, S, I, S])
    f.AddPath(1, 3, [S, S, S])
    p = f.GetFSMPaths()
    assert p[0].fsm_nodes == nodes((0, 0), (1, 1), (2, 1), (3, 1), (4, 1), (5, -1))
    assert p[1].op_reprs == [I, S, S, I, S]
    assert p[1].fsm_nodes == nodes((0, 0), (1, 0), (2, 2), (3, 2), (4, 2), (5, -1))
    assert p[2].op_reprs == [I, S, S, S, I]
    assert p[2].fsm_nodes == nodes((0, 0), (1, 0), (2, 3), (3, 3), (4, -1), (5, -1))
    assert kFSMReadyStatIdx == 0 and kFSMFinalStatIdx == -1


# --- GenMatRepr (fsm.cc:208-336) ----------------------------------------------
def _fsm(n, paths):
    f = FSM(n)
    for h, t, ops in paths:
        f.AddPath(h, t, ops)
    return f


GEN_MAT_CASES = [
    (1, [(0, 0, [I])], [mat(1, 1, {(0, 0): I})]),
    (1, [(0, 0, [S])], [mat(1, 1, {(0, 0): S})]),
    (1, [(0, 0, [S]), (0, 0, [OpRepr(2)])], [mat(1, 1, {(0, 0): S + OpRepr(2)})]),
    (2, [(0, 0, [S]), (1, 1, [S])],
     [mat(1, 2, {(0, 0): I, (0, 1): S}), mat(2, 1, {(0, 0): S, (1, 0): I})]),
    (2, [(0, 1, [S, S]), (0, 1, [S, S])],
     [mat(1, 2, {(0, 0): S, (0, 1): S}), mat(2, 1, {(0, 0): S, (1, 0): S})]),
    (4, [(0, 1, [S, S]), (1, 2, [S, S]), (2, 3, [S, S])],
     [mat(1, 2, {(0, 0): I, (0, 1): S}), mat(2, 3, {(0, 0): I, (0, 1): S, (1, 2): S}),
      mat(3, 2, {(0, 1): S, (1, 0): S, (2, 0): I}), mat(2, 1, {(0, 0): I, (1, 0): S})]),
    (5, [(0, 4, [S, I, I, I, S]), (1, 4, [S, S, I, S]), (1, 3, [S, S, S])],
     [mat(1, 2, {(0, 0): I, (0, 1): S}), mat(2, 3, {(0, 1): S, (0, 2): S, (1, 0): I}),
      mat(3, 3, {(0, 0): I, (1, 1): S, (2, 2): S}),
      mat(3, 3, {(0, 1): I, (1, 2): I, (2, 0): S}),
      mat(3, 1, {(0, 0): I, (1, 0): S, (2, 0): S})]),
]


@pytest.mark.parametrize("n,paths,bchmk", GEN_MAT_CASES)
def test_gen_mat_repr(n, paths, bchmk):
    assert _fsm(n, paths).GenMatRepr() == bchmk


# --- GenCompressedMatRepr (fsm.cc:339-527) -----------------------------------
def _compressed_cases():
    j1, j2 = 1, 2
    s = 1
    cases = [
        (1, [(0, 0, [I])], [mat(1, 1, {(0, 0): I})]),
        (1, [(0, 0, [S])], [mat(1, 1, {(0, 0): S})]),
        (2, [(0, 0, [S]), (1, 1, [S])],
         [mat(1, 2, {(0, 0): I, (0, 1): S}), mat(2, 1, {(0, 0): S, (1, 0): I})]),
        (2, [(0, 1, [S, S]), (0, 1, [S, S])],
         [mat(1, 1, {(0, 0): S}), mat(1, 1, {(0, 0): S + S})]),
        (4, [(0, 1, [S, S]), (1, 2, [S, S]), (2, 3, [S, S])],
         [mat(1, 2, {(0, 0): S, (0, 1): I}), mat(2, 3, {(0, 2): S, (1, 0): I, (1, 1): S}),
          mat(3, 2, {(0, 0): S, (1, 1): S, (2, 1): I}), mat(2, 1, {(0, 0): S, (1, 0): I})]),
        (5, [(0, 4, [S, I, I, I, S]), (1, 4, [S, S, I, S]), (1, 3, [S, S, S])],
         [mat(1, 2, {(0, 0): I, (0, 1): S}), mat(2, 2, {(0, 1): S, (1, 0): I}),
          mat(2, 2, {(0, 0): I, (1, 1): S}), mat(2, 2, {(0, 1): I, (1, 0): S, (1, 1): I}),
          mat(2, 1, {(0, 0): I, (1, 0): S})]),
        (4, [(0, 1, [OpRepr(j1, s), S]), (0, 2, [OpRepr(j1, s), I, S]),
             (1, 3, [OpRepr(j1, s), I, S]), (2, 3, [OpRepr(j1, s), S]),
             (0, 3, [OpRepr(j2, s), I, I, S]), (1, 2, [OpRepr(j2, s), S])],
         [mat(1, 2, {(0, 0): I, (0, 1): S}),
          mat(2, 4, {(0, 0): OpRepr(j1, kIdOpLabel), (0, 3): S, (1, 1): OpRepr(j1, s),
                     (1, 2): I}),
          mat(4, 2, {(0, 0): S, (1, 1): I, (2, 0): OpRepr(j2, kIdOpLabel),
                     (2, 1): OpRepr(j1, s), (3, 0): OpRepr(j1, kIdOpLabel),
                     (3, 1): OpRepr(j2, s)}),
          mat(2, 1, {(0, 0): S, (1, 0): I})]),
    ]
    j, k, sx, sy, sz = 1, 2, 1, 2, 3
    cases.append((
        3, [(0, 1, [OpRepr(j, sx), OpRepr(sx)]), (0, 1, [OpRepr(j, sy), OpRepr(sy)]),
            (0, 1, [OpRepr(j, sz), OpRepr(sz)]), (1, 2, [OpRepr(j, sx), OpRepr(sx)]),
            (1, 2, [OpRepr(j, sy), OpRepr(sy)]), (1, 2, [OpRepr(j, sz), OpRepr(sz)]),
            (0, 1, [OpRepr(k, sx), OpRepr(sx)]), (1, 2, [OpRepr(k, sz), OpRepr(sz)])],
        _case7_bchmk(j, k, sx, sy, sz)))
    return cases


def _case7_bchmk(j, k, sx, sy, sz):
    return [mat(1, 4, {(0, 0): OpRepr([k, j], [sx, sx]), (0, 1): OpRepr(j, sy),
                       (0, 2): OpRepr(j, sz), (0, 3): I}),
            mat(4, 4, {(0, 3): OpRepr(sx), (1, 3): OpRepr(sy), (2, 3): OpRepr(sz),
                       (3, 0): OpRepr(j, sx), (3, 1): OpRepr(j, sy),
                       (3, 2): OpRepr([j, k], [sz, sz])}),
            mat(4, 1, {(0, 0): OpRepr(sx), (1, 0): OpRepr(sy), (2, 0): OpRepr(sz), (3, 0): I})]


@pytest.mark.parametrize("n,paths,bchmk", _compressed_cases())
def test_gen_compressed_mat_repr(n, paths, bchmk):
    assert _fsm(n, paths).GenCompressedMatRepr() == bchmk


def test_label_convertor():
    c = LabelConvertor(1.0, key=float)
    assert [c.Convert(v) for v in (1, 1.0, 1., 1.000)] == [0, 0, 0, 0]
    assert c.Convert(2.0) == 1 and c.Convert(2.0) == 1 and c.Convert(1.) == 0


# --- MPOGenerator.AddTerm -> compressed matrices (test_mpogen.cc:69-246) -----
def _spin_half():
    out = Index([((-1,), 1), ((1,), 1)], OUT)
    pin = out.inverse()

    def op(entries):
        t = GQTensor([pin, out], (0,))
        for (a, b), v in entries.items():
            t[a, b] = v
        return t
    sz = op({(0, 0): -0.5, (1, 1): 0.5})
    return out, sz


def _gen(n):
    out, sz = _spin_half()
    return MPOGenerator(SiteVec(n, out), (0,)), sz


def _comp(gen):
    return gen.GetFSM().GenCompressedMatRepr()


def test_add_term_case1():
    g, sz = _gen(2)
    g.AddTerm(1.0, [sz], [0])
    assert _comp(g) == [mat(1, 1, {(0, 0): OpRepr(1)}), mat(1, 1, {(0, 0): I})]
    g, sz = _gen(2)
    g.AddTerm(1.0, [sz], [0])
    g.AddTerm(0.0, [sz], [0])
    assert _comp(g) == [mat(1, 1, {(0, 0): OpRepr(1)}), mat(1, 1, {(0, 0): I})]


def test_add_term_case2():
    g, sz = _gen(2)
    g.AddTerm(1.0, [sz, sz], [0, 1])
    g.AddTerm(1.0, [sz, sz], [0, 1])
    assert _comp(g) == [mat(1, 1, {(0, 0): S}), mat(1, 1, {(0, 0): S + S})]


def test_add_term_case3():
    g, sz = _gen(4)
    for i in range(3):
        g.AddTerm(1.0, [sz, sz], [i, i + 1])
    assert _comp(g) == [mat(1, 2, {(0, 0): S, (0, 1): I}),
                        mat(2, 3, {(0, 2): S, (1, 0): I, (1, 1): S}),
                        mat(3, 2, {(0, 0): S, (1, 1): S, (2, 1): I}),
                        mat(2, 1, {(0, 0): S, (1, 0): I})]


def test_add_term_case4():
    g, sz = _gen(5)
    g.AddTerm(1.0, [sz, sz], [0, 4])
    g.AddTerm(1.0, [sz, sz, sz], [1, 2, 4])
    g.AddTerm(1.0, [sz, sz, sz], [1, 2, 3])
    assert _comp(g) == [mat(1, 2, {(0, 0): I, (0, 1): S}),
                        mat(2, 2, {(0, 1): S, (1, 0): I}),
                        mat(2, 2, {(0, 0): I, (1, 1): S}),
                        mat(2, 2, {(0, 1): I, (1, 0): S, (1, 1): I}),
                        mat(2, 1, {(0, 0): I, (1, 0): S})]


def test_add_term_case5():
    j1, j2, s = 1, 2, 1
    g, sz = _gen(4)
    ja, jb = 0.5, 2.0
    for a, b in ((0, 1), (0, 2), (1, 3), (2, 3)):
        g.AddTerm(ja, [sz, sz], [a, b])
    for a, b in ((0, 3), (1, 2)):
        g.AddTerm(jb, [sz, sz], [a, b])
    assert _comp(g) == [
        mat(1, 2, {(0, 0): I, (0, 1): S}),
        mat(2, 4, {(0, 0): OpRepr(j1, kIdOpLabel), (0, 3): S, (1, 1): OpRepr(j1, s), (1, 2): I}),
        mat(4, 2, {(0, 0): S, (1, 1): I, (2, 0): OpRepr(j2, kIdOpLabel), (2, 1): OpRepr(j1, s),
                   (3, 0): OpRepr(j1, kIdOpLabel), (3, 1): OpRepr(j2, s)}),
        mat(2, 1, {(0, 0): S, (1, 0): I})]


def test_add_term_case6():
    """The reference's case uses complex S^x, S^y, S^z; the compressed
    matrices depend only on which operators are distinct, so three distinct
    real operators stand in for them (i S^y is real), on a local space with
    a single quantum-number sector so that S^x and S^y are allowed."""
    out = Index([((0,), 2)], OUT)
    pin = out.inverse()

    def op(entries):
        t = GQTensor([pin, out], (0,))
        for (a, b), v in entries.items():
            t[a, b] = v
        return t
    g = MPOGenerator(SiteVec(3, out), (0,))
    sx = op({(0, 1): 1.0, (1, 0): 1.0})
    isy = op({(0, 1): 1.0, (1, 0): -1.0})
    sz = op({(0, 0): -0.5, (1, 1): 0.5})
    J, K = 0.5, 2.0
    for o in (sx, isy, sz):
        g.AddTerm(J, [o, o], [0, 1])
    for o in (sx, isy, sz):
        g.AddTerm(J, [o, o], [1, 2])
    g.AddTerm(K, [sx, sx], [0, 1])
    g.AddTerm(K, [sz, sz], [1, 2])
    assert _comp(g) == _case7_bchmk(1, 2, 1, 2, 3)


def test_gen_realises_coefficients_on_the_matrices():
    """Gen on case 5: the MPO contracts to the operator sum, and its bulk bond
    dimension is the compressed one (4)."""
    g, sz = _gen(4)
    ja, jb = 0.5, 2.0
    pairs = [(0, 1, ja), (0, 2, ja), (1, 3, ja), (2, 3, ja), (0, 3, jb), (1, 2, jb)]
    for a, b, J in pairs:
        g.AddTerm(J, [sz, sz], [a, b])
    mpo = g.Gen()
    assert g.bond_dims == [2, 4, 2]
    from test_mpogen import _dense_mpo, _site_op
    d = sz.to_dense()
    h = sum(J * _site_op(d, a, 4) @ _site_op(d, b, 4) for a, b, J in pairs)
    np.testing.assert_allclose(_dense_mpo(mpo), h, atol=1e-14)
