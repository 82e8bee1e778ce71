"""The MPO generator: the MPO it produces, contracted to a dense operator,
equals the Hamiltonian summed term by term (Heisenberg chain, a J1-J2
cylinder with longer-range terms, a Hubbard chain with Jordan-Wigner
strings), and the bond dimensions of the reference's models are the
counts of ``fsm.h:167-176`` in the bulk (Heisenberg 5, Hubbard 6; the
bonds next to the chain ends carry fewer automaton states)."""
import numpy as np

from mps2_gb300 import hamiltonians as H
from _convert import to_oracle


def _dense_mpo(mpo):
    """Contract head (p_in, r, p_out), bulk (l, p_in, p_out, r) and tail
    (p_in, l, p_out) into the operator matrix over all sites."""
    ws = [to_oracle(w).to_dense() for w in mpo]
    n = len(ws)
    # acc[a, b, r]: a = combined p_in, b = combined p_out
    acc = np.transpose(ws[0], (0, 2, 1))          # (p_in, p_out, r)
    for i in range(1, n - 1):
        w = ws[i]                                  # (l, p_in, p_out, r)
        acc = np.einsum("abl,lcdr->acbdr", acc, w)
        s = acc.shape
        acc = acc.reshape(s[0] * s[1], s[2] * s[3], s[4])
    w = ws[-1]                                     # (p_in, l, p_out)
    acc = np.einsum("abl,cld->acbd", acc, w)
    s = acc.shape
    return acc.reshape(s[0] * s[1], s[2] * s[3])


def _site_op(o, i, n):
    m = np.array([[1.0]])
    for k in range(n):
        m = np.kron(m, o if k == i else np.eye(o.shape[0]))
    return m


def _heisenberg_dense(n, pairs):
    _, ops = H.spin_half_ops()
    sz = to_oracle(ops["sz"]).to_dense()
    sp = to_oracle(ops["sp"]).to_dense()
    sm = to_oracle(ops["sm"]).to_dense()
    h = np.zeros((2 ** n, 2 ** n))
    for i, j, J in pairs:
        h += J * _site_op(sz, i, n) @ _site_op(sz, j, n)
        h += 0.5 * J * (_site_op(sp, i, n) @ _site_op(sm, j, n) +
                        _site_op(sm, i, n) @ _site_op(sp, j, n))
    return h


def test_heisenberg_chain_mpo_is_the_hamiltonian():
    n = 6
    sv, mpo, qn0, gen = H.heisenberg_chain(n)
    h = _heisenberg_dense(n, [(i, i + 1, 1.0) for i in range(n - 1)])
    np.testing.assert_allclose(_dense_mpo(mpo), h, atol=1e-13)
    assert max(w.indices[-1].dim for w in mpo[1:-1]) == 5   # bulk bonds; the ends need fewer


def test_j1j2_cylinder_mpo_is_the_hamiltonian():
    pairs = H.j1j2_cylinder_pairs(3, 2, 1.0, 0.5)
    n = 6
    sv, mpo, qn0, gen = H.heisenberg_pairs(n, pairs)
    np.testing.assert_allclose(_dense_mpo(mpo), _heisenberg_dense(n, pairs), atol=1e-13)


def test_hubbard_chain_mpo_is_the_hamiltonian():
    """4 sites, t=1, U=8: the MPO against the same operator sum built from
    the site operators with the Jordan-Wigner string in between."""
    n = 4
    sv, mpo, qn0, gen = H.hubbard_chain(n, 1.0, 8.0)
    _, o = H.hubbard_ops()
    d = {k: to_oracle(v).to_dense() for k, v in o.items()}
    dim = 4 ** n

    def chain(ops_at):
        m = np.array([[1.0]])
        for k in range(n):
            m = np.kron(m, ops_at.get(k, np.eye(4)))
        return m
    h = np.zeros((dim, dim))
    for s in range(n):
        h += 8.0 * chain({s: d["nupdn"]})
    for a in range(n - 1):
        b = a + 1
        h += chain({a: -1.0 * d["adagupf"], b: d["aup"]})
        h += chain({a: -1.0 * d["adagdn"], b: d["fadn"]})
        h += chain({a: d["naupf"], b: -1.0 * d["adagup"]})
        h += chain({a: d["nadn"], b: -1.0 * d["fadagdn"]})
    np.testing.assert_allclose(_dense_mpo(mpo), h, atol=1e-12)
    assert max(w.indices[-1].dim for w in mpo[1:-1]) == 6


def test_random_terms_mpo_is_the_sum_of_terms():
    """Seeded random Hamiltonians on 5 sites: one- to three-site operator
    strings (S^z, S^+, S^-, identity inside), coefficients drawn from a small
    set so that coefficient labels repeat and the compression moves shared
    coefficients between matrices.  Only charge-conserving strings are kept.
    The generated MPO, contracted, equals the sum of the terms."""
    from mps2_gb300.mpogen import MPOGenerator
    from mps2_gb300.site_vec import SiteVec
    pb, ops = H.spin_half_ops()
    d = {k: to_oracle(v).to_dense() for k, v in ops.items()}
    charge = {"sz": 0, "sp": 1, "sm": -1, "id": 0}
    rng = np.random.default_rng(20240)
    n = 5
    for trial in range(12):
        gen = MPOGenerator(SiteVec(n, pb), (0,))
        h = np.zeros((2 ** n, 2 ** n))
        coefs = [0.5, -1.25, 2.0, 0.5, 1.0]
        seen_one_site = set()
        for _ in range(rng.integers(4, 12)):
            k = int(rng.integers(1, 4))
            sites = sorted(rng.choice(n, size=k, replace=False).tolist())
            names = [str(rng.choice(["sz", "sp", "sm"])) for _ in sites]
            if sum(charge[x] for x in names) != 0:
                continue
            c = float(rng.choice(coefs))
            gen.AddTerm(c, [ops[x] for x in names], sites)
            if k == 1:  # the reference keeps one copy of an identical one-site term
                if (names[0], sites[0], c) in seen_one_site:
                    continue
                seen_one_site.add((names[0], sites[0], c))
            m = np.array([[1.0]])
            for s in range(n):
                m = np.kron(m, d[names[sites.index(s)]] if s in sites else np.eye(2))
            h += c * m
        if not np.any(h):
            continue
        mpo = gen.Gen()
        np.testing.assert_allclose(_dense_mpo(mpo), h, atol=1e-13, err_msg=f"trial {trial}")


def test_identical_one_site_term_counts_once():
    """The reference's FSM keeps an existing element when the added one is
    equal to it (``fsm.h:230-239``), so the same one-site term added twice
    is counted once, while two equal two-site terms add up (their paths
    run through different middle states)."""
    from mps2_gb300.mpogen import MPOGenerator
    from mps2_gb300.site_vec import SiteVec
    pb, ops = H.spin_half_ops()
    sz = to_oracle(ops["sz"]).to_dense()
    gen = MPOGenerator(SiteVec(3, pb), (0,))
    gen.AddTerm(0.5, [ops["sz"]], [1])
    gen.AddTerm(0.5, [ops["sz"]], [1])
    gen.AddTerm(1.0, [ops["sz"], ops["sz"]], [0, 2])
    gen.AddTerm(1.0, [ops["sz"], ops["sz"]], [0, 2])
    want = 0.5 * _site_op(sz, 1, 3) + 2.0 * _site_op(sz, 0, 3) @ _site_op(sz, 2, 3)
    np.testing.assert_allclose(_dense_mpo(gen.Gen()), want, atol=1e-14)
