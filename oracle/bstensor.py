"""FP64 CPU oracle: block-sparse, quantum-number-labelled tensors.

TEST INFRASTRUCTURE ONLY.  This package is the correctness checker for the
GPU library in ``mps2_gb300``.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it; the product never
does.

The reference (gqmps2) does all of its tensor arithmetic inside the external
GraceQ/tensor library ("gqten"), which is not vendored and whose version is
unpinned (``external/CMakeLists.txt:10``, ``doc/index.md:35``).  What follows
is a restatement of the behaviour visible at gqmps2's call sites:

* ``Contract(a, b, {axes_a, axes_b}, &c)`` -- tensordot over matching
  quantum-number sectors; output legs are a's free legs (in order) followed
  by b's free legs (call sites ``two_site_update_finite_vmps_impl.h:118-129,
  243, 272, 276, 290-317``; ``lanczos_solver_impl.h:231-254``).
* ``Dag`` -- flip every leg direction, negate the divergence (real numbers:
  no conjugation needed).
* ``Normalize`` / ``LinearCombine`` / full contraction with ``Dag`` as the
  inner product (``lanczos_solver_impl.h:120, 135-141, 151-160, 215``).
* ``SVD(t, ldims, ldiv, trunc_err, Dmin, Dmax, ...)`` with global truncation
  (``two_site_update_finite_vmps_impl.h:258-263``); the truncation rule is
  spelled out in :func:`svd`.

Parity is pinned by the golden ground-state energies of the reference's own
end-to-end tests (``tests/test_algorithm/test_two_site_update_finite_vmps.cc``)
and by the Lanczos-vs-dense-diagonalisation check of
``tests/test_algorithm/test_lanczos_solver.cc:111``.

Conventions
-----------
* A quantum number (QN) is a tuple of ints (one entry per U(1) charge).
* Leg direction: ``OUT = +1``, ``IN = -1``.  A block with sector coordinates
  ``c`` is allowed when ``sum_i dir_i * qn_i(c_i) == div``.
* Blocks are dense row-major ``numpy.float64`` arrays keyed by the tuple of
  sector positions.
"""
from __future__ import annotations

import itertools
from typing import Dict, List, Sequence, Tuple

import numpy as np

OUT = 1
IN = -1

# Singular values at or below ZERO_SV_RTOL * (largest singular value) are
# treated as exact zeros by the truncating SVD.  They can still be kept (the
# reference keeps min(Dmax, #values)), but their singular vectors -- an
# arbitrary completion in LAPACK -- are replaced by a canonical one.
ZERO_SV_RTOL = 1e-13


def qn_add(a, b):
    return tuple(x + y for x, y in zip(a, b))


def qn_sub(a, b):
    return tuple(x - y for x, y in zip(a, b))


def qn_neg(a):
    return tuple(-x for x in a)


def qn_scale(s, a):
    return tuple(s * x for x in a)


class Index:
    """One tensor leg: a direction and an ordered list of (QN, dim) sectors."""

    __slots__ = ("dir", "qns", "dims")

    def __init__(self, sectors: Sequence[Tuple[tuple, int]], dir: int):
        self.dir = int(dir)
        self.qns = [tuple(int(v) for v in q) for q, _ in sectors]
        self.dims = [int(d) for _, d in sectors]

    @property
    def dim(self) -> int:
        return sum(self.dims)

    @property
    def nsec(self) -> int:
        return len(self.dims)

    def inverse(self) -> "Index":
        return Index(list(zip(self.qns, self.dims)), -self.dir)

    def sectors(self):
        return list(zip(self.qns, self.dims))

    def sector_offsets(self):
        return np.concatenate([[0], np.cumsum(self.dims)]).astype(int)

    def coor_to_sector(self, coor: int) -> Tuple[int, int]:
        """Actual (dense) coordinate -> (sector position, offset inside)."""
        for s, d in enumerate(self.dims):
            if coor < d:
                return s, coor
            coor -= d
        raise IndexError("coordinate out of range")

    def __eq__(self, other):
        return (isinstance(other, Index) and self.dir == other.dir
                and self.qns == other.qns and self.dims == other.dims)

    def __repr__(self):
        return f"Index(dir={self.dir}, {self.sectors()})"


class BSTensor:
    """Block-sparse tensor: legs, divergence and the present dense blocks."""

    def __init__(self, indices: Sequence[Index], div=None, blocks=None):
        self.indices: List[Index] = list(indices)
        self.blocks: Dict[tuple, np.ndarray] = dict(blocks or {})
        self.div = None if div is None else tuple(div)
        if self.div is None and self.blocks:
            self.div = self.block_div(next(iter(self.blocks)))

    # ---- structure -------------------------------------------------------
    @property
    def rank(self) -> int:
        return len(self.indices)

    @property
    def shape(self):
        return tuple(ix.dim for ix in self.indices)

    def block_div(self, coords) -> tuple:
        nq = len(self.indices[0].qns[0])
        q = (0,) * nq
        for ix, c in zip(self.indices, coords):
            q = qn_add(q, qn_scale(ix.dir, ix.qns[c]))
        return q

    def block_shape(self, coords):
        return tuple(ix.dims[c] for ix, c in zip(self.indices, coords))

    def allowed_coords(self, div=None):
        div = self.div if div is None else tuple(div)
        out = []
        for coords in itertools.product(*[range(ix.nsec) for ix in self.indices]):
            if self.block_div(coords) == div:
                out.append(coords)
        return out

    def size(self) -> int:
        return sum(b.size for b in self.blocks.values())

    # ---- element access (dense coordinates) ------------------------------
    def __setitem__(self, coors, value):
        secs = [ix.coor_to_sector(c) for ix, c in zip(self.indices, coors)]
        bc = tuple(s for s, _ in secs)
        inner = tuple(o for _, o in secs)
        if bc not in self.blocks:
            d = self.block_div(bc)
            if self.div is None:
                self.div = d
            elif d != self.div:
                raise ValueError("element breaks the tensor's divergence")
            self.blocks[bc] = np.zeros(self.block_shape(bc))
        self.blocks[bc][inner] = value

    def __getitem__(self, coors):
        secs = [ix.coor_to_sector(c) for ix, c in zip(self.indices, coors)]
        bc = tuple(s for s, _ in secs)
        if bc not in self.blocks:
            return 0.0
        return float(self.blocks[bc][tuple(o for _, o in secs)])

    def to_dense(self) -> np.ndarray:
        out = np.zeros(self.shape)
        offs = [ix.sector_offsets() for ix in self.indices]
        for bc, b in self.blocks.items():
            sl = tuple(slice(o[c], o[c] + d) for o, c, d in zip(offs, bc, b.shape))
            out[sl] = b
        return out

    def copy(self) -> "BSTensor":
        return BSTensor(self.indices, self.div,
                        {k: v.copy() for k, v in self.blocks.items()})

    # ---- arithmetic ------------------------------------------------------
    def norm(self) -> float:
        return float(np.sqrt(sum(float(np.vdot(b, b)) for b in self.blocks.values())))

    def normalize(self) -> float:
        """gqten ``Normalize``: scale to unit 2-norm, return the old norm."""
        n = self.norm()
        if n != 0.0:
            for k in self.blocks:
                self.blocks[k] = self.blocks[k] / n
        return n

    def scale(self, s: float) -> "BSTensor":
        return BSTensor(self.indices, self.div,
                        {k: v * s for k, v in self.blocks.items()})

    def transpose(self, perm) -> "BSTensor":
        return BSTensor([self.indices[p] for p in perm], self.div,
                        {tuple(k[p] for p in perm): np.ascontiguousarray(v.transpose(perm))
                         for k, v in self.blocks.items()})


def dag(t: BSTensor) -> BSTensor:
    """gqten ``Dag`` for real tensors: invert every leg, negate the div."""
    return BSTensor([ix.inverse() for ix in t.indices],
                    None if t.div is None else qn_neg(t.div),
                    {k: v.copy() for k, v in t.blocks.items()})


def contract(a: BSTensor, b: BSTensor, axes_a: Sequence[int],
             axes_b: Sequence[int]) -> BSTensor:
    """gqten ``Contract``: sum over matching sectors of the contracted legs.

    Output legs are a's free legs (ascending) then b's free legs (ascending),
    as at ``lanczos_solver_impl.h:231-234`` where the leg positions of every
    intermediate follow from that rule.
    """
    axes_a = list(axes_a)
    axes_b = list(axes_b)
    for ia, ib in zip(axes_a, axes_b):
        if a.indices[ia].inverse() != b.indices[ib]:
            raise ValueError(f"legs {ia} and {ib} cannot be contracted")
    free_a = [i for i in range(a.rank) if i not in axes_a]
    free_b = [i for i in range(b.rank) if i not in axes_b]
    out_idx = [a.indices[i] for i in free_a] + [b.indices[i] for i in free_b]
    div = None
    if a.div is not None and b.div is not None:
        div = qn_add(a.div, b.div)
    # matricise: a -> (free, contracted), b -> (contracted, free)
    perm_a = free_a + axes_a
    perm_b = axes_b + free_b
    bgroups: Dict[tuple, list] = {}
    for cb, vb in b.blocks.items():
        key = tuple(cb[i] for i in axes_b)
        kdim = int(np.prod([vb.shape[i] for i in axes_b])) if axes_b else 1
        bm = np.ascontiguousarray(vb.transpose(perm_b)).reshape(kdim, -1)
        fshape = tuple(vb.shape[i] for i in free_b)
        bgroups.setdefault(key, []).append((tuple(cb[i] for i in free_b), bm, fshape))
    out: Dict[tuple, np.ndarray] = {}
    for ca, va in a.blocks.items():
        key = tuple(ca[i] for i in axes_a)
        grp = bgroups.get(key)
        if not grp:
            continue
        kdim = int(np.prod([va.shape[i] for i in axes_a])) if axes_a else 1
        am = np.ascontiguousarray(va.transpose(perm_a)).reshape(-1, kdim)
        afc = tuple(ca[i] for i in free_a)
        afs = tuple(va.shape[i] for i in free_a)
        for bfc, bm, bfs in grp:
            oc = afc + bfc
            r = (am @ bm).reshape(afs + bfs)
            if oc in out:
                out[oc] += r
            else:
                out[oc] = r
    if not out_idx:  # scalar result
        s = sum(float(v) for v in out.values())
        t = BSTensor([], div, {(): np.array(s)})
        return t
    return BSTensor(out_idx, div, out)


def inner(a: BSTensor, b: BSTensor) -> float:
    """<a|b> = full contraction of Dag(a) with b over all legs in order."""
    s = 0.0
    for k, v in a.blocks.items():
        w = b.blocks.get(k)
        if w is not None:
            s += float(np.vdot(v, w))
    return s


def linear_combine(coefs, tensors, beta: float = 0.0, out: BSTensor = None) -> BSTensor:
    """gqten ``LinearCombine``: out = beta*out + sum_i coefs[i]*tensors[i].

    Block sets are united; missing blocks count as zero.
    """
    ref = out if out is not None else tensors[0]
    res: Dict[tuple, np.ndarray] = {}
    if out is not None and beta != 0.0:
        for k, v in out.blocks.items():
            res[k] = beta * v
    for c, t in zip(coefs, tensors):
        for k, v in t.blocks.items():
            if k in res:
                res[k] = res[k] + c * v
            else:
                res[k] = c * v
    return BSTensor(ref.indices, ref.div if ref.div is not None else tensors[0].div, res)


# ---------------------------------------------------------------------------
# Truncating SVD
# ---------------------------------------------------------------------------
class SVDResult:
    def __init__(self, u, s, vt, trunc_err, D, svals):
        self.u = u
        self.s = s            # list of (sector position, kept values) in bond order
        self.vt = vt
        self.trunc_err = trunc_err
        self.D = D
        self.svals = svals    # all kept singular values, bond order


def _left_qn(t: BSTensor, coords, ldims):
    nq = len(t.indices[0].qns[0])
    q = (0,) * nq
    for ix, c in zip(t.indices[:ldims], coords[:ldims]):
        q = qn_add(q, qn_scale(ix.dir, ix.qns[c]))
    return q


def fix_sign(u: np.ndarray, vt: np.ndarray):
    """Gauge convention: the largest-|.| entry of each left singular vector
    (first one on ties) is made positive; the right vector follows."""
    if u.size == 0:
        return u, vt
    idx = np.argmax(np.abs(u), axis=0)
    sgn = np.sign(u[idx, np.arange(u.shape[1])])
    sgn[sgn == 0] = 1.0
    return u * sgn[None, :], vt * sgn[:, None]


def select_kept(all_s: np.ndarray, trunc_err: float, dmin: int, dmax: int):
    """Global truncation over every sector's singular values.

    Values at or below ``ZERO_SV_RTOL * s_max`` must already be exact zeros
    (see :func:`svd`).  Values are ranked largest first (ties: earlier
    sector, then earlier position).  With ``W = sum s^2``, the kept count D
    is the smallest number in ``[Dmin, Dmax]`` whose discarded weight
    ``sum_{i>=D} s_i^2 / W`` is at most ``trunc_err``, capped by Dmax and by
    the number of values (zeros included, as the reference keeps
    ``min(Dmax, #values)`` when ``Dmin == Dmax``).
    Returns (order, D, actual_trunc_err) where ``order`` ranks all values.
    """
    n = all_s.size
    order = np.argsort(-all_s, kind="stable")
    ranked = all_s[order]
    if n == 0 or ranked[0] <= 0.0:
        return order, min(n, max(1, min(dmin, dmax))), 0.0
    sq = ranked * ranked
    # tail[i] = sum_{j>=i} sq[j], accumulated from the smallest value up
    tail = np.zeros(n + 1)
    acc = 0.0
    for i in range(n - 1, -1, -1):
        acc += float(sq[i])
        tail[i] = acc
    total = float(tail[0])
    dcap = min(dmax, n)
    D = dcap
    lo = max(1, min(dmin, dcap))
    for d in range(lo, dcap + 1):
        if tail[d] / total <= trunc_err:
            D = d
            break
    err = float(tail[D] / total)
    return order, D, err


def null_completion(q_nz: np.ndarray, dim: int, k: int, group: int = 0,
                    side: int = 0) -> np.ndarray:
    """``k`` orthonormal vectors orthogonal to the ``r`` orthonormal columns
    of ``q_nz`` (``dim x r``): columns ``r .. r+k-1`` of the orthogonal
    factor of the complete Householder QR of ``q_nz`` (LAPACK ``dgeqrf`` +
    ``dorgqr`` conventions), i.e. the unit vectors e_r .. e_{r+k-1} carried
    through the r reflectors -- the basis states of the group that the
    nonzero vectors leave, made orthogonal to them.  O(dim r (r + k)) work;
    exactly orthonormal whatever the overlap of the unit vectors with
    ``q_nz``.  With r = 0 it is the first k unit vectors.  Signed zeros of
    ``q_nz`` are made +0.0 first: a reflector's sign follows its pivot's,
    and an exact zero pivot counts as positive (LAPACK would read its sign
    bit).  (``group`` and ``side`` do not enter.)"""
    if k == 0:
        return np.zeros((dim, 0))
    r = q_nz.shape[1]
    if r == 0:
        return np.eye(dim, k)
    q_nz = np.where(q_nz == 0.0, 0.0, q_nz)
    qf = np.linalg.qr(q_nz, mode="complete")[0]
    return np.ascontiguousarray(qf[:, r:r + k])


def svd(t: BSTensor, ldims: int, ldiv, trunc_err: float, dmin: int, dmax: int) -> SVDResult:
    """Restatement of gqten's truncating ``SVD`` as called at
    ``two_site_update_finite_vmps_impl.h:258-263``.

    * The tensor is matricised with its first ``ldims`` legs as rows.  Every
      block allowed by the tensor's divergence takes part (absent blocks are
      zero).  Blocks whose row legs carry the same new-bond charge
      ``q = ldiv - sum_{i<ldims} dir_i q_i`` form one dense matrix; its rows
      are the row-leg sector tuples of the group in ascending order, its
      columns likewise.
    * Every group is decomposed (LAPACK ``gesdd``).  Values at or below
      ``ZERO_SV_RTOL * s_max`` (global maximum) become exact zeros.
    * The kept values are chosen by :func:`select_kept`.  Kept nonzero
      values take the LAPACK singular vectors with the sign convention of
      :func:`fix_sign`; kept zero values take the canonical completion of
      :func:`null_completion` on both sides (LAPACK's own choice for them
      is arbitrary).
    * The new bond's sectors are the groups with at least one kept value,
      ascending in charge.  U carries divergence ``ldiv``, S is diagonal
      with divergence zero, Vt takes the remainder.  S is not renormalised.
    """
    ldiv = tuple(ldiv)
    row_idx = t.indices[:ldims]
    col_idx = t.indices[ldims:]
    groups: Dict[tuple, dict] = {}
    for coords in t.allowed_coords():
        q = qn_sub(ldiv, _left_qn(t, coords, ldims))
        g = groups.setdefault(q, {"rows": {}, "cols": {}, "blocks": []})
        rc, cc = coords[:ldims], coords[ldims:]
        g["rows"].setdefault(rc, int(np.prod([ix.dims[c] for ix, c in zip(row_idx, rc)])))
        g["cols"].setdefault(cc, int(np.prod([ix.dims[c] for ix, c in zip(col_idx, cc)])))
        blk = t.blocks.get(coords)
        if blk is not None:
            g["blocks"].append((rc, cc, blk))
    qs = sorted(groups)
    dec = []
    all_s = []
    for q in qs:
        g = groups[q]
        rows = sorted(g["rows"])
        cols = sorted(g["cols"])
        roff, off = {}, 0
        for r in rows:
            roff[r] = off
            off += g["rows"][r]
        m = off
        coff, off = {}, 0
        for c in cols:
            coff[c] = off
            off += g["cols"][c]
        n = off
        mat = np.zeros((m, n))
        for rc, cc, blk in g["blocks"]:
            mr, nc = g["rows"][rc], g["cols"][cc]
            mat[roff[rc]:roff[rc] + mr, coff[cc]:coff[cc] + nc] = blk.reshape(mr, nc)
        u, s, vt = np.linalg.svd(mat, full_matrices=False)
        dec.append([q, rows, cols, roff, coff, u, s, vt, m, n])
        all_s.append(s)
    flat = np.concatenate(all_s) if all_s else np.zeros(0)
    smax = float(flat.max()) if flat.size else 0.0
    flat = np.where(flat > ZERO_SV_RTOL * smax, flat, 0.0)
    order, D, err = select_kept(flat, trunc_err, dmin, dmax)
    keep = np.zeros(flat.size, dtype=bool)
    keep[order[:D]] = True
    sectors, masks, svals_g = [], [], []
    pos = 0
    for d in dec:
        ns = d[6].size
        kmask = keep[pos:pos + ns]
        svals_g.append(flat[pos:pos + ns])
        pos += ns
        masks.append(kmask)
        if kmask.any():
            sectors.append((d[0], int(kmask.sum())))
    new_out = Index(sectors, OUT)
    new_in = new_out.inverse()
    ub, sb, vb = {}, {}, {}
    svals = []
    sec = 0
    for gi, (d, kmask, sg) in enumerate(zip(dec, masks, svals_g)):
        if not kmask.any():
            continue
        q, rows, cols, roff, coff, u, s, vt, m, n = d
        nzmask = sg > 0.0
        keep_nz = kmask & nzmask
        k_zero = int((kmask & ~nzmask).sum())
        u_nz_all = u[:, nzmask]
        v_nz_all = vt[nzmask, :].T
        uk, vk = fix_sign(u[:, keep_nz], vt[keep_nz, :])
        if k_zero:
            uz = null_completion(u_nz_all, m, k_zero, gi, 0)
            vz = null_completion(v_nz_all, n, k_zero, gi, 1)
            uk = np.concatenate([uk, uz], axis=1)
            vk = np.concatenate([vk, vz.T], axis=0)
        sk = np.concatenate([sg[keep_nz], np.zeros(k_zero)])
        svals.append(sk)
        for r in rows:
            shape = tuple(ix.dims[c] for ix, c in zip(row_idx, r))
            blk = uk[roff[r]:roff[r] + int(np.prod(shape)), :]
            ub[r + (sec,)] = blk.reshape(shape + (sk.size,)).copy()
        for c in cols:
            shape = tuple(ix.dims[cc] for ix, cc in zip(col_idx, c))
            blk = vk[:, coff[c]:coff[c] + int(np.prod(shape))]
            vb[(sec,) + c] = blk.reshape((sk.size,) + shape).copy()
        sb[(sec, sec)] = np.diag(sk)
        sec += 1
    nq = len(ldiv)
    u_t = BSTensor(row_idx + [new_out], ldiv, ub)
    s_t = BSTensor([new_in, new_out], (0,) * nq, sb)
    vdiv = qn_sub(t.div, ldiv) if t.div is not None else None
    v_t = BSTensor([new_in] + col_idx, vdiv, vb)
    return SVDResult(u_t, s_t, v_t, err, D,
                     np.concatenate(svals) if svals else np.zeros(0))


def svd_full(t: BSTensor, ldims: int, ldiv) -> SVDResult:
    """Untruncated SVD (``mock_gqten::SVD``, ``utilities.h:26-57``)."""
    return svd(t, ldims, ldiv, 0.0, 1 << 30, 1 << 30)
