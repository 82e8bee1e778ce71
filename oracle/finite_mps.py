"""FP64 restatement of the finite-MPS canonicalisation and truncation.

Test infrastructure only (the checker of the device implementation).
Follows ``include/gqmps2/one_dim_tn/mps/finite_mps/finite_mps.h``:

* ``centralize``: ``FiniteMPS::Centralize`` (:149-161) with
  ``LeftCanonicalize_``/``LeftCanonicalizeTen_`` (:164-200) and
  ``RightCanonicalize_``/``RightCanonicalizeTen_`` (:203-248): untruncated
  SVD (``mock_gqten::SVD``, ``utilities.h:26-57``) of one site tensor, the
  orthonormal factor stays, S.Vt (or U.S) is pushed into the neighbour;
  tensors already canonical in the right direction are skipped.
* ``truncate_mps``: ``TruncateMPS`` (:251-300): centralise to site 0,
  normalise it, then a left-to-right pass of truncating SVDs whose S is
  normalised before it is pushed right.
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np

from .bstensor import BSTensor, contract, svd, svd_full

NONE, LEFT, RIGHT = 0, 1, 2


def _scaled_vt(res) -> BSTensor:
    """S.Vt of an SVD result (S along Vt's first leg)."""
    vt = res.vt
    out = BSTensor(vt.indices, vt.div, {})
    offs = np.cumsum([0] + list(vt.indices[0].dims))
    s = np.asarray(res.svals)
    for k, b in vt.blocks.items():
        sh = [1] * b.ndim
        sh[0] = -1
        out.blocks[k] = b * s[offs[k[0]]:offs[k[0] + 1]].reshape(sh)
    return out


def _u_scaled(res) -> BSTensor:
    """U.S of an SVD result (S along U's last leg)."""
    u = res.u
    out = BSTensor(u.indices, u.div, {})
    last = len(u.indices) - 1
    offs = np.cumsum([0] + list(u.indices[last].dims))
    s = np.asarray(res.svals)
    for k, b in u.blocks.items():
        sh = [1] * b.ndim
        sh[-1] = -1
        out.blocks[k] = b * s[offs[k[last]]:offs[k[last] + 1]].reshape(sh)
    return out


def left_canonicalize_ten(mps: List[BSTensor], cano: List[int], i: int) -> None:
    """``LeftCanonicalizeTen_`` (:178-200)."""
    ldims = 1 if i == 0 else 2
    res = svd_full(mps[i], ldims, mps[i].div)
    mps[i] = res.u
    mps[i + 1] = contract(_scaled_vt(res), mps[i + 1], [1], [0])
    cano[i] = LEFT
    cano[i + 1] = NONE


def right_canonicalize_ten(mps: List[BSTensor], cano: List[int], i: int) -> None:
    """``RightCanonicalizeTen_`` (:217-248): the row leg is the left bond and
    the row divergence is zero."""
    zero = tuple(0 for _ in mps[i].div)
    res = svd_full(mps[i], 1, zero)
    mps[i] = res.vt
    axis = 1 if i - 1 == 0 else 2
    mps[i - 1] = contract(mps[i - 1], _u_scaled(res), [axis], [0])
    cano[i] = RIGHT
    cano[i - 1] = NONE


def centralize(mps: List[BSTensor], cano: List[int], center: int) -> None:
    """``Centralize`` (:149-161)."""
    n = len(mps)
    if center != 0:
        stop = center - 1
        start = None
        for i in range(0, stop + 1):
            start = i
            if cano[i] != LEFT:
                break
            if i == stop:
                start = None
        if start is not None:
            for i in range(start, stop + 1):
                left_canonicalize_ten(mps, cano, i)
    if center != n - 1:
        stop = center + 1
        start = None
        for i in range(n - 1, stop - 1, -1):
            start = i
            if cano[i] != RIGHT:
                break
            if i == stop:
                start = None
        if start is not None:
            for i in range(start, stop - 1, -1):
                right_canonicalize_ten(mps, cano, i)


def truncate_mps(mps: List[BSTensor], cano: List[int], trunc_err: float, dmin: int,
                 dmax: int) -> List[Tuple[float, int]]:
    """``TruncateMPS`` (:251-300); returns (truncation error, D) per bond."""
    n = len(mps)
    centralize(mps, cano, 0)
    nrm = np.sqrt(sum(float(np.sum(b * b)) for b in mps[0].blocks.values()))
    mps[0] = BSTensor(mps[0].indices, mps[0].div, {k: b / nrm for k, b in mps[0].blocks.items()})
    out = []
    for i in range(n - 1):
        ldims = 1 if i == 0 else 2
        res = svd(mps[i], ldims, mps[i].div, trunc_err, dmin, dmax)
        out.append((res.trunc_err, res.D))
        s = np.asarray(res.svals)
        res.svals = list(s / np.sqrt(np.sum(s * s)))
        mps[i] = res.u
        mps[i + 1] = contract(_scaled_vt(res), mps[i + 1], [1], [0])
    # every site was written through the reference's non-const accessor,
    # which marks it as not canonical
    for i in range(n):
        cano[i] = NONE
    return out
