"""Local Hilbert spaces of a 1-D system (gqmps2 ``SiteVec``).

Mirrors ``include/gqmps2/site_vec.h:37-132``: every site carries an
OUT-directed physical index and an identity operator on it.
"""
from __future__ import annotations

from typing import Sequence, Union

import numpy as np

from .tensor import GQTensor, Index, OUT


def SetIndexDirOut(ix: Index) -> Index:
    """``site_vec.h:37-43``: the physical index is stored OUT-directed."""
    return ix if ix.dir == OUT else ix.inverse()


def GenIdOp(pb_out: Index) -> GQTensor:
    """``site_vec.h:47-53``: identity on one site, legs (in, out)."""
    op = GQTensor([pb_out.inverse(), pb_out])
    for i in range(pb_out.dim):
        op[i, i] = 1.0
    return op


class SiteVec:
    """``SiteVec(N, local_hilbert_space)`` or ``SiteVec([index per site])``."""

    def __init__(self, n_or_list: Union[int, Sequence[Index]], pb: Index = None):
        if isinstance(n_or_list, int):
            if pb is None:
                raise ValueError("SiteVec(N, index) needs the local index")
            sites = [SetIndexDirOut(pb)] * n_or_list
        else:
            sites = [SetIndexDirOut(ix) for ix in n_or_list]
        self.sites = list(sites)
        self.size = len(self.sites)
        self.id_ops = [GenIdOp(ix) for ix in self.sites]
