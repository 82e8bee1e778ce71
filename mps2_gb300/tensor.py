"""Host-side block-sparse tensor container (the boundary data format).

This mirrors the parts of GraceQ/tensor's ``GQTensor``/``Index``/``QN`` that
gqmps2's user code touches: building local operators element by element
(``did({0, 0}) = 1`` in ``tests/test_algorithm/test_two_site_update_finite_vmps.cc:105-110``),
``InverseIndex``, ``Div``, and handing MPS/MPO tensors to the solver.  All
arithmetic happens on the GPU inside ``libgqmps2_gb300.so``; this class only
holds data.

Conventions shared with the C ABI (``include/gqmps2_gb300.h``):

* a quantum number is a tuple of ``nq`` ints (U(1)^nq charges);
* leg direction ``OUT = +1``, ``IN = -1``; a block with sector coordinates
  ``c`` is allowed when ``sum_i dir_i * qn_i(c_i) == div``;
* blocks are dense row-major float64 arrays, exchanged in ascending
  lexicographic order of their sector coordinates ("block order").
"""
from __future__ import annotations

import itertools
from typing import Dict, List, Sequence, Tuple

import numpy as np

OUT = 1
IN = -1


def _qadd(a, b):
    return tuple(x + y for x, y in zip(a, b))


def _qscale(s, a):
    return tuple(s * x for x in a)


class QN(tuple):
    """A U(1)^n quantum number; ``QN(1, 0)`` for (N=1, Sz=0)."""

    def __new__(cls, *vals):
        if len(vals) == 1 and isinstance(vals[0], (tuple, list)):
            vals = tuple(vals[0])
        return super().__new__(cls, tuple(int(v) for v in vals))

    def __add__(self, other):
        return QN(_qadd(self, other))

    def __sub__(self, other):
        return QN(tuple(x - y for x, y in zip(self, other)))

    def __neg__(self):
        return QN(tuple(-x for x in self))


class Index:
    """A tensor leg: direction plus ordered (QN, degeneracy) sectors."""

    __slots__ = ("dir", "qns", "dims")

    def __init__(self, sectors: Sequence[Tuple[Sequence[int], int]], dir: int):
        if dir not in (IN, OUT):
            raise ValueError("direction must be IN (-1) or OUT (+1)")
        self.dir = int(dir)
        self.qns = [QN(q) for q, _ in sectors]
        self.dims = [int(d) for _, d in sectors]
        if any(d <= 0 for d in self.dims):
            raise ValueError("sector dimensions must be positive")

    @property
    def dim(self) -> int:
        return sum(self.dims)

    @property
    def nsec(self) -> int:
        return len(self.dims)

    @property
    def nq(self) -> int:
        return len(self.qns[0]) if self.qns else 0

    def sectors(self):
        return list(zip(self.qns, self.dims))

    def inverse(self) -> "Index":
        return Index(self.sectors(), -self.dir)

    def coor_to_sector(self, coor: int) -> Tuple[int, int]:
        if coor < 0:
            raise IndexError("negative coordinate")
        for s, d in enumerate(self.dims):
            if coor < d:
                return s, coor
            coor -= d
        raise IndexError("coordinate out of range")

    def qn_of_coor(self, coor: int) -> QN:
        return self.qns[self.coor_to_sector(coor)[0]]

    def __eq__(self, other):
        return (isinstance(other, Index) and self.dir == other.dir
                and self.qns == other.qns and self.dims == other.dims)

    def __hash__(self):
        return hash((self.dir, tuple(self.qns), tuple(self.dims)))

    def __repr__(self):
        return f"Index({self.sectors()}, {'OUT' if self.dir == OUT else 'IN'})"


def InverseIndex(ix: Index) -> Index:
    return ix.inverse()


class GQTensor:
    """Host block-sparse tensor (data only)."""

    def __init__(self, indices: Sequence[Index] = (), div=None, blocks=None):
        self.indices: List[Index] = list(indices)
        self.blocks: Dict[tuple, np.ndarray] = {}
        self.div = None if div is None else QN(div)
        if blocks:
            for k, v in blocks.items():
                self.blocks[tuple(int(c) for c in k)] = np.ascontiguousarray(v, dtype=np.float64)
            if self.div is None:
                self.div = self.block_div(next(iter(self.blocks)))

    @property
    def rank(self) -> int:
        return len(self.indices)

    @property
    def nq(self) -> int:
        return self.indices[0].nq if self.indices else 0

    @property
    def shape(self):
        return tuple(ix.dim for ix in self.indices)

    def is_default(self) -> bool:
        return self.rank == 0

    def block_div(self, coords) -> QN:
        q = (0,) * self.nq
        for ix, c in zip(self.indices, coords):
            q = _qadd(q, _qscale(ix.dir, ix.qns[c]))
        return QN(q)

    def block_shape(self, coords):
        return tuple(ix.dims[c] for ix, c in zip(self.indices, coords))

    def allowed_coords(self, div=None):
        div = self.div if div is None else QN(div)
        return [c for c in itertools.product(*[range(ix.nsec) for ix in self.indices])
                if self.block_div(c) == div]

    def __setitem__(self, coors, value):
        if not isinstance(coors, tuple):
            coors = (coors,)
        secs = [ix.coor_to_sector(c) for ix, c in zip(self.indices, coors)]
        bc = tuple(s for s, _ in secs)
        if bc not in self.blocks:
            d = self.block_div(bc)
            if self.div is None:
                self.div = d
            elif d != self.div:
                raise ValueError("element breaks the tensor's quantum-number divergence")
            self.blocks[bc] = np.zeros(self.block_shape(bc))
        self.blocks[bc][tuple(o for _, o in secs)] = value

    def __getitem__(self, coors):
        if not isinstance(coors, tuple):
            coors = (coors,)
        secs = [ix.coor_to_sector(c) for ix, c in zip(self.indices, coors)]
        bc = tuple(s for s, _ in secs)
        blk = self.blocks.get(bc)
        if blk is None:
            return 0.0
        return float(blk[tuple(o for _, o in secs)])

    def __mul__(self, s):
        return GQTensor(self.indices, self.div, {k: v * s for k, v in self.blocks.items()})

    __rmul__ = __mul__

    def __neg__(self):
        return self * -1.0

    def to_dense(self) -> np.ndarray:
        out = np.zeros(self.shape)
        offs = [np.concatenate([[0], np.cumsum(ix.dims)]) for ix in self.indices]
        for bc, b in self.blocks.items():
            sl = tuple(slice(o[c], o[c] + d) for o, c, d in zip(offs, bc, b.shape))
            out[sl] = b
        return out

    def sorted_block_coords(self):
        return sorted(self.blocks)

    def size(self) -> int:
        return sum(b.size for b in self.blocks.values())

    def copy(self) -> "GQTensor":
        return GQTensor(self.indices, self.div, {k: v.copy() for k, v in self.blocks.items()})

    def dense_equal(self, other, tol=0.0) -> bool:
        if self.indices != other.indices:
            return False
        return bool(np.max(np.abs(self.to_dense() - other.to_dense()), initial=0.0) <= tol)


def Div(t: GQTensor) -> QN:
    """Divergence of a tensor (zero QN for a tensor without blocks)."""
    if t.div is None:
        return QN((0,) * t.nq)
    return t.div
