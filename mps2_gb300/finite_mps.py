"""Finite MPS container, initialisers and the on-disk tensor layout.

* ``FiniteMPS`` mirrors ``one_dim_tn/mps/finite_mps/finite_mps.h:51-140``:
  a vector of site tensors that may be empty (the solver takes and returns
  the state through ``mps_path``), with ``Dump``/``Load`` of
  ``mps/mps.h:69-107``.
* File naming follows the reference: ``<mps_path>/mps_ten<i>.gqten``
  (``GenMPSTenName``, ``mps/mps.h:31-34``) and
  ``<temp_path>/{l,r}env<len>.gqten`` (``GenEnvTenName``,
  ``two_site_update_finite_vmps_impl.h:55-61``).  The byte layout inside a
  file is this project's own (gqten's stream format is not part of the
  reference tree); it is documented in :func:`write_tensor`.
* ``DirectStateInitMps`` restates ``finite_mps_init.h:216-262``.
"""
from __future__ import annotations

import os
import struct
from typing import List, Optional, Sequence

import numpy as np

from .site_vec import SiteVec
from .tensor import GQTensor, Index, IN, OUT, QN

kMpsPath = "mps"
kRuntimeTempPath = ".temp"
kEnvFileBaseName = "env"
kMpsTenBaseName = "mps_ten"
kGQTenFileSuffix = "gqten"

_MAGIC = b"GQTB"
_VERSION = 1


def GenMPSTenName(mps_path: str, idx: int) -> str:
    return f"{mps_path}/{kMpsTenBaseName}{idx}.{kGQTenFileSuffix}"


def GenEnvTenName(dir: str, blk_len: int, temp_path: str) -> str:
    return f"{temp_path}/{dir}{kEnvFileBaseName}{blk_len}.{kGQTenFileSuffix}"


def write_tensor(t: GQTensor, path: str) -> None:
    """Binary layout (little endian):

    ``"GQTB"``, u32 version=1, u32 rank, u32 nq, i32[nq] div;
    per leg: i32 dir (+1 OUT / -1 IN), u32 nsec, nsec x (i32[nq] qn, i64 dim);
    u64 nblocks; nblocks x u32[rank] sector coordinates (block order:
    ascending lexicographic); then every block's float64 data, row-major,
    in the same order.
    """
    nq = t.nq
    div = t.div if t.div is not None else QN((0,) * nq)
    coords = t.sorted_block_coords()
    with open(path, "wb") as f:
        f.write(_MAGIC)
        f.write(struct.pack("<III", _VERSION, t.rank, nq))
        f.write(struct.pack(f"<{nq}i", *div))
        for ix in t.indices:
            f.write(struct.pack("<iI", ix.dir, ix.nsec))
            for q, d in ix.sectors():
                f.write(struct.pack(f"<{nq}iq", *q, d))
        f.write(struct.pack("<Q", len(coords)))
        for c in coords:
            f.write(struct.pack(f"<{t.rank}I", *c))
        for c in coords:
            f.write(np.ascontiguousarray(t.blocks[c], dtype="<f8").tobytes())


def read_tensor(path: str) -> GQTensor:
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:4] != _MAGIC:
        raise ValueError(f"{path}: not a tensor file")
    off = 4
    ver, rank, nq = struct.unpack_from("<III", buf, off)
    off += 12
    if ver != _VERSION:
        raise ValueError(f"{path}: unsupported version {ver}")
    div = struct.unpack_from(f"<{nq}i", buf, off)
    off += 4 * nq
    indices = []
    for _ in range(rank):
        d, nsec = struct.unpack_from("<iI", buf, off)
        off += 8
        secs = []
        for _ in range(nsec):
            vals = struct.unpack_from(f"<{nq}iq", buf, off)
            off += 4 * nq + 8
            secs.append((vals[:nq], vals[nq]))
        indices.append(Index(secs, d))
    (nblk,) = struct.unpack_from("<Q", buf, off)
    off += 8
    coords = []
    for _ in range(nblk):
        coords.append(struct.unpack_from(f"<{rank}I", buf, off))
        off += 4 * rank
    t = GQTensor(indices, div)
    for c in coords:
        shape = t.block_shape(c)
        n = int(np.prod(shape))
        t.blocks[tuple(c)] = np.frombuffer(buf, dtype="<f8", count=n, offset=off).reshape(shape).copy()
        off += 8 * n
    if off != len(buf):
        raise ValueError(f"{path}: trailing bytes")
    return t


kUncentralizedCenterIdx = -1


class FiniteMPS:
    """A finite MPS: ``N`` optional site tensors plus the site information.

    As the reference's non-const accessors do (``finite_mps.h:67-89``),
    assigning a site tensor marks that site non-canonical and the MPS
    uncentralised; ``Centralize`` and the initialisers set both afterwards."""

    # canonical types of the site tensors (``MPSTenCanoType``)
    NONE, LEFT, RIGHT = 0, 1, 2

    def __init__(self, site_vec: SiteVec):
        self.site_vec = site_vec
        self.tens: List[Optional[GQTensor]] = [None] * site_vec.size
        self.center = kUncentralizedCenterIdx
        self.tens_cano_type = [FiniteMPS.NONE] * site_vec.size

    def GetCenter(self) -> int:
        return self.center

    def GetTensCanoType(self) -> List[int]:
        return list(self.tens_cano_type)

    def GetTenCanoType(self, i: int) -> int:
        return self.tens_cano_type[i]

    def Centralize(self, target_center: int) -> None:
        """``FiniteMPS::Centralize`` (``finite_mps.h:149-248``) on the GPU:
        the site tensors are uploaded, canonicalised by device SVDs and
        contractions, and downloaded again."""
        from .vmps import mps_centralize
        mps_centralize(self, target_center)
        self.center = target_center

    def size(self) -> int:
        return len(self.tens)

    __len__ = size

    def __getitem__(self, i) -> GQTensor:
        t = self.tens[i]
        if t is None:
            raise KeyError(f"site {i} is not loaded")
        return t

    def __setitem__(self, i, t: GQTensor):
        self.tens[i] = t
        self.tens_cano_type[i] = FiniteMPS.NONE
        self.center = kUncentralizedCenterIdx

    def empty(self) -> bool:
        return all(t is None for t in self.tens)

    def clear(self):
        self.tens = [None] * len(self.tens)

    def dealloc(self, i):
        self.tens[i] = None

    def GetSitesInfo(self) -> SiteVec:
        return self.site_vec

    def LoadTen(self, i: int, file: str) -> None:
        """``TenVec::LoadTen`` (``ten_vec.h:50-55``)."""
        self.tens[i] = read_tensor(file)

    def DumpTen(self, i: int, file: str, release_mem: bool = False) -> None:
        """``TenVec::DumpTen`` (``ten_vec.h:63-85``)."""
        write_tensor(self[i], file)
        if release_mem:
            self.tens[i] = None

    def Dump(self, mps_path: str = kMpsPath, release_mem: bool = False) -> None:
        os.makedirs(mps_path, exist_ok=True)
        for i, t in enumerate(self.tens):
            write_tensor(t, GenMPSTenName(mps_path, i))
            if release_mem:
                self.tens[i] = None

    def Load(self, mps_path: str = kMpsPath) -> None:
        for i in range(len(self.tens)):
            self.tens[i] = read_tensor(GenMPSTenName(mps_path, i))


def DirectStateInitMps(mps: FiniteMPS, stat_labs: Sequence[int], zero_div) -> None:
    """``finite_mps_init.h:216-262``: bond-dimension-1 product state.

    The head tensor carries the total charge; the bond charge to the right
    of site i is the sum of the site charges right of i.  The result is
    already right-canonical (every site tensor is a single 1), which is
    what the reference's trailing ``Centralize(0)`` produces for it.
    """
    zero_div = QN(zero_div)
    N = mps.size()
    if N != len(stat_labs):
        raise ValueError("one state label per site")
    pb = mps.site_vec.sites
    qs = [pb[i].qn_of_coor(stat_labs[i]) for i in range(N)]
    div = qs[0]
    for q in qs[1:]:
        div = div + q
    rvb = Index([(div - qs[0], 1)], OUT)
    t0 = GQTensor([pb[0], rvb])
    t0[stat_labs[0], 0] = 1.0
    mps[0] = t0
    for i in range(1, N - 1):
        lvb = rvb.inverse()
        rq = zero_div - qs[i] + lvb.qns[0]
        rvb = Index([(rq, 1)], OUT)
        t = GQTensor([lvb, pb[i], rvb])
        t[0, stat_labs[i], 0] = 1.0
        mps[i] = t
    lvb = rvb.inverse()
    t = GQTensor([lvb, pb[N - 1]])
    t[0, stat_labs[N - 1]] = 1.0
    mps[N - 1] = t
    mps.center = 0
    mps.tens_cano_type = [FiniteMPS.NONE] + [FiniteMPS.RIGHT] * (N - 1)


def extend_direct_random_tensors(mps: FiniteMPS, stat_labs_set: Sequence[Sequence[int]],
                                 zero_div, enlarged_dim: int, seed: int = 0) -> List[GQTensor]:
    """The site tensors of ``ExtendDirectRandomInitMps``
    (``finite_mps_init.h:269-330``) before its final ``Centralize(0)``: a
    sum of the product states ``stat_labs_set[j]``, each bond carrying one
    sector of dimension ``enlarged_dim`` per product state (the charge that
    product state puts on that bond), every allowed block filled with random
    values.  The head tensor carries the total charge of the first product
    state.  GraceQ/tensor's ``Random`` (its generator and distribution) is
    not in the reference tree; this uses numpy's PCG64 seeded with ``seed``
    and values uniform in [0, 1)."""
    zero_div = QN(zero_div)
    N = mps.size()
    nfuse = len(stat_labs_set)
    if nfuse < 1:
        raise ValueError("at least one product state")
    if any(len(labs) != N for labs in stat_labs_set):
        raise ValueError("one state label per site in every product state")
    if enlarged_dim < 1:
        raise ValueError("enlarged_dim must be positive")
    rng = np.random.default_rng(seed)
    pb = mps.site_vec.sites

    def random_fill(t: GQTensor) -> GQTensor:
        for c in t.allowed_coords(t.div):
            t.blocks[c] = rng.random(t.block_shape(c))
        return t

    div = pb[0].qn_of_coor(stat_labs_set[0][0])
    for i in range(1, N):
        div = div + pb[i].qn_of_coor(stat_labs_set[0][i])
    rq = [div - pb[0].qn_of_coor(stat_labs_set[j][0]) for j in range(nfuse)]
    rvb = Index([(q, enlarged_dim) for q in rq], OUT)
    tens = [random_fill(GQTensor([pb[0], rvb], div))]
    for i in range(1, N - 1):
        lvb = rvb.inverse()
        # lvb's sector j (coordinate j * enlarged_dim) carries product state j
        rq = [zero_div - pb[i].qn_of_coor(stat_labs_set[j][i]) +
              lvb.qn_of_coor(j * enlarged_dim) for j in range(nfuse)]
        rvb = Index([(q, enlarged_dim) for q in rq], OUT)
        tens.append(random_fill(GQTensor([lvb, pb[i], rvb], zero_div)))
    tens.append(random_fill(GQTensor([rvb.inverse(), pb[N - 1]], zero_div)))
    return tens


def ExtendDirectRandomInitMps(mps: FiniteMPS, stat_labs_set: Sequence[Sequence[int]], zero_div,
                              enlarged_dim: int, seed: int = 0) -> None:
    """``ExtendDirectRandomInitMps`` (``finite_mps_init.h:269-330``): the
    random sum of product states of :func:`extend_direct_random_tensors`,
    centralised at site 0 on the GPU, the head tensor normalised."""
    tens = extend_direct_random_tensors(mps, stat_labs_set, zero_div, enlarged_dim, seed)
    for i, t in enumerate(tens):
        mps[i] = t
    mps.Centralize(0)
    t0 = mps[0]
    nrm = float(np.sqrt(sum(float(np.sum(b * b)) for b in t0.blocks.values())))
    if nrm > 0.0:
        for k in t0.blocks:
            t0.blocks[k] = t0.blocks[k] / nrm
    # the reference normalises through the writing accessor, which marks the
    # site non-canonical and the MPS uncentralised
    mps.tens_cano_type[0] = FiniteMPS.NONE
    mps.center = kUncentralizedCenterIdx
