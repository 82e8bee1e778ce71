"""Model builders used by the tests and the benchmark.

Each builder returns ``(site_vec, mpo, zero_div)`` built with
:class:`MPOGenerator`, with the local operators exactly as the reference's
end-to-end tests define them
(``tests/test_algorithm/test_two_site_update_finite_vmps.cc``).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np

from .mpogen import MPOGenerator
from .site_vec import SiteVec
from .tensor import GQTensor, Index, IN, OUT, QN


# ---------------------------------------------------------------------------
# spin-1/2 with U(1) Sz (charges in units of 1/2: up=+1, down=-1)
# ---------------------------------------------------------------------------
def spin_half_ops():
    """Operators of ``test_two_site_update_finite_vmps.cc:86-110``."""
    pb_out = Index([(QN(1), 1), (QN(-1), 1)], OUT)
    pb_in = pb_out.inverse()
    ops = {k: GQTensor([pb_in, pb_out]) for k in ("id", "sz", "sp", "sm")}
    ops["id"][0, 0] = 1
    ops["id"][1, 1] = 1
    ops["sz"][0, 0] = 0.5
    ops["sz"][1, 1] = -0.5
    ops["sp"][0, 1] = 1
    ops["sm"][1, 0] = 1
    return pb_out, ops


def heisenberg_pairs(N: int, pairs: Sequence[Tuple[int, int, float]],
                     delta: float = 1.0, ising_only: bool = False):
    """H = sum_(i,j,J) J [Delta Sz_i Sz_j + (S+_i S-_j + S-_i S+_j)/2]."""
    pb_out, ops = spin_half_ops()
    sv = SiteVec(N, pb_out)
    qn0 = QN(0)
    gen = MPOGenerator(sv, qn0)
    for i, j, J in pairs:
        if i > j:
            i, j = j, i
        gen.AddTerm(J * delta, [ops["sz"], ops["sz"]], [i, j])
        if not ising_only:
            gen.AddTerm(0.5 * J, [ops["sp"], ops["sm"]], [i, j])
            gen.AddTerm(0.5 * J, [ops["sm"], ops["sp"]], [i, j])
    return sv, gen.Gen(), qn0, gen


def heisenberg_chain(N: int, J: float = 1.0, delta: float = 1.0):
    return heisenberg_pairs(N, [(i, i + 1, J) for i in range(N - 1)], delta)


def snake_index(x: int, y: int, Ly: int) -> int:
    """Snake ordering of an Lx x Ly cylinder: even columns go up, odd down."""
    return x * Ly + (y if x % 2 == 0 else Ly - 1 - y)


def j1j2_cylinder_pairs(Lx: int, Ly: int, J1: float, J2: float):
    """Open in x, periodic in y (cylinder), snake ordering."""
    pairs = {}

    def add(a, b, J):
        if a == b:
            return
        key = (min(a, b), max(a, b))
        pairs[key] = pairs.get(key, 0.0) + J

    for x in range(Lx):
        for y in range(Ly):
            s = snake_index(x, y, Ly)
            if Ly > 2 or y + 1 < Ly:
                add(s, snake_index(x, (y + 1) % Ly, Ly), J1)
            if x + 1 < Lx:
                add(s, snake_index(x + 1, y, Ly), J1)
                add(s, snake_index(x + 1, (y + 1) % Ly, Ly), J2)
                add(s, snake_index(x + 1, (y - 1) % Ly, Ly), J2)
    return [(a, b, J) for (a, b), J in sorted(pairs.items())]


# ---------------------------------------------------------------------------
# Hubbard with U(1)xU(1) (N_up, N_dn), basis {0, up, dn, updn}
# ---------------------------------------------------------------------------
def kitaev_simple_pairs(Nx: int = 4, Ny: int = 2):
    """The zz bonds of the ``2DKitaevSimpleCase`` lattice
    (``test_two_site_update_finite_vmps.cc:311-325``): for every odd column
    x and every y, the bond between honeycomb sites (x, y) and
    (x - 1, y + 1), site index Ny * (x mod Nx) + (y mod Ny), ordered."""
    pairs = []
    for x in range(Nx):
        for y in range(Ny):
            if x % 2 == 1:
                s0 = Ny * (x % Nx) + y % Ny
                s1 = Ny * ((x - 1) % Nx) + (y + 1) % Ny
                pairs.append((min(s0, s1), max(s0, s1), 1.0))
    return pairs


def hubbard_ops():
    """Operators of ``test_two_site_update_finite_vmps.cc:796-859``."""
    pb_out = Index([(QN(0, 0), 1), (QN(1, 0), 1), (QN(0, 1), 1), (QN(1, 1), 1)], OUT)
    pb_in = pb_out.inverse()
    names = ["f", "nupdn", "adagupf", "aup", "adagdn", "fadn", "naupf", "adagup",
             "nadn", "fadagdn"]
    o = {k: GQTensor([pb_in, pb_out]) for k in names}
    o["f"][0, 0] = 1
    o["f"][1, 1] = -1
    o["f"][2, 2] = -1
    o["f"][3, 3] = 1
    o["nupdn"][3, 3] = 1
    o["adagupf"][1, 0] = 1
    o["adagupf"][3, 2] = -1
    o["aup"][0, 1] = 1
    o["aup"][2, 3] = 1
    o["adagdn"][2, 0] = 1
    o["adagdn"][3, 1] = 1
    o["fadn"][0, 2] = 1
    o["fadn"][1, 3] = -1
    o["naupf"][0, 1] = 1
    o["naupf"][2, 3] = -1
    o["adagup"][1, 0] = 1
    o["adagup"][3, 2] = 1
    o["nadn"][0, 2] = -1
    o["nadn"][1, 3] = -1
    o["fadagdn"][2, 0] = -1
    o["fadagdn"][3, 1] = 1
    return pb_out, o


def hubbard_bonds(N: int, bonds: Sequence[Tuple[int, int, float]], U: float):
    """Hubbard model on the given hopping bonds, written like the reference
    test at ``:888-944`` (hopping with a Jordan-Wigner string ``f``)."""
    pb_out, o = hubbard_ops()
    sv = SiteVec(N, pb_out)
    qn0 = QN(0, 0)
    gen = MPOGenerator(sv, qn0)
    for s in range(N):
        gen.AddTerm(U, o["nupdn"], s)
    for a, b, t in bonds:
        if a > b:
            a, b = b, a
        gen.AddTerm(1.0, -t * o["adagupf"], a, o["aup"], b, o["f"])
        gen.AddTerm(1.0, -t * o["adagdn"], a, o["fadn"], b, o["f"])
        gen.AddTerm(1.0, o["naupf"], a, -t * o["adagup"], b, o["f"])
        gen.AddTerm(1.0, o["nadn"], a, -t * o["fadagdn"], b, o["f"])
    return sv, gen.Gen(), qn0, gen


def hubbard_chain(N: int, t: float = 1.0, U: float = 8.0):
    return hubbard_bonds(N, [(i, i + 1, t) for i in range(N - 1)], U)


def hubbard_2x2_reference():
    """The ``HubbardSystem.2Dcase`` lattice (``:888-944``): 2x2, t0=1,
    t1=0.5 on the diagonals, U=2."""
    Nx = Ny = 2
    t0, t1 = 1.0, 0.5
    bonds = []

    def idx(i, j):
        return i * Ny + j

    for i in range(Nx):
        for j in range(Ny):
            s0 = idx(i, j)
            if i != Nx - 1:
                bonds.append((s0, idx(i + 1, j), t0))
            if j != Ny - 1:
                bonds.append((s0, idx(i, j + 1), t0))
            if j != Ny - 1:
                if i != 0:
                    bonds.append((s0, idx(i - 1, j + 1), t1))
                if i != Nx - 1:
                    bonds.append((s0, idx(i + 1, j + 1), t1))
    return hubbard_bonds(Nx * Ny, bonds, 2.0)


# ---------------------------------------------------------------------------
# t-J with U(1)xU(1) (N, Sz), basis {up, dn, empty}
# ---------------------------------------------------------------------------
def tj_ops():
    """Operators of ``test_two_site_update_finite_vmps.cc:493-551``."""
    pb_out = Index([(QN(1, 1), 1), (QN(1, -1), 1), (QN(0, 0), 1)], OUT)
    pb_in = pb_out.inverse()
    names = ["f", "sz", "sp", "sm", "cup", "cdagup", "cdn", "cdagdn"]
    o = {k: GQTensor([pb_in, pb_out]) for k in names}
    o["f"][0, 0] = -1
    o["f"][1, 1] = -1
    o["f"][2, 2] = 1
    o["sz"][0, 0] = 0.5
    o["sz"][1, 1] = -0.5
    o["sp"][1, 0] = 1
    o["sm"][0, 1] = 1
    o["cup"][0, 2] = 1
    o["cdagup"][2, 0] = 1
    o["cdn"][1, 2] = 1
    o["cdagdn"][2, 1] = 1
    return pb_out, o


def tj_bonds(N: int, bonds, t: float = 3.0, J: float = 1.0):
    pb_out, o = tj_ops()
    sv = SiteVec(N, pb_out)
    qn0 = QN(0, 0)
    gen = MPOGenerator(sv, qn0)
    for a, b in bonds:
        gen.AddTerm(-t, o["cdagup"], a, o["cup"], b, o["f"])
        gen.AddTerm(-t, o["cdagdn"], a, o["cdn"], b, o["f"])
        gen.AddTerm(-t, o["cup"], a, o["cdagup"], b, o["f"])
        gen.AddTerm(-t, o["cdn"], a, o["cdagdn"], b, o["f"])
        gen.AddTerm(J, o["sz"], a, o["sz"], b)
        gen.AddTerm(J / 2, o["sp"], a, o["sm"], b)
        gen.AddTerm(J / 2, o["sm"], a, o["sp"], b)
    return sv, gen.Gen(), qn0, gen


# ---------------------------------------------------------------------------
# Kondo double chain (non-uniform sites, U(1) Sz with a single sector)
# ---------------------------------------------------------------------------
def kondo_double_chain(Nx: int = 4, t: float = 0.25, Jk: float = 1.0, Jz: float = 0.5):
    """``TestKondoInsulatorSystem`` (``:962-1115``)."""
    N = 2 * Nx
    pbE = Index([(QN(0), 4)], OUT)
    pbL = Index([(QN(0), 2)], OUT)
    iE, iL = pbE.inverse(), pbL.inverse()
    E = {k: GQTensor([iE, pbE]) for k in
         ("sz", "sp", "sm", "bupcF", "bupaF", "Fbdnc", "Fbdna", "bupc", "bupa", "bdnc", "bdna")}
    Lo = {k: GQTensor([iL, pbL]) for k in ("Sz", "Sp", "Sm")}
    E["sz"][0, 0] = 0.5
    E["sz"][1, 1] = -0.5
    E["sp"][0, 1] = 1.0
    E["sm"][1, 0] = 1.0
    E["bupcF"][2, 1] = -1
    E["bupcF"][0, 3] = 1
    E["Fbdnc"][2, 0] = 1
    E["Fbdnc"][1, 3] = -1
    E["bupaF"][1, 2] = 1
    E["bupaF"][3, 0] = -1
    E["Fbdna"][0, 2] = -1
    E["Fbdna"][3, 1] = 1
    E["bupc"][2, 1] = 1
    E["bupc"][0, 3] = 1
    E["bdnc"][2, 0] = 1
    E["bdnc"][1, 3] = 1
    E["bupa"][1, 2] = 1
    E["bupa"][3, 0] = 1
    E["bdna"][0, 2] = 1
    E["bdna"][3, 1] = 1
    Lo["Sz"][0, 0] = 0.5
    Lo["Sz"][1, 1] = -0.5
    Lo["Sp"][0, 1] = 1.0
    Lo["Sm"][1, 0] = 1.0
    pb = [pbE if i % 2 == 0 else pbL for i in range(N)]
    sv = SiteVec(pb)
    qn0 = QN(0)
    gen = MPOGenerator(sv, qn0)
    for i in range(0, N - 2, 2):
        gen.AddTerm(-t, E["bupcF"], i, E["bupa"], i + 2)
        gen.AddTerm(-t, E["bdnc"], i, E["Fbdna"], i + 2)
        gen.AddTerm(t, E["bupaF"], i, E["bupc"], i + 2)
        gen.AddTerm(t, E["bdna"], i, E["Fbdnc"], i + 2)
        gen.AddTerm(Jz, Lo["Sz"], i + 1, Lo["Sz"], i + 3)
    for i in range(0, N, 2):
        gen.AddTerm(Jk, E["sz"], i, Lo["Sz"], i + 1)
        gen.AddTerm(Jk / 2, E["sp"], i, Lo["Sm"], i + 1)
        gen.AddTerm(Jk / 2, E["sm"], i, Lo["Sp"], i + 1)
    return sv, gen.Gen(), qn0, gen


def neel_shuffled_labels(N: int, seed: int = 0) -> List[int]:
    """Neel labels (N/2 up, N/2 down) with the site order shuffled by a
    seeded generator; the total Sz stays 0."""
    labs = [i % 2 for i in range(N)]
    rng = np.random.default_rng(seed)
    rng.shuffle(labs)
    return [int(v) for v in labs]
