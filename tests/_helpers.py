"""Shared test helpers: random block-sparse tensors, oracle states, errors."""
import itertools

import numpy as np

import oracle
from mps2_gb300.tensor import GQTensor, Index, IN, OUT
from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
from oracle.lanczos import LanczosParams as OLP
from oracle.vmps import SweepParams as OSP
from _convert import from_oracle, to_oracle


def random_index(rng, nsec, qrange, dmax, dir, nq=1):
    qs = set()
    while len(qs) < nsec:
        qs.add(tuple(int(v) for v in rng.integers(-qrange, qrange + 1, size=nq)))
    return Index([(q, int(rng.integers(1, dmax + 1))) for q in sorted(qs)], dir)


def random_tensor(rng, indices, div, fill=1.0):
    """Random blocks on a `fill` fraction of the allowed blocks (at least
    one block whenever the divergence allows any)."""
    t = GQTensor(indices, div)
    allowed = t.allowed_coords(div)
    for c in allowed:
        if rng.random() <= fill:
            t.blocks[c] = rng.standard_normal(t.block_shape(c))
    if allowed and not t.blocks:
        c = allowed[int(rng.integers(len(allowed)))]
        t.blocks[c] = rng.standard_normal(t.block_shape(c))
    return t


def first_allowed_div(indices):
    """A divergence for which these legs allow at least one block."""
    t = GQTensor(indices)
    return t.block_div(tuple(0 for _ in indices))


def rel_err(gpu: GQTensor, ref) -> float:
    """||gpu - ref|| / ||ref|| over the union of blocks (absent = zero)."""
    num = 0.0
    den = 0.0
    keys = set(gpu.blocks) | set(ref.blocks)
    for k in keys:
        a = gpu.blocks.get(k)
        b = ref.blocks.get(k)
        if a is None:
            a = np.zeros_like(b)
        if b is None:
            b = np.zeros_like(a)
        num += float(np.sum((a - b) ** 2))
        den += float(np.sum(b ** 2))
    return float(np.sqrt(num / den)) if den > 0 else float(np.sqrt(num))


def oracle_state(build, labels, sweeps, D, lanczos=(1e-9, 50)):
    """Run the oracle for `sweeps` sweeps and return (mps, mpo, envs) as
    oracle tensors, to take realistic effective Hamiltonians from."""
    sv, mpo, qn0, _ = build()
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, labels, qn0)
    om = [to_oracle(t) for t in mps.tens]
    oo = [to_oracle(t) for t in mpo]
    envs = {}
    if sweeps > 0:
        oracle.two_site_finite_vmps(om, oo, OSP(sweeps, D, D, 0.0, OLP(*lanczos)), envs=envs)
    else:
        oracle.init_envs(om, oo, envs)
    return om, oo, envs
