"""FP64 restatement of the finite-MPS measurements -- test infrastructure
only (the checker of ``mps2_gb300.measure``).

Follows ``one_dim_tn/mps/finite_mps/finite_mps_measu.h``: ``OneSiteOpAvg``
(:366-402), ``OpsVecAvg`` (:462-526) and ``CtrctMidTen`` (:528-554), with
``Centralize`` from ``oracle.finite_mps``.  Each function returns the plain
list of averages.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np

from .bstensor import BSTensor, contract, dag
from .finite_mps import centralize


def _scalar(t: BSTensor) -> float:
    return float(sum(float(np.sum(b)) for b in t.blocks.values()))


def one_site_avg(cent: BSTensor, op: BSTensor, site: int, n: int) -> float:
    if site == 0:
        x1, y1, x2, y2 = [0], [0], [0, 1], [1, 0]
    elif site == n - 1:
        x1, y1, x2, y2 = [1], [0], [0, 1], [0, 1]
    else:
        x1, y1, x2, y2 = [1], [0], [0, 2, 1], [0, 1, 2]
    temp = contract(cent, op, x1, y1)
    return _scalar(contract(temp, dag(cent), x2, y2))


def measure_one_site(mps: List[BSTensor], cano: List[int], op: BSTensor) -> List[float]:
    n = len(mps)
    out = []
    for i in range(n):
        centralize(mps, cano, i)
        out.append(one_site_avg(mps[i], op, i, n))
    return out


def ops_vec_avg(mps: List[BSTensor], ops: Sequence[BSTensor], head: int, tail: int) -> float:
    n = len(mps)
    if head == 0:
        a1, a2, a3 = [0], [1], [0]
    else:
        a1, a2, a3 = [1], [0, 2], [0, 1]
    t = contract(contract(mps[head], ops[0], a1, [0]), dag(mps[head]), a2, a3)
    for i in range(head + 1, tail):
        t1 = contract(mps[i], t, [0], [0])
        t2 = contract(t1, ops[i - head], [0], [0])
        t = contract(t2, dag(mps[i]), [1, 2], [0, 1])
    if tail == n - 1:
        b1, b2 = [0, 1], [0, 1]
    else:
        b1, b2 = [0, 1, 2], [2, 0, 1]
    t2 = contract(mps[tail], t, [0], [0])
    t3 = contract(t2, ops[-1], [0], [0])
    return _scalar(contract(t3, dag(mps[tail]), b1, b2))


def measure_two_site(mps: List[BSTensor], cano: List[int], a: BSTensor, b: BSTensor,
                     inst: BSTensor, sites_set) -> List[float]:
    """<A_i inst ... inst B_j> for each (i, j)."""
    out = []
    for i, j in sites_set:
        centralize(mps, cano, i)
        ops = [a] + [inst] * (j - i - 1) + [b]
        out.append(ops_vec_avg(mps, ops, i, j))
    return out
