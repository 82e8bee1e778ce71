"""Conversions between the product's host tensors and the oracle's."""
import oracle
from mps2_gb300.tensor import GQTensor, Index


def to_oracle(t: GQTensor) -> "oracle.BSTensor":
    idx = [oracle.Index([(tuple(q), d) for q, d in ix.sectors()], ix.dir) for ix in t.indices]
    return oracle.BSTensor(idx, None if t.div is None else tuple(t.div),
                           {k: v.copy() for k, v in t.blocks.items()})


def from_oracle(t) -> GQTensor:
    idx = [Index(ix.sectors(), ix.dir) for ix in t.indices]
    return GQTensor(idx, t.div, {k: v.copy() for k, v in t.blocks.items()})
