"""The 5-site MPS of ``test_finite_mps.cc:30-63`` (U(1) charge N): random
blocks with the reference's divergences."""
from mps2_gb300.tensor import GQTensor, IN, Index, OUT, QN
from _helpers import random_tensor


def reference_mps_tensors(rng, divs=(1, 1, 0, 0, 0)):
    q = [QN(0), QN(1), QN(2)]
    pb_out = Index([(q[0], 1), (q[1], 1)], OUT)
    vb01_out = Index([(q[0], 1), (q[1], 1)], OUT)
    vb012_out = Index([(q[0], 1), (q[1], 2), (q[2], 1)], OUT)
    legs = [[pb_out, vb01_out],
            [vb01_out.inverse(), pb_out, vb012_out],
            [vb012_out.inverse(), pb_out, vb012_out],
            [vb012_out.inverse(), pb_out, vb01_out],
            [vb01_out.inverse(), pb_out]]
    return [random_tensor(rng, l, (d,)) for l, d in zip(legs, divs)], pb_out
