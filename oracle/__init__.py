"""FP64 CPU oracle for the two-site DMRG hot path -- TEST INFRASTRUCTURE ONLY.

Imported only by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py``; the product never imports, links or runs it.
"""
from .bstensor import (BSTensor, Index, IN, OUT, contract, dag, inner,  # noqa: F401
                       linear_combine, svd, svd_full)
from .lanczos import LanczosParams, lanczos_solver  # noqa: F401
from .vmps import SweepParams, two_site_finite_vmps, init_envs  # noqa: F401
