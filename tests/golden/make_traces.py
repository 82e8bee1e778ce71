"""Write the oracle's per-update DMRG traces used by the GPU parity tests.

Each trace is the FP64 oracle (``oracle/``, the CPU restatement of gqmps2's
``TwoSiteFiniteVMPS``) run on one workload, with every two-site update's
site, direction, energy E0, truncation error, kept bond dimension D,
Lanczos iteration count and entanglement entropy S (the fields of the
reference's per-update log line, ``two_site_update_finite_vmps_impl.h:329-338``),
plus the energy at the end of each sweep.

Workloads:
* ``heisenberg_L20_D200``: spin-1/2 Heisenberg open chain, L=20, J=1, U(1)
  Sz, total Sz=0, Neel labels with the site order shuffled by seed 0,
  Dmin=Dmax=200, 4 sweeps, Lanczos (1e-9, 100), trunc_err 0;
* ``hubbard_L16_D128``: Fermi-Hubbard open chain, L=16, t=1, U=8, half
  filling, U(1)xU(1) (N, Sz), alternating up/down product state,
  Dmin=Dmax=128, 4 sweeps, Lanczos (1e-9, 100), trunc_err 0.

Run from the repository root: ``python tests/golden/make_traces.py [name ...]``.
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def workloads():
    from mps2_gb300 import hamiltonians as H
    return {
        "heisenberg_L20_D200": dict(build=lambda: H.heisenberg_chain(20),
                                    labels=H.neel_shuffled_labels(20, 0),
                                    sweeps=4, D=200, lanczos=(1e-9, 100)),
        "hubbard_L16_D128": dict(build=lambda: H.hubbard_chain(16, 1.0, 8.0),
                                 labels=[1 if i % 2 == 0 else 2 for i in range(16)],
                                 sweeps=4, D=128, lanczos=(1e-9, 100)),
    }


def trace(name):
    import oracle
    from _convert import to_oracle
    from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
    from oracle.lanczos import LanczosParams as OLP
    from oracle.vmps import SweepParams as OSP
    w = workloads()[name]
    sv, mpo, qn0, _ = w["build"]()
    mps = FiniteMPS(sv)
    DirectStateInitMps(mps, w["labels"], qn0)
    om = [to_oracle(t) for t in mps.tens]
    oo = [to_oracle(t) for t in mpo]
    stats, sweep_e = [], []
    t0 = time.perf_counter()
    oracle.two_site_finite_vmps(om, oo, OSP(w["sweeps"], w["D"], w["D"], 0.0, OLP(*w["lanczos"])),
                                stats=stats, sweep_energies=sweep_e)
    return {
        "workload": name, "L": len(mpo), "D": w["D"], "sweeps": w["sweeps"],
        "lanczos": list(w["lanczos"]), "labels": w["labels"],
        "oracle_seconds": time.perf_counter() - t0,
        "sweep_energies": sweep_e,
        "updates": [{"site": s.site, "dir": s.dir, "e0": s.e0, "trunc_err": s.trunc_err,
                     "D": s.D, "iters": s.iters, "ee": s.ee} for s in stats],
    }


def main(names):
    for name in names or workloads():
        tr = trace(name)
        path = os.path.join(HERE, f"trace_{name}.json")
        with open(path, "w") as f:
            json.dump(tr, f, indent=0)
        print(f"{path}: {len(tr['updates'])} updates, E={tr['sweep_energies']}, "
              f"{tr['oracle_seconds']:.0f}s")


if __name__ == "__main__":
    main(sys.argv[1:])
