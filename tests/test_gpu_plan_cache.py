"""Contraction plans kept per lane (``mps2_gb300/csrc/contract.cu``): the
same sweeps run with the plan cache (default) and without it
(``GQ_NO_PLAN_CACHE``) give bitwise identical energies and states."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import json, sys, hashlib
import numpy as np
sys.path.insert(0, ROOT)
from mps2_gb300 import hamiltonians as H, _lib
from mps2_gb300.finite_mps import DirectStateInitMps, FiniteMPS
from mps2_gb300.vmps import (DMRGState, LanczosParams, SweepParams, profile_enable,
                             profile_read)
_lib.check(_lib.load().gq_init(0))
N = 12
sv, mpo, qn0, _ = H.hubbard_chain(N, 1.0, 8.0)
mps = FiniteMPS(sv)
DirectStateInitMps(mps, [1 if i % 2 == 0 else 2 for i in range(N)], qn0)
st = DMRGState(mps.tens, mpo)
st.init_envs("fp64tc")
out = []
for k, (D, prec) in enumerate([(32, "tf32x3"), (64, "tf32x3"), (64, "tf32x3"), (64, "fp64")]):
    if k == 2:
        profile_enable(True)
    e, stats = st.sweep(SweepParams(1, D, D, 0.0, LanczosParams(1e-10, 40), precision=prec))
    if k == 2:
        plans = profile_read("host_plan")
        profile_enable(False)
    out.append(e.hex())
h = hashlib.sha256()
for i in range(N):
    t = st.get_mps(i)
    for key in sorted(t.blocks):
        h.update(np.ascontiguousarray(t.blocks[key]).tobytes())
print(json.dumps({"energies": out, "state": h.hexdigest(), "plan_ms": plans[1],
                  "plans": plans[0]}))
'''


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "-c", SCRIPT.replace("ROOT", repr(ROOT))],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.gpu
def test_plan_cache_gives_identical_sweeps():
    a = _run({})
    b = _run({"GQ_NO_PLAN_CACHE": "1"})
    assert a["energies"] == b["energies"]
    assert a["state"] == b["state"]
    assert a["plans"] == b["plans"] and a["plans"] > 0
