"""The device-checked debug library (libmpsgb300_checked.so, MPSG_DEVICE_CHECKS): every offset the
copy engine decodes is recomputed by plain division and every address is checked against its
task's span. A workload that runs the row, tile and gather copy modes through permutes, fusions,
contractions, both H_eff paths, environment updates and a short sweep records no violation and
still matches the oracle."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKLOAD = r"""
import json, sys
import numpy as np
sys.path.insert(0, ROOT); sys.path.insert(0, ROOT + "/tests")
import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from oracle import mps as om
from oracle import symtensors as st
assert mg.checked_library(), mg._lib.LIB_PATH
mg.device_checks(reset=True)
conv = lambda sp: tuple(st.VectorSpace(V.sectors, V.isdual) for V in sp)
errs = {}
for chi, nq in ((64, 9), (256, 15)):
    (sv, sl, sr), flats = gd.heff_inputs_host(chi, 0.5, 1911, nq)
    O = [st.from_flat(0, conv(s), f) for s, f in zip((sv, sl, sr), flats)]
    W = om.xxz_u1mpo(3, 0.5)[1]
    want = st.flatten(om.applymps2site(O[0], O[1], O[2], W, W))
    v, eL, eR, W1, W2 = gd.heff_problem(chi, 0.5, 1911, ncharges=nq)
    got = mg.applymps2site(v, eL, eR, W1, W2, precision=0).to_flat()
    errs[f"heff_fp64_{chi}"] = float(np.linalg.norm(got - want) / np.linalg.norm(want))
    got4 = mg.Heff2(v, eL, eR, W1, W2, precision=4)(v).to_flat()
    errs[f"heff_s4_{chi}"] = float(np.linalg.norm(got4 - want) / np.linalg.norm(want))
    for perm in ((2, 1, 4, 3), (4, 3, 2, 1), (1, 3, 2, 4)):
        p = mg.permutelegs(v, perm).to_flat()
        q = st.flatten(st.permutelegs(O[0], perm))
        errs[f"perm_{chi}_{perm}"] = float(np.max(np.abs(p - q)))
    f = mg.fuselegs(v, 2, 2, False)
    back = mg.splitleg(f, 2, v.space[1:3]).to_flat()
    errs[f"fuse_split_{chi}"] = float(np.max(np.abs(back - flats[0])))
from helpers import to_device
lx, chi = 12, 16
sites = gd.random_mps_host(lx, lx // 2, chi, seed=3)
mo = om.MPState([st.from_flat(c, conv(sp), f) for c, sp, f in sites], 0)
om.center_at(mo, 1)
md = gd.MPState([to_device(A) for A in mo.As], center=1)
Wo, Wd = om.xxz_u1mpo(lx, 1.0), gd.xxz_u1mpo(lx, 1.0)
eo, ed = om.initialenv(mo, Wo), gd.initialenv(md, Wd)
kw = dict(maxdim=chi, tol=1e-10, lanczostol=1e-7, krylovdim=4, krylovmaxiter=8, tieband=1e-12)
e_o = om.dmrg2sitesweep(mo, Wo, eo, **kw)
e_d = gd.dmrg2sitesweep(md, Wd, ed, **kw)
errs["sweep"] = float(np.max(np.abs(np.array(e_d) - np.array(e_o)) / np.abs(np.array(e_o))))
n, first = mg.device_checks()
print(json.dumps({"violations": n, "first": first, "errs": errs}))
"""


def test_checked_library_records_no_violation():
    env = dict(os.environ)
    r = subprocess.run([sys.executable, "-m", "mps_gb300.build", "--checked"], cwd=ROOT,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    env["MPSG_LIBRARY"] = "checked"
    code = WORKLOAD.replace("ROOT", repr(ROOT))
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["violations"] == 0, out["first"]
    e = out["errs"]
    for k, x in e.items():
        if k.startswith("heff_fp64") or k == "sweep":
            assert x <= 1e-10, (k, x)
        elif k.startswith("heff_s4"):
            assert x <= 1e-7, (k, x)
        else:
            assert x == 0.0, (k, x)
