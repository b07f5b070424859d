"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

Writes `heff_chi16.npz` (an H_eff application at chi=16 over 5 charges: inputs and output) and
`sweep_L10.npz` (one 2-site DMRG sweep of the L=10 Heisenberg chain, chi<=16: initial MPS and the
3L-5 energies).  Inputs are drawn from seeded Philox streams; the outputs are the oracle's.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mps_gb300 import dmrg as gd  # noqa: E402  (host-side input generators only)
from oracle import mps as om  # noqa: E402
from oracle import symtensors as st  # noqa: E402


def conv(sp):
    return tuple(st.VectorSpace(V.sectors, V.isdual) for V in sp)


def heff_fixture():
    chi, nq, delta = 16, 5, 0.5
    (sv, sl, sr), flats = gd.heff_inputs_host(chi, delta, 1911, nq)
    O = [st.from_flat(0, conv(s), f) for s, f in zip((sv, sl, sr), flats)]
    W = om.xxz_u1mpo(3, delta)[1]
    out = st.flatten(om.applymps2site(O[0], O[1], O[2], W, W))
    np.savez_compressed(os.path.join(HERE, "heff_chi16.npz"), chi=chi, nq=nq, delta=delta,
                        v=flats[0], envL=flats[1], envR=flats[2], out=out)


def sweep_fixture():
    lx, chi = 10, 16
    sites = gd.random_mps_host(lx, lx // 2, chi, seed=7)
    mps = om.MPState([st.from_flat(c, conv(sp), f) for c, sp, f in sites], 0)
    om.center_at(mps, 1)
    Ws = om.xxz_u1mpo(lx, 1.0)
    env = om.initialenv(mps, Ws)
    es = om.dmrg2sitesweep(mps, Ws, env, maxdim=chi, tol=1e-10, lanczostol=1e-7, krylovdim=4,
                           krylovmaxiter=8, tieband=1e-12)
    np.savez_compressed(os.path.join(HERE, "sweep_L10.npz"), lx=lx, chi=chi, seed=7,
                        energies=np.array(es))


if __name__ == "__main__":
    heff_fixture()
    sweep_fixture()
    print("golden fixtures written to", HERE)
