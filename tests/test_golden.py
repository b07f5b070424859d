"""Golden fixtures (tests/golden/, written by tests/golden/make_golden.py from the oracle).

CPU: the oracle still reproduces the committed vectors bit for bit.  GPU: the library's FP64
path reproduces them within 1e-12 (H_eff) and 1e-10 (the energies of a DMRG sweep) without
running the oracle.
"""
import os

import numpy as np
import pytest

from mps_gb300 import dmrg as gd
from oracle import mps as om
from oracle import symtensors as st

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def conv(sp):
    return tuple(st.VectorSpace(V.sectors, V.isdual) for V in sp)


def test_oracle_reproduces_heff_fixture():
    g = np.load(os.path.join(GOLD, "heff_chi16.npz"))
    (sv, sl, sr), flats = gd.heff_inputs_host(int(g["chi"]), float(g["delta"]), 1911, int(g["nq"]))
    for f, name in zip(flats, ("v", "envL", "envR")):
        assert np.array_equal(f, g[name])
    O = [st.from_flat(0, conv(s), f) for s, f in zip((sv, sl, sr), flats)]
    W = om.xxz_u1mpo(3, float(g["delta"]))[1]
    assert np.array_equal(st.flatten(om.applymps2site(O[0], O[1], O[2], W, W)), g["out"])


def test_oracle_reproduces_sweep_fixture():
    g = np.load(os.path.join(GOLD, "sweep_L10.npz"))
    lx, chi = int(g["lx"]), int(g["chi"])
    sites = gd.random_mps_host(lx, lx // 2, chi, seed=int(g["seed"]))
    mps = om.MPState([st.from_flat(c, conv(sp), f) for c, sp, f in sites], 0)
    om.center_at(mps, 1)
    Ws = om.xxz_u1mpo(lx, 1.0)
    env = om.initialenv(mps, Ws)
    es = om.dmrg2sitesweep(mps, Ws, env, maxdim=chi, tol=1e-10, lanczostol=1e-7, krylovdim=4,
                           krylovmaxiter=8, tieband=1e-12)
    # (LAPACK eigen-solvers inside: the last bits may depend on the BLAS thread count)
    np.testing.assert_allclose(np.array(es), g["energies"], rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_library_matches_heff_fixture():
    import mps_gb300 as mg
    g = np.load(os.path.join(GOLD, "heff_chi16.npz"))
    D = gd.heff_problem(int(g["chi"]), float(g["delta"]), 1911, ncharges=int(g["nq"]))
    got = mg.applymps2site(*D, precision=0).to_flat()
    assert np.linalg.norm(got - g["out"]) <= 1e-12 * np.linalg.norm(g["out"])


@pytest.mark.gpu
def test_library_matches_sweep_fixture():
    g = np.load(os.path.join(GOLD, "sweep_L10.npz"))
    lx, chi = int(g["lx"]), int(g["chi"])
    sites = gd.random_mps_host(lx, lx // 2, chi, seed=int(g["seed"]))
    mps = gd.mps_from_host(sites)
    gd.center_at(mps, 1)
    Ws = gd.xxz_u1mpo(lx, 1.0)
    env = gd.initialenv(mps, Ws)
    es = gd.dmrg2sitesweep(mps, Ws, env, maxdim=chi, tol=1e-10, lanczostol=1e-7, krylovdim=4,
                           krylovmaxiter=8, tieband=1e-12)
    np.testing.assert_allclose(es, g["energies"], rtol=1e-10, atol=0)
