"""2-site DMRG on a Heisenberg cylinder with the generated lattice MPO (the config of a width-W
cylinder with w = 2 + 3(W + 2) channels), against exact diagonalisation of the same terms."""
import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from mps_gb300 import lattice as lt

from test_lattice_cpu import dense_from_terms

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg", [dict(precision=0, energy_precision=0, env_precision=0, svd="exact"),
                                 dict(precision=4, energy_precision=7, env_precision=7, svd="gram")])
def test_cylinder_dmrg_matches_exact_diagonalisation(cfg):
    width, length = 3, 4
    n = width * length
    terms = lt.cylinder_heisenberg_terms(width, length)
    Ws = lt.device_mpo(n, terms)
    mps = gd.mps_from_host(gd.random_mps_host(n, n // 2, 64, seed=2))
    gd.center_at(mps, 1)
    env = gd.initialenv(mps, Ws)
    for _ in range(4):
        es = gd.dmrg2sitesweep(mps, Ws, env, maxdim=64, tol=1e-12, lanczostol=1e-10,
                               krylovdim=6, krylovmaxiter=30, tieband=1e-9, **cfg)
    H = dense_from_terms(n, terms)
    pop = np.array([bin(k).count("1") for k in range(2 ** n)])
    idx = np.where(pop == n // 2)[0]
    e0 = np.linalg.eigvalsh(H[np.ix_(idx, idx)])[0]
    assert abs(es[-1] - e0) < 1e-9 * abs(e0)


def test_triangular_ladder_with_ring_exchange_dmrg_matches_exact_diagonalisation():
    """The (2, 5) triangular ladder with four-spin ring exchange (MPO bond dimension up to 86,
    33 product terms per plaquette): DMRG at full bond dimension = ED."""
    ly, lx = 2, 5
    n = ly * lx
    terms = lt.triangular_terms(ly, lx, 0.3, 1.0, 1.0, 0.4, 0.7, 0.0)
    Ws = lt.device_mpo(n, terms)
    assert max(W.space[0].dim() for W in Ws) == 86
    mps = gd.mps_from_host(gd.random_mps_host(n, n // 2, 32, seed=5))
    gd.center_at(mps, 1)
    env = gd.initialenv(mps, Ws)
    for _ in range(4):
        es = gd.dmrg2sitesweep(mps, Ws, env, maxdim=32, tol=1e-12, lanczostol=1e-10,
                               krylovdim=6, krylovmaxiter=30, tieband=1e-9)
    H = lt.dense_mpo(lt.mpo_blocks(n, terms))
    pop = np.array([bin(k).count("1") for k in range(2 ** n)])
    idx = np.where(pop == n // 2)[0]
    e0 = np.linalg.eigvalsh(H[np.ix_(idx, idx)])[0]
    assert abs(es[-1] - e0) < 1e-9 * abs(e0)
