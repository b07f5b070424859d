"""Lattice MPOs (the role of src/mpogen.jl:153-352): the finite-state-machine U(1) MPO, contracted
to a dense matrix on the host, equals the Hamiltonian assembled directly from its terms by
Kronecker products; bond dimensions count the open terms."""
import numpy as np
import pytest

from mps_gb300 import lattice as lt


def dense_from_terms(n, terms):
    """Sum over terms of kron(op at each site, identity elsewhere); site 0 most significant,
    basis (down, up)."""
    H = np.zeros((2 ** n, 2 ** n))
    for sites, ops, amp in terms:
        mats = [np.eye(2)] * n
        mats = list(mats)
        for s, o in zip(sites, ops):
            mats[s] = lt.OPS[o][0]
        M = mats[0]
        for m in mats[1:]:
            M = np.kron(M, m)
        H += amp * M
    return H


def test_chain_mpo_equals_dense_xxz():
    n = 6
    terms = lt.chain_xxz_terms(n, 0.7)
    H = lt.dense_mpo(lt.mpo_blocks(n, terms))
    np.testing.assert_allclose(H, dense_from_terms(n, terms), atol=1e-14)
    # the XXZ chain needs 2 + 3 channels on every inner bond (the reference's w = 5)
    for (Vl, _, Vr, _), _ in lt.mpo_blocks(n, terms)[1:-1]:
        assert sum(Vl[1]) == 5


@pytest.mark.parametrize("width,length", [(3, 2), (4, 2), (2, 3)])
def test_cylinder_mpo_equals_dense(width, length):
    n = width * length
    terms = lt.cylinder_heisenberg_terms(width, length)
    H = lt.dense_mpo(lt.mpo_blocks(n, terms))
    np.testing.assert_allclose(H, dense_from_terms(n, terms), atol=1e-13)
    # Heisenberg: H commutes with the total Sz (U(1)) and is symmetric
    np.testing.assert_allclose(H, H.T, atol=1e-14)


def test_cylinder_bond_dimension():
    """6 x 24 cylinder: a cut at a column boundary crosses the 6 bonds along the length
    (3 terms each, w = 2 + 18 = 20); a cut inside a column also crosses one bond around the
    circumference and the wrap bond (w = 26)."""
    width, length = 6, 24
    terms = lt.cylinder_heisenberg_terms(width, length)
    tens = lt.mpo_blocks(width * length, terms)
    dims = [sum(Vr[1]) for (_, _, Vr, _), _ in tens]
    assert dims[width - 1] == 20 and dims[2 * width - 1] == 20
    assert max(dims) == 2 + 3 * (width + 2)
    assert dims[-1] == 1


def test_bad_terms_rejected():
    with pytest.raises(ValueError):
        lt.mpo_blocks(4, [((2, 1), ("P", "M"), 1.0)])
    with pytest.raises(ValueError):
        lt.mpo_blocks(3, [((1, 3), ("Z", "Z"), 1.0)])
