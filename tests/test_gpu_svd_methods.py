"""Per-sector factorisations on the GPU: the exact thin SVD (QR iteration, sectors factorised
concurrently) and the density-matrix truncation (eigen-decomposition of the Gram matrix of each
sector block), against the oracle's SVD (src/symtools.jl:1-35, src/mpsutils.jl:116-179).
"""
import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from oracle import symtensors as st
from oracle.symtensors import U1Space, dual_space as dual

from helpers import to_device, to_oracle, assert_tensor_close, relerr

pytestmark = pytest.mark.gpu


def spectrum_tensor(V1, V2, rng, lo=-6.0):
    """Rank-2 tensor whose blocks have singular values 10^linspace(0, lo) times a block scale,
    random singular vectors (so the spectrum, and a clear truncation gap, are known)."""
    sects, sizes = st.allsectorsandsizes(0, (V1, V2))
    blocks = {}
    for k, (s, (m, n)) in enumerate(zip(sects, sizes)):
        r = min(m, n)
        U, _ = np.linalg.qr(rng.standard_normal((m, r)))
        W, _ = np.linalg.qr(rng.standard_normal((n, r)))
        sv = 10.0 ** np.linspace(0.0, lo, r) * (0.5 + 0.5 / (k + 1))
        blocks[s] = (U * sv) @ W.T
    return st.SymTensor(0, (V1, V2), blocks)


SHAPES = [  # tall, wide and square sectors, more sectors than solver lanes
    (U1Space((0, 120), (1, 40), (2, 200), (3, 7), (4, 90), (5, 64)),
     dual(U1Space((0, 60), (1, 110), (2, 150), (3, 9), (4, 90), (5, 1)))),
    (U1Space((-1, 33), (0, 257), (1, 5)), dual(U1Space((-1, 300), (0, 12), (1, 5)))),
]


@pytest.mark.parametrize("shape", range(len(SHAPES)))
def test_exact_svd_concurrent_sectors(shape):
    rng = np.random.default_rng(10 + shape)
    A = spectrum_tensor(*SHAPES[shape], rng, lo=-3.0)
    Ad = to_device(A)
    u0, s0, v0 = st.svd_(A)
    u, s, v = mg._svd_(Ad)
    assert_tensor_close(mg.matmul(mg.matmul(u, s), v), A, rtol=1e-12)
    sd = to_oracle(s)
    for key in s0.blocks:
        np.testing.assert_allclose(np.diag(sd.blocks[key]), s0.blocks[key].diagonal()
                                   if s0.blocks[key].ndim == 2 else s0.blocks[key],
                                   rtol=1e-12, atol=1e-14)
    for maxdim, tol in [(300, 1e-12), (57, 1e-12), (1000, 1e-2)]:
        u0, s0, v0 = st.svdtrunc(A, maxdim=maxdim, tol=tol, tieband=1e-12)
        u, s, v = mg.svdtrunc(Ad, maxdim=maxdim, tol=tol, tieband=1e-12)
        assert s.space == tuple(mg.VectorSpace(V.sectors, V.isdual) for V in s0.space)
        P0 = st.matmul(st.matmul(u0, s0), v0)
        assert_tensor_close(mg.matmul(mg.matmul(u, s), v), P0, rtol=1e-11)


def gram_checks(A, Ad, method, maxdim, tol):
    u0, s0, v0 = st.svdtrunc(A, maxdim=maxdim, tol=tol, tieband=1e-12)
    u, s, v = mg.svdtrunc(Ad, maxdim=maxdim, tol=tol, tieband=1e-12, method=method)
    # same kept sectors and bond dimensions as the exact truncation
    assert s.space == tuple(mg.VectorSpace(V.sectors, V.isdual) for V in s0.space)
    # singular values: absolute error about eps * max(S)^2 / S
    smax = max(float(np.max(np.abs(b))) for b in s0.blocks.values())
    sd = to_oracle(s)
    for key, b in s0.blocks.items():
        want = np.diag(b) if b.ndim == 2 else b
        got = np.diag(sd.blocks[key])
        assert np.all(np.abs(got - want) <= 1e-13 * smax * smax / want + 1e-15), key
    # the orthonormal factor is orthonormal to rounding
    if method == "gram_left":
        G = mg.contract(mg.dual(u), (-1, 1), u, (-1, 2))
    else:
        G = mg.contract(v, (1, -1), mg.dual(v), (2, -1))
    Gd = st.array(to_oracle(G))
    np.testing.assert_allclose(Gd, np.eye(Gd.shape[0]), atol=1e-13)
    # u s v is the projection on the kept subspace: equal to the exact truncation up to the
    # subspace error of the Gram eigenvectors, about eps * max(S) / min(kept S)
    smin = min(float(np.min(b)) for b in s0.blocks.values())
    P0 = st.matmul(st.matmul(u0, s0), v0)
    P = mg.matmul(mg.matmul(u, s), v)
    assert relerr(P.to_flat(), st.flatten(P0)) <= max(1e-12, 5e-15 * smax / smin)


@pytest.mark.parametrize("method", ["gram_left", "gram_right"])
@pytest.mark.parametrize("shape", range(len(SHAPES)))
def test_gram_truncation_matches_exact(method, shape):
    rng = np.random.default_rng(20 + shape)
    A = spectrum_tensor(*SHAPES[shape], rng, lo=-6.0)
    Ad = to_device(A)
    for maxdim, tol in [(120, 1e-10), (400, 1e-4), (25, 1e-10)]:
        gram_checks(A, Ad, method, maxdim, tol)


def test_gram_truncation_all_below_tol_raises_like_reference():
    rng = np.random.default_rng(2)
    A = spectrum_tensor(U1Space((0, 5)), dual(U1Space((0, 4))), rng)
    with pytest.raises(mg.MPSGError) as e:
        mg.svdtrunc(to_device(A), maxdim=4, tol=1e6, method="gram_left")
    assert e.value.code == 6


def test_sweep_with_gram_truncation_matches_exact_sweep():
    """Two sweeps of the L=16 Heisenberg chain (chi <= 32) with the density-matrix truncation
    against the exact-SVD sweep on the device, from the same canonical MPS. Here maxdim decides
    every truncation (cut values far above the Gram resolution of ~1e-8 * max S), so the bond
    spaces agree exactly; the tie band keeps SU(2) multiplets cut by maxdim out of the noise."""
    lx, chi = 16, 32
    Ws = gd.xxz_u1mpo(lx, 1.0)
    host = gd.random_mps_host(lx, lx // 2, chi, seed=3)
    runs = {}
    for svd in ("exact", "gram"):
        mps = gd.mps_from_host(host)
        gd.center_at(mps, 1)
        env = gd.initialenv(mps, Ws)
        es = []
        for _ in range(2):
            es.append(gd.dmrg2sitesweep(mps, Ws, env, maxdim=chi, tol=1e-10, lanczostol=1e-9,
                                        krylovdim=4, krylovmaxiter=8, svd=svd, tieband=1e-9))
        runs[svd] = (es, [A.space for A in mps.As])
    np.testing.assert_allclose(runs["gram"][0][-1], runs["exact"][0][-1], rtol=1e-9, atol=0)
    assert runs["gram"][1] == runs["exact"][1]
