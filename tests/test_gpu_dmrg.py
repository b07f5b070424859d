"""GPU parity of the factorisation, Krylov and sweep layers against the oracle (FP64 path).

* per-sector SVD and svdtrunc (src/symtools.jl:1-35, src/mpsutils.jl:116-179);
* the Lanczos eigensolver at the KrylovKit boundary (src/dmrg.jl:77-82) — same restart logic in
  oracle and library, so eigenvalues and operation counts must agree;
* full 2-site DMRG sweeps (src/dmrg.jl:58-179): the L=32 Heisenberg chain, chi <= 64, cutoff
  1e-10, Krylov dimension 4, four sweeps, every post-truncation energy within 1e-10 relative.
"""
import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from oracle import symtensors as st
from oracle import mps as om
from oracle.symtensors import U1Space, dual_space as dual

from helpers import to_device, to_oracle, rand_tensor, assert_tensor_close, relerr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("charge", [0, 1, -1])
def test_svd_reconstruction_and_values(charge):
    rng = np.random.default_rng(40 + charge)
    V1 = U1Space((0, 20), (1, 33), (2, 41))
    V2 = U1Space((0, 44), (-1, 25), (-2, 12), (-3, 30))
    A = rand_tensor(charge, (V1, V2), rng)
    u, s, v = mg._svd_(to_device(A))
    assert s.isdiagonal()
    R = mg.matmul(mg.matmul(u, s), v)
    assert_tensor_close(R, A, rtol=1e-12)
    u0, s0, v0 = st.svd_(A)
    for sec, blk in s0.blocks.items():
        got = np.diag(s.blocks[sec])
        np.testing.assert_allclose(got, blk, rtol=1e-12, atol=1e-13 * blk[0])
    # u is a left isometry in every sector
    for sec, blk in u.blocks.items():
        np.testing.assert_allclose(blk.T @ blk, np.eye(blk.shape[1]), atol=1e-12)


def test_svdtrunc_matches_oracle():
    rng = np.random.default_rng(77)
    V1 = U1Space((0, 30), (1, 50), (2, 40))
    V2 = dual(U1Space((0, 35), (1, 45), (2, 20)))
    A = rand_tensor(0, (V1, V2), rng)
    for maxdim, tol in [(40, 1e-12), (200, 5.0), (7, 1e-12)]:
        u0, s0, v0 = st.svdtrunc(A, maxdim=maxdim, tol=tol, tieband=1e-12)
        u, s, v = mg.svdtrunc(to_device(A), maxdim=maxdim, tol=tol, tieband=1e-12)
        assert s.space == tuple(mg.VectorSpace(V.sectors, V.isdual) for V in s0.space)
        assert u.space[1] == mg.VectorSpace(u0.space[1].sectors, u0.space[1].isdual)
        P0 = st.matmul(st.matmul(u0, s0), v0)
        assert_tensor_close(mg.matmul(mg.matmul(u, s), v), P0, rtol=1e-11)
        assert abs(mg.norm(s) - st.norm(s0)) < 1e-12 * st.norm(s0)


def test_svdtrunc_all_below_tol_raises_like_reference():
    rng = np.random.default_rng(1)
    A = rand_tensor(0, (U1Space((0, 3)), dual(U1Space((0, 3)))), rng)
    with pytest.raises(mg.MPSGError) as e:
        mg.svdtrunc(to_device(A), maxdim=4, tol=1e6)
    assert e.value.code == 6


def oracle_mps(sites):
    conv = lambda sp: tuple(st.VectorSpace(V.sectors, V.isdual) for V in sp)
    return om.MPState([st.from_flat(c, conv(sp), f) for c, sp, f in sites], 0)


def test_center_at_matches_oracle():
    sites = gd.random_mps_host(10, 5, 12, seed=5)
    mo = oracle_mps(sites)
    md = gd.mps_from_host(sites)
    om.center_at(mo, 1)
    gd.center_at(md, 1)
    # gauge-invariant check: the normalised two-site wavefunction at the left edge
    for k in range(len(mo)):
        assert md.As[k].space == tuple(mg.VectorSpace(V.sectors, V.isdual) for V in mo.As[k].space)
    for k in range(1, len(mo)):  # right-canonical sites: A A^dagger = 1 on the left bond
        Ad = md.As[k]
        G = mg.contract(Ad, (1, -1, -2), mg.dual(Ad), (2, -1, -2))
        Gd = st.array(to_oracle(G))
        np.testing.assert_allclose(Gd, np.eye(Gd.shape[0]), atol=1e-12)
    e0 = st.contract(mo.As[0], (1, 2, -1), mo.As[1], (-1, 3, 4))
    e1 = mg.contract(md.As[0], (1, 2, -1), md.As[1], (-1, 3, 4))
    assert abs(st.norm(e0) - mg.norm(e1)) < 1e-12 * st.norm(e0)


def heisenberg_setup(lx, chi, seed=1911):
    """Oracle MPS canonicalised on the CPU; the device MPS is uploaded from the same tensors so
    that gauge-dependent objects (environments, eigenvectors) compare elementwise."""
    sites = gd.random_mps_host(lx, lx // 2, chi, seed=seed)
    mo = oracle_mps(sites)
    om.center_at(mo, 1)
    md = gd.MPState([to_device(A) for A in mo.As], center=1)
    Wo, Wd = om.xxz_u1mpo(lx, 1.0), gd.xxz_u1mpo(lx, 1.0)
    return mo, md, Wo, Wd, om.initialenv(mo, Wo), gd.initialenv(md, Wd)


def test_initialenv_matches_oracle():
    mo, md, Wo, Wd, eo, ed = heisenberg_setup(10, 16)
    for k in range(1, len(eo)):
        assert_tensor_close(ed[k], eo[k], rtol=1e-12)


def test_eigsolve_matches_oracle():
    mo, md, Wo, Wd, eo, ed = heisenberg_setup(12, 16)
    l = 1
    AAo = st.contract(mo.As[0], (1, 2, -1), mo.As[1], (-1, 3, 4))
    AAd = mg.contract(md.As[0], (1, 2, -1), md.As[1], (-1, 3, 4))
    fo = lambda x: om.applymps2site(x, eo[l - 1], eo[l + 2], Wo[l - 1], Wo[l])
    for kd, mi in [(4, 8), (6, 3)]:
        E0, x0, info0 = om.eigsolve_lanczos(fo, AAo, krylovdim=kd, maxiter=mi, tol=1e-9)
        E1, x1, info1 = mg.eigsolve_heff2(AAd, ed[l - 1], ed[l + 2], Wd[l - 1], Wd[l],
                                          krylovdim=kd, maxiter=mi, tol=1e-9)
        assert abs(E0 - E1) <= 1e-10 * abs(E0)
        assert (info1.numops, info1.numiter) == (info0.numops, info0.numiter)
        ov = abs(st.dot(x0, to_oracle(x1)))
        assert abs(ov - 1.0) < 1e-8


def run_sweeps(lx, chi, nsweeps, tieband=1e-12):
    mo, md, Wo, Wd, eo, ed = heisenberg_setup(lx, chi)
    kw = dict(maxdim=chi, tol=1e-10, lanczostol=1e-7, krylovdim=4, krylovmaxiter=8,
              tieband=tieband)
    out = []
    for _ in range(nsweeps):
        so, sd = [], []
        e_o = om.dmrg2sitesweep(mo, Wo, eo, stats=so, **kw)
        e_d = gd.dmrg2sitesweep(md, Wd, ed, stats=sd, **kw)
        out.append((e_o, e_d, so, sd))
    return out, md


def test_dmrg_sweep_small_chain():
    out, _ = run_sweeps(12, 16, 2)
    for e_o, e_d, so, sd in out:
        assert len(e_d) == 3 * 12 - 5
        np.testing.assert_allclose(e_d, e_o, rtol=1e-10, atol=0)


def test_mixed_sweep_energies_within_1e10_of_fp64():
    """The mixed sweep configuration (5-slice Krylov matvecs, 7-slice energy and environment
    contractions, density-matrix truncation with its second-level decomposition) against the
    FP64 drop-in sweep (FP64 everywhere, exact per-sector SVD) from the same canonical MPS:
    every post-truncation energy of both sweeps within 1e-10 relative, including the first
    sweep from the random state, where Lanczos solves stop at maxiter before converging. Bond
    dimensions agree to a few states: where the absolute cutoff (1e-10) decides, values at the
    cutoff may round either way."""
    lx, chi = 20, 96
    _, md, _, Wd, _, ed = heisenberg_setup(lx, chi, seed=11)
    # SU(2) multiplets give exactly equal singular values in different charge sectors; the tie
    # band makes the sector that keeps a state cut by maxdim independent of rounding noise
    kw = dict(maxdim=chi, tol=1e-10, lanczostol=1e-8, krylovdim=4, krylovmaxiter=8,
              tieband=1e-9)
    cfgs = {"fp64": dict(precision=0, energy_precision=0, env_precision=0, svd="exact"),
            "mixed": dict(precision=5, energy_precision=7, env_precision=7, svd="gram")}
    res = {}
    for name, cfg in cfgs.items():
        mps = gd.MPState([mg.copy(A) for A in md.As], center=1)
        env = [None if e is None else mg.copy(e) for e in ed]
        es = [gd.dmrg2sitesweep(mps, Wd, env, **kw, **cfg) for _ in range(2)]
        res[name] = (es, [A.space for A in mps.As])
    (first_mx, last_mx), (first_64, last_64) = res["mixed"][0], res["fp64"][0]
    np.testing.assert_allclose(first_mx, first_64, rtol=1e-10, atol=0)
    np.testing.assert_allclose(last_mx, last_64, rtol=1e-10, atol=0)
    for sp_mx, sp_64 in zip(res["mixed"][1], res["fp64"][1]):  # dims within a few states
        assert abs(sp_mx[2].dim() - sp_64[2].dim()) <= 8


def test_dmrg_heisenberg_L32_chi64_four_sweeps():
    """The chi<=64 Heisenberg-chain workload: every post-truncation energy of every sweep within
    1e-10 relative of the oracle, final energy below the L=32 OBC ground energy bound."""
    out, md = run_sweeps(32, 64, 4)
    for e_o, e_d, so, sd in out:
        np.testing.assert_allclose(e_d, e_o, rtol=1e-10, atol=0)
    assert out[-1][1][-1] < -13.99
    # bond dimensions stay bounded by maxdim
    for A in md.As:
        assert A.space[0].dim() <= 64 and A.space[2].dim() <= 64


def test_context_outlives_tensors_in_any_release_order():
    ctx = mg.Context(0)
    t = mg.fill(2.0, 0, (mg.U1Space((0, 3)), mg.dual(mg.U1Space((0, 3)))), ctx)
    ctx.close()  # the tensor keeps the device context alive
    assert np.array_equal(t.to_flat(), np.full(9, 2.0))
    del t


def test_independent_chains_concurrently_equal_one_by_one():
    """Chains driven concurrently (one context and stream each) give exactly the energies of the
    same chains run one after the other: the kernels are deterministic and the contexts share
    nothing but the device."""
    specs = [(12, 0.3, 24), (16, 1.0, 32), (14, 1.4, 16)]
    o = gd.SweepOptions(tol=1e-10, lanczostol=1e-8, krylovdim=4, krylovmaxiter=8, precision=4,
                        energy_precision=7, env_precision=7, svd="gram")
    one = gd.run_chains(specs, 2, o, threads=1)
    many = gd.run_chains(specs, 2, o, threads=len(specs))
    assert one == many
    assert all(e < 0 for e in one)


@pytest.mark.parametrize("mode", ["async", "blocking"])
def test_sweep_with_offloaded_environments_is_bit_identical(mode):
    """A sweep whose environments live in a 3-entry device window (the rest in host memory,
    moved by asynchronous copies with prefetch, or by blocking ones) gives exactly the energies
    of the all-resident sweep."""
    from mps_gb300.envstore import OffloadedEnvs
    lx, chi = 16, 32
    _, md, _, Wd, _, ed = heisenberg_setup(lx, chi, seed=3)
    res = []
    for window in (None, 3):
        mps = gd.MPState([mg.copy(A) for A in md.As], center=1)
        env = [None if e is None else mg.copy(e) for e in ed]
        if window:
            load = (lambda c, s, f: mg.from_flat(c, s, f)) if mode == "blocking" else None
            env = OffloadedEnvs(env, window=window, load=load)
        es = gd.dmrg2sitesweep(mps, Wd, env, maxdim=chi, tol=1e-10, krylovdim=4,
                               krylovmaxiter=8)
        res.append(es)
        if window:
            assert env.downloads > 0 and env.uploads > 0
            assert env.prefetches > 0 and env.clean_evictions > 0
            if mode == "async":  # blocking prefetches finish at once: nothing is pending
                assert env.prefetch_hits > 0
    assert res[0] == res[1]
