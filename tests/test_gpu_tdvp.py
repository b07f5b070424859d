"""Symmetric complex TDVP on the GPU: the per-sector complex SVD against the oracle, the sweeps
against the dense TDVP oracle (src/tdvp.jl restated), conservation laws on a truncated chain."""
import numpy as np
import pytest

import mps_gb300 as mg
from helpers import dense_site, oracle_ops, rand_tensor, to_device, to_oracle
from mps_gb300 import ctensor as ct
from mps_gb300 import dmrg as gd
from mps_gb300 import tdvp as td
from oracle import mps as om
from oracle import symtensors as st
from oracle import tdvp as ot
from oracle.symtensors import U1Space, dual_space

pytestmark = pytest.mark.gpu

DELTA, DT = 0.5, 0.05


def random_state(lx, m, chimax, seed):
    rng = np.random.default_rng(seed)
    d = U1Space((0, 1), (1, 1))
    Vl = U1Space((0, 1))
    As = []
    for site in range(1, lx + 1):
        Vr = U1Space(*om.binomial_bond_dims(lx, site, m, chimax))
        As.append(rand_tensor(0, (Vl, d, dual_space(Vr)), rng))
        Vl = Vr
    mps = om.center_at(om.MPState(As, 0), 1)
    mps.As[0] = st.scaled(mps.As[0], 1.0 / st.norm(mps.As[0]))
    return mps


@pytest.mark.parametrize("truncate", [False, True])
def test_svd_complex_matches_oracle(truncate):
    rng = np.random.default_rng(11)
    Vr = U1Space((0, 7), (1, 20), (2, 5), (3, 1))
    Vc = U1Space((0, 12), (1, 9), (2, 5), (3, 3), isdual=True)
    re = rand_tensor(0, (Vr, Vc), rng)
    im = rand_tensor(0, (Vr, Vc), rng)
    ure, uim, s, vre, vim = mg.svd_complex(to_device(re), to_device(im), maxdim=20, tol=1e-3,
                                           truncate=truncate)
    M = st.SymTensor(0, (Vr, Vc), {k: re.blocks[k] + 1j * im.blocks[k] for k in re.blocks},
                     check=False)
    if truncate:
        u0, s0, v0 = st.svdtrunc(M, maxdim=20, tol=1e-3)
    else:
        u0, s0, v0 = st.svd_(M)
    assert s.space == tuple(mg.VectorSpace(V.sectors, V.isdual) for V in s0.space)
    so = to_oracle(s)
    for k, b in s0.blocks.items():
        np.testing.assert_allclose(np.diag(so.blocks[k]), b, rtol=1e-12, atol=1e-12)
    u = {k: to_oracle(ure).blocks[k] + 1j * to_oracle(uim).blocks[k]
         for k in to_oracle(ure).blocks}
    v = {k: to_oracle(vre).blocks[k] + 1j * to_oracle(vim).blocks[k]
         for k in to_oracle(vre).blocks}
    for (c1, c2), b in s0.blocks.items():
        U, V = u[(c1, c1)], v[(c2, c2)]
        np.testing.assert_allclose(U.conj().T @ U, np.eye(len(b)), atol=1e-12)
        np.testing.assert_allclose(V @ V.conj().T, np.eye(len(b)), atol=1e-12)
        # the kept part of the product equals the oracle's (singular vectors are unique up to a
        # phase per vector, the product is not)
        ref = u0.blocks[(c1, c1)] @ np.diag(b) @ v0.blocks[(c2, c2)]
        np.testing.assert_allclose(U @ np.diag(b) @ V, ref, atol=1e-11)


@pytest.mark.parametrize("kind,turning", [("1site", "symmetric"), ("1site", "reference"),
                                          ("2site", "symmetric"), ("2site", "reference")])
def test_gpu_tdvp_matches_dense_oracle(kind, turning):
    lx, m = 8, 4
    mps = random_state(lx, m, 1 << 20, seed=5)
    As_d = [st.array(A).astype(complex) for A in mps.As]
    Ws_d = [st.array(W).astype(complex) for W in om.xxz_u1mpo(lx, DELTA)]
    env_d = ot.initialenv(As_d, Ws_d)
    ops = ct.gpu_ops()
    Ws = gd.xxz_u1mpo(lx, DELTA)
    As = [ct.CTensor(to_device(A)) for A in mps.As]
    env = td.initialenv(ops, As, Ws)
    for _ in range(2):
        if kind == "1site":
            ot.tdvp1sitesweep(DT, As_d, Ws_d, env_d, turning=turning)
            td.tdvp1sitesweep(ops, DT, As, Ws, env, turning=turning)
        else:
            ot.tdvp2sitesweep(DT, As_d, Ws_d, env_d, maxdim=64, tol=1e-14, turning=turning)
            td.tdvp2sitesweep(ops, DT, As, Ws, env, maxdim=64, tol=1e-14, turning=turning)
    psi_d = ot.state_vector(As_d)
    psi = ot.state_vector([dense_site(ops, A) for A in As])
    assert np.linalg.norm(psi - psi_d) < 1e-10
    if turning == "symmetric":  # full bond dimension: the exact evolution by 4 dt
        H = om.xxz_hamiltonian(lx, DELTA)
        w, Q = np.linalg.eigh(H)
        psi0 = ot.state_vector([st.array(A).astype(complex) for A in mps.As])
        ex = Q @ (np.exp(-4j * DT * w) * (Q.conj().T @ psi0))
        assert np.linalg.norm(psi - ex) < 1e-10


def _energy(ops, As, Ws, env):
    """<psi|H|psi> / <psi|psi> of a center-1 MPS from its environments (the 1-site H_eff)."""
    A = As[0]
    hv = td.apply1(ops, A, env[0], env[2], Ws[0])
    return (ct.cdot(ops, A, hv) / ct.cdot(ops, A, A)).real


def test_gpu_tdvp_conservation_and_backend_agreement_on_a_truncated_chain():
    """1-site TDVP on a truncated bond dimension stays on the manifold: it conserves the norm
    and the energy (to the Krylov tolerance). The GPU run and the same host code on the oracle's
    operations agree to rounding."""
    lx, m, chi = 14, 7, 12
    mps = random_state(lx, m, chi, seed=9)
    ops_g, ops_o = ct.gpu_ops(), oracle_ops()
    Ws_g, Ws_o = gd.xxz_u1mpo(lx, DELTA), om.xxz_u1mpo(lx, DELTA)
    As_g = [ct.CTensor(to_device(A)) for A in mps.As]
    As_o = [ct.CTensor(A) for A in mps.As]
    env_g = td.initialenv(ops_g, As_g, Ws_g)
    env_o = td.initialenv(ops_o, As_o, Ws_o)
    e0 = _energy(ops_g, As_g, Ws_g, env_g)
    for _ in range(3):
        td.tdvp1sitesweep(ops_g, DT, As_g, Ws_g, env_g, turning="symmetric")
        td.tdvp1sitesweep(ops_o, DT, As_o, Ws_o, env_o, turning="symmetric")
    assert abs(td.norm2(ops_g, As_g) - 1.0) < 1e-10
    assert abs(_energy(ops_g, As_g, Ws_g, env_g) - e0) < 1e-9
    # site tensors differ by bond gauges (singular vectors are unique up to a phase each); the
    # state is gauge invariant
    psi_g = ot.state_vector([dense_site(ops_g, A) for A in As_g])
    psi_o = ot.state_vector([dense_site(ops_o, A) for A in As_o])
    assert np.linalg.norm(psi_g - psi_o) < 1e-10
    sz_g = td.site_operator(ops_g, mg.VectorSpace(((0, 1), (1, 1))), {0: -0.5, 1: 0.5})
    sz_o = td.site_operator(ops_o, U1Space((0, 1), (1, 1)), {0: -0.5, 1: 0.5})
    for i, j in ((1, 2), (4, 9), (7, 14)):
        g = td.expectation(ops_g, As_g, {i: sz_g, j: sz_g})
        o = td.expectation(ops_o, As_o, {i: sz_o, j: sz_o})
        assert abs(g - o) < 1e-11


def test_batched_dots_and_lincomb():
    rng = np.random.default_rng(3)
    V = U1Space((0, 5), (1, 7), (2, 3))
    W = U1Space((0, 4), (1, 2), isdual=True)
    ts = [rand_tensor(1, (V, W), rng) for _ in range(5)]
    gs = [to_device(t) for t in ts]
    got = mg.dots(gs[:4], gs[1:])
    want = [float(np.vdot(st.flatten(a), st.flatten(b))) for a, b in zip(ts[:4], ts[1:])]
    np.testing.assert_allclose(got, want, rtol=1e-14)
    assert got == [mg.dot(a, b) for a, b in zip(gs[:4], gs[1:])]
    c = [0.5, -2.0, 3.25]
    out = mg.lincomb(c, gs[:3], mg.similar(gs[0]))
    ref = sum(ci * st.flatten(t) for ci, t in zip(c, ts[:3]))
    np.testing.assert_allclose(out.to_flat(), ref, rtol=1e-14, atol=1e-14)
    mg.lincomb([1.0, -1.0], [gs[3], gs[4]], gs[3])  # out aliases an operand
    np.testing.assert_allclose(gs[3].to_flat(), st.flatten(ts[3]) - st.flatten(ts[4]), atol=1e-14)
    with pytest.raises(mg.SpaceMismatch):
        mg.lincomb([1.0], [to_device(rand_tensor(0, (V, W), rng))], gs[0])


@pytest.mark.parametrize("sa,sb,real_b", [(1.0, 1.0, False), (-1.0, 1.0, False),
                                          (1.0, -1.0, False), (-1.0, 1.0, True)])
def test_contract_complex_matches_complex_oracle(sa, sb, real_b):
    rng = np.random.default_rng(17)
    V1, V2 = U1Space((0, 3), (1, 4), (2, 2)), U1Space((0, 2), (1, 5))
    V3 = U1Space((-1, 2), (0, 3), (1, 2))
    ar, ai = rand_tensor(0, (V1, V2, V3), rng), rand_tensor(0, (V1, V2, V3), rng)
    V4 = U1Space((0, 3), (1, 2))
    br, bi = rand_tensor(0, (dual_space(V3), dual_space(V2), V4), rng), \
        rand_tensor(0, (dual_space(V3), dual_space(V2), V4), rng)
    cplx = lambda r, i, s: st.SymTensor(r.charge, r.space,
                                        {k: r.blocks[k] + 1j * s * i.blocks[k] for k in r.blocks},
                                        check=False)
    A = cplx(ar, ai, sa)
    B = st.SymTensor(br.charge, br.space, {k: br.blocks[k] + 0j for k in br.blocks},
                     check=False) if real_b else cplx(br, bi, sb)
    want = st.contract(A, (1, -2, -1), B, (-1, -2, 2))
    cr, ci = mg.contract_complex(to_device(ar), to_device(ai), sa, (1, -2, -1), to_device(br),
                                 None if real_b else to_device(bi), sb, (-1, -2, 2))
    got = cr.to_flat() + 1j * ci.to_flat()
    ref = st.flatten(want)
    assert np.linalg.norm(got - ref) < 1e-13 * np.linalg.norm(ref)
    # a full contraction with the conjugated dual gives the complex number |A|^2
    z = mg.contract_complex(to_device(ar), to_device(ai), sa, (-1, -2, -3),
                            mg.dual(to_device(ar)), mg.dual(to_device(ai)), -sa, (-1, -2, -3))
    zz = sum(np.sum(A.blocks[k] * np.conj(A.blocks[k])) for k in A.blocks)
    assert abs(z - zz) < 1e-12 * abs(zz)
