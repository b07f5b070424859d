"""CPU oracle: MPS / MPO containers and the algorithms of the 2-site DMRG hot path, restated from
amiragha/mps in NumPy float64.

TEST INFRASTRUCTURE ONLY (see ``oracle/symtensors.py``).  The Krylov eigensolver is KrylovKit's
``eigsolve`` in the reference, an unvendored and unpinned dependency; ``eigsolve_lanczos`` below
restates its published thick-restart Lanczos scheme (KrylovKit ``Lanczos``: full
reorthogonalisation, convergence tested when the basis reaches ``krylovdim``, restart keeping
``div(3*krylovdim + 2*converged, 5)`` Ritz vectors).  Results at that boundary are therefore
"parity unpinned": no reference test fixes them.
"""
from __future__ import annotations

import math

import numpy as np

from . import symtensors as st
from .symtensors import U1Space, dual_space, contract, SymTensor


# ---------------------------------------------------------------------------------------------
# MPO  (src/symmpo.jl:45-97)
# ---------------------------------------------------------------------------------------------
def xxz_u1mpo(lx: int, delta: float = 1.0):
    """U(1) XXZ MPO with bond space (-1=>1, 0=>3, 1=>1) and site space (0=>1, 1=>1)."""
    V0 = U1Space((0, 1))
    V = U1Space((-1, 1), (0, 3), (1, 1))
    d = U1Space((0, 1), (1, 1))
    space = (V, d, dual_space(V), dual_space(d))
    Wbeg = st.fill(0.0, 0, (V0,) + space[1:])
    W = st.fill(0.0, 0, space)
    Wend = st.fill(0.0, 0, space[:2] + (V0, space[3]))
    mat0 = np.array([[1.0, 0.0, 0.0], [delta * -0.5, 0.0, 0.0], [0.0, -0.5, 1.0]])
    mat1 = np.array([[1.0, 0.0, 0.0], [delta * 0.5, 0.0, 0.0], [0.0, 0.5, 1.0]])
    F = dict(order="F")
    W[(0, 0, 0, 0)] = mat0.reshape((3, 1, 3, 1), **F)
    W[(0, 1, 0, 1)] = mat1.reshape((3, 1, 3, 1), **F)
    W[(0, 1, 1, 0)] = np.array([0.0, 0.0, 1.0]).reshape((3, 1, 1, 1), **F)
    W[(0, 0, -1, 1)] = np.array([0.0, 0.0, 1.0]).reshape((3, 1, 1, 1), **F)
    W[(1, 0, 0, 1)] = 0.5 * np.array([1.0, 0.0, 0.0]).reshape((1, 1, 3, 1), **F)
    W[(-1, 1, 0, 0)] = 0.5 * np.array([1.0, 0.0, 0.0]).reshape((1, 1, 3, 1), **F)
    Wbeg[(0, 0, 0, 0)] = mat0[2, :].reshape((1, 1, 3, 1), **F)
    Wbeg[(0, 1, 0, 1)] = mat1[2, :].reshape((1, 1, 3, 1), **F)
    Wbeg[(0, 1, 1, 0)] = np.ones((1, 1, 1, 1))
    Wbeg[(0, 0, -1, 1)] = np.ones((1, 1, 1, 1))
    Wend[(0, 0, 0, 0)] = mat0[:, 0].reshape((3, 1, 1, 1), **F)
    Wend[(0, 1, 0, 1)] = mat1[:, 0].reshape((3, 1, 1, 1), **F)
    Wend[(-1, 1, 0, 0)] = 0.5 * np.ones((1, 1, 1, 1))
    Wend[(1, 0, 0, 1)] = 0.5 * np.ones((1, 1, 1, 1))
    return [Wbeg] + [W] * (lx - 2) + [Wend]


def xxz_hamiltonian(lx: int, delta: float = 1.0) -> np.ndarray:
    """Dense open-chain XXZ Hamiltonian built by Kronecker products (src/xxz.jl:13-37) with the
    spin-1/2 operators of src/spin_definitions.jl:7-16 (basis index 1 = up)."""
    sz = np.diag([0.5, -0.5])
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm = sp.T.copy()
    term = 0.5 * (np.kron(sp, sm) + np.kron(sm, sp)) + delta * np.kron(sz, sz)
    H = term
    for i in range(3, lx + 1):
        H = np.kron(H, np.eye(2)) + np.kron(np.eye(2 ** (i - 2)), term)
    return H


# ---------------------------------------------------------------------------------------------
# MPS  (src/symmps.jl)
# ---------------------------------------------------------------------------------------------
class MPState:
    """``MPState``: site tensors (Vl, d, dual(Vr)) and the orthogonality center (symmps.jl:1-4)."""

    def __init__(self, As, center: int = 0):
        self.As = list(As)
        self.center = center

    def __len__(self):
        return len(self.As)


def _pushleft(mps: MPState, l: int):
    """``_pushleft!`` (symmps.jl:167-174); ``l`` is 1-based."""
    A = mps.As[l - 1]
    u, s, v = st.svd_(st.fuselegs(A, 2, 2))
    mps.As[l - 1] = st.splitleg(v, 2, A.space[1:3])
    mps.As[l - 2] = contract(mps.As[l - 2], (1, 2, -1), st.matmul(u, s), (-1, 3))


def _pushright(mps: MPState, l: int):
    """``_pushright!`` (symmps.jl:176-183)."""
    A = mps.As[l - 1]
    u, s, v = st.svd_(st.fuselegs(A, 1, 2))
    mps.As[l - 1] = st.splitleg(u, 1, A.space[0:2])
    mps.As[l] = contract(st.matmul(s, v), (1, -1), mps.As[l], (-1, 2, 3))


def center_at(mps: MPState, center: int) -> MPState:
    """``center_at!`` (symmps.jl:185-200)."""
    x1, xL = 1, len(mps)
    if mps.center > 0:
        x1 = xL = mps.center
    for p in range(x1, center):
        _pushright(mps, p)
    for p in range(xL, center, -1):
        _pushleft(mps, p)
    mps.center = center
    return mps


# ---------------------------------------------------------------------------------------------
# Effective Hamiltonian and environments  (src/apply.jl)
# ---------------------------------------------------------------------------------------------
def applymps2site(v, envL, envR, W1, W2):
    """``_applymps2site`` for SymTensors: four chained contractions (apply.jl:93-105)."""
    t = contract(envL, (-1, 2, 1), v, (-1, 3, 4, 5))
    t = contract(t, (1, -1, -2, 4, 5), W1, (-1, 2, 3, -2))
    t = contract(t, (1, 2, -1, -2, 5), W2, (-1, 3, 4, -2))
    return contract(t, (1, 2, 3, -1, -2), envR, (-2, -1, 4))


def mpsupdateright(renv, mat, hmpo):
    """``_mpsupdateright`` (apply.jl:17-25)."""
    t = contract(renv, (-1, 3, 4), mat, (1, 2, -1))
    t = contract(t, (1, -1, -2, 4), hmpo, (3, 2, -2, -1))
    return contract(t, (1, -1, 2, -2), st.dual(mat), (3, -1, -2))


def mpsupdateleft(lenv, mat, hmpo):
    """``_mpsupdateleft`` (apply.jl:49-58)."""
    t = contract(lenv, (-1, 3, 4), mat, (-1, 2, 1))
    t = contract(t, (1, -1, -2, 4), hmpo, (-2, 2, 3, -1))
    return contract(t, (1, -1, 2, -2), st.dual(mat), (-2, -1, 3))


def initialenv(mps: MPState, mpo, at: int = 1):
    """Boundary environments filled with ones, then right updates down to ``at`` (dmrg.jl:9-36)."""
    if mps.center != at:
        raise st.SpaceMismatch(f"MPS center has to be {at}")
    lx = len(mps)
    env = [None] * (lx + 2)
    lVa = mps.As[0].space[0]
    rVa = dual_space(mps.As[-1].space[2])
    lVw = mpo[0].space[0]
    rVw = dual_space(mpo[-1].space[2])
    env[0] = st.fill(1.0, 0, (dual_space(lVa), dual_space(lVw), lVa))
    env[lx + 1] = st.fill(1.0, 0, (rVa, rVw, dual_space(rVa)))
    for l in range(lx, at - 1, -1):
        env[l] = mpsupdateright(env[l + 1], mps.As[l - 1], mpo[l - 1])
    for l in range(1, at):
        env[l] = mpsupdateleft(env[l - 1], mps.As[l - 1], mpo[l - 1])
    return env


# ---------------------------------------------------------------------------------------------
# Thick-restart Lanczos (KrylovKit ``eigsolve(f, x0, 1, :SR, ishermitian=true, ...)`` semantics)
# ---------------------------------------------------------------------------------------------
class LanczosInfo:
    def __init__(self, normres, numiter, numops, converged):
        self.normres = normres
        self.numiter = numiter
        self.numops = numops
        self.converged = converged


def _lincomb(vecs, coeffs):
    out = st.scaled(vecs[0], float(coeffs[0]))
    for v, c in zip(vecs[1:], coeffs[1:]):
        st.axpy(float(c), v, out)
    return out


def _orthogonalize(w, V):
    """Classical Gram-Schmidt applied twice; returns the summed coefficients."""
    h = np.zeros(len(V))
    for _ in range(2):
        c = np.array([float(np.real(st.dot(v, w))) for v in V])
        for v, cj in zip(V, c):
            st.axpy(-cj, v, w)
        h += c
    return h


def eigsolve_lanczos(f, x0, krylovdim: int = 5, maxiter: int = 8, tol: float = 1e-7):
    """Lowest eigenpair of the symmetric linear map ``f`` starting from ``x0``.

    Returns ``(theta, x, info)``.  The projected matrix ``H`` is a tridiagonal matrix that becomes
    an arrowhead block after every thick restart.  Convergence (residual ``beta*|u_K|`` at most
    ``tol``) is tested only when the basis is full or the residual norm ``beta`` drops to ``tol``.
    """
    beta0 = st.norm(x0)
    V = [st.scaled(x0, 1.0 / beta0)]
    w = f(V[0])
    numops, numiter = 1, 1
    h = _orthogonalize(w, V)
    H = np.zeros((krylovdim + 1, krylovdim + 1))
    H[0, 0] = h[0]
    r, beta = w, st.norm(w)
    arrow = False  # True right after a restart: the couplings of the next vector are set
    while True:
        K = len(V)
        if K == krylovdim or beta <= tol:
            D, U = np.linalg.eigh(H[:K, :K])
            normres = abs(beta * U[K - 1, 0])
            converged = normres <= tol
            if converged or beta <= tol or numiter >= maxiter:
                x = _lincomb(V, U[:, 0])
                st.rmul(x, 1.0 / st.norm(x))
                return float(D[0]), x, LanczosInfo(normres, numiter, numops, converged)
            keep = max(1, (3 * krylovdim + 2 * int(converged)) // 5)
            Vn = [_lincomb(V, U[:, i]) for i in range(keep)]
            Hn = np.zeros_like(H)
            for i in range(keep):
                Hn[i, i] = D[i]
                Hn[keep, i] = Hn[i, keep] = beta * U[K - 1, i]
            V, H = Vn, Hn
            numiter += 1
            arrow = True
            K = keep
        # expand the basis by the normalised residual
        v = st.scaled(r, 1.0 / beta)
        if arrow:
            arrow = False
        else:
            H[K, K - 1] = H[K - 1, K] = beta
        V.append(v)
        w = f(v)
        numops += 1
        h = _orthogonalize(w, V)
        H[K, K] = h[K]
        r, beta = w, st.norm(w)


# ---------------------------------------------------------------------------------------------
# 2-site DMRG sweep  (src/dmrg.jl:58-179)
# ---------------------------------------------------------------------------------------------
def _heff(env, Ws, l):
    return lambda x: applymps2site(x, env[l - 1], env[l + 2], Ws[l - 1], Ws[l])


def _truncate_and_energy(v, AA, env, Ws, l, maxdim, tol, tieband):
    u, s, vt = st.svdtrunc(st.symmatrix(v, [1, 2], [3, 4]), maxdim=maxdim, tol=tol,
                           tieband=tieband)
    truncerr = 1.0 - st.norm(s)
    st.rmul(s, 1.0 / st.norm(s))
    usv = st.matmul(st.matmul(u, s), vt)
    AA = st.splitleg(st.splitleg(usv, 2, AA.space[2:4]), 1, AA.space[0:2])
    e = float(np.real(st.dot(AA, _heff(env, Ws, l)(AA))))
    return u, s, vt, AA, e, truncerr


def dmrg2sitesweep(mps: MPState, Ws, env, maxdim=200, tol=1e-9, lanczostol=1e-7, krylovdim=5,
                   krylovmaxiter=8, tieband=0.0, stats=None):
    """One left-to-right-to-left sweep; returns the reference's list of post-truncation energies
    (3L-5 entries, the right-to-left loop pushes its energy twice, dmrg.jl:132,156)."""
    lx = len(mps)
    if mps.center != 1:
        raise st.SpaceMismatch("The center of MPS has to be 1 for dmrg L->R->L")
    energies = []
    A = mps.As[0]
    eig = dict(krylovdim=krylovdim, maxiter=krylovmaxiter, tol=lanczostol)
    for l in range(1, lx - 1):
        AA = contract(A, (1, 2, -1), mps.As[l], (-1, 3, 4))
        _, v, info = eigsolve_lanczos(_heff(env, Ws, l), AA, **eig)
        if stats is not None:
            stats.append(info)
        u, s, vt, AA, e, _ = _truncate_and_energy(v, AA, env, Ws, l, maxdim, tol, tieband)
        energies.append(e)
        mps.As[l - 1] = st.splitleg(u, 1, A.space[0:2])
        env[l] = mpsupdateleft(env[l - 1], mps.As[l - 1], Ws[l - 1])
        A = st.splitleg(st.matmul(s, vt), 2, AA.space[2:4])
    l = lx - 1
    AA = contract(A, (1, 2, -1), mps.As[l], (-1, 3, 4))
    _, v, info = eigsolve_lanczos(_heff(env, Ws, l), AA, **eig)
    if stats is not None:
        stats.append(info)
    e = None
    for l in range(lx - 1, 1, -1):
        u, s, vt, AA, e, _ = _truncate_and_energy(v, AA, env, Ws, l, maxdim, tol, tieband)
        energies.append(e)
        mps.As[l] = st.splitleg(vt, 2, AA.space[2:4])
        env[l + 1] = mpsupdateright(env[l + 2], mps.As[l], Ws[l])
        A = st.splitleg(st.matmul(u, s), 1, AA.space[0:2])
        AA = contract(mps.As[l - 2], (1, 2, -1), A, (-1, 3, 4))
        _, v, info = eigsolve_lanczos(_heff(env, Ws, l - 1), AA, **eig)
        if stats is not None:
            stats.append(info)
        energies.append(e)
    l = 1
    u, s, vt, AA, e, _ = _truncate_and_energy(v, AA, env, Ws, l, maxdim, tol, tieband)
    energies.append(e)
    mps.As[1] = st.splitleg(vt, 2, AA.space[2:4])
    env[2] = mpsupdateright(env[3], mps.As[1], Ws[1])
    mps.As[0] = st.splitleg(st.matmul(u, s), 1, AA.space[0:2])
    return energies


def binomial_bond_dims(lx, site, M, chimax, d=2):
    """Bond charges between ``site`` and ``site+1`` as in symmps.jl:59-62, each with dimension
    min(chimax, #left states, #right states) for d = 2."""
    cmin = max(0, M - (d - 1) * (lx - site))
    cmax = min(M, (d - 1) * site)
    return [(c, max(1, min(chimax, math.comb(site, c), math.comb(lx - site, M - c))))
            for c in range(cmin, cmax + 1)]


# ---------------------------------------------------------------------------------------------
# The chi-dimensional two-site H_eff input (synthetic: the reference publishes no dataset).  Legs
# follow the reference's conventions: v (Vl, d, d, dual(Vr)) as a two-site MPS tensor
# (symmps.jl:63-64), envL (dual(Vl), dual(Vw), Vl) and envR (Vr, Vw, dual(Vr)) (dmrg.jl:25-26),
# W the middle XXZ MPO tensor (symmpo.jl:45-97).
# ---------------------------------------------------------------------------------------------
def binomial_profile(chi: int, ncharges: int = 25):
    """Bond dimensions per charge: chi * C(n-1, k) / 2^(n-1), at least one state per charge,
    rounded by largest remainder in mirror-symmetric pairs so that they sum to chi."""
    n = ncharges - 1
    exact = [chi * math.comb(n, k) / 2.0 ** n for k in range(ncharges)]
    dims = [max(1, int(math.floor(x))) for x in exact]
    left = chi - sum(dims)
    rank = sorted(range(ncharges), key=lambda k: (-(exact[k] - math.floor(exact[k])),
                                                  abs(k - n / 2)))
    sgn = 1 if left > 0 else -1
    for i in range(10 * ncharges):
        if left == 0:
            break
        k = rank[i % ncharges]
        m = n - k
        if k == m:
            if dims[k] + sgn >= 1:
                dims[k] += sgn
                left -= sgn
        elif abs(left) >= 2 and dims[k] + sgn >= 1 and dims[m] + sgn >= 1:
            dims[k] += sgn
            dims[m] += sgn
            left -= 2 * sgn
    if left != 0:
        dims[n // 2] += left
    return dims


def heff_workload(chi: int, delta: float = 0.5, seed: int = 1911, ncharges: int = 25):
    """(v, envL, envR, W, W) of the two-site H_eff benchmark: both bonds carry charges
    0..ncharges-1 with the binomial profile of ``chi`` states, the site space is (0=>1, 1=>1),
    and every block of v, envL, envR (in that order, each in reference block order, each block
    column-major) is drawn N(0,1) from one Philox(seed) stream."""
    Vb = st.VectorSpace([(k, dk) for k, dk in enumerate(binomial_profile(chi, ncharges))])
    d = U1Space((0, 1), (1, 1))
    Vw = U1Space((-1, 1), (0, 3), (1, 1))
    spaces = ((Vb, d, d, dual_space(Vb)), (dual_space(Vb), dual_space(Vw), Vb),
              (Vb, Vw, dual_space(Vb)))
    rng = np.random.Generator(np.random.Philox(seed))
    out = []
    for sp in spaces:
        sects, sizes = st.allsectorsandsizes(0, sp)
        n = sum(int(np.prod(z)) for z in sizes)
        out.append(st.from_flat(0, sp, rng.standard_normal(n)))
    W = xxz_u1mpo(3, delta)[1]
    return out[0], out[1], out[2], W, W


def heff_flops(v, envL, envR, W1, W2) -> float:
    """Algorithmic flops (sum of 2*M*N*K over the sector GEMMs) of one ``applymps2site`` in the
    reference's contraction order, counted by running it once."""
    with st.FlopCount() as fc:
        applymps2site(v, envL, envR, W1, W2)
    return fc.flops
