"""CPU oracle: dense complex time evolution of an MPS (src/tdvp.jl) and the Krylov exponential.

TEST INFRASTRUCTURE ONLY: the checker of the library's symmetric TDVP. Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` may import it.

The reference's TDVP is dense (``Array{T,3}`` site tensors, ``@tensor`` contractions): this
module restates it on NumPy arrays with Julia's index conventions (site tensor A[l, o, r], MPO
tensor W[m_left, o_out, m_right, o_in], environments env[ket, mpo, bra]).

``exponentiate`` stands for KrylovKit.exponentiate(f, t, x; ishermitian=true) (an external
package, not vendored and unpinned; the call sites are src/tdvp.jl:27,40,52,68,78,122,139,153,
172,184). It is restated from the published Lanczos exponential-integrator scheme: a Lanczos
basis with full reorthogonalisation; the exponential of the small tridiagonal matrix through
its eigen-decomposition; the a-posteriori error beta_m |e_m^T exp(tau T) e_1| decides the
Krylov dimension; a step that the full basis cannot take within tol is cut in halves. The
library implements the same scheme (its reorthogonalisation is classical Gram-Schmidt twice with
batched dot products, this one modified Gram-Schmidt twice: both are full reorthogonalisation),
so results agree to rounding; parity against a Julia run is unpinned (Julia is absent).

Turning point of a sweep: the reference evolves the last site (1-site) or the last pair (2-site)
once, by dt, between the left-to-right and the right-to-left half-sweeps (src/tdvp.jl:45-48,
145-148), while every other piece is evolved twice by dt. ``turning="reference"`` reproduces
that; ``turning="symmetric"`` evolves the turning piece by 2 dt, which makes the sweep the
symmetric composition of the two first-order projector-splitting half-sweeps, i.e. exact time
evolution by 2 dt when the bond dimensions are full (tested against exact diagonalisation).
"""
from __future__ import annotations

import numpy as np

TURNING = ("reference", "symmetric")


# ---------------------------------------------------------------------------------------------
# dense effective Hamiltonians and environment updates (src/apply.jl)
# ---------------------------------------------------------------------------------------------
def applymps0site(lam, envL, envR):
    """``_applymps0site`` (apply.jl:2-7): A[d,d'] = envL[u,m,d] lam[u,u'] envR[u',m,d']."""
    return np.einsum("umd,uv,vme->de", envL, lam, envR, optimize=True)


def mpsupdateright(renv, mat, hmpo):
    """``_mpsupdateright`` (apply.jl:9-15):
    R[u,m,d] = renv[u',m',d'] mat[u,o,u'] hmpo[m,o',m',o] conj(mat)[d,o',d']."""
    return np.einsum("abc,uoa,mpbo,dpc->umd", renv, mat, hmpo, mat.conj(), optimize=True)


def mpsupdateleft(lenv, mat, hmpo):
    """``_mpsupdateleft`` (apply.jl:41-47):
    L[u,m,d] = lenv[u',m',d'] mat[u',o,u] hmpo[m',o',m,o] conj(mat)[d',o',d]."""
    return np.einsum("abc,aou,bpmo,cpd->umd", lenv, mat, hmpo, mat.conj(), optimize=True)


def applymps1site(v, envL, envR, hmpo):
    """``_applymps1site`` (apply.jl:70-78):
    v[l,o,r] = envL[l',ml,l] v[l',o',r'] hmpo[ml,o,mr,o'] envR[r',mr,r]."""
    return np.einsum("aml,apb,monp,bnr->lor", envL, v, hmpo, envR, optimize=True)


def applymps2site(v, envL, envR, hmpoL, hmpoR):
    """``_applymps2site`` (apply.jl:80-91)."""
    return np.einsum("aml,apqb,mxnp,nyrq,brc->lxyc", envL, v, hmpoL, hmpoR, envR, optimize=True)


def initialenv(As, Ws):
    """Dense ``initialenv`` at center 1 (dmrg.jl:9-36): boundaries of ones, right updates."""
    lx = len(As)
    env = [None] * (lx + 2)
    env[0] = np.ones((As[0].shape[0], Ws[0].shape[0], As[0].shape[0]), dtype=complex)
    env[lx + 1] = np.ones((As[-1].shape[2], Ws[-1].shape[2], As[-1].shape[2]), dtype=complex)
    for l in range(lx, 0, -1):
        env[l] = mpsupdateright(env[l + 1], As[l - 1], Ws[l - 1])
    return env


# ---------------------------------------------------------------------------------------------
# Krylov exponential (KrylovKit.exponentiate, ishermitian=true)
# ---------------------------------------------------------------------------------------------
class ExpInfo:
    def __init__(self, numops, numsteps, converged):
        self.numops = numops
        self.numsteps = numsteps
        self.converged = converged


def _expT(alphas, betas, tau):
    """exp(tau T) e_1 for the real symmetric tridiagonal T(alphas, betas)."""
    m = len(alphas)
    T = np.diag(np.asarray(alphas, dtype=float))
    for i in range(m - 1):
        T[i, i + 1] = T[i + 1, i] = betas[i]
    w, Q = np.linalg.eigh(T)
    return Q @ (np.exp(tau * w) * Q[0, :])


def exponentiate(f, t, x, krylovdim: int = 30, tol: float = 1e-12, maxiter: int = 100):
    """exp(t f) x for a Hermitian linear map f, t complex. Returns (y, ExpInfo)."""
    shape = x.shape
    xv = np.asarray(x, dtype=complex).reshape(-1)
    scale = float(np.linalg.norm(xv))
    if scale == 0.0:
        return np.zeros(shape, dtype=complex), ExpInfo(0, 0, True)
    v = xv / scale
    left = 1.0
    numops = numsteps = 0
    converged = True
    while left > 0.0 and numsteps < maxiter:
        numsteps += 1
        V = [v]
        alphas, betas = [], []
        step = None
        for j in range(krylovdim):
            w = np.asarray(f(V[j].reshape(shape)), dtype=complex).reshape(-1)
            numops += 1
            a = float(np.real(np.vdot(V[j], w)))
            w = w - a * V[j]
            if j > 0:
                w = w - betas[j - 1] * V[j - 1]
            for _ in range(2):  # full reorthogonalisation, twice
                for u in V:
                    w = w - np.vdot(u, w) * u
            b = float(np.linalg.norm(w))
            alphas.append(a)
            m = j + 1
            tau = left
            c = _expT(alphas, betas, tau * t)
            err = b * abs(c[m - 1]) * scale
            if err <= tol or b <= 1e-14 * max(1.0, abs(a)):
                step = tau
                break
            if m == krylovdim:
                while err > tol and tau > 1e-6 * left:
                    tau *= 0.5
                    c = _expT(alphas, betas, tau * t)
                    err = b * abs(c[m - 1]) * scale
                if err > tol:
                    converged = False
                step = tau
                break
            betas.append(b)
            V.append(w / b)
        y = sum(c[i] * V[i] for i in range(len(c))) * scale
        left = max(0.0, left - step) if step < left else 0.0
        scale = float(np.linalg.norm(y))
        v = y / scale
    if left > 0.0:
        converged = False
    return (v * scale).reshape(shape), ExpInfo(numops, numsteps, converged)


# ---------------------------------------------------------------------------------------------
# sweeps (src/tdvp.jl)
# ---------------------------------------------------------------------------------------------
def _qr_left(A):
    """Q, R of reshape(A, Dl*d, Dr) with Q reshaped back (tdvp.jl:35-36)."""
    Dl, d, Dr = A.shape
    Q, R = np.linalg.qr(A.reshape(Dl * d, Dr, order="F"))
    return Q.reshape(Dl, d, Q.shape[1], order="F"), R


def _qr_right(A):
    """Q, Lambda of transpose(reshape(A, Dl, d*Dr)) (tdvp.jl:61-64)."""
    Dl, d, Dr = A.shape
    Q, R = np.linalg.qr(A.reshape(Dl, d * Dr, order="F").T)
    return Q.T.reshape(Q.shape[1], d, Dr, order="F"), R.T


def tdvp1sitesweep(dt, As, Ws, env, turning: str = "reference", krylovdim: int = 30,
                   tol: float = 1e-12):
    """``tdvp1sitesweep!`` (tdvp.jl:12-89) on a center-1 dense MPS; As and env are updated in
    place and returned. ``turning`` is explained in the module docstring."""
    if turning not in TURNING:
        raise ValueError(turning)
    lx = len(As)
    ex = lambda fn, t, x: exponentiate(fn, t, x, krylovdim=krylovdim, tol=tol)[0]
    A = As[0]
    for l in range(1, lx):
        A = ex(lambda v: applymps1site(v, env[l - 1], env[l + 1], Ws[l - 1]), -1j * dt, A)
        Q, lam = _qr_left(A)
        As[l - 1] = Q
        env[l] = mpsupdateleft(env[l - 1], Q, Ws[l - 1])
        lam = ex(lambda v: applymps0site(v, env[l], env[l + 1]), 1j * dt, lam)
        A = np.einsum("lm,mor->lor", lam, As[l])
    l = lx
    t_turn = 2 * dt if turning == "symmetric" else dt
    A = ex(lambda v: applymps1site(v, env[l - 1], env[l + 1], Ws[l - 1]), -1j * t_turn, A)
    for l in range(lx - 1, 0, -1):
        Q, lam = _qr_right(A)
        As[l] = Q
        env[l + 1] = mpsupdateright(env[l + 2], Q, Ws[l])
        lam = ex(lambda v: applymps0site(v, env[l], env[l + 1]), 1j * dt, lam)
        A = np.einsum("lom,mr->lor", As[l - 1], lam)
        A = ex(lambda v: applymps1site(v, env[l - 1], env[l + 1], Ws[l - 1]), -1j * dt, A)
    As[0] = A
    return As, env


def svdtrunc_dense(M, maxdim: int, tol: float):
    """Dense ``svdtrunc`` (mpsutils.jl:34-41): n = min(maxdim, #{S > S[1] tol}) (a RELATIVE
    tol, unlike the symmetric method's absolute one)."""
    U, S, Vh = np.linalg.svd(M, full_matrices=False)
    k = int(min(maxdim, np.sum(S > S[0] * tol)))
    if k == 0:
        raise ValueError("The largest singular value is smaller than tol!")
    return U[:, :k], S[:k], Vh[:k, :]


def tdvp2sitesweep(dt, As, Ws, env, maxdim: int = 200, tol: float = 1e-14,
                   turning: str = "reference", krylovdim: int = 30, ktol: float = 1e-12):
    """``tdvp2sitesweep!`` (tdvp.jl:105-210) on a center-1 dense MPS, in place."""
    if turning not in TURNING:
        raise ValueError(turning)
    lx = len(As)
    ex = lambda fn, t, x: exponentiate(fn, t, x, krylovdim=krylovdim, tol=ktol)[0]
    A = As[0]
    for l in range(1, lx - 1):
        AA = np.einsum("abm,mcd->abcd", A, As[l])
        AA = ex(lambda v: applymps2site(v, env[l - 1], env[l + 2], Ws[l - 1], Ws[l]), -1j * dt,
                AA)
        s0, s1, s2, s3 = AA.shape
        u, s, v = svdtrunc_dense(AA.reshape(s0 * s1, s2 * s3, order="F"), maxdim, tol)
        As[l - 1] = u.reshape(s0, s1, len(s), order="F")
        env[l] = mpsupdateleft(env[l - 1], As[l - 1], Ws[l - 1])
        lam = (s[:, None] * v).reshape(len(s), s2, s3, order="F")
        lam = ex(lambda x: applymps1site(x, env[l], env[l + 2], Ws[l]), 1j * dt, lam)
        A = lam
    l = lx - 1
    t_turn = 2 * dt if turning == "symmetric" else dt
    AA = np.einsum("abm,mcd->abcd", A, As[l])
    AA = ex(lambda v: applymps2site(v, env[l - 1], env[l + 2], Ws[l - 1], Ws[l]), -1j * t_turn,
            AA)
    for l in range(lx - 1, 1, -1):
        s0, s1, s2, s3 = AA.shape
        u, s, v = svdtrunc_dense(AA.reshape(s0 * s1, s2 * s3, order="F"), maxdim, tol)
        As[l] = v.reshape(len(s), s2, s3, order="F")
        env[l + 1] = mpsupdateright(env[l + 2], As[l], Ws[l])
        lam = (u * s[None, :]).reshape(s0, s1, len(s), order="F")
        lam = ex(lambda x: applymps1site(x, env[l - 1], env[l + 1], Ws[l - 1]), 1j * dt, lam)
        AA = np.einsum("abm,mcd->abcd", As[l - 2], lam)
        AA = ex(lambda v: applymps2site(v, env[l - 2], env[l + 1], Ws[l - 2], Ws[l - 1]),
                -1j * dt, AA)
    s0, s1, s2, s3 = AA.shape
    u, s, v = svdtrunc_dense(AA.reshape(s0 * s1, s2 * s3, order="F"), maxdim, tol)
    As[1] = v.reshape(len(s), s2, s3, order="F")
    env[2] = mpsupdateright(env[3], As[1], Ws[1])
    As[0] = (u * s[None, :]).reshape(s0, s1, len(s), order="F")
    return As, env


# ---------------------------------------------------------------------------------------------
# dense helpers for checks
# ---------------------------------------------------------------------------------------------
def state_vector(As):
    """The full state vector of a dense MPS with boundary dims 1 (site 1 most significant)."""
    psi = As[0]
    for A in As[1:]:
        psi = np.tensordot(psi, A, axes=([psi.ndim - 1], [0]))
    return psi.reshape(-1)


def szsz(psi, lx, i, j):
    """<psi| Sz_i Sz_j |psi> / <psi|psi> on a 2^lx state vector (basis: 0 = down, 1 = up)."""
    idx = np.arange(2 ** lx)
    zi = ((idx >> (lx - i)) & 1) - 0.5
    zj = ((idx >> (lx - j)) & 1) - 0.5
    p = np.abs(psi) ** 2
    return float(np.sum(p * zi * zj) / np.sum(p))
