"""Derivatives of TDVP-evolved observables with respect to a Hamiltonian coupling.

The reference evolves MPS with the time-dependent variational principle (src/tdvp.jl:12-89).
The quantity here is, e.g., d<Sz_i Sz_j>(t)/dDelta of an XXZ chain after 1-site TDVP. A single
scalar parameter is a forward-mode (tangent) derivative: every quantity of the sweep in
``mps_gb300.tdvp`` carries its derivative with respect to the coupling, propagated through each
step by the chain rule, so one tangent sweep costs a fixed multiple of a plain sweep and stores
nothing beyond the current state and environments (no tape, no recomputation). The result is
the exact derivative of the discrete algorithm's output (up to the Krylov tolerances).

Steps and their tangents (``d`` = derivative with respect to the coupling, W the MPO, dW its
derivative, H_eff built from the environments L, R and W):

* Krylov exponential x' = exp(t F) x with F Hermitian and dF its derivative (the H_eff built with
  one of dL, dR, dW in place of L, R, W). The derivative of exp(t F) x in the direction dF is the
  top block of exp(t M) [dx; x] for the block-triangular M = [[F, dF], [0, F]]; M is not
  Hermitian, so ``exponentiate_tangent`` runs Arnoldi with full reorthogonalisation on pairs of
  tensors and exponentiates the small Hessenberg matrix on the host, with the error estimate
  and step halving of ``ctensor.exponentiate``. The value x' itself comes from the plain
  Lanczos exponential, so the forward state is the one ``tdvp1sitesweep`` computes.
* Gauge move M = Q lam (per-sector SVD, Q = u isometric, lam = s v): the tangent with
  Q^H dQ = 0, i.e. dQ = (1 - Q Q^H) dM v^H s^-1 and dlam = Q^H dM (right-to-left: M = lam Q,
  dlam = dM Q^H, dQ = s^-1 u^H dM (1 - Q^H Q)). Any other choice differs by a gauge
  transformation of the MPS, which TDVP carries covariantly and no observable sees.
* Environments: the four-term product rule over (environment, ket, MPO, bra) of
  ``_mpsupdateleft`` / ``_mpsupdateright`` (src/apply.jl:17-58).
* Observables: <psi|O|psi> / <psi|psi> by transfer matrices with their tangents.

Reverse mode (``evolve_with_adjoint``) gives the gradient with respect to every MPO tensor and
every initial site tensor at once (many couplings, or a cost on the initial state). The forward
sweeps keep only the MPS at the start of each sweep. Backward, sweep by sweep from the last, the
environments are rebuilt from that checkpoint, the sweep is replayed on a tape (the same
operations as ``tdvp1sitesweep``) and the cotangents are propagated through it. The adjoint of
a Krylov exponential y = exp(t F) x is x_bar = exp(conj(t) F) y_bar, plus, for the operands of
F, a Gauss-Legendre quadrature of int_0^1 <exp(s conj(t) F) y_bar, dF exp((1-s) t F) x> ds. All
quadrature vectors of one step come from two Krylov integrations (``exponentiate_family``).
"""
from __future__ import annotations

import numpy as np

from .ctensor import (CTensor, Ops, cdual, ccontract, cdots, cfuselegs, clincomb,
                      cmatmul_real, cmatmul_real_right, cnorm, cscale, cspace, csplitleg, csvd,
                      cdownload, creal, exponentiate)
from .tdvp import TURNING, _transfer, apply0, apply1


# ---------------------------------------------------------------------------------------------
# small helpers: None stands for a zero tangent
# ---------------------------------------------------------------------------------------------
def _sum(ops: Ops, terms):
    """sum of (coefficient, CTensor or None) terms; None when every term is None."""
    terms = [(z, X) for z, X in terms if X is not None]
    if not terms:
        return None
    if len(terms) == 1 and terms[0][0] == 1.0:
        return terms[0][1]
    return clincomb(ops, terms)


def _diag_inverse(ops: Ops, s):
    """The inverse of the SVD's real diagonal s as a map back: legs (dual(s_2), dual(s_1)),
    block (c2, c1) = diag(1 / s_(c1, c2)) (zero where s is zero: a pseudo-inverse), so that
    X * s^-1 contracts with a leg s_2 and s^-1 * Y with a leg s_1. Blocks of s are the diagonals
    (1-d) or dense square blocks."""
    blocks = {}
    for key, b in s.blocks.items():
        b = np.asarray(b, dtype=np.float64)
        d = b if b.ndim == 1 else np.diagonal(b)
        inv = np.where(d != 0.0, 1.0 / np.where(d != 0.0, d, 1.0), 0.0)
        blocks[(key[1], key[0])] = np.diag(inv)
    V1, V2 = ops.space(s)
    return ops.from_blocks(s.charge, (ops.dual_space(V2), ops.dual_space(V1)), blocks)


def _mm(ops, X, Y):
    """Matrix product X * Y of complex rank-2 tensors (last leg of X with first of Y)."""
    return ccontract(ops, X, (1, -1), Y, (-1, 2))


def _dag_mm(ops, X, Y):
    """X^H * Y (first legs contracted, X conjugated)."""
    return ccontract(ops, cdual(ops, X), (-1, 1), Y, (-1, 2))


def _mm_dag(ops, X, Y):
    """X * Y^H (last legs contracted, Y conjugated)."""
    return ccontract(ops, X, (1, -1), cdual(ops, Y), (2, -1))


def updateleft4(ops: Ops, env, Aket, W, Abra):
    """``_mpsupdateleft`` (src/apply.jl:49-58) with separate ket and bra site tensors."""
    t = ccontract(ops, env, (-1, 3, 4), Aket, (-1, 2, 1))
    t = ccontract(ops, t, (1, -1, -2, 4), W, (-2, 2, 3, -1))
    return ccontract(ops, t, (1, -1, 2, -2), cdual(ops, Abra), (-2, -1, 3))


def updateright4(ops: Ops, env, Aket, W, Abra):
    """``_mpsupdateright`` (src/apply.jl:17-25) with separate ket and bra site tensors."""
    t = ccontract(ops, env, (-1, 3, 4), Aket, (1, 2, -1))
    t = ccontract(ops, t, (1, -1, -2, 4), W, (3, 2, -2, -1))
    return ccontract(ops, t, (1, -1, 2, -2), cdual(ops, Abra), (3, -1, -2))


def _env_tangent(ops, upd, env, denv, A, dA, W, dW):
    """Product rule of an environment update over (environment, ket, MPO, bra)."""
    return _sum(ops, [
        (1.0, None if denv is None else upd(ops, denv, A, W, A)),
        (1.0, None if dA is None else upd(ops, env, dA, W, A)),
        (1.0, None if dW is None else upd(ops, env, A, dW, A)),
        (1.0, None if dA is None else upd(ops, env, A, W, dA))])


# ---------------------------------------------------------------------------------------------
# the derivative of a Krylov exponential
# ---------------------------------------------------------------------------------------------
def _pair_dots(ops, V, w):
    a = cdots(ops, [v[0] for v in V], w[0])
    b = cdots(ops, [v[1] for v in V], w[1])
    return [x + y for x, y in zip(a, b)]


def _pair_comb(ops, terms):
    return (clincomb(ops, [(z, p[0]) for z, p in terms]),
            clincomb(ops, [(z, p[1]) for z, p in terms]))


def _pair_norm(ops, p):
    return float(np.hypot(cnorm(ops, p[0]), cnorm(ops, p[1])))


def exponentiate_tangent(ops: Ops, f, df, t, x, dx, krylovdim: int = 30, tol: float = 1e-12,
                         maxiter: int = 100):
    """d/dp [exp(t F(p)) x(p)] = the top block of exp(t M) [dx; x], M = [[F, dF], [0, F]]
    (f applies F, df applies dF, dx may be None for a constant x): Arnoldi with classical
    Gram-Schmidt applied twice on pairs of complex tensors, exp of the Hessenberg matrix on the
    host (scipy), a-posteriori error h_{m+1,m} |e_m^T exp(tau t H_m) e_1| |[dx; x]| per step
    and step halving when the basis cannot reach tol. Returns (tangent, numops, converged)."""
    from scipy.linalg import expm
    if dx is None:
        dx = cscale(ops, x, 0.0)
    v = (dx, x)
    scale = _pair_norm(ops, v)
    if scale == 0.0:
        return dx, 0, True
    v = _pair_comb(ops, [(1.0 / scale, v)])

    def M(p):
        fx, fy = f(p[0]), f(p[1])
        return (clincomb(ops, [(1.0, fx), (1.0, df(p[1]))]), fy)

    left = 1.0
    numops = steps = 0
    converged = True
    y = v
    while left > 0.0 and steps < maxiter:
        steps += 1
        V = [v]
        H = np.zeros((krylovdim + 1, krylovdim), dtype=complex)
        step = None
        c = None
        for j in range(krylovdim):
            w = M(V[j])
            numops += 1
            for _ in range(2):
                coef = _pair_dots(ops, V, w)
                H[:j + 1, j] += coef
                w = _pair_comb(ops, [(1.0, w)] + [(-cu, u) for cu, u in zip(coef, V)])
            b = _pair_norm(ops, w)
            m = j + 1
            tau = left
            E = expm(tau * t * H[:m, :m])
            c = E[:, 0]
            err = b * abs(c[m - 1]) * scale
            if err <= tol or b <= 1e-14 * max(1.0, abs(H[j, j])):
                step = tau
                break
            if m == krylovdim:
                while err > tol and tau > 1e-6 * left:
                    tau *= 0.5
                    c = expm(tau * t * H[:m, :m])[:, 0]
                    err = b * abs(c[m - 1]) * scale
                if err > tol:
                    converged = False
                step = tau
                break
            H[j + 1, j] = b
            V.append(_pair_comb(ops, [(1.0 / b, w)]))
        y = _pair_comb(ops, [(complex(c[i]) * scale, V[i]) for i in range(len(c))])
        left = left - step if step < left else 0.0
        scale = _pair_norm(ops, y)
        v = _pair_comb(ops, [(1.0 / scale, y)])
    if left > 0.0:
        converged = False
    return y[0], numops, converged


class TangentStats:
    def __init__(self):
        self.exponentials = 0
        self.matvecs = 0
        self.unconverged = 0

    def add(self, numops, converged):
        self.exponentials += 1
        self.matvecs += numops
        self.unconverged += 0 if converged else 1


def _expo_pair(ops, f, df, t, x, dx, krylovdim, tol, stats):
    """(exp(t F) x by the plain Lanczos exponential, its tangent)."""
    y, info = exponentiate(ops, f, t, x, krylovdim=krylovdim, tol=tol)
    dy, nops, ok = exponentiate_tangent(ops, f, df, t, x, dx, krylovdim=krylovdim, tol=tol)
    if stats is not None:
        stats.add(info.numops + nops, info.converged and ok)
    return y, dy


def _h1_tangent(ops, L, dL, R, dR, W, dW):
    """x -> dH_eff x for the 1-site H_eff (src/apply.jl:70-78)."""
    def df(x):
        return _sum(ops, [(1.0, None if dL is None else apply1(ops, x, dL, R, W)),
                          (1.0, None if dR is None else apply1(ops, x, L, dR, W)),
                          (1.0, None if dW is None else apply1(ops, x, L, R, dW))]) or \
            cscale(ops, x, 0.0)
    return df


def _h0_tangent(ops, L, dL, R, dR):
    """x -> dH_eff x for the 0-site H_eff (src/apply.jl:2-7)."""
    def df(x):
        return _sum(ops, [(1.0, None if dL is None else apply0(ops, x, dL, R)),
                          (1.0, None if dR is None else apply0(ops, x, L, dR))]) or \
            cscale(ops, x, 0.0)
    return df


# ---------------------------------------------------------------------------------------------
# environments, sweeps, observables
# ---------------------------------------------------------------------------------------------
def initialenv_tangent(ops: Ops, As, dAs, Ws, dWs, env):
    """Tangents of the environments built by ``tdvp.initialenv`` (right environments from the
    right end; the boundary ones are constant)."""
    lx = len(As)
    denv = [None] * (lx + 2)
    for l in range(lx, 0, -1):
        denv[l] = _env_tangent(ops, updateright4, env[l + 1], denv[l + 1], As[l - 1],
                               dAs[l - 1], Ws[l - 1], dWs[l - 1])
    return denv


def tdvp1sitesweep_tangent(ops: Ops, dt: float, As, dAs, Ws, dWs, env, denv,
                           turning: str = "reference", krylovdim: int = 30, tol: float = 1e-12,
                           stats: TangentStats | None = None):
    """``tdvp.tdvp1sitesweep`` (src/tdvp.jl:12-89) with every site tensor and environment
    carrying its derivative with respect to the coupling (``dAs``, ``denv``: lists of CTensor
    or None; ``dWs``: the MPO's derivative, real tensors or None). All four lists are updated
    in place; the state is the plain sweep's."""
    if turning not in TURNING:
        raise ValueError(f"turning must be one of {TURNING}")
    lx = len(As)
    As[:] = [creal(A) for A in As]
    A, dA = As[0], dAs[0]
    for l in range(1, lx):
        L, R = env[l - 1], env[l + 1]
        A, dA = _expo_pair(ops, lambda v: apply1(ops, v, L, R, Ws[l - 1]),
                           _h1_tangent(ops, L, denv[l - 1], R, denv[l + 1], Ws[l - 1],
                                       dWs[l - 1]), -1j * dt, A, dA, krylovdim, tol, stats)
        M = cfuselegs(ops, A, 1, 2)
        u, s, v = csvd(ops, M)  # as _pushright!, src/symmps.jl:176-183
        sp = cspace(ops, A)[0:2]
        Q = csplitleg(ops, u, 1, sp)
        lam = cmatmul_real(ops, s, v)
        dQ = dlam = None
        if dA is not None:
            dM = cfuselegs(ops, dA, 1, 2)
            Y = cmatmul_real_right(ops, _mm_dag(ops, dM, v), _diag_inverse(ops, s))
            dQf = clincomb(ops, [(1.0, Y), (-1.0, _mm(ops, u, _dag_mm(ops, u, Y)))])
            dQ = csplitleg(ops, dQf, 1, sp)
            dlam = _dag_mm(ops, u, dM)
        As[l - 1], dAs[l - 1] = Q, dQ
        env[l] = updateleft4(ops, env[l - 1], Q, Ws[l - 1], Q)
        denv[l] = _env_tangent(ops, updateleft4, env[l - 1], denv[l - 1], Q, dQ, Ws[l - 1],
                               dWs[l - 1])
        L0, R0 = env[l], env[l + 1]
        lam, dlam = _expo_pair(ops, lambda x: apply0(ops, x, L0, R0),
                               _h0_tangent(ops, L0, denv[l], R0, denv[l + 1]), 1j * dt, lam,
                               dlam, krylovdim, tol, stats)
        A = ccontract(ops, lam, (1, -1), As[l], (-1, 2, 3))
        dA = _sum(ops, [(1.0, None if dlam is None else ccontract(ops, dlam, (1, -1), As[l],
                                                                   (-1, 2, 3))),
                        (1.0, None if dAs[l] is None else ccontract(ops, lam, (1, -1), dAs[l],
                                                                     (-1, 2, 3)))])
    t_turn = 2.0 * dt if turning == "symmetric" else dt
    L, R = env[lx - 1], env[lx + 1]
    A, dA = _expo_pair(ops, lambda v: apply1(ops, v, L, R, Ws[lx - 1]),
                       _h1_tangent(ops, L, denv[lx - 1], R, denv[lx + 1], Ws[lx - 1],
                                   dWs[lx - 1]), -1j * t_turn, A, dA, krylovdim, tol, stats)
    for l in range(lx - 1, 0, -1):
        M = cfuselegs(ops, A, 2, 2)
        u, s, v = csvd(ops, M)  # as _pushleft!, src/symmps.jl:167-174
        sp = cspace(ops, A)[1:3]
        Q = csplitleg(ops, v, 2, sp)
        lam = cmatmul_real_right(ops, u, s)
        dQ = dlam = None
        if dA is not None:
            dM = cfuselegs(ops, dA, 2, 2)
            dlam = _mm_dag(ops, dM, v)
            Y = cmatmul_real(ops, _diag_inverse(ops, s), _dag_mm(ops, u, dM))
            dQf = clincomb(ops, [(1.0, Y), (-1.0, _mm(ops, _mm_dag(ops, Y, v), v))])
            dQ = csplitleg(ops, dQf, 2, sp)
        As[l], dAs[l] = Q, dQ
        env[l + 1] = updateright4(ops, env[l + 2], Q, Ws[l], Q)
        denv[l + 1] = _env_tangent(ops, updateright4, env[l + 2], denv[l + 2], Q, dQ, Ws[l],
                                   dWs[l])
        L0, R0 = env[l], env[l + 1]
        lam, dlam = _expo_pair(ops, lambda x: apply0(ops, x, L0, R0),
                               _h0_tangent(ops, L0, denv[l], R0, denv[l + 1]), 1j * dt, lam,
                               dlam, krylovdim, tol, stats)
        A = ccontract(ops, As[l - 1], (1, 2, -1), lam, (-1, 3))
        dA = _sum(ops, [(1.0, None if dlam is None else ccontract(ops, As[l - 1], (1, 2, -1),
                                                                   dlam, (-1, 3))),
                        (1.0, None if dAs[l - 1] is None else ccontract(ops, dAs[l - 1],
                                                                         (1, 2, -1), lam,
                                                                         (-1, 3)))])
        L, R = env[l - 1], env[l + 1]
        A, dA = _expo_pair(ops, lambda x: apply1(ops, x, L, R, Ws[l - 1]),
                           _h1_tangent(ops, L, denv[l - 1], R, denv[l + 1], Ws[l - 1],
                                       dWs[l - 1]), -1j * dt, A, dA, krylovdim, tol, stats)
    As[0], dAs[0] = A, dA
    return As, dAs, env, denv


def _transfer_bra_ket(ops: Ops, L, Abra, Aket, op=None):
    """L <- L . conj(Abra) [. op] . Aket (``tdvp._transfer`` with separate bra and ket)."""
    t = ccontract(ops, L, (-1, 1), cdual(ops, Abra), (-1, 2, 3))
    if op is not None:
        t = ccontract(ops, t, (1, -1, 3), op, (-1, 2))
    return ccontract(ops, t, (-1, -2, 1), Aket, (-1, -2, 2))


def expectation_tangent(ops: Ops, As, dAs, site_ops: dict):
    """(<psi|O|psi> / <psi|psi>, its derivative) for O = prod_x site_ops[x] (1-based sites)."""
    V0 = cspace(ops, As[0])[0]
    L0 = CTensor(ops.fill(1.0, 0, (V0, ops.dual_space(V0))))
    L, N, dL, dN = L0, L0, None, None
    for x, (A, dA) in enumerate(zip(As, dAs), start=1):
        op = site_ops.get(x)
        nL = _transfer(ops, L, A, op)
        nN = _transfer(ops, N, A)
        dL = _sum(ops, [(1.0, None if dL is None else _transfer(ops, dL, A, op)),
                        (1.0, None if dA is None else _transfer_bra_ket(ops, L, A, dA, op)),
                        (1.0, None if dA is None else _transfer_bra_ket(ops, L, dA, A, op))])
        dN = _sum(ops, [(1.0, None if dN is None else _transfer(ops, dN, A)),
                        (1.0, None if dA is None else _transfer_bra_ket(ops, N, A, dA)),
                        (1.0, None if dA is None else _transfer_bra_ket(ops, N, dA, A))])
        L, N = nL, nN
    total = lambda T: 0.0 if T is None else complex(cdownload(ops, T).sum())
    num, den = total(L), total(N)
    dnum, dden = total(dL), total(dN)
    return num / den, (dnum * den - num * dden) / den ** 2


def evolve_with_tangent(ops: Ops, As, Ws, dWs, dt: float, sweeps: int, site_ops: dict,
                        turning: str = "symmetric", krylovdim: int = 30, tol: float = 1e-12,
                        stats: TangentStats | None = None):
    """Evolve the center-1 MPS ``As`` (list of CTensor, modified in place) by ``sweeps`` 1-site
    TDVP sweeps of dt under the MPO Ws, carrying tangents with respect to the coupling whose
    MPO derivative is dWs (the initial state does not depend on it). Returns (<O>(t),
    d<O>(t)/dp) for O = prod site_ops."""
    from .tdvp import initialenv
    env = initialenv(ops, As, Ws)
    dAs = [None] * len(As)
    denv = initialenv_tangent(ops, As, dAs, Ws, dWs, env)
    for _ in range(sweeps):
        tdvp1sitesweep_tangent(ops, dt, As, dAs, Ws, dWs, env, denv, turning=turning,
                               krylovdim=krylovdim, tol=tol, stats=stats)
    return expectation_tangent(ops, As, dAs, site_ops)


# ---------------------------------------------------------------------------------------------
# reverse mode: adjoints of the sweep, environments recomputed from per-sweep checkpoints
# ---------------------------------------------------------------------------------------------
_FRESH = 1000  # offset of the negative labels that pair legs in an adjoint contraction


def _cscale_any(ops, X, z):
    return clincomb(ops, [(complex(z), X)])


def _contract_vjp_one(ops, ix, Y, iy, dC):
    """Cotangent of X in C = ccontract(X, ix, Y, iy) for the cotangent dC (dL = Re<dC, dC_>):
    dX = dC contracted with conj(Y) (``cdual``: conjugated, dual spaces) on the legs C took
    from Y; a full contraction (C a number) gives dX = dC * conj(Y) in X's leg order."""
    if not any(lab > 0 for lab in ix + iy):
        if tuple(ix) != tuple(iy):
            raise ValueError("full contraction adjoint needs matching leg order")
        return _cscale_any(ops, cdual(ops, Y), dC)
    nC = sum(1 for lab in ix + iy if lab > 0)
    idx_dc = []
    for p in range(1, nC + 1):
        idx_dc.append(ix.index(p) + 1 if p in ix else -(_FRESH + p))
    idx_y = [-(_FRESH + lab) if lab > 0 else ix.index(lab) + 1 for lab in iy]
    return ccontract(ops, dC, tuple(idx_dc), cdual(ops, Y), tuple(idx_y))


class _Tape:
    """Records the sweep's primitive operations with their adjoints; ``backward`` propagates
    cotangents (dL = Re <x_bar, dx>) from seeds to every recorded input, matched by identity."""

    def __init__(self, ops):
        self.ops = ops
        self.rec = []

    def contract(self, A, ia, B, ib):
        ia, ib = tuple(int(x) for x in ia), tuple(int(x) for x in ib)
        C = ccontract(self.ops, A, ia, B, ib)
        ops = self.ops
        self.rec.append(((A, B), (C,), lambda g: (_contract_vjp_one(ops, ia, B, ib, g[0]),
                                                   _contract_vjp_one(ops, ib, A, ia, g[0]))))
        return C

    def dual(self, A):
        D = cdual(self.ops, A)
        ops = self.ops
        self.rec.append(((A,), (D,), lambda g: (cdual(ops, g[0]),)))
        return D

    def fuse(self, A, l, n):
        M = cfuselegs(self.ops, A, l, n)
        sp = cspace(self.ops, A)[l - 1:l - 1 + n]
        ops = self.ops
        self.rec.append(((A,), (M,), lambda g: (csplitleg(ops, g[0], l, sp),)))
        return M

    def split(self, M, l, sp):
        A = csplitleg(self.ops, M, l, sp)
        ops, n = self.ops, len(sp)
        self.rec.append(((M,), (A,), lambda g: (cfuselegs(ops, g[0], l, n),)))
        return A

    def custom(self, inputs, outputs, vjp):
        self.rec.append((tuple(inputs), tuple(outputs), vjp))

    def backward(self, seeds):
        ops = self.ops
        grads = {}

        def acc(x, g):
            if g is None or x is None:
                return
            k = id(x)
            grads[k] = g if k not in grads else clincomb(ops, [(1.0, grads[k]), (1.0, g)])

        for x, g in seeds:
            acc(x, g)
        for inputs, outputs, vjp in reversed(self.rec):
            gs = [grads.get(id(o)) for o in outputs]
            if all(g is None for g in gs):
                continue
            for i, o in enumerate(outputs):  # an output's cotangent is consumed here
                if gs[i] is None:
                    gs[i] = cscale(ops, o, 0.0)
            for x, g in zip(inputs, vjp(gs)):
                acc(x, g)
        return lambda x: grads.get(id(x))


def _gauss_legendre(q):
    x, w = np.polynomial.legendre.leggauss(q)
    return 0.5 * (x + 1.0), 0.5 * w


def _apply_tape(ops, kind, v, L, R, W):
    """The 1-site (kind 1) or 0-site (kind 0) H_eff of ``tdvp`` on a private tape."""
    tp = _Tape(ops)
    if kind == 1:  # apply1
        t = tp.contract(L, (-1, 2, 1), v, (-1, 3, 4))
        t = tp.contract(t, (1, -1, -2, 4), W, (-1, 2, 3, -2))
        out = tp.contract(t, (1, 2, -1, -2), R, (-2, -1, 3))
    else:  # apply0
        t = tp.contract(L, (-1, 2, 1), v, (-1, 3))
        out = tp.contract(t, (1, -1, -2), R, (-2, -1, 2))
    return tp, out


def exponentiate_family(ops: Ops, f, t, x, fracs, krylovdim: int = 30, tol: float = 1e-12,
                        maxiter: int = 100):
    """[exp(p t f) x for p in fracs] (0 <= p <= 1, f Hermitian) from the Lanczos bases of one
    integration of exp(t f) x: the same Krylov recurrence, a-posteriori error control and step
    halving as ``ctensor.exponentiate``; every p that falls in a restart segment is evaluated
    from that segment's basis (exp of the tridiagonal at the partial time), so the whole family
    costs what the single exponential costs. Returns (list, ExpInfo); ``converged`` also checks
    each p's own error estimate."""
    from .ctensor import ExpInfo, _expT
    fr = [float(p) for p in fracs]
    if any(p < 0.0 or p > 1.0 for p in fr):
        raise ValueError("fractions must lie in [0, 1]")
    out = {p: x for p in fr if p == 0.0}
    scale = cnorm(ops, x)
    if scale == 0.0:
        return [x for _ in fr], ExpInfo(0, 0, True)
    pending = sorted(set(p for p in fr if p > 0.0))
    v = cscale(ops, x, 1.0 / scale)
    start = 0.0
    numops = numsteps = 0
    converged = True
    while pending and numsteps < maxiter:
        numsteps += 1
        V = [v]
        alphas, betas = [], []
        left = 1.0 - start
        step, b = None, 0.0
        for j in range(krylovdim):
            w = f(V[j])
            numops += 1
            a = 0.0
            for rep in range(2):
                coef = cdots(ops, V, w)
                if rep == 0:
                    a = coef[j].real
                w = clincomb(ops, [(1.0, w)] + [(-cu, u) for cu, u in zip(coef, V)])
            b = cnorm(ops, w)
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
            V.append(cscale(ops, w, 1.0 / b))
        end = 1.0 if step >= left else start + step
        m = len(alphas)
        while pending and pending[0] <= end:
            p = pending.pop(0)
            cp = _expT(alphas, betas, (p - start) * t)
            if b * abs(cp[m - 1]) * scale > tol and b > 1e-14 * max(1.0, abs(alphas[-1])):
                converged = False
            out[p] = clincomb(ops, [(complex(cp[i]) * scale, V[i]) for i in range(m)])
        if not pending:
            break
        y = clincomb(ops, [(complex(c[i]) * scale, V[i]) for i in range(m)])
        start = end
        scale = cnorm(ops, y)
        v = cscale(ops, y, 1.0 / scale)
    if pending:
        converged = False
        for p in pending:
            out[p] = cscale(ops, x, 0.0)
    return [out[p] for p in fr], ExpInfo(numops, numsteps, converged)


def _expo_vjp(ops, kind, L, R, W, tau, x, ybar, krylovdim, tol, quad):
    """Adjoint of y = exp(tau F) x, F the Hermitian H_eff built from (L, R, W):
    x_bar = exp(conj(tau) F) y_bar, and for the operands of F the gradient of
    Re tau int_0^1 <exp(s conj(tau) F) y_bar, dF exp((1-s) tau F) x> ds by Gauss-Legendre
    quadrature (``quad`` nodes), each node one adjoint of the H_eff's contractions. The node
    vectors come from two Krylov integrations (``exponentiate_family`` of y_bar under conj(tau),
    which also gives x_bar, and of x under tau). Returns (x_bar, gL, gR, gW, ExpInfo list)."""
    if kind == 1:
        f = lambda v: apply1(ops, v, L, R, W)
    else:
        f = lambda v: apply0(ops, v, L, R)
    s_nodes, weights = _gauss_legendre(quad)
    us, iu = exponentiate_family(ops, f, np.conj(tau), ybar, list(s_nodes) + [1.0],
                                 krylovdim=krylovdim, tol=tol)
    vs, iv = exponentiate_family(ops, f, tau, x, [1.0 - s for s in s_nodes],
                                 krylovdim=krylovdim, tol=tol)
    xbar = us[-1]
    gL = gR = gW = None
    for u, v, w in zip(us, vs, weights):
        tp, out = _apply_tape(ops, kind, v, L, R, W)
        grad = tp.backward([(out, cscale(ops, u, w * np.conj(tau)))])
        gL = _sum(ops, [(1.0, gL), (1.0, grad(L))])
        gR = _sum(ops, [(1.0, gR), (1.0, grad(R))])
        if kind == 1:
            gW = _sum(ops, [(1.0, gW), (1.0, grad(W))])
    return xbar, gL, gR, gW, (iu, iv)


def _same_shape_inverse(ops, s):
    """s^-1 with s's own legs and sectors (block (c1, c2) = diag(1 / s_(c1, c2)))."""
    blocks = {}
    for key, b in s.blocks.items():
        b = np.asarray(b, dtype=np.float64)
        d = b if b.ndim == 1 else np.diagonal(b)
        blocks[key] = np.diag(np.where(d != 0.0, 1.0 / np.where(d != 0.0, d, 1.0), 0.0))
    return ops.from_blocks(s.charge, ops.space(s), blocks)


def _sweep_taped(ops, tp, dt, As, Ws, env, turning, krylovdim, tol, quad, stats):
    """``tdvp.tdvp1sitesweep`` on a tape (same operations, same state); As and env in place."""
    lx = len(As)
    As[:] = [creal(A) for A in As]

    def expo(kind, l_env, r_env, W, tau, x):
        L, R = env[l_env], env[r_env]
        f = (lambda v: apply1(ops, v, L, R, W)) if kind == 1 else (lambda v: apply0(ops, v, L, R))
        y, info = exponentiate(ops, f, tau, x, krylovdim=krylovdim, tol=tol)
        if stats is not None:
            stats.add(info.numops, info.converged)
        ins = (x, L, R) + ((W,) if kind == 1 else ())

        def vjp(g, kind=kind, L=L, R=R, W=W, tau=tau, x=x):
            xb, gL, gR, gW, infos = _expo_vjp(ops, kind, L, R, W, tau, x, g[0], krylovdim,
                                              tol, quad)
            if stats is not None:
                for info in infos:
                    stats.add(info.numops, info.converged)
            return (xb, gL, gR) + ((gW,) if kind == 1 else ())
        tp.custom(ins, (y,), vjp)
        return y

    def gauge(A, left):
        M = tp.fuse(A, 1, 2) if left else tp.fuse(A, 2, 2)
        u, s, v = csvd(ops, M)
        sinv = _same_shape_inverse(ops, s)
        if left:
            Qf, lam = u, cmatmul_real(ops, s, v)

            def vjp(g, u=u, v=v, sinv=sinv):
                Qb, lb = g
                Y = _mm(ops, Qb, cmatmul_real(ops, sinv, v))
                Y = clincomb(ops, [(1.0, Y), (-1.0, _mm(ops, u, _dag_mm(ops, u, Y)))])
                return (clincomb(ops, [(1.0, Y), (1.0, _mm(ops, u, lb))]),)
        else:
            Qf, lam = v, cmatmul_real_right(ops, u, s)

            def vjp(g, u=u, v=v, sinv=sinv):
                Qb, lb = g
                Z = _mm(ops, cmatmul_real_right(ops, u, sinv), Qb)
                Z = clincomb(ops, [(1.0, Z), (-1.0, _mm(ops, _mm_dag(ops, Z, v), v))])
                return (clincomb(ops, [(1.0, Z), (1.0, _mm(ops, lb, v))]),)
        tp.custom((M,), (Qf, lam), vjp)
        return Qf, lam

    def upd_left(e, Q, W):
        t = tp.contract(e, (-1, 3, 4), Q, (-1, 2, 1))
        t = tp.contract(t, (1, -1, -2, 4), W, (-2, 2, 3, -1))
        return tp.contract(t, (1, -1, 2, -2), tp.dual(Q), (-2, -1, 3))

    def upd_right(e, Q, W):
        t = tp.contract(e, (-1, 3, 4), Q, (1, 2, -1))
        t = tp.contract(t, (1, -1, -2, 4), W, (3, 2, -2, -1))
        return tp.contract(t, (1, -1, 2, -2), tp.dual(Q), (3, -1, -2))

    A = As[0]
    for l in range(1, lx):
        A = expo(1, l - 1, l + 1, Ws[l - 1], -1j * dt, A)
        Qf, lam = gauge(A, True)
        Q = tp.split(Qf, 1, cspace(ops, A)[0:2])
        As[l - 1] = Q
        env[l] = upd_left(env[l - 1], Q, Ws[l - 1])
        lam = expo(0, l, l + 1, None, 1j * dt, lam)
        A = tp.contract(lam, (1, -1), As[l], (-1, 2, 3))
    t_turn = 2.0 * dt if turning == "symmetric" else dt
    A = expo(1, lx - 1, lx + 1, Ws[lx - 1], -1j * t_turn, A)
    for l in range(lx - 1, 0, -1):
        Qf, lam = gauge(A, False)
        Q = tp.split(Qf, 2, cspace(ops, A)[1:3])
        As[l] = Q
        env[l + 1] = upd_right(env[l + 2], Q, Ws[l])
        lam = expo(0, l, l + 1, None, 1j * dt, lam)
        A = tp.contract(As[l - 1], (1, 2, -1), lam, (-1, 3))
        A = expo(1, l - 1, l + 1, Ws[l - 1], -1j * dt, A)
    As[0] = A
    return As, env


def _initialenv_taped(ops, tp, As, Ws):
    """``tdvp.initialenv`` on a tape (the right environments as functions of As and Ws)."""
    lx = len(As)
    env = [None] * (lx + 2)
    lVa = cspace(ops, As[0])[0]
    rVa = ops.dual_space(cspace(ops, As[-1])[2])
    lVw = ops.space(Ws[0])[0]
    rVw = ops.dual_space(ops.space(Ws[-1])[2])
    env[0] = CTensor(ops.fill(1.0, 0, (ops.dual_space(lVa), ops.dual_space(lVw), lVa)))
    env[lx + 1] = CTensor(ops.fill(1.0, 0, (rVa, rVw, ops.dual_space(rVa))))
    for l in range(lx, 0, -1):
        t = tp.contract(env[l + 1], (-1, 3, 4), As[l - 1], (1, 2, -1))
        t = tp.contract(t, (1, -1, -2, 4), Ws[l - 1], (3, 2, -2, -1))
        env[l] = tp.contract(t, (1, -1, 2, -2), tp.dual(As[l - 1]), (3, -1, -2))
    return env


def _expectation_taped(ops, tp, As, site_ops):
    """(num, den) = (<psi|O|psi>, <psi|psi>) as numbers on the tape (transfers, then the sum of
    the last transfer's entries as a contraction with ones)."""
    V0 = cspace(ops, As[0])[0]
    L0 = CTensor(ops.fill(1.0, 0, (V0, ops.dual_space(V0))))
    L, N = L0, L0

    def transfer(T, A, op):
        t = tp.contract(T, (-1, 1), tp.dual(A), (-1, 2, 3))
        if op is not None:
            t = tp.contract(t, (1, -1, 3), op, (-1, 2))
        return tp.contract(t, (-1, -2, 1), A, (-1, -2, 2))

    for x, A in enumerate(As, start=1):
        L = transfer(L, A, site_ops.get(x))
        N = transfer(N, A, None)
    sp = cspace(ops, L)
    ones = CTensor(ops.fill(1.0, 0, tuple(ops.dual_space(V) for V in sp)))
    num = tp.contract(L, (-1, -2), ones, (-1, -2))
    den = tp.contract(N, (-1, -2), ones, (-1, -2))
    return num, den, L, N


def evolve_with_adjoint(ops: Ops, As, Ws, dt: float, sweeps: int, site_ops: dict,
                        turning: str = "symmetric", krylovdim: int = 30, tol: float = 1e-12,
                        quad: int = 8, stats: TangentStats | None = None):
    """Reverse mode of ``sweeps`` 1-site TDVP sweeps of the center-1 MPS ``As`` under the MPO
    ``Ws``, for C = Re <psi|O|psi> / <psi|psi> (O = prod site_ops) at the end. Forward: the
    plain sweeps, keeping only the MPS at the start of each sweep (checkpoints; the MPO and the
    site operators are the other inputs). Backward, sweep by sweep from the last: the
    environments are recomputed from the checkpoint, the sweep is replayed on a tape and the
    cotangents pass through it (adjoint contractions, the gauge moves' adjoints, and for every
    Krylov exponential exp(conj(t) F) on the cotangent plus a Gauss-Legendre quadrature of its
    coupling gradient). Returns (C, grad_W, grad_A0): cotangents of every MPO tensor (real part
    is the gradient for a real MPO) and of every initial site tensor. ``As`` ends evolved."""
    from .tdvp import initialenv, tdvp1sitesweep
    if turning not in TURNING:
        raise ValueError(f"turning must be one of {TURNING}")
    # cotangents are kept per tensor object: sites that share one MPO tensor (a uniform chain)
    # get their own copy so that each site's gradient is returned separately
    Ws = [ops.lincomb([(1.0, W)]) for W in Ws]
    checkpoints = []
    env = initialenv(ops, As, Ws)
    for _ in range(sweeps):
        checkpoints.append([creal(A) for A in As])
        tdvp1sitesweep(ops, dt, As, Ws, env, turning=turning, krylovdim=krylovdim, tol=tol)
    # the observable and its cotangents on the final state
    tp = _Tape(ops)
    final = list(As)
    out_num, out_den, _, _ = _expectation_taped(ops, tp, final, site_ops)
    num, den = complex(out_num), complex(out_den)
    C = num / den
    # L = Re(num / den): cotangents conj(dL/dnum), conj(dL/dden) of the recorded scalars
    gnum = np.conj(1.0 / den)
    gden = np.conj(-num / den ** 2)
    g = tp.backward([(out_num, gnum), (out_den, gden)])
    cot = [g(A) for A in final]
    gW = [g(W) for W in Ws]
    for k in range(sweeps - 1, -1, -1):
        start = [creal(A) for A in checkpoints[k]]
        tp = _Tape(ops)
        work = list(start)
        env0 = _initialenv_taped(ops, tp, work, Ws)
        env = list(env0)
        _sweep_taped(ops, tp, dt, work, Ws, env, turning, krylovdim, tol, quad, stats)
        seeds = [(A, c) for A, c in zip(work, cot) if c is not None]
        g = tp.backward(seeds)
        cot = [g(A) for A in start]
        gW = [_sum(ops, [(1.0, a), (1.0, g(W))]) for a, W in zip(gW, Ws)]
    return C, gW, cot
