"""Time-dependent variational principle on U(1) block-sparse complex MPS (src/tdvp.jl).

The reference evolves dense complex MPS (``@tensor`` on ``Array``s, src/tdvp.jl:12-210,
src/apply.jl:2-91). Here the same sweeps run on symmetric tensors, so time evolution of a
charge-conserving Hamiltonian (XXZ, lattice MPOs) goes through the block-sparse contraction
engine: each effective Hamiltonian is a chain of complex contractions
(``ctensor.ccontract``, i.e. real contractions on the GPU), the Krylov exponential is
``ctensor.exponentiate`` and the gauge moves are per-sector complex SVDs (``mpsg_svd_complex``;
the reference uses a dense QR, tdvp.jl:35,61, an SVD gives the same isometry up to a unitary on
the bond, which the evolved state does not depend on).

Index conventions follow the reference's symmetric kernels: site tensor (Vl, d, dual(Vr)),
MPO tensor (V, d_out, dual(V), dual(d_in)), left environment (ket, mpo, bra) from
``_mpsupdateleft`` (src/apply.jl:49-58) and right environment from ``_mpsupdateright``
(:17-25), both with the bra conjugated. The 1-site and 0-site effective Hamiltonians are the
dense ones of src/apply.jl:2-7,70-78 written as contractions in the order of the symmetric
``_applymps2site`` (:93-105).

Turning point: ``turning="reference"`` evolves the last site (pair) once by dt between the
half-sweeps, as src/tdvp.jl:45-48,145-148 do; ``turning="symmetric"`` evolves it by 2 dt, which
makes a sweep the symmetric composition of the two projector-splitting half-sweeps (exact
evolution by 2 dt at full bond dimension).
"""
from __future__ import annotations

from .ctensor import (CTensor, Ops, cdual, ccontract, cdownload, cfuselegs, cmatmul_real,
                      cmatmul_real_right, creal, cspace, csplitleg, csvd, csymmatrix,
                      exponentiate)

TURNING = ("reference", "symmetric")


# ---------------------------------------------------------------------------------------------
# effective Hamiltonians and environments
# ---------------------------------------------------------------------------------------------
def apply0(ops: Ops, lam, envL, envR):
    """0-site: A[d,d'] = envL[u,m,d] lam[u,u'] envR[u',m,d'] (src/apply.jl:2-7)."""
    t = ccontract(ops, envL, (-1, 2, 1), lam, (-1, 3))
    return ccontract(ops, t, (1, -1, -2), envR, (-2, -1, 2))


def apply1(ops: Ops, v, envL, envR, W):
    """1-site: v[l,o,r] = envL[l',ml,l] v[l',o',r'] W[ml,o,mr,o'] envR[r',mr,r]
    (src/apply.jl:70-78)."""
    t = ccontract(ops, envL, (-1, 2, 1), v, (-1, 3, 4))
    t = ccontract(ops, t, (1, -1, -2, 4), W, (-1, 2, 3, -2))
    return ccontract(ops, t, (1, 2, -1, -2), envR, (-2, -1, 3))


def apply2(ops: Ops, v, envL, envR, W1, W2):
    """2-site: the chain of ``_applymps2site`` (src/apply.jl:93-105) on complex tensors."""
    t = ccontract(ops, envL, (-1, 2, 1), v, (-1, 3, 4, 5))
    t = ccontract(ops, t, (1, -1, -2, 4, 5), W1, (-1, 2, 3, -2))
    t = ccontract(ops, t, (1, 2, -1, -2, 5), W2, (-1, 3, 4, -2))
    return ccontract(ops, t, (1, 2, 3, -1, -2), envR, (-2, -1, 4))


def updateleft(ops: Ops, env, A, W):
    """``_mpsupdateleft`` (src/apply.jl:49-58) with the conjugated bra."""
    t = ccontract(ops, env, (-1, 3, 4), A, (-1, 2, 1))
    t = ccontract(ops, t, (1, -1, -2, 4), W, (-2, 2, 3, -1))
    return ccontract(ops, t, (1, -1, 2, -2), cdual(ops, A), (-2, -1, 3))


def updateright(ops: Ops, env, A, W):
    """``_mpsupdateright`` (src/apply.jl:17-25) with the conjugated bra."""
    t = ccontract(ops, env, (-1, 3, 4), A, (1, 2, -1))
    t = ccontract(ops, t, (1, -1, -2, 4), W, (3, 2, -2, -1))
    return ccontract(ops, t, (1, -1, 2, -2), cdual(ops, A), (3, -1, -2))


def initialenv(ops: Ops, As, Ws):
    """``initialenv(mps, mpo)`` at center 1 (src/dmrg.jl:9-36) for a complex MPS."""
    lx = len(As)
    env = [None] * (lx + 2)
    lVa = cspace(ops, As[0])[0]
    rVa = ops.dual_space(cspace(ops, As[-1])[2])
    lVw = ops.space(Ws[0])[0]
    rVw = ops.dual_space(ops.space(Ws[-1])[2])
    env[0] = CTensor(ops.fill(1.0, 0, (ops.dual_space(lVa), ops.dual_space(lVw), lVa)))
    env[lx + 1] = CTensor(ops.fill(1.0, 0, (rVa, rVw, ops.dual_space(rVa))))
    for l in range(lx, 0, -1):
        env[l] = updateright(ops, env[l + 1], As[l - 1], Ws[l - 1])
    return env


# ---------------------------------------------------------------------------------------------
# sweeps (src/tdvp.jl)
# ---------------------------------------------------------------------------------------------
class TDVPStats:
    def __init__(self):
        self.exponentials = 0
        self.matvecs = 0
        self.unconverged = 0

    def add(self, info):
        self.exponentials += 1
        self.matvecs += info.numops
        self.unconverged += 0 if info.converged else 1


def _expo(ops, f, t, x, krylovdim, tol, stats):
    y, info = exponentiate(ops, f, t, x, krylovdim=krylovdim, tol=tol)
    if stats is not None:
        stats.add(info)
    return y


def tdvp1sitesweep(ops: Ops, dt: float, As, Ws, env, turning: str = "reference",
                   krylovdim: int = 30, tol: float = 1e-12, stats: TDVPStats | None = None):
    """``tdvp1sitesweep!`` (src/tdvp.jl:12-89) on a center-1 complex MPS (list of CTensor,
    site 1 first); ``As`` and ``env`` are updated in place and returned."""
    if turning not in TURNING:
        raise ValueError(f"turning must be one of {TURNING}")
    lx = len(As)
    As[:] = [creal(A) for A in As]
    A = As[0]
    for l in range(1, lx):
        A = _expo(ops, lambda v: apply1(ops, v, env[l - 1], env[l + 1], Ws[l - 1]), -1j * dt, A,
                  krylovdim, tol, stats)
        u, s, v = csvd(ops, cfuselegs(ops, A, 1, 2))  # as _pushright!, src/symmps.jl:176-183
        Q = csplitleg(ops, u, 1, cspace(ops, A)[0:2])
        As[l - 1] = Q
        env[l] = updateleft(ops, env[l - 1], Q, Ws[l - 1])
        lam = cmatmul_real(ops, s, v)
        lam = _expo(ops, lambda x: apply0(ops, x, env[l], env[l + 1]), 1j * dt, lam, krylovdim,
                    tol, stats)
        A = ccontract(ops, lam, (1, -1), As[l], (-1, 2, 3))
    t_turn = 2.0 * dt if turning == "symmetric" else dt
    A = _expo(ops, lambda v: apply1(ops, v, env[lx - 1], env[lx + 1], Ws[lx - 1]), -1j * t_turn,
              A, krylovdim, tol, stats)
    for l in range(lx - 1, 0, -1):
        u, s, v = csvd(ops, cfuselegs(ops, A, 2, 2))  # as _pushleft!, src/symmps.jl:167-174
        Q = csplitleg(ops, v, 2, cspace(ops, A)[1:3])
        As[l] = Q
        env[l + 1] = updateright(ops, env[l + 2], Q, Ws[l])
        lam = cmatmul_real_right(ops, u, s)
        lam = _expo(ops, lambda x: apply0(ops, x, env[l], env[l + 1]), 1j * dt, lam, krylovdim,
                    tol, stats)
        A = ccontract(ops, As[l - 1], (1, 2, -1), lam, (-1, 3))
        A = _expo(ops, lambda v: apply1(ops, v, env[l - 1], env[l + 1], Ws[l - 1]), -1j * dt, A,
                  krylovdim, tol, stats)
    As[0] = A
    return As, env


def tdvp2sitesweep(ops: Ops, dt: float, As, Ws, env, maxdim: int = 200, tol: float = 1e-14,
                   tieband: float = 0.0, turning: str = "reference", krylovdim: int = 30,
                   ktol: float = 1e-12, stats: TDVPStats | None = None):
    """``tdvp2sitesweep!`` (src/tdvp.jl:105-210) on a center-1 complex MPS, in place; the
    truncation is the symmetric ``svdtrunc`` rule (absolute ``tol``, src/mpsutils.jl:89-112)."""
    if turning not in TURNING:
        raise ValueError(f"turning must be one of {TURNING}")
    lx = len(As)
    As[:] = [creal(A) for A in As]

    def split(AA):
        sp = cspace(ops, AA)
        u, s, v = csvd(ops, csymmatrix(ops, AA, [1, 2], [3, 4]), truncate=True, maxdim=maxdim,
                       tol=tol, tieband=tieband)
        return sp, u, s, v

    A = As[0]
    for l in range(1, lx - 1):
        AA = ccontract(ops, A, (1, 2, -1), As[l], (-1, 3, 4))
        AA = _expo(ops, lambda v: apply2(ops, v, env[l - 1], env[l + 2], Ws[l - 1], Ws[l]),
                   -1j * dt, AA, krylovdim, ktol, stats)
        sp, u, s, v = split(AA)
        As[l - 1] = csplitleg(ops, u, 1, sp[0:2])
        env[l] = updateleft(ops, env[l - 1], As[l - 1], Ws[l - 1])
        lam = csplitleg(ops, cmatmul_real(ops, s, v), 2, sp[2:4])
        A = _expo(ops, lambda x: apply1(ops, x, env[l], env[l + 2], Ws[l]), 1j * dt, lam,
                  krylovdim, ktol, stats)
    l = lx - 1
    t_turn = 2.0 * dt if turning == "symmetric" else dt
    AA = ccontract(ops, A, (1, 2, -1), As[l], (-1, 3, 4))
    AA = _expo(ops, lambda v: apply2(ops, v, env[l - 1], env[l + 2], Ws[l - 1], Ws[l]),
               -1j * t_turn, AA, krylovdim, ktol, stats)
    for l in range(lx - 1, 1, -1):
        sp, u, s, v = split(AA)
        As[l] = csplitleg(ops, v, 2, sp[2:4])
        env[l + 1] = updateright(ops, env[l + 2], As[l], Ws[l])
        lam = csplitleg(ops, cmatmul_real_right(ops, u, s), 1, sp[0:2])
        lam = _expo(ops, lambda x: apply1(ops, x, env[l - 1], env[l + 1], Ws[l - 1]), 1j * dt,
                    lam, krylovdim, ktol, stats)
        AA = ccontract(ops, As[l - 2], (1, 2, -1), lam, (-1, 3, 4))
        AA = _expo(ops, lambda v: apply2(ops, v, env[l - 2], env[l + 1], Ws[l - 2], Ws[l - 1]),
                   -1j * dt, AA, krylovdim, ktol, stats)
    sp, u, s, v = split(AA)
    As[1] = csplitleg(ops, v, 2, sp[2:4])
    env[2] = updateright(ops, env[3], As[1], Ws[1])
    As[0] = csplitleg(ops, cmatmul_real_right(ops, u, s), 1, sp[0:2])
    return As, env


# ---------------------------------------------------------------------------------------------
# measurements (src/symmps.jl:265-371, generalised to complex states)
# ---------------------------------------------------------------------------------------------
def site_operator(ops: Ops, dspace, diag_or_matrix, charge: int = 0):
    """A site operator with legs (d, dual(d)) and the given charge (the SymMatrix ops of
    src/symmps.jl:265-343): either a dict {site charge: diagonal value} (charge 0), or a dense
    d x d matrix <out|op|in> in the charge-ordered site basis, of which the blocks with
    c_out - c_in = charge are kept (e.g. S+ with charge +1, S- with charge -1)."""
    blocks = {}
    if isinstance(diag_or_matrix, dict):
        if charge != 0:
            raise ValueError("a diagonal operator has charge 0")
        for c, _ in dspace.sectors:
            b = diag_or_matrix[c]
            blocks[(c, c)] = [[b]] if not hasattr(b, "__len__") else b
    else:
        import numpy as np
        m = np.asarray(diag_or_matrix, dtype=float)
        start, p = {}, 0
        for c, n in dspace.sectors:
            start[c] = (p, n)
            p += n
        for co, (po, no) in start.items():
            for ci, (pi, ni) in start.items():
                if co - ci == charge:
                    blocks[(co, ci)] = m[po:po + no, pi:pi + ni]
    return ops.from_blocks(charge, (dspace, ops.dual_space(dspace)), blocks)


def _transfer(ops: Ops, L, A, op=None):
    """L (bra, ket) <- L . conj(A) [. op] . A, the step of measure(mps, op1, op2, x1, x2)
    (src/symmps.jl:298-318)."""
    t = ccontract(ops, L, (-1, 1), cdual(ops, A), (-1, 2, 3))
    if op is not None:
        t = ccontract(ops, t, (1, -1, 3), op, (-1, 2))
    return ccontract(ops, t, (-1, -2, 1), A, (-1, -2, 2))


def expectation(ops: Ops, As, site_ops: dict) -> complex:
    """<psi| prod_x op_x |psi> / <psi|psi> by one left-to-right transfer (no gauge assumption);
    ``site_ops`` maps 1-based sites to charge-0 operators."""
    V0 = cspace(ops, As[0])[0]
    L0 = CTensor(ops.fill(1.0, 0, (V0, ops.dual_space(V0))))
    L, N = L0, L0
    for x, A in enumerate(As, start=1):
        L = _transfer(ops, L, A, site_ops.get(x))
        N = _transfer(ops, N, A)
    num = complex(cdownload(ops, L).sum())
    den = complex(cdownload(ops, N).sum())
    return num / den


def energy(ops: Ops, As, Ws, env) -> float:
    """<psi|H|psi> / <psi|psi> of a center-1 MPS from its environments (1-site H_eff at site 1)."""
    from .ctensor import cdot
    A = As[0]
    hv = apply1(ops, A, env[0], env[2], Ws[0])
    return (cdot(ops, A, hv) / cdot(ops, A, A)).real


def norm2(ops: Ops, As) -> float:
    V0 = cspace(ops, As[0])[0]
    N = CTensor(ops.fill(1.0, 0, (V0, ops.dual_space(V0))))
    for A in As:
        N = _transfer(ops, N, A)
    return float(cdownload(ops, N).sum().real)
