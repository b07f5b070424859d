"""Measurements on MPS (src/symmps.jl:202-221,245-371,452-482): local and two-point expectation
values, MPO expectation values, overlaps, norms and Schmidt spectra.

Every function takes real MPS (site tensors as library ``SymTensor``s) or complex ones
(``ctensor.CTensor``, e.g. from time evolution) and runs as block-sparse contractions on the GPU
(``ops`` defaults to the library's operations). Expectation values are computed by left-to-right
transfer without moving the orthogonality center: <psi|O|psi> unnormalised, the value the
reference returns for its (normalised, canonical) states, without mutating the MPS.
"""
from __future__ import annotations

import numpy as np

from . import ctensor as ct
from . import tdvp as td


def _ops(ops):
    return ops if ops is not None else ct.gpu_ops()


def _sites(mps):
    return list(mps.As) if hasattr(mps, "As") else list(mps)


def _left_boundary(ops, A):
    V0 = ct.cspace(ops, A)[0]
    return ct.CTensor(ops.fill(1.0, 0, (V0, ops.dual_space(V0))))


def _close(ops, L) -> complex:
    return complex(ct.cdownload(ops, L).sum())


def _value(z: complex, real_input: bool):
    return z.real if real_input else z


def _is_real(As):
    return all(not isinstance(A, ct.CTensor) or A.im is None for A in As)


def _right_closures(ops, As):
    """R[x] for x = 1..L+1: the sites x..L of <psi|psi> closed at the right boundary, legs
    (ket, bra) of the bond left of site x; R[L+1] is the boundary of ones."""
    lx = len(As)
    Vend = ops.dual_space(ct.cspace(ops, As[-1])[2])
    R = [None] * (lx + 2)
    R[lx + 1] = ct.CTensor(ops.fill(1.0, 0, (Vend, ops.dual_space(Vend))))
    for x in range(lx, 1, -1):
        A = As[x - 1]
        t = ct.ccontract(ops, A, (1, 2, -1), R[x + 1], (-1, 3))
        R[x] = ct.ccontract(ops, t, (1, -1, -2), ct.cdual(ops, A), (2, -1, -2))
    return R


def _prefixes(ops, As):
    """L[x] for x = 0..L-1: sites 1..x of <psi|psi> (legs (bra, ket) of the bond right of x)."""
    L = _left_boundary(ops, As[0])
    out = [L]
    for A in As[:-1]:
        L = td._transfer(ops, L, A)
        out.append(L)
    return out


def _join(ops, L, R):
    return complex(ct.ccontract(ops, L, (-1, -2), R, (-2, -1)))


def measure_site(mps, op, l: int | None = None, ops=None) -> dict:
    """measure(mps, op, l) / measure(mps, op) (src/symmps.jl:245-282): {site: <psi|op_site|psi>}
    for one site or every site. ``op`` is a charge-0 tensor with legs (d, dual(d))."""
    ops = _ops(ops)
    As = _sites(mps)
    real = _is_real(As)
    sites = [l] if l is not None else list(range(1, len(As) + 1))
    for x in sites:
        if not 1 <= x <= len(As):
            raise ValueError(f"site {x} outside 1..{len(As)}")
    P, R = _prefixes(ops, As), _right_closures(ops, As)
    return {x: _value(_join(ops, td._transfer(ops, P[x - 1], As[x - 1], op), R[x + 1]), real)
            for x in sites}


def measure_pairs(mps, op1, op2, x1: int | None = None, x2: int | None = None,
                  ops=None) -> dict:
    """measure(mps, op1, op2, x1, x2) / measure(mps, op1, op2) (src/symmps.jl:284-343):
    {(x1, x2): <psi|op1_x1 op2_x2|psi>} for one pair or every pair x1 < x2."""
    ops = _ops(ops)
    As = _sites(mps)
    lx = len(As)
    real = _is_real(As)
    if x1 is not None:
        if x2 is None or not (0 < x1 < x2 <= lx):
            raise ValueError("need 0 < x1 < x2 <= L")
        pairs = {x1: {x2}}
    else:
        pairs = {a: set(range(a + 1, lx + 1)) for a in range(1, lx)}
    P, R = _prefixes(ops, As), _right_closures(ops, As)
    out = {}
    for a, bs in pairs.items():
        L1 = td._transfer(ops, P[a - 1], As[a - 1], op1)
        for x in range(a + 1, max(bs) + 1):
            if x in bs:
                L2 = td._transfer(ops, L1, As[x - 1], op2)
                out[(a, x)] = _value(_join(ops, L2, R[x + 1]), real)
            L1 = td._transfer(ops, L1, As[x - 1])
    return out


def measure_mpo(mps, Ws, ops=None) -> dict:
    """measure(mps, mpo) (src/symmps.jl:354-371): {1: <psi|W|psi>} by left environment updates
    (the network of _mpsupdateleft, src/apply.jl:49-58)."""
    ops = _ops(ops)
    As = _sites(mps)
    if len(Ws) != len(As):
        raise ValueError("MPO and MPS lengths differ")
    lVa = ct.cspace(ops, As[0])[0]
    lVw = ops.space(Ws[0])[0]
    L = ct.CTensor(ops.fill(1.0, 0, (ops.dual_space(lVa), ops.dual_space(lVw), lVa)))
    for A, W in zip(As, Ws):
        L = td.updateleft(ops, L, A, W)
    return {1: _value(_close(ops, L), _is_real(As))}


def overlap(mps1, mps2, ops=None):
    """overlap(mps1, mps2) = <psi_2|psi_1> (src/symmps.jl:452-473), not normalised."""
    ops = _ops(ops)
    A1, A2 = _sites(mps1), _sites(mps2)
    if len(A1) != len(A2):
        raise ValueError("MPS lengths differ")
    V0 = ct.cspace(ops, A1[0])[0]
    L = ct.CTensor(ops.fill(1.0, 0, (V0, ops.dual_space(V0))))
    for A, B in zip(A1, A2):
        t = ct.ccontract(ops, L, (-1, 1), ct.cdual(ops, B), (-1, 2, 3))
        L = ct.ccontract(ops, t, (-1, -2, 1), A, (-1, -2, 2))
    return _value(_close(ops, L), _is_real(A1) and _is_real(A2))


def norm(mps, ops=None) -> float:
    """norm(mps) = sqrt(Re <psi|psi>) (src/symmps.jl:482)."""
    return float(np.sqrt(max(np.real(overlap(mps, mps, ops)), 0.0)))


def schmidtvalues(mps, ops=None):
    """schmidtvalues(mps) (src/symmps.jl:202-218): the singular values across every bond,
    descending, from a left-to-right sweep of SVDs on a copy of the gauge (the MPS is not
    modified). The state must have its orthogonality center at site 1."""
    ops = _ops(ops)
    As = _sites(mps)
    A = ct.creal(As[0])
    values = []
    for l in range(1, len(As)):
        u, s, v = ct.csvd(ops, ct.cfuselegs(ops, A, 1, 2))
        values.append(np.sort(_diag_values(s))[::-1])
        A = ct.ccontract(ops, ct.cmatmul_real(ops, s, v), (1, -1), As[l], (-1, 2, 3))
    return values


def _diag_values(s):
    """The diagonal entries of a diagonal tensor (dense square blocks on the device, or 1-d
    blocks)."""
    blocks = s.blocks() if callable(getattr(s, "blocks", None)) else s.blocks
    out = []
    for b in blocks.values():
        b = np.asarray(b)
        out.extend(np.diag(b) if b.ndim == 2 else b)
    return np.asarray(out)


def entanglemententropy(mps, ops=None):
    """entanglemententropy(mps) (src/symmps.jl:221): -sum p log p with p = s^2 at every bond."""
    out = []
    for s in schmidtvalues(mps, ops):
        p = np.asarray(s) ** 2
        p = p[p > 0]
        out.append(float(-np.sum(p * np.log(p))))
    return out
