"""Model inputs and DMRG drivers on the GPU library (host side of TensorNetAlgs / symmpo.jl).

* ``xxz_u1mpo`` mirrors src/symmpo.jl:45-97 (U(1) XXZ MPO, bond space (-1=>1, 0=>3, 1=>1)).
* ``binomial_profile`` / ``heff_problem`` build the chi-dimensional H_eff workload: bond spaces
  over 25 charges with a binomial profile, random N(0,1) blocks from a seeded Philox stream.
"""
from __future__ import annotations

import math

import numpy as np

from . import symtensors as mg
from .symtensors import VectorSpace, U1Space, dual

MPO_BOND = ((-1, 1), (0, 3), (1, 1))
SITE = ((0, 1), (1, 1))


def binomial_profile(chi: int, ncharges: int = 25):
    """Dimensions chi*C(n-1,k)/2^(n-1) rounded by largest remainder with a floor of one state per
    charge; symmetric in k and summing to chi."""
    n = ncharges - 1
    q = [chi * math.comb(n, k) / 2.0 ** n for k in range(ncharges)]
    base = [max(1, int(math.floor(x))) for x in q]
    deficit = chi - sum(base)
    # hand out (or take back) states in symmetric pairs by remainder, centre charge last
    order = sorted(range(ncharges), key=lambda k: (-(q[k] - math.floor(q[k])), abs(k - n / 2)))
    step = 1 if deficit > 0 else -1
    i = 0
    while deficit != 0 and i < 10 * ncharges:
        k = order[i % ncharges]
        mirror = n - k
        if k == mirror:
            if abs(deficit) >= 1 and base[k] + step >= 1:
                base[k] += step
                deficit -= step
        elif abs(deficit) >= 2 and base[k] + step >= 1 and base[mirror] + step >= 1:
            base[k] += step
            base[mirror] += step
            deficit -= 2 * step
        i += 1
    if deficit != 0:
        base[n // 2] += deficit
    return base


def xxz_blocks(delta: float, kind: str):
    """Blocks of the XXZ MPO tensors of src/symmpo.jl:45-97: ``kind`` = 'beg', 'mid' or 'end'.
    Returns (space, {sector: block}) with zero blocks for the remaining allowed sectors."""
    mat0 = np.array([[1.0, 0.0, 0.0], [-0.5 * delta, 0.0, 0.0], [0.0, -0.5, 1.0]])
    mat1 = np.array([[1.0, 0.0, 0.0], [0.5 * delta, 0.0, 0.0], [0.0, 0.5, 1.0]])
    V0 = U1Space((0, 1))
    V = U1Space(*MPO_BOND)
    d = U1Space(*SITE)
    F = dict(order="F")
    if kind == "mid":
        space = (V, d, dual(V), dual(d))
        set_ = {
            (0, 0, 0, 0): mat0.reshape((3, 1, 3, 1), **F),
            (0, 1, 0, 1): mat1.reshape((3, 1, 3, 1), **F),
            (0, 1, 1, 0): np.array([0.0, 0.0, 1.0]).reshape((3, 1, 1, 1), **F),
            (0, 0, -1, 1): np.array([0.0, 0.0, 1.0]).reshape((3, 1, 1, 1), **F),
            (1, 0, 0, 1): 0.5 * np.array([1.0, 0.0, 0.0]).reshape((1, 1, 3, 1), **F),
            (-1, 1, 0, 0): 0.5 * np.array([1.0, 0.0, 0.0]).reshape((1, 1, 3, 1), **F),
        }
    elif kind == "beg":
        space = (V0, d, dual(V), dual(d))
        set_ = {
            (0, 0, 0, 0): mat0[2, :].reshape((1, 1, 3, 1), **F),
            (0, 1, 0, 1): mat1[2, :].reshape((1, 1, 3, 1), **F),
            (0, 1, 1, 0): np.ones((1, 1, 1, 1)),
            (0, 0, -1, 1): np.ones((1, 1, 1, 1)),
        }
    elif kind == "end":
        space = (V, d, V0, dual(d))
        set_ = {
            (0, 0, 0, 0): mat0[:, 0].reshape((3, 1, 1, 1), **F),
            (0, 1, 0, 1): mat1[:, 0].reshape((3, 1, 1, 1), **F),
            (-1, 1, 0, 0): 0.5 * np.ones((1, 1, 1, 1)),
            (1, 0, 0, 1): 0.5 * np.ones((1, 1, 1, 1)),
        }
    else:
        raise ValueError(kind)
    return space, set_


def _tensor_from_partial_blocks(space, blocks, charge=0, ctx=None, meta_only=False):
    m = mg.meta(charge, space)
    if meta_only:
        return m
    flat = np.zeros(m.numel())
    for s, z, o in zip(m.sectors(), m.block_sizes(), m.offsets()):
        if s in blocks:
            b = np.asarray(blocks[s], dtype=np.float64)
            if tuple(b.shape) != tuple(z):
                raise mg.SpaceMismatch(2, f"SizeMismatch() at {s}")
            flat[o:o + b.size] = b.ravel(order="F")
    unknown = set(blocks) - set(m.sectors())
    if unknown:
        raise mg.SpaceMismatch(2, f"Block doesn't exist: {sorted(unknown)}")
    return mg.from_flat(charge, space, flat, ctx)


def xxz_u1mpo(lx: int, delta: float = 1.0, ctx=None, meta_only=False):
    """``xxz_u1mpo(Float64, lx, 2, delta)`` (src/symmpo.jl:45-97) as device tensors."""
    out = []
    for site in range(1, lx + 1):
        kind = "beg" if site == 1 else ("end" if site == lx else "mid")
        sp, bl = xxz_blocks(delta, kind)
        out.append(_tensor_from_partial_blocks(sp, bl, ctx=ctx, meta_only=meta_only))
    return out


def heff_spaces(chi: int, ncharges: int = 25):
    """Spaces of the chi-dimensional two-site H_eff workload (v, envL, envR, W1, W2)."""
    Vb = VectorSpace([(k, d) for k, d in enumerate(binomial_profile(chi, ncharges))])
    d = U1Space(*SITE)
    Vw = U1Space(*MPO_BOND)
    v = (Vb, d, d, dual(Vb))
    envL = (dual(Vb), dual(Vw), Vb)
    envR = (Vb, Vw, dual(Vb))
    return v, envL, envR


def heff_inputs_host(chi: int, delta: float = 0.5, seed: int = 1911, ncharges: int = 25):
    """Flat float64 arrays (reference block order) of v, envL, envR plus the W structure, drawn
    from a Philox stream so that the oracle and the device get identical inputs."""
    sv, sl, sr = heff_spaces(chi, ncharges)
    rng = np.random.Generator(np.random.Philox(seed))
    flats = []
    for sp in (sv, sl, sr):
        n = mg.meta(0, sp).numel()
        flats.append(rng.standard_normal(n))
    return (sv, sl, sr), flats


def heff_problem(chi: int, delta: float = 0.5, seed: int = 1911, ctx=None, meta_only=False,
                 ncharges: int = 25):
    """(v, envL, envR, W1, W2) of the chi-dimensional H_eff matvec workload."""
    (sv, sl, sr), flats = (heff_spaces(chi, ncharges), None) if meta_only else \
        heff_inputs_host(chi, delta, seed, ncharges)
    sp, bl = xxz_blocks(delta, "mid")
    W = _tensor_from_partial_blocks(sp, bl, ctx=ctx, meta_only=meta_only)
    if meta_only:
        return (mg.meta(0, sv), mg.meta(0, sl), mg.meta(0, sr), W, W)
    v, eL, eR = (mg.from_flat(0, s, f, ctx) for s, f in zip((sv, sl, sr), flats))
    return v, eL, eR, W, W


HEFF_STEPS = (((-1, 2, 1), (-1, 3, 4, 5)), ((1, -1, -2, 4, 5), (-1, 2, 3, -2)),
              ((1, 2, -1, -2, 5), (-1, 3, 4, -2)), ((1, 2, 3, -1, -2), (-2, -1, 4)))


def heff_flops_meta(v, envL, envR, W1, W2):
    """Planned algorithmic flops (sum of 2*M*N*K) of the four H_eff contractions
    (src/apply.jl:99-103), from structure-only tensors."""
    partners = (v, W1, W2, envR)
    t = envL
    total = 0.0
    for k, ((ia, ib), B) in enumerate(zip(HEFF_STEPS, partners)):
        if k == 0:
            total += mg.contract_flops(envL, ia, v, ib)
            t = mg.contract(envL, ia, v, ib)
        else:
            total += mg.contract_flops(t, ia, B, ib)
            t = mg.contract(t, ia, B, ib)
    return total
