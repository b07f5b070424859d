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


# ---------------------------------------------------------------------------------------------
# MPS (src/symmps.jl) and the 2-site DMRG sweep (src/dmrg.jl) on device tensors
# ---------------------------------------------------------------------------------------------
class MPState:
    """``MPState``: site tensors (Vl, d, dual(Vr)) and the orthogonality center (symmps.jl:1-4)."""

    def __init__(self, As, center: int = 0):
        self.As = list(As)
        self.center = center

    def __len__(self):
        return len(self.As)


def bond_dims(lx, site, M, chimax):
    """Charges of the bond right of ``site`` as in src/symmps.jl:59-62 (d = 2), each with
    dimension min(chimax, #left states, #right states)."""
    cmin = max(0, M - (lx - site))
    cmax = min(M, site)
    return [(c, max(1, min(chimax, math.comb(site, c), math.comb(lx - site, M - c))))
            for c in range(cmin, cmax + 1)]


def random_mps_host(lx: int, M: int, chimax: int, seed: int = 1911):
    """(charge, spaces, flat) per site of a random U(1) MPS with total charge M: blocks N(0,1)
    from a Philox stream in reference block order."""
    rng = np.random.Generator(np.random.Philox(seed))
    d = U1Space(*SITE)
    Vl = U1Space((0, 1))
    out = []
    for site in range(1, lx + 1):
        Vr = VectorSpace(bond_dims(lx, site, M, chimax))
        sp = (Vl, d, dual(Vr))
        n = mg.meta(0, sp).numel()
        out.append((0, sp, rng.standard_normal(n)))
        Vl = Vr
    return out


def binomial_bond_dims(lx, site, M, chimax):
    """Charges of the bond right of ``site`` with a total dimension of about ``chimax``: each
    charge c gets chimax * w_c / sum(w) states (w_c = C(site, c) C(lx - site, M - c), the number
    of basis states through that charge), at least 1 and at most the exact count."""
    exact = bond_dims(lx, site, M, 1 << 62)
    if sum(d for _, d in exact) <= chimax:
        return exact
    w = [math.comb(site, c) * math.comb(lx - site, M - c) for c, _ in exact]
    tot = float(sum(w))
    return [(c, max(1, min(d, int(round(chimax * wc / tot))))) for (c, d), wc in zip(exact, w)]


def binomial_mps_host(lx: int, M: int, chimax: int, seed: int = 1911):
    """Like random_mps_host but with bond dimensions from binomial_bond_dims, so every bond
    holds about chimax states in total (the workload of a sweep at fixed maximal chi)."""
    rng = np.random.Generator(np.random.Philox(seed))
    d = U1Space(*SITE)
    Vl = U1Space((0, 1))
    out = []
    for site in range(1, lx + 1):
        Vr = VectorSpace(binomial_bond_dims(lx, site, M, chimax))
        sp = (Vl, d, dual(Vr))
        n = mg.meta(0, sp).numel()
        out.append((0, sp, rng.standard_normal(n)))
        Vl = Vr
    return out


def mps_from_host(sites, ctx=None) -> MPState:
    return MPState([mg.from_flat(c, sp, f, ctx) for c, sp, f in sites], center=0)


def _factor(M, keep, svd):
    """Full (untruncated) per-sector factorisation M = u s v with the ``keep`` factor
    orthonormal: the exact SVD (_svd_) or the density-matrix method."""
    if svd == "exact":
        return mg._svd_(M)
    return mg.svdtrunc(M, maxdim=max(M.size()), tol=0.0, method="gram_" + keep)


def _pushleft(mps: MPState, l: int, svd="exact", normalize=False):
    """``_pushleft!`` (src/symmps.jl:167-174), 1-based ``l``."""
    A = mps.As[l - 1]
    u, s, v = _factor(mg.fuselegs(A, 2, 2), "right", svd)
    if normalize:
        mg.rmul(s, 1.0 / mg.norm(s))
    mps.As[l - 1] = mg.splitleg(v, 2, A.space[1:3])
    mps.As[l - 2] = mg.contract(mps.As[l - 2], (1, 2, -1), mg.matmul(u, s, precision=0), (-1, 3),
                                precision=0)


def _pushright(mps: MPState, l: int, svd="exact", normalize=False):
    """``_pushright!`` (src/symmps.jl:176-183)."""
    A = mps.As[l - 1]
    u, s, v = _factor(mg.fuselegs(A, 1, 2), "left", svd)
    if normalize:
        mg.rmul(s, 1.0 / mg.norm(s))
    mps.As[l - 1] = mg.splitleg(u, 1, A.space[0:2])
    mps.As[l] = mg.contract(mg.matmul(s, v, precision=0), (1, -1), mps.As[l], (-1, 2, 3),
                            precision=0)


def center_at(mps: MPState, center: int, svd: str = "exact",
              normalize: bool = False) -> MPState:
    """``center_at!`` (src/symmps.jl:185-200). ``svd="gram"`` canonicalises with the
    density-matrix factorisation (same bond spaces, orthonormal site tensors). ``normalize``
    rescales the singular values passed on at every step to unit norm: the state keeps its
    direction while its norm, which for a long random MPS grows or shrinks geometrically (and
    whose Gram matrices square it), stays 1."""
    x1, xL = 1, len(mps)
    if mps.center > 0:
        x1 = xL = mps.center
    for p in range(x1, center):
        _pushright(mps, p, svd, normalize)
    for p in range(xL, center, -1):
        _pushleft(mps, p, svd, normalize)
    mps.center = center
    return mps


def initialenv(mps: MPState, Ws, at: int = 1, precision: int = 0):
    """``initialenv`` (src/dmrg.jl:9-36): boundary environments of ones, then right updates."""
    if mps.center != at:
        raise mg.SpaceMismatch(2, f"MPS center has to be {at}")
    lx = len(mps)
    ctx = mps.As[0].ctx
    env = [None] * (lx + 2)
    lVa = mps.As[0].space[0]
    rVa = dual(mps.As[-1].space[2])
    lVw = Ws[0].space[0]
    rVw = dual(Ws[-1].space[2])
    env[0] = mg.fill(1.0, 0, (dual(lVa), dual(lVw), lVa), ctx)
    env[lx + 1] = mg.fill(1.0, 0, (rVa, rVw, dual(rVa)), ctx)
    for l in range(lx, at - 1, -1):
        env[l] = mg.mpsupdateright(env[l + 1], mps.As[l - 1], Ws[l - 1], precision=precision)
    for l in range(1, at):
        env[l] = mg.mpsupdateleft(env[l - 1], mps.As[l - 1], Ws[l - 1], precision=precision)
    return env


class SweepOptions:
    """Keyword arguments of ``dmrg2sitesweep!`` (src/dmrg.jl:58-66) plus the precision split:
    ``precision`` for the Krylov matvecs, ``energy_precision`` for the post-truncation energy
    matvec (dmrg.jl:92-93) and ``env_precision`` for environment updates. ``svd`` selects the
    truncation: "exact" per-sector SVD (the reference's svdtrunc) or "gram", the density-matrix
    truncation that keeps the new site tensor orthonormal (u going right, v going left)."""

    def __init__(self, maxdim=200, tol=1e-9, lanczostol=1e-7, krylovdim=5, krylovmaxiter=8,
                 tieband=0.0, precision=0, energy_precision=0, env_precision=0, svd="exact"):
        if svd not in ("exact", "gram"):
            raise ValueError(f"svd must be 'exact' or 'gram', not {svd!r}")
        self.svd = svd
        self.maxdim = maxdim
        self.tol = tol
        self.lanczostol = lanczostol
        self.krylovdim = krylovdim
        self.krylovmaxiter = krylovmaxiter
        self.tieband = tieband
        self.precision = precision
        self.energy_precision = energy_precision
        self.env_precision = env_precision


def _truncate_and_energy(v, AA, env, Ws, l, o: SweepOptions, keep="left", tick=None):
    """svdtrunc + normalisation + post-truncation energy (dmrg.jl:88-93); ``keep`` names the
    factor that becomes the new (orthonormal) site tensor."""
    import time
    t = time.perf_counter()
    method = "exact" if o.svd == "exact" else "gram_" + keep
    u, s, vt = mg.svdtrunc(mg.SymMatrix(v, [1, 2], [3, 4]), maxdim=o.maxdim, tol=o.tol,
                           tieband=o.tieband, method=method)
    if tick:
        t = tick("svdtrunc", t)
    ns = mg.norm(s)
    truncerr = 1.0 - ns
    mg.rmul(s, 1.0 / ns)
    usv = mg.matmul(mg.matmul(u, s, precision=0), vt, precision=0)
    AA = mg.splitleg(mg.splitleg(usv, 2, AA.space[2:4]), 1, AA.space[0:2])
    e = mg.dot(AA, mg.applymps2site(AA, env[l - 1], env[l + 2], Ws[l - 1], Ws[l],
                                    precision=o.energy_precision))
    if tick:
        tick("energy", t)
    return u, s, vt, AA, e, truncerr


def _prefetch(env, i):
    """Hint to an environment store that keeps entries off the device (``OffloadedEnvs``):
    entry ``i`` is read soon. Plain lists ignore it."""
    f = getattr(env, "prefetch", None)
    if f is not None and 0 <= i < len(env):
        f(i)


def _eig(AA, env, Ws, l, o: SweepOptions, stats):
    e, v, info = mg.eigsolve_heff2(AA, env[l - 1], env[l + 2], Ws[l - 1], Ws[l],
                                   krylovdim=o.krylovdim, maxiter=o.krylovmaxiter,
                                   tol=o.lanczostol, precision=o.precision)
    if stats is not None:
        stats.append(info)
    return v


class PhaseTimer:
    """Wall time per sweep phase (eigensolve, svdtrunc, energy, environment update), each phase
    closed by a device synchronisation; pass one as ``timing=`` to dmrg2sitesweep."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.s = {}

    def __call__(self, name, t0):
        import time
        self.ctx.synchronize()
        t1 = time.perf_counter()
        self.s[name] = self.s.get(name, 0.0) + (t1 - t0)
        return t1


def sweep_steps(mps: MPState, Ws, env, o: SweepOptions, timing: PhaseTimer | None = None):
    """``dmrg2sitesweep!`` (src/dmrg.jl:58-179) as a generator: before each of the sweep's
    eigensolves it yields ``(AA, l)`` (the two-site tensor and the 1-based bond; the operator is
    that of env[l-1], env[l+2], Ws[l-1], Ws[l]) and takes the ground-state vector sent back.
    Returns the energy list. ``dmrg2sitesweep`` answers each request with its own eigensolve;
    a lock-step driver answers the requests of many chains with one batched eigensolve."""
    import time
    tick = (lambda name, t0: timing(name, t0)) if timing else (lambda name, t0: t0)
    now = time.perf_counter
    lx = len(mps)
    if mps.center != 1:
        raise mg.SpaceMismatch(2, "The center of MPS has to be 1 for dmrg L->R->L")
    energies = []
    A = mps.As[0]
    t = now()
    for l in range(1, lx - 1):
        _prefetch(env, l + 3)  # the right environment of the next bond
        AA = mg.contract(A, (1, 2, -1), mps.As[l], (-1, 3, 4), precision=0)
        v = yield AA, l
        t = tick("eigsolve", t)
        u, s, vt, AA, e, _ = _truncate_and_energy(v, AA, env, Ws, l, o, tick=timing)
        energies.append(e)
        t = now()
        mps.As[l - 1] = mg.splitleg(u, 1, A.space[0:2])
        env[l] = mg.mpsupdateleft(env[l - 1], mps.As[l - 1], Ws[l - 1], precision=o.env_precision)
        A = mg.splitleg(mg.matmul(s, vt, precision=0), 2, AA.space[2:4])
        t = tick("environment", t)
    l = lx - 1
    AA = mg.contract(A, (1, 2, -1), mps.As[l], (-1, 3, 4), precision=0)
    v = yield AA, l
    t = tick("eigsolve", t)
    e = None
    for l in range(lx - 1, 1, -1):
        _prefetch(env, l - 2)  # the left environment of the next bond
        u, s, vt, AA, e, _ = _truncate_and_energy(v, AA, env, Ws, l, o, keep="right",
                                                  tick=timing)
        energies.append(e)
        t = now()
        mps.As[l] = mg.splitleg(vt, 2, AA.space[2:4])
        env[l + 1] = mg.mpsupdateright(env[l + 2], mps.As[l], Ws[l], precision=o.env_precision)
        A = mg.splitleg(mg.matmul(u, s, precision=0), 1, AA.space[0:2])
        t = tick("environment", t)
        AA = mg.contract(mps.As[l - 2], (1, 2, -1), A, (-1, 3, 4), precision=0)
        v = yield AA, l - 1
        t = tick("eigsolve", t)
        energies.append(e)
    l = 1
    u, s, vt, AA, e, _ = _truncate_and_energy(v, AA, env, Ws, l, o, keep="right", tick=timing)
    t = now()
    energies.append(e)
    mps.As[1] = mg.splitleg(vt, 2, AA.space[2:4])
    env[2] = mg.mpsupdateright(env[3], mps.As[1], Ws[1], precision=o.env_precision)
    mps.As[0] = mg.splitleg(mg.matmul(u, s, precision=0), 1, AA.space[0:2])
    tick("environment", t)
    return energies


def dmrg2sitesweep(mps: MPState, Ws, env, opts: SweepOptions | None = None, stats=None,
                   timing: PhaseTimer | None = None, **kw):
    """``dmrg2sitesweep!`` (src/dmrg.jl:58-179): one left-to-right-to-left sweep on the GPU.
    Returns the reference's energy list (3L-5 post-truncation energies; the right-to-left loop
    pushes each energy twice, dmrg.jl:132,156). ``timing`` (a PhaseTimer) accumulates the wall
    time of the eigensolves, truncations (svdtrunc), post-truncation energies and environment
    updates."""
    o = opts or SweepOptions(**kw)
    gen = sweep_steps(mps, Ws, env, o, timing)
    try:
        AA, l = next(gen)
        while True:
            AA, l = gen.send(_eig(AA, env, Ws, l, o, stats))
    except StopIteration as stop:
        return stop.value


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


# ---------------------------------------------------------------------------------------------
# many independent chains (the batched workload): one context (CUDA stream) per chain
# ---------------------------------------------------------------------------------------------
def chain_ensemble(n: int, seed: int = 1911, lengths=(32, 128), deltas=(0.0, 1.5),
                   chis=(128, 256, 512, 1024)):
    """(L, Delta, maxdim) of n independent XXZ chains: L uniform over the even lengths in
    ``lengths``, Delta uniform in ``deltas``, maxdim drawn from ``chis`` (Philox ``seed``)."""
    rng = np.random.Generator(np.random.Philox(seed))
    out = []
    for _ in range(n):
        L = 2 * int(rng.integers(lengths[0] // 2, lengths[1] // 2 + 1))
        out.append((L, float(rng.uniform(*deltas)), int(rng.choice(chis))))
    return out


def run_chains(specs, nsweeps: int, opts: SweepOptions, threads: int | None = None,
               device: int = 0, seed: int = 7):
    """2-site DMRG on independent chains (L, Delta, maxdim), each with its own context, so its
    kernels go to its own CUDA stream; ``threads`` host threads drive them (1 = one after the
    other). Every chain starts from a random binomial-profile MPS (Philox seed + index),
    canonicalised and with environments built, then runs ``nsweeps`` sweeps. Returns the last
    post-truncation energy of each chain."""
    from concurrent.futures import ThreadPoolExecutor

    results = [None] * len(specs)

    def work(i):
        L, delta, chi = specs[i]
        ctx = mg.Context(device)
        Ws = xxz_u1mpo(L, delta, ctx=ctx)
        mps = mps_from_host(binomial_mps_host(L, L // 2, chi, seed + i), ctx)
        center_at(mps, 1, svd=opts.svd, normalize=True)  # long random chains: keep the norm 1
        env = initialenv(mps, Ws)
        o = SweepOptions(**{**opts.__dict__, "maxdim": chi})
        es = None
        for _ in range(nsweeps):
            es = dmrg2sitesweep(mps, Ws, env, o)
        ctx.synchronize()
        results[i] = es[-1]

    with ThreadPoolExecutor(max_workers=max(1, threads or len(specs))) as ex:
        list(ex.map(work, range(len(specs))))
    return results


def _chain_sweeps(mps, Ws, env, o, nsweeps):
    es = None
    for _ in range(nsweeps):
        es = yield from sweep_steps(mps, Ws, env, o)
    return es


def run_chains_lockstep(specs, nsweeps: int, opts: SweepOptions, device: int = 0, seed: int = 7,
                        graph: bool = True, stats=None, max_batch: int = 128,
                        wait_all: bool = True):
    """2-site DMRG on independent chains (L, Delta, maxdim) with batched eigensolves. Every
    chain runs its sweeps on its own context and host thread (as ``run_chains``), as a
    ``sweep_steps`` generator, and prepares its share of each eigensolve there (host planning
    and W folds, ``Heff2.prepare``); one batcher answers all requests waiting at that moment
    with ONE batched Lanczos on its own context (``HeffBatch.from_prepared``:
    every Krylov application one grouped launch per phase for all those chains, replayed from a
    CUDA graph, split GEMMs with tuned tiles; FP64 recurrences). With ``wait_all`` the batcher
    waits until every chain still sweeping has a request (lock step); otherwise it takes what is
    waiting (then without graph capture: the other chains' threads keep working meanwhile).
    Same start states as ``run_chains`` (Philox seed + index). Returns the last
    post-truncation energy of each chain; ``stats`` (a dict) collects batch counts, chains per
    batch, batcher times and the tuner's runs and hits."""
    import threading
    import time
    if opts.precision < 2:
        raise ValueError("batched eigensolves run the split-precision Krylov matvecs: "
                         "precision >= 2")
    n = len(specs)
    bctx = mg.Context(device)
    cv = threading.Condition()
    waiting, answers = {}, {}
    release = []  # the batcher's vectors, dropped by the batcher between its own launches
    active = set(range(n))
    results = [None] * n
    failed = []
    record = {"batches": 0, "chains_per_batch": [], "batch_build_s": 0.0,
              "batched_eigsolve_s": 0.0}

    def chain(i):
        try:
            L, delta, chi = specs[i]
            ctx = mg.Context(device)
            Ws = xxz_u1mpo(L, delta, ctx=ctx)
            mps = mps_from_host(binomial_mps_host(L, L // 2, chi, seed + i), ctx)
            center_at(mps, 1, svd=opts.svd, normalize=True)
            env = initialenv(mps, Ws)
            o = SweepOptions(**{**opts.__dict__, "maxdim": chi})
            gen = _chain_sweeps(mps, Ws, env, o, nsweeps)
            req = next(gen)
            while True:
                AA, l = req
                # this chain's share of the batch (host planning and W folds) on its own context
                op = mg.Heff2.prepare(AA, env[l - 1], env[l + 2], Ws[l - 1], Ws[l],
                                      precision=opts.precision)
                ctx.synchronize()  # the batcher's stream reads these tensors
                with cv:
                    waiting[i] = (op, AA)
                    cv.notify_all()
                    cv.wait_for(lambda: i in answers or failed)
                    if failed:
                        return
                    v = answers.pop(i)
                del op
                vec = mg.copy(v, ctx)
                ctx.synchronize()
                with cv:  # freed on the batcher's stream: only the batcher may release it
                    release.append(v)
                del v
                try:
                    req = gen.send(vec)
                except StopIteration as stop:
                    results[i] = stop.value[-1]
                    return
        except BaseException as e:  # noqa: BLE001 (re-raised in the caller)
            with cv:
                failed.append(e)
                cv.notify_all()
        finally:
            with cv:
                active.discard(i)
                cv.notify_all()

    def batcher():
        try:
            while True:
                with cv:
                    cv.wait_for(lambda: failed or not active or
                                (waiting and (not wait_all or len(waiting) >= len(active))))
                    if failed or (not active and not waiting):
                        return
                    batch = dict(waiting)
                    waiting.clear()
                    release.clear()
                ids = sorted(batch)
                for k in range(0, len(ids), max_batch):
                    part = ids[k:k + max_batch]
                    t0 = time.perf_counter()
                    # dynamic batches run uncaptured: the other chains' threads keep issuing
                    # their own work (first launches load kernels) while a capture would run
                    B = mg.HeffBatch.from_prepared([batch[i][0] for i in part], bctx,
                                                   graph=graph and wait_all)
                    bctx.synchronize()  # the chains' operators may go once this is done
                    t1 = time.perf_counter()
                    _, vecs, _ = B.eigsolve([batch[i][1] for i in part],
                                            krylovdim=opts.krylovdim,
                                            maxiter=opts.krylovmaxiter, tol=opts.lanczostol)
                    del B
                    bctx.synchronize()
                    record["batch_build_s"] += t1 - t0
                    record["batched_eigsolve_s"] += time.perf_counter() - t1
                    record["batches"] += 1
                    record["chains_per_batch"].append(len(part))
                    with cv:
                        answers.update(zip(part, vecs))
                        cv.notify_all()
        except BaseException as e:  # noqa: BLE001
            with cv:
                failed.append(e)
                cv.notify_all()

    threads = [threading.Thread(target=chain, args=(i,)) for i in range(n)]
    tb = threading.Thread(target=batcher)
    for t in threads:
        t.start()
    tb.start()
    for t in threads:
        t.join()
    tb.join()
    if failed:
        raise failed[0]
    if stats is not None:
        runs, hits = mg.tuner(bctx)
        stats.update({**record, "tuner_runs": runs, "tuner_hits": hits})
    return results
