"""U(1) MPOs of spin-1/2 Hamiltonians on lattices (the role of ``_generatempo_sym``,
src/mpogen.jl:153-352), built on the host as sector blocks.

A Hamiltonian is a list of terms, each a product of single-site operators (S+, S-, Sz, with
U(1) charges +1, -1, 0 on the site space (0 => down, 1 => up)) on increasing sites with an
amplitude. The MPO is a finite-state machine on the bond: a "done" channel (charge 0, all terms
finished), a "start" channel (charge 0, nothing placed yet) and one channel per term that has
started and not finished, carrying the charge of the operators placed so far. At each site a
term starts (start -> its channel), passes (identity), continues (operator, channel -> channel)
or finishes (operator, channel -> done); single-site terms go from start to done. The bond
dimension is 2 + the number of terms crossing the bond, as in the reference (one channel per
open term, no compression). Channels are ordered by charge, and within a charge: done first,
open terms in the order they started, start last.

``cylinder_heisenberg_terms`` gives the J1 Heisenberg model on a W x L cylinder (periodic
around the circumference, open along the length) with the column-major site order of the
reference (y fastest, src/model3.jl:86-87): bond dimension 2 + 3 W. ``j1j2_chain_terms`` and
``triangular_terms`` give the reference's j1j2 chain and triangular-lattice spin models
(src/spinmodels.jl:14-110), the latter with its four-spin ring exchange, expanded into products
of single-site operators by ``ring_exchange_terms``.
"""
from __future__ import annotations

import numpy as np

SZ = np.diag([-0.5, 0.5])             # basis (down, up) = charges (0, 1)
SP = np.array([[0.0, 0.0], [1.0, 0.0]])  # down -> up, charge +1
SM = SP.T.copy()                      # charge -1
EYE = np.eye(2)
OPS = {"Z": (SZ, 0), "P": (SP, 1), "M": (SM, -1), "I": (EYE, 0)}


def heisenberg_bond_terms(i, j, J=1.0, delta=1.0):
    """J (S+_i S-_j / 2 + S-_i S+_j / 2 + delta Sz_i Sz_j) with i < j."""
    if i > j:
        i, j = j, i
    return [((i, j), ("P", "M"), 0.5 * J), ((i, j), ("M", "P"), 0.5 * J),
            ((i, j), ("Z", "Z"), J * delta)]


def cylinder_heisenberg_terms(width, length, J=1.0):
    """J1 Heisenberg terms on a width x length cylinder, sites numbered x*width + y (0-based)."""
    site = lambda x, y: x * width + y
    terms = []
    for x in range(length):
        for y in range(width):
            if width > 2 or y + 1 < width:  # around the circumference (a 2-wide ring is one bond)
                terms += heisenberg_bond_terms(site(x, y), site(x, (y + 1) % width), J)
            if x + 1 < length:
                terms += heisenberg_bond_terms(site(x, y), site(x + 1, y), J)
    return terms


def j1j2_chain_terms(lx, j1, j2):
    """Heisenberg chain with nearest (j1) and next-nearest (j2) neighbour couplings, open ends
    (``j1j2model``, src/spinmodels.jl:14-40)."""
    terms = []
    for i in range(lx):
        if j1 != 0 and i + 1 < lx:
            terms += heisenberg_bond_terms(i, i + 1, j1)
        if j2 != 0 and i + 2 < lx:
            terms += heisenberg_bond_terms(i, i + 2, j2)
    return terms


def _op_basis_expansion(H, n):
    """Amplitudes of an n-site operator (2^n x 2^n, site 0 most significant) on the products of
    Sz, S+, S-, 1: the four are orthogonal under tr(A^T B), so each amplitude is a trace ratio
    (the decomposition of ``nbodyopexpansion``, src/spin_definitions.jl:86-130)."""
    names = ("Z", "P", "M", "I")
    out = []
    for idx in np.ndindex(*(4,) * n):
        M = np.ones((1, 1))
        norm = 1.0
        for k in idx:
            op = OPS[names[k]][0]
            M = np.kron(M, op)
            norm *= float(np.sum(op * op))
        amp = float(np.sum(M * H)) / norm
        if abs(amp) > 1e-14:
            out.append((tuple(names[k] for k in idx), amp))
    return out


def _ring_matrix(n):
    """C + C^-1 for the cyclic shift of n spins (``ringexchangeoperator``,
    src/spin_definitions.jl:74-84): a basis state's bits rotate by one place."""
    P = np.zeros((2 ** n, 2 ** n))
    for j in range(2 ** n):
        i = (j >> 1) | ((j & 1) << (n - 1))
        P[i, j] = 1.0
    return P + P.T


_RING4 = None


def ring_exchange_terms(sites, k):
    """k (C + C^-1 - 1/4) on four sites in their cyclic order (the reference's ring term R4,
    src/spinmodels.jl:79-81): traceless, so every product term has at least one non-identity
    factor; identity factors are dropped and the factors sorted by site."""
    global _RING4
    if _RING4 is None:
        _RING4 = _op_basis_expansion(_ring_matrix(4) - 0.25 * np.eye(16), 4)
    terms = []
    for names, amp in _RING4:
        pairs = sorted((s, o) for s, o in zip(sites, names) if o != "I")
        terms.append((tuple(s for s, _ in pairs), tuple(o for _, o in pairs), k * amp))
    return terms


def triangular_terms(ly, lx, j1, j2, j3, k1=0.0, k2=0.0, k3=0.0, periodic_y=False):
    """Spin-1/2 model on the ly x lx triangular lattice (``triangularspinmodel``,
    src/spinmodels.jl:42-110): Heisenberg couplings j1, j2, j3 along the (dy, dx) offsets (0, 1),
    (1, 0), (1, -1) and ring exchanges k1, k2, k3 on the plaquettes given there, sites numbered
    x * ly + y (y fastest), open along x, open or periodic (ly > 2) along y."""
    if periodic_y and ly <= 2:
        raise ValueError("periodic y needs ly > 2")

    def site(y, x):
        if periodic_y:
            y %= ly
        if not (0 <= y < ly and 0 <= x < lx):
            return None
        return x * ly + y

    bonds = ((j1, (0, 1)), (j2, (1, 0)), (j3, (1, -1)))
    rings = ((k1, ((0, 0), (0, 1), (1, 1), (1, 0))), (k2, ((0, 0), (0, 1), (1, 0), (1, -1))),
             (k3, ((0, 0), (1, 0), (0, 1), (-1, 1))))
    terms = []
    for x in range(lx):
        for y in range(ly):
            for J, (dy, dx) in bonds:
                t = site(y + dy, x + dx)
                if J != 0 and t is not None:
                    terms += heisenberg_bond_terms(site(y, x), t, J)
            for K, offs in rings:
                ss = [site(y + dy, x + dx) for dy, dx in offs]
                if K != 0 and None not in ss:
                    terms += ring_exchange_terms(ss, K)
    return terms


def chain_xxz_terms(lx, delta):
    terms = []
    for i in range(lx - 1):
        terms += heisenberg_bond_terms(i, i + 1, 1.0, delta)
    return terms


def mpo_blocks(n_sites, terms, share_prefixes=False):
    """Per site: (space, {sector: block}) of the MPO tensor W(Vl, d, dual(Vr), dual(d)).
    Spaces are (charges, dims, isdual) triples per leg, usable with VectorSpace.

    By default every open term has its own channel, as in the reference. With
    ``share_prefixes`` a channel stands for the operators placed so far: open terms with the
    same placed (site, operator) sequence share it until they diverge, and each term's amplitude
    sits on its finishing edge (summed over terms with the same full sequence). Every path from
    the start channel to the done channel is then the sequence of exactly one distinct term, so
    the MPO is the same Hamiltonian with fewer channels."""
    terms = sorted(((tuple(s), tuple(o), float(a)) for s, o, a in terms), key=lambda t: t[0])
    for s, o, _ in terms:
        if len(s) != len(o) or list(s) != sorted(s) or len(set(s)) != len(s):
            raise ValueError(f"term sites must increase: {s}")
        if s[-1] >= n_sites:
            raise ValueError(f"term beyond the lattice: {s}")

    def key(k, p):  # the channel of term k once its first p operators are placed
        if not share_prefixes:
            return ("t", k)
        s, o, _ = terms[k]
        return ("p",) + tuple(zip(s[:p], o[:p]))

    def channels(open_terms):
        seen, out = set(), []
        for k, p, c in open_terms:
            name = key(k, p)
            if name not in seen:
                seen.add(name)
                out.append((c, name))
        return out

    open_terms = []  # (term index, next op position, accumulated charge), in start order
    out = []
    ti = 0
    for n in range(n_sites):
        # left channels: [(charge, name)]: done, open terms (or prefixes), start
        left = []
        if n > 0:
            left.append((0, "done"))
            left += channels(open_terms)
        left.append((0, "start"))
        trans = {}  # (left name, right name, op) -> amplitude

        def add(ln, rn, op, amp, finishing):
            if finishing:  # amplitudes of terms with the same full sequence add up
                trans[(ln, rn, op)] = trans.get((ln, rn, op), 0.0) + amp
            else:  # an edge shared by several terms has weight 1
                trans[(ln, rn, op)] = amp

        new_open = []
        if n > 0:
            add("done", "done", "I", 1.0, False)
        for (k, p, c) in open_terms:
            s, o, a = terms[k]
            if s[p] == n:
                if p == len(s) - 1:
                    add(key(k, p), "done", o[p], a, True)
                else:
                    add(key(k, p), key(k, p + 1), o[p], 1.0, False)
                    new_open.append((k, p + 1, c + OPS[o[p]][1]))
            else:
                add(key(k, p), key(k, p), "I", 1.0, False)
                new_open.append((k, p, c))
        while ti < len(terms) and terms[ti][0][0] == n:
            s, o, a = terms[ti]
            if len(s) == 1:
                add("start", "done", o[0], a, True)
            else:
                add("start", key(ti, 1), o[0], 1.0, False)
                new_open.append((ti, 1, OPS[o[0]][1]))
            ti += 1
        if n < n_sites - 1:
            add("start", "start", "I", 1.0, False)
        open_terms = new_open
        right = [(0, "done")] + channels(open_terms)
        if n < n_sites - 1:
            right.append((0, "start"))
        else:
            if open_terms:
                raise ValueError("terms still open at the last site")
            right = [(0, "done")]
        if n == 0:
            left = [(0, "start")]
        out.append(_site_tensor(left, right, [(l, r, op, a) for (l, r, op), a in trans.items()]))
    return out


def _index(channels):
    """charge -> ordered names, and name -> (charge, position within the charge)."""
    by = {}
    for c, name in channels:
        by.setdefault(c, []).append(name)
    pos = {name: (c, by[c].index(name)) for c, names in by.items() for name in names}
    return by, pos


def _site_tensor(left, right, trans):
    lby, lpos = _index(left)
    rby, rpos = _index(right)
    Vl = (sorted(lby), [len(lby[c]) for c in sorted(lby)], False)
    Vr = (sorted(rby), [len(rby[c]) for c in sorted(rby)], True)
    d = ([0, 1], [1, 1], False)
    dd = ([0, 1], [1, 1], True)
    blocks = {}
    for ln, rn, opname, amp in trans:
        op, q = OPS[opname]
        cl, il = lpos[ln]
        cr, ir = rpos[rn]
        if cr != cl + q:
            raise ValueError("channel charge does not follow the operator charge")
        for s in (0, 1):
            for sp in (0, 1):
                v = op[s, sp]
                if v == 0.0:
                    continue
                sec = (cl, s, cr, sp)
                if sec not in blocks:
                    blocks[sec] = np.zeros((len(lby[cl]), 1, len(rby[cr]), 1))
                blocks[sec][il, 0, ir, 0] += amp * v
    return (Vl, d, Vr, dd), blocks


def device_mpo(n_sites, terms, ctx=None, meta_only=False, share_prefixes=False):
    """The MPO of ``terms`` as library tensors W(Vl, d, dual(Vr), dual(d)) (zero blocks for the
    allowed sectors no term touches); ``share_prefixes`` as in ``mpo_blocks``."""
    from . import symtensors as mg
    from .dmrg import _tensor_from_partial_blocks
    out = []
    for legs, blocks in mpo_blocks(n_sites, terms, share_prefixes=share_prefixes):
        sp = tuple(mg.VectorSpace(list(zip(c, dims)), isd) for c, dims, isd in legs)
        out.append(_tensor_from_partial_blocks(sp, blocks, ctx=ctx, meta_only=meta_only))
    return out


def dense_mpo(site_tensors):
    """The full 2^n x 2^n matrix of an MPO given as mpo_blocks output (host check, small n).
    Basis index bits: site 0 is the most significant, 1 = up."""
    mats = []
    for (Vl, _, Vr, _), blocks in site_tensors:
        lo = {c: o for c, o in zip(Vl[0], np.cumsum([0] + Vl[1][:-1]))}
        ro = {c: o for c, o in zip(Vr[0], np.cumsum([0] + Vr[1][:-1]))}
        W = np.zeros((sum(Vl[1]), 2, sum(Vr[1]), 2))
        for (cl, s, cr, sp), b in blocks.items():
            W[lo[cl]:lo[cl] + b.shape[0], s, ro[cr]:ro[cr] + b.shape[2], sp] = b[:, 0, :, 0]
        mats.append(W)
    # contract: T[a, s..., b, s'...]; basis up = index 1 in the site space
    T = mats[0][0]  # (s, b, s')
    H = np.einsum("sbt->bst", T)  # (b, s, s')
    for W in mats[1:]:
        H = np.einsum("bIJ,bscp->cIsJp", H, W)
        nb = H.shape[0]
        H = H.reshape(nb, H.shape[1] * 2, H.shape[3] * 2)
    return H[0]
