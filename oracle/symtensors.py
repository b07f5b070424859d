"""CPU oracle: a NumPy (float64 / complex128) restatement of the SymTensors layer of amiragha/mps.

TEST INFRASTRUCTURE ONLY.  This module is the checker for the GPU library: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``
may import it.  Nothing in ``mps_gb300`` imports or calls it.

Every function follows one reference routine and cites it (paths are relative to the reference
project root).  Leg positions are 1-based and index tuples are ncon-style, exactly as in the
reference, so tests written against this module read like the reference's own tests.

Representation
--------------
* A U(1) charge is a Python ``int`` (``src/group.jl:12-34``).
* A sector is a tuple of raw charge labels, one per leg.  Sectors are ordered column-major: the
  LAST leg is the slowest, i.e. by the reversed tuple (``src/sector.jl:35-36``).
* A block is an ``ndarray`` whose values are indexed like the Julia array (the memory order of
  numpy is irrelevant here; every reshape uses ``order='F'`` to keep Julia's column-major
  semantics).
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "VectorSpace", "U1Space", "dual_space", "isdual_pair", "fuse", "mapcharges_space",
    "allsectorsandsizes", "sector_key", "SymTensor", "SymDiagonal", "permutelegs", "fuselegs",
    "splitleg", "symmatrix", "symvector", "matmul", "split_matrix", "contract",
    "contract_index_perm", "dual", "array", "fill", "fill_linearindex", "eye", "from_blocks",
    "dot", "norm", "axpy", "axpby", "rmul", "scaled", "similar_zeros", "svd_", "svdtrunc",
    "truncatedsizes", "flatten", "from_flat", "SpaceMismatch", "FlopCount",
]


class FlopCount:
    """Context manager that sums the algorithmic flops of the sector GEMMs ``matmul`` performs
    while it is active: 2*M*N*K for every output block whose two partner blocks exist
    (contract.jl:284-291); allowed sectors without a partner (contract.jl:292-294) cost nothing.
    This is the flop count of the reference's own contraction order, which the benchmark's
    GFLOP/s figures use.  ``FlopCount().flops`` after the ``with`` block holds the total."""

    _active: list = []

    def __init__(self):
        self.flops = 0.0

    def __enter__(self):
        FlopCount._active.append(self)
        return self

    def __exit__(self, *exc):
        FlopCount._active.remove(self)
        return False


class SpaceMismatch(Exception):
    """Raised where the reference throws ``SpaceMismatch``/``SectorMismatch``/``error(...)``."""


# ---------------------------------------------------------------------------------------------
# Vector spaces  (src/vspace.jl)
# ---------------------------------------------------------------------------------------------
class VectorSpace:
    """Graded space charge -> dim with an ``isdual`` flag (``src/vspace.jl:5-18``)."""

    __slots__ = ("sectors", "isdual")

    def __init__(self, pairs, isdual: bool = False):
        pairs = [(int(c), int(d)) for c, d in pairs]
        charges = [c for c, _ in pairs]
        if len(set(charges)) != len(charges):  # vspace.jl:8-9
            raise SpaceMismatch(f"duplicate charges! {pairs}")
        for _, d in pairs:  # vspace.jl:11-13
            if d <= 0:
                raise SpaceMismatch("space dimension can only be positive!")
        self.sectors = tuple(sorted(pairs))  # SortedDict keeps keys ascending
        self.isdual = bool(isdual)

    def charges(self):
        return [c for c, _ in self.sectors]

    def dims(self):
        return [d for _, d in self.sectors]

    def dim(self, charge=None) -> int:
        """``dim(V, c)`` is 0 for an absent charge; ``dim(V)`` is the total (vspace.jl:42-45)."""
        if charge is None:
            return sum(self.dims())
        for c, d in self.sectors:
            if c == charge:
                return d
        return 0

    def __len__(self):
        return len(self.sectors)

    def __iter__(self):
        return iter(self.sectors)

    def __eq__(self, other):  # vspace.jl:29-34
        return (isinstance(other, VectorSpace) and self.sectors == other.sectors
                and self.isdual == other.isdual)

    def __hash__(self):
        return hash((self.sectors, self.isdual))

    def layout(self):
        """Dense index range of every charge, in charge order (vspace.jl:56-73)."""
        out, p = {}, 0
        for c, d in self.sectors:
            out[c] = (p, p + d)
            p += d
        return out

    def __repr__(self):
        tag = "'" if self.isdual else ""
        inner = ", ".join(f"{c}{tag}=>{d}" for c, d in self.sectors)
        return f"U1Space{'†' if self.isdual else ''}({inner})"


def U1Space(*pairs, isdual: bool = False) -> VectorSpace:
    """``U1Space(c=>d, ...)`` (vspace.jl:75-76)."""
    if len(pairs) == 1 and not isinstance(pairs[0], tuple):
        pairs = tuple(pairs[0])
    return VectorSpace(pairs, isdual)


def dual_space(V: VectorSpace) -> VectorSpace:
    """``dual(V)``: same labels, flipped flag (vspace.jl:53)."""
    return VectorSpace(V.sectors, not V.isdual)


def isdual_pair(V1: VectorSpace, V2: VectorSpace) -> bool:
    """``isdual(V1, V2)``: equal sectors, opposite flags (vspace.jl:24-25)."""
    return V1.sectors == V2.sectors and V1.isdual != V2.isdual


def mapcharges_space(f, V: VectorSpace) -> VectorSpace:
    """``mapcharges(f, V)`` (vspace.jl:141-148)."""
    mapped = [f(c) for c in V.charges()]
    if len(set(mapped)) != len(mapped):
        raise SpaceMismatch("mapping charges creates duplicates!")
    return VectorSpace([(f(c), d) for c, d in V.sectors], V.isdual)


def _eff(c: int, isdual: bool) -> int:
    return -c if isdual else c


def fuse(_dual: bool, Vs) -> VectorSpace:
    """Tensor product of spaces, fused right to left (vspace.jl:109-138)."""
    Vs = tuple(Vs)
    N = len(Vs)
    if N < 2:
        if _dual == Vs[0].isdual:
            return Vs[0]
        return dual_space(mapcharges_space(lambda x: -x, Vs[0]))
    if N > 2:
        return fuse(_dual, Vs[:N - 2] + (fuse(_dual, Vs[N - 2:]),))
    acc: dict[int, int] = {}
    for c2, d2 in Vs[1]:
        e2 = _eff(c2, Vs[1].isdual)
        for c1, d1 in Vs[0]:
            e1 = _eff(c1, Vs[0].isdual)
            c = -(e1 + e2) if _dual else e1 + e2
            acc[c] = acc.get(c, 0) + d1 * d2
    return VectorSpace(sorted(acc.items()), _dual)


# ---------------------------------------------------------------------------------------------
# Sectors  (src/sector.jl)
# ---------------------------------------------------------------------------------------------
def sector_key(s):
    """Column-major sector order: compare reversed tuples (sector.jl:35-36)."""
    return tuple(reversed(s))


def sector_sum(s, dualinfo) -> int:
    """``sum(s, dualinfo)``: effective charge of a sector (sector.jl:14-20)."""
    return sum(_eff(c, d) for c, d in zip(s, dualinfo))


def allsectorsandsizes(charge: int, Vs):
    """All sectors of ``Vs`` adding up to ``charge``, sorted, with block sizes (sector.jl:69-92)."""
    Vs = tuple(Vs)
    N = len(Vs)
    if N < 2:
        c = _eff(charge, Vs[0].isdual)
        d = Vs[0].dim(c)
        if d > 0:
            return [(c,)], [(d,)]
        return [], []
    sects, sizes = [], []
    for c, d in Vs[N - 1]:
        ec = _eff(c, Vs[N - 1].isdual)
        sh, zh = allsectorsandsizes(charge - ec, Vs[:N - 1])
        for s, z in zip(sh, zh):
            sects.append(s + (c,))
            sizes.append(z + (d,))
    return sects, sizes


def _stable_sortperm(keys):
    """Julia ``sortperm`` is stable (its ``Perm`` ordering breaks ties by index)."""
    return sorted(range(len(keys)), key=lambda i: (keys[i], i))


# ---------------------------------------------------------------------------------------------
# SymTensor container  (src/symtensor.jl)
# ---------------------------------------------------------------------------------------------
class SymTensor:
    """Block-sparse tensor: charge, leg spaces and sorted sector -> block map (symtensor.jl:12-30).

    ``blocks`` is a dict kept in reference sector order (insertion order == sorted order).
    """

    __slots__ = ("charge", "space", "blocks")

    def __init__(self, charge: int, space, blocks, check: bool = True):
        self.charge = int(charge)
        self.space = tuple(space)
        items = sorted(blocks.items(), key=lambda kv: sector_key(kv[0]))
        self.blocks = {tuple(int(c) for c in s): b for s, b in items}
        if check:  # symtensor.jl:20-26
            sects, sizes = allsectorsandsizes(self.charge, self.space)
            if len(sects) != len(self.blocks):
                raise SpaceMismatch(f"SectorMismatch: {len(self.blocks)} blocks vs {len(sects)}")
            for (s, b), s0, z0 in zip(self.blocks.items(), sects, sizes):
                if s != s0:
                    raise SpaceMismatch(f"SectorMismatch(), {s} vs {s0}")
                if tuple(np.shape(b)) != tuple(z0):
                    raise SpaceMismatch(f"SizeMismatch() {np.shape(b)} vs {z0} at {s}")

    @property
    def rank(self):
        return len(self.space)

    def sectors(self):
        return list(self.blocks.keys())

    def size(self):
        return tuple(V.dim() for V in self.space)

    @property
    def dtype(self):
        for b in self.blocks.values():
            return np.asarray(b).dtype
        return np.dtype(np.float64)

    def issimilar(self, other) -> bool:  # symtensor.jl:93-94
        return self.charge == other.charge and self.space == other.space

    def __eq__(self, other):  # exact equality (symtensor.jl:96-97)
        if not self.issimilar(other) or list(self.blocks) != list(other.blocks):
            return False
        return all(np.array_equal(self.blocks[s], other.blocks[s]) for s in self.blocks)

    def isapprox(self, other, rtol=1e-8, atol=0.0) -> bool:
        if not self.issimilar(other) or list(self.blocks) != list(other.blocks):
            return False
        return all(np.allclose(self.blocks[s], other.blocks[s], rtol=rtol, atol=atol)
                   for s in self.blocks)

    def __getitem__(self, s):
        return self.blocks[tuple(s)]

    def __setitem__(self, s, blk):  # symtensor.jl:124-130
        s = tuple(s)
        if s not in self.blocks:
            raise SpaceMismatch("Block doesn't exist")
        self.blocks[s] = np.asarray(blk)


class SymDiagonal(SymTensor):
    """Block-diagonal singular values: blocks are 1-d arrays (symtensor.jl:47-66)."""

    def __init__(self, charge, space, diag_blocks):
        SymTensor.__init__(self, charge, space, {}, check=False)
        items = sorted(diag_blocks.items(), key=lambda kv: sector_key(kv[0]))
        self.blocks = {tuple(s): np.asarray(b, dtype=np.float64) for s, b in items}

    def as_dense(self) -> SymTensor:
        return SymTensor(self.charge, self.space,
                         {s: np.diag(b) for s, b in self.blocks.items()}, check=False)

    def diag(self):  # symtensor.jl:71
        return np.sort(np.concatenate([b for b in self.blocks.values()]))[::-1]


def from_blocks(charge, space, blocks) -> SymTensor:
    return SymTensor(charge, space, blocks)


def fill(x, charge, space) -> SymTensor:
    """``fill(x, charge, space)`` (symtensor.jl:157-164)."""
    sects, sizes = allsectorsandsizes(charge, space)
    dt = np.result_type(type(x), np.float64) if not isinstance(x, (int, np.integer)) else np.int64
    return SymTensor(charge, space, {s: np.full(z, x, dtype=dt) for s, z in zip(sects, sizes)})


def fill_linearindex(charge, space) -> SymTensor:
    """Blocks hold 1, 2, 3, ... in sector then column-major order (symtensor.jl:173-183)."""
    sects, sizes = allsectorsandsizes(charge, space)
    blocks, p = {}, 0
    for s, z in zip(sects, sizes):
        n = int(np.prod(z))
        blocks[s] = np.arange(p + 1, p + n + 1, dtype=np.int64).reshape(z, order="F")
        p += n
    return SymTensor(charge, space, blocks)


def eye(V: VectorSpace, dtype=np.float64) -> SymTensor:
    """Identity on ``(V, dual(V))`` (symtensor.jl:188-191)."""
    return SymTensor(0, (V, dual_space(V)),
                     {(c, c): np.eye(d, dtype=dtype) for c, d in V.sectors}, check=False)


def dual(A: SymTensor) -> SymTensor:
    """``dual(A)``: negated charge, flipped leg flags, same labels and blocks (symtensor.jl:201-212).

    The reference does not conjugate the blocks in either branch; that is reproduced here.
    """
    if isinstance(A, SymDiagonal):
        out = SymDiagonal(-A.charge, tuple(dual_space(V) for V in A.space), A.blocks)
        return out
    return SymTensor(-A.charge, tuple(dual_space(V) for V in A.space), dict(A.blocks),
                     check=False)


def array(A: SymTensor) -> np.ndarray:
    """Dense embedding; every leg laid out in charge order (symtensor.jl:236-242)."""
    if isinstance(A, SymDiagonal):
        A = A.as_dense()
    out = np.zeros(A.size(), dtype=A.dtype)
    lays = [V.layout() for V in A.space]
    for s, b in A.blocks.items():
        idx = tuple(slice(*lays[i][s[i]]) for i in range(len(s)))
        out[idx] = b
    return out


# ---------------------------------------------------------------------------------------------
# Vector operations used by the Krylov solver  (symtensor.jl:244-323)
# ---------------------------------------------------------------------------------------------
def scaled(A: SymTensor, a) -> SymTensor:
    """``A * a`` (symtensor.jl:244-248)."""
    if isinstance(A, SymDiagonal):
        return SymDiagonal(A.charge, A.space, {s: a * b for s, b in A.blocks.items()})
    return SymTensor(A.charge, A.space, {s: a * b for s, b in A.blocks.items()}, check=False)


def similar_zeros(A: SymTensor) -> SymTensor:
    return SymTensor(A.charge, A.space, {s: np.zeros_like(b) for s, b in A.blocks.items()},
                     check=False)


def rmul(A: SymTensor, a) -> SymTensor:
    """In-place ``rmul!(A, a)`` (symtensor.jl:280-285)."""
    for s in A.blocks:
        A.blocks[s] = A.blocks[s] * a
    return A


def axpy(a, A: SymTensor, B: SymTensor) -> SymTensor:
    """``axpy!(a, A, B)``: B <- a*A + B (symtensor.jl:288-296)."""
    if not A.issimilar(B):
        raise SpaceMismatch("axpy! The two matrices are not simliar!")
    for s in B.blocks:
        B.blocks[s] = a * A.blocks[s] + B.blocks[s]
    return B


def axpby(a, A: SymTensor, b, B: SymTensor) -> SymTensor:
    """``axpby!(a, A, b, B)``: B <- a*A + b*B (symtensor.jl:299-308)."""
    if not A.issimilar(B):
        raise SpaceMismatch("axpy! The two matrices are not simliar!")
    for s in B.blocks:
        B.blocks[s] = a * A.blocks[s] + b * B.blocks[s]
    return B


def dot(A: SymTensor, B: SymTensor):
    """Inner product conjugating the first argument, summed block by block (symtensor.jl:314-318)."""
    if not A.issimilar(B):
        raise SpaceMismatch("The two SymTensors have to be similar to dot!")
    return sum(np.vdot(np.asarray(A.blocks[s]).ravel(order="F"),
                       np.asarray(B.blocks[s]).ravel(order="F")) for s in A.blocks)


def norm(A: SymTensor) -> float:
    """``sqrt(Float64(dot(A, A)))`` (symtensor.jl:321-323)."""
    return float(np.sqrt(np.real(dot(A, A))))


# ---------------------------------------------------------------------------------------------
# Releg  (src/symreleg.jl)
# ---------------------------------------------------------------------------------------------
def permutelegs(A: SymTensor, perm) -> SymTensor:
    """Permute legs, 1-based ``perm`` (symreleg.jl:34-51)."""
    N = A.rank
    perm = [int(p) for p in perm]
    if sorted(perm) != list(range(1, N + 1)):
        raise SpaceMismatch("Not a valid permutation!")
    if perm == list(range(1, N + 1)):
        return A
    p0 = [p - 1 for p in perm]
    space = tuple(A.space[i] for i in p0)
    if isinstance(A, SymDiagonal):  # symreleg.jl:45-46
        return SymDiagonal(A.charge, space, A.blocks)
    blocks = {tuple(s[i] for i in p0): np.transpose(b, p0) for s, b in A.blocks.items()}
    return SymTensor(A.charge, space, blocks, check=False)


def fuselegs(A: SymTensor, l: int, n: int = 2, _dual: bool = False) -> SymTensor:
    """Fuse legs ``l..l+n-1`` (1-based) into one graded leg (symreleg.jl:79-146)."""
    N = A.rank
    if not (0 < l < N + 2 - n):
        raise SpaceMismatch(f"fuselegs {l} to {l + n - 1} for size {N}")
    if n < 2 and _dual == A.space[l - 1].isdual:
        return A
    i0, i1 = l - 1, l - 1 + n
    dualinfo = [V.isdual for V in A.space[i0:i1]]
    csects = A.sectors()
    fsects = []
    for s in csects:
        fc = sector_sum(s[i0:i1], dualinfo)
        if _dual:
            fc = -fc
        fsects.append(s[:i0] + (fc,) + s[i1:])
    sperm = _stable_sortperm([sector_key(f) for f in fsects])
    semits = [csects[i] for i in sperm]
    Vf = fuse(_dual, A.space[i0:i1])
    space = A.space[:i0] + (Vf,) + A.space[i1:]
    sects, sizes = allsectorsandsizes(A.charge, space)
    blocks, ptr = {}, 0
    for sect, z in zip(sects, sizes):
        blk = np.empty(z, dtype=A.dtype)
        p = 0
        while p < z[i0]:
            src = A.blocks[semits[ptr]]
            s = src.shape
            fd = int(np.prod(s[i0:i1]))
            idx = [slice(None)] * len(z)
            idx[i0] = slice(p, p + fd)
            blk[tuple(idx)] = src.reshape(s[:i0] + (fd,) + s[i1:], order="F")
            p += fd
            ptr += 1
        blocks[sect] = blk
    return SymTensor(A.charge, space, blocks, check=False)


def splitleg(A: SymTensor, l: int, space) -> SymTensor:
    """Split leg ``l`` (1-based) into the given spaces (symreleg.jl:160-214)."""
    N = A.rank
    space = tuple(space)
    if not (0 < l <= N):
        raise SpaceMismatch(f"integer l not in range {l}, {N}")
    if len(space) == 1:
        if A.space[l - 1] != space[0]:
            raise SpaceMismatch(f"SpaceMismatch {A.space[l - 1]}, {space[0]}")
        return A
    i = l - 1
    sects = A.sectors()
    order = _stable_sortperm([s[i] for s in sects])
    blocks = {}
    for k in order:
        s = sects[k]
        charge = _eff(s[i], A.space[i].isdual)
        pats, sizes = allsectorsandsizes(charge, space)
        old = A.blocks[s]
        sh = old.shape
        pivot = 0
        for pat, z in zip(pats, sizes):
            sl = int(np.prod(z))
            idx = [slice(None)] * N
            idx[i] = slice(pivot, pivot + sl)
            blocks[s[:i] + pat + s[i + 1:]] = old[tuple(idx)].reshape(sh[:i] + z + sh[i + 1:],
                                                                      order="F")
            pivot += sl
    new_space = A.space[:i] + space + A.space[i + 1:]
    return SymTensor(A.charge, new_space, blocks, check=False)


# ---------------------------------------------------------------------------------------------
# Contraction  (src/contract.jl)
# ---------------------------------------------------------------------------------------------
def contract_index_perm(indexset):
    """Remaining legs (sorted by target), contracted legs (sorted by |label|) and targets
    (contract.jl:82-99).  Positions are 1-based."""
    rems, cons, cons_order, tofinals = [], [], [], []
    for i, idx in enumerate(indexset, start=1):
        if idx < 0:
            cons.append(i)
            cons_order.append(idx)
        else:
            rems.append(i)
            tofinals.append(idx)
    perm = _stable_sortperm(tofinals)
    cperm = _stable_sortperm([abs(x) for x in cons_order])
    return [rems[p] for p in perm], [cons[p] for p in cperm], [tofinals[p] for p in perm]


def symmatrix(A: SymTensor, rowidxs, colidxs) -> SymTensor:
    """Permute and fuse into a block-diagonal matrix, rows fused with ``fuse(false)``, columns
    with ``fuse(true)`` (contract.jl:112-171)."""
    N = A.rank
    rowidxs, colidxs = list(rowidxs), list(colidxs)
    idxperm = rowidxs + colidxs
    if sorted(idxperm) != list(range(1, N + 1)):
        raise SpaceMismatch("Incorrect index set for conversion to SymMatrix!")
    if not rowidxs:
        raise SpaceMismatch("empty row for matrix not allowed!")
    if not colidxs:
        raise SpaceMismatch("empty col for matrix not allowed!")
    n = len(rowidxs)
    p0 = [p - 1 for p in idxperm]
    rowdual = [A.space[i - 1].isdual for i in rowidxs]
    coldual = [A.space[i - 1].isdual for i in colidxs]
    orig = A.sectors()
    csects = [tuple(s[i] for i in p0) for s in orig]
    sperm1 = _stable_sortperm([sector_key(c) for c in csects])
    fsects = []
    for i in range(len(csects)):
        sec = csects[sperm1[i]]
        c1 = sector_sum(sec[:n], rowdual)
        c2 = -sector_sum(sec[n:], coldual)
        fsects.append((c1, c2))
    sperm2 = _stable_sortperm([sector_key(f) for f in fsects])
    semits = [orig[sperm1[j]] for j in sperm2]
    space = (fuse(False, [A.space[i - 1] for i in rowidxs]),
             fuse(True, [A.space[i - 1] for i in colidxs]))
    sects, sizes = allsectorsandsizes(A.charge, space)
    blocks, ptr = {}, 0
    for sect, (rlim, clim) in zip(sects, sizes):
        blk = np.empty((rlim, clim), dtype=A.dtype)
        pc = 0
        while pc < clim:
            pr = 0
            fdc = 0
            while pr < rlim:
                ablk = np.transpose(A.blocks[semits[ptr]], p0)
                s = ablk.shape
                fdr = int(np.prod(s[:n]))
                fdc = int(np.prod(s[n:]))
                blk[pr:pr + fdr, pc:pc + fdc] = ablk.reshape((fdr, fdc), order="F")
                pr += fdr
                ptr += 1
            pc += fdc
        blocks[sect] = blk
    return SymTensor(A.charge, space, blocks, check=False)


def symvector(A: SymTensor, perm, _dual: bool) -> SymTensor:
    """Permute then fuse every leg into one (contract.jl:101-110)."""
    N = A.rank
    if sorted(perm) != list(range(1, N + 1)):
        raise SpaceMismatch("Incorrect index set for conversion to SymVector!")
    return fuselegs(permutelegs(A, perm), 1, N, _dual)


def matmul(A: SymTensor, B: SymTensor) -> SymTensor:
    """Per-sector block GEMM; allowed sectors without a partner get zero blocks
    (contract.jl:234-298).  ``A``/``B`` may be SymDiagonal."""
    if not isdual_pair(A.space[1], B.space[0]):
        raise SpaceMismatch(f"not contractible! {A.space[1]} and {B.space[0]}")
    charge = A.charge + B.charge
    space = (A.space[0], B.space[1])
    sects, sizes = allsectorsandsizes(charge, space)
    dt = np.result_type(A.dtype, B.dtype)
    blocks = {}
    for (c1, c2), z in zip(sects, sizes):
        _c1 = _eff(c1, A.space[0].isdual)
        _c2 = _eff(c2, B.space[1].isdual)
        if A.space[1].isdual:
            sa = (c1, -A.charge + _c1)
            sb = (B.charge - _c2, c2)
        else:
            sa = (c1, A.charge - _c1)
            sb = (-B.charge + _c2, c2)
        if sa in A.blocks and sb in B.blocks:
            a, b = _blockmat(A, sa), _blockmat(B, sb)
            for fc in FlopCount._active:
                fc.flops += 2.0 * a.shape[0] * b.shape[1] * a.shape[1]
            blocks[(c1, c2)] = a @ b
        else:
            blocks[(c1, c2)] = np.zeros(z, dtype=dt)
    return SymTensor(charge, space, blocks, check=False)


def _blockmat(A, s):
    b = A.blocks[s]
    if isinstance(A, SymDiagonal):
        return np.diag(b)
    return b


def split_matrix(A: SymTensor, rlegs, clegs) -> SymTensor:
    """Cut every fused block of a SymMatrix back into unfused sectors (contract.jl:187-224)."""
    rlegs, clegs = tuple(rlegs), tuple(clegs)
    blocks = {}
    for (c1, c2), blk in A.blocks.items():
        c1 = _eff(c1, A.space[0].isdual)
        c2 = _eff(c2, A.space[1].isdual)
        rpats, rsizes = allsectorsandsizes(c1, rlegs)
        cpats, csizes = allsectorsandsizes(c2, clegs)
        pc = 0
        for cp, cz in zip(cpats, csizes):
            csl = int(np.prod(cz))
            pr = 0
            for rp, rz in zip(rpats, rsizes):
                rsl = int(np.prod(rz))
                blocks[rp + cp] = blk[pr:pr + rsl, pc:pc + csl].reshape(rz + cz, order="F")
                pr += rsl
            pc += csl
    return SymTensor(A.charge, rlegs + clegs, blocks, check=False)


def _invperm(p):
    out = [0] * len(p)
    for i, v in enumerate(p, start=1):
        out[v - 1] = i
    return out


def contract(A: SymTensor, idxA, B: SymTensor, idxB):
    """ncon-style contraction: permute-fuse both operands, per-sector GEMM, split, permute
    (contract.jl:11-47).  Returns a scalar when every leg is contracted."""
    remsA, consA, tofA = contract_index_perm(idxA)
    remsB, consB, tofB = contract_index_perm(idxB)
    if not remsA:
        _A = symvector(A, consA, False)
        if not remsB:
            _B = symvector(B, consB, True)
            if not isdual_pair(_A.space[0], _B.space[0]):  # contract.jl:226-228
                raise SpaceMismatch("not contractible!")
            # contract.jl:230-231 multiplies the first blocks elementwise and sums
            if not _A.blocks or not _B.blocks:
                return 0.0
            a = next(iter(_A.blocks.values()))
            b = next(iter(_B.blocks.values()))
            return np.sum(a * b)
        # contract.jl:30-32 calls `*` on a rank-1 and a rank-2 tensor, which has no method
        raise SpaceMismatch("contract with no remaining leg on the first operand is unsupported")
    if not remsB:
        # contract.jl:39-41 has the same missing method
        raise SpaceMismatch("contract with no remaining leg on the second operand is unsupported")
    _A = symmatrix(A, remsA, consA)
    _B = symmatrix(B, consB, remsB)
    C = split_matrix(matmul(_A, _B), [A.space[i - 1] for i in remsA],
                     [B.space[i - 1] for i in remsB])
    return permutelegs(C, _invperm(tofA + tofB))


# ---------------------------------------------------------------------------------------------
# Factorisations  (src/symtools.jl, src/mpsutils.jl)
# ---------------------------------------------------------------------------------------------
def svd_(A: SymTensor):
    """Per-sector thin SVD (symtools.jl:1-35).  Returns u, s (SymDiagonal), v."""
    ub, sb, vb = {}, {}, {}
    midl, midr = {}, {}
    for (c1, c2), blk in A.blocks.items():
        U, S, Vt = np.linalg.svd(blk, full_matrices=False)
        ub[(c1, c1)] = U
        sb[(c1, c2)] = S
        vb[(c2, c2)] = Vt
        midl[c1] = len(S)
        midr[c2] = len(S)
    Vl = VectorSpace(sorted(midl.items()), A.space[0].isdual)
    Vr = VectorSpace(sorted(midr.items()), A.space[1].isdual)
    u = SymTensor(0, (A.space[0], dual_space(Vl)), ub, check=False)
    s = SymDiagonal(A.charge, (Vl, Vr), sb)
    v = SymTensor(0, (dual_space(Vr), A.space[1]), vb, check=False)
    return u, s, v


def truncatedsizes(S, maxdim: int = 200, tol: float = 1e-14, tieband: float = 0.0):
    """Greedy global pick of the ``maxdim`` largest values above the ABSOLUTE ``tol``; ties go to
    the first sector (mpsutils.jl:89-112, Julia ``findmax`` returns the first maximum).

    ``tieband`` = 0 is the reference rule.  A positive band treats candidates within
    ``tieband * max(S)`` of the current maximum as equal and takes the lowest sector index among
    them, which makes the choice independent of round-off between two SVD implementations.
    """
    nS = len(S)
    pointers = [0] * nS
    c = [float(S[i][0]) for i in range(nS)]
    total = sum(len(s) for s in S)
    band = tieband * max(c) if (tieband > 0 and c) else 0.0
    for n in range(1, min(maxdim, total) + 1):
        m = max(c)
        if band > 0:
            index = next(i for i in range(nS) if c[i] >= m - band)
            m = c[index]
        else:
            index = c.index(m)
        if m < tol:
            if n == 1:
                raise SpaceMismatch(f"The largest singular value is smaller than tol! {m} < {tol}")
            break
        if pointers[index] + 1 >= len(S[index]):
            pointers[index] += 1
            c[index] = 0.0
        else:
            pointers[index] += 1
            c[index] = float(S[index][pointers[index]])
    return pointers


def svdtrunc(A: SymTensor, maxdim: int | None = None, tol: float = 1e-12, tieband: float = 0.0):
    """Per-sector SVD, global greedy truncation, zero-kept sectors dropped (mpsutils.jl:116-179)."""
    if maxdim is None:
        maxdim = max(A.size())
    su, ss, sv, bu, bs, bv = [], [], [], [], [], []
    for (c1, c2), blk in A.blocks.items():
        su.append((c1, c1))
        ss.append((c1, c2))
        sv.append((c2, c2))
        U, S, Vt = np.linalg.svd(blk, full_matrices=False)
        bu.append(U)
        bs.append(S)
        bv.append(Vt)
    ns = truncatedsizes(bs, maxdim=maxdim, tol=tol, tieband=tieband)
    keep = [i for i, k in enumerate(ns) if k > 0]
    Vl = VectorSpace([(ss[i][0], ns[i]) for i in keep], A.space[0].isdual)
    Vr = VectorSpace([(ss[i][1], ns[i]) for i in keep], A.space[1].isdual)
    u = SymTensor(0, (A.space[0], dual_space(Vl)),
                  {su[i]: bu[i][:, :ns[i]] for i in keep}, check=False)
    s = SymDiagonal(A.charge, (Vl, Vr), {ss[i]: bs[i][:ns[i]] for i in keep})
    v = SymTensor(0, (dual_space(Vr), A.space[1]),
                  {sv[i]: bv[i][:ns[i], :] for i in keep}, check=False)
    return u, s, v


# ---------------------------------------------------------------------------------------------
# Flat interchange with the device library: blocks in reference order, each column-major
# ---------------------------------------------------------------------------------------------
def flatten(A: SymTensor) -> np.ndarray:
    if not A.blocks:
        return np.zeros(0)
    return np.concatenate([np.asarray(b).ravel(order="F") for b in A.blocks.values()])


def from_flat(charge, space, flat) -> SymTensor:
    sects, sizes = allsectorsandsizes(charge, space)
    blocks, p = {}, 0
    flat = np.asarray(flat)
    for s, z in zip(sects, sizes):
        n = int(np.prod(z))
        blocks[s] = flat[p:p + n].reshape(z, order="F")
        p += n
    if p != flat.size:
        raise SpaceMismatch(f"flat length {flat.size} != tensor size {p}")
    return SymTensor(charge, space, blocks)
