"""Host-side mirror of the SymTensors API of amiragha/mps, backed by the GB300 C ABI.

Names, argument meaning (1-based leg positions, ncon-style index tuples) and error behaviour
follow the reference (src/SymTensors.jl:26-81); every tensor lives on the device and every
operation runs as CUDA kernels of ``libmpsgb300.so``.  The only host work is bookkeeping
metadata and copying flat arrays in or out.

``precision`` arguments select the block-GEMM arithmetic: 0 = FP64 (the reference's Float64
path), s >= 2 = split precision with s bf16 slices (FP32 accumulation, FP64 epilogue).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import call, i32arr, i64arr, SpaceMismatch, MPSGError

__all__ = [
    "VectorSpace", "U1Space", "Context", "get_context", "SymTensor", "dual", "zeros", "fill",
    "from_flat", "from_blocks", "meta", "permutelegs", "fuselegs", "splitleg", "SymMatrix",
    "matmul", "contract", "contract_complex", "contract_flops", "dot", "norm", "axpy", "axpby",
    "rmul", "mul",
    "similar", "copy", "fill_", "applymps2site", "applymps2site_host", "applymps2site_flops",
    "mpsupdateleft",
    "mpsupdateright", "SpaceMismatch", "MPSGError", "set_default_precision", "_svd_",
    "svdtrunc", "svd_complex", "dots", "lincomb", "truncatedsizes", "small_eigh",
    "eigsolve_heff2", "EigInfo", "Heff2", "HeffBatch", "tuner", "set_split_tuning", "HostBuffer", "Copy", "download_async",
    "upload_async", "device_checks", "checked_library",
]


# ---------------------------------------------------------------------------------------------
# spaces (src/vspace.jl)
# ---------------------------------------------------------------------------------------------
class VectorSpace:
    """Graded space charge -> dim with an ``isdual`` flag (value type; src/vspace.jl:5-18)."""

    __slots__ = ("sectors", "isdual")

    def __init__(self, pairs, isdual: bool = False):
        pairs = sorted((int(c), int(d)) for c, d in pairs)
        for i in range(1, len(pairs)):
            if pairs[i][0] == pairs[i - 1][0]:
                raise SpaceMismatch(_lib.ERR_SPACE_MISMATCH, f"duplicate charges! {pairs}")
        for _, d in pairs:
            if d <= 0:
                raise SpaceMismatch(_lib.ERR_SPACE_MISMATCH, "space dimension can only be positive!")
        self.sectors = tuple(pairs)
        self.isdual = bool(isdual)

    def charges(self):
        return [c for c, _ in self.sectors]

    def dims(self):
        return [d for _, d in self.sectors]

    def dim(self, charge=None) -> int:
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

    def __eq__(self, other):
        return (isinstance(other, VectorSpace) and self.sectors == other.sectors
                and self.isdual == other.isdual)

    def __hash__(self):
        return hash((self.sectors, self.isdual))

    def __repr__(self):
        tag = "'" if self.isdual else ""
        inner = ", ".join(f"{c}{tag}=>{d}" for c, d in self.sectors)
        return f"U1Space{'†' if self.isdual else ''}({inner})"


def U1Space(*pairs, isdual: bool = False) -> VectorSpace:
    """``U1Space(c=>d, ...)`` (src/vspace.jl:75-76): ``U1Space((0, 1), (1, 2))``."""
    if len(pairs) == 1 and not isinstance(pairs[0], tuple):
        pairs = tuple(pairs[0])
    return VectorSpace(pairs, isdual)


def _space_args(spaces):
    spaces = list(spaces)
    nsect = [len(V) for V in spaces]
    charges = [c for V in spaces for c in V.charges()]
    dims = [d for V in spaces for d in V.dims()]
    isd = [int(V.isdual) for V in spaces]
    return len(spaces), i32arr(nsect), i32arr(charges), i64arr(dims), i32arr(isd)


# ---------------------------------------------------------------------------------------------
# context
# ---------------------------------------------------------------------------------------------
_DEFAULT_PRECISION = 0


def set_default_precision(p: int):
    """Default block-GEMM arithmetic for calls that do not pass ``precision``."""
    global _DEFAULT_PRECISION
    _DEFAULT_PRECISION = int(p)


def _prec(p):
    return _DEFAULT_PRECISION if p is None else int(p)


class Context:
    """One GPU, one CUDA stream and the plan caches of the library."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        call("mpsg_ctx_create", device, C.byref(h))
        self._h = h
        self.device = device
        self._free = _lib.lib.mpsg_ctx_destroy

    @property
    def handle(self):
        return self._h

    def synchronize(self):
        call("mpsg_ctx_synchronize", self._h)

    def counters(self):
        """(kernel launches, algorithmic GEMM flops) issued so far on this context."""
        n = C.c_int64()
        f = C.c_double()
        call("mpsg_ctx_counters", self._h, C.byref(n), C.byref(f))
        return n.value, f.value

    def clear_caches(self):
        call("mpsg_ctx_clear_caches", self._h)

    def stream(self) -> int:
        """The context's cudaStream_t as an integer."""
        s = C.c_void_p()
        call("mpsg_ctx_stream", self._h, C.byref(s))
        return s.value or 0

    KERNEL_KINDS = {"copy": 0, "gemm_f64": 1, "gemm_split": 2, "pack": 3, "vec": 4,
                    "pack_slices": 5}

    def set_timing(self, enable: bool):
        """Bracket every kernel launch with CUDA events (resets the accumulated times)."""
        call("mpsg_ctx_set_timing", self._h, int(bool(enable)))

    def kernel_time(self, kind: str):
        """(summed milliseconds, launches, algorithmic flops) of one kernel class since timing
        was enabled."""
        ms = C.c_double()
        n = C.c_int64()
        f = C.c_double()
        call("mpsg_ctx_kernel_time", self._h, self.KERNEL_KINDS[kind], C.byref(ms), C.byref(n),
             C.byref(f))
        return ms.value, n.value, f.value

    def close(self):
        if self._h:
            self._free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_contexts: dict[int, Context] = {}


def get_context(device: int = 0) -> Context:
    if device not in _contexts:
        _contexts[device] = Context(device)
    return _contexts[device]


# ---------------------------------------------------------------------------------------------
# tensors (src/symtensor.jl)
# ---------------------------------------------------------------------------------------------
class SymTensor:
    """Device-resident block-sparse tensor.  ``ctx is None`` marks a structure-only tensor
    (sector table without data), which the planning functions accept on any host."""

    __slots__ = ("_h", "ctx", "_space", "_charge", "_sect", "__weakref__")

    def __init__(self, handle, ctx):
        self._h = handle
        self.ctx = ctx
        self._space = None
        self._charge = None
        self._sect = None

    def __del__(self):
        try:
            if self._h:
                _lib.lib.mpsg_tensor_free(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def is_meta(self) -> bool:
        return self.ctx is None

    @property
    def charge(self) -> int:
        if self._charge is None:
            c = C.c_int32()
            call("mpsg_tensor_charge", self._h, C.byref(c))
            self._charge = c.value
        return self._charge

    @property
    def rank(self) -> int:
        n = C.c_int32()
        call("mpsg_tensor_rank", self._h, C.byref(n))
        return n.value

    @property
    def space(self):
        if self._space is None:
            sp = []
            for leg in range(1, self.rank + 1):
                n = C.c_int32()
                d = C.c_int32()
                call("mpsg_tensor_space", self._h, leg, C.byref(n), None, None, C.byref(d))
                ch = (C.c_int32 * n.value)()
                dm = (C.c_int64 * n.value)()
                call("mpsg_tensor_space", self._h, leg, None, ch, dm, None)
                sp.append(VectorSpace(zip(list(ch), list(dm)), bool(d.value)))
            self._space = tuple(sp)
        return self._space

    def numel(self) -> int:
        ne = C.c_int64()
        call("mpsg_tensor_numel", self._h, None, C.byref(ne))
        return ne.value

    def nblocks(self) -> int:
        nb = C.c_int64()
        call("mpsg_tensor_numel", self._h, C.byref(nb), None)
        return nb.value

    def size(self):
        return tuple(V.dim() for V in self.space)

    def _sector_table(self):
        if self._sect is None:
            nb, N = self.nblocks(), self.rank
            lab = (C.c_int32 * max(1, nb * N))()
            sz = (C.c_int64 * max(1, nb * N))()
            off = (C.c_int64 * max(1, nb))()
            call("mpsg_tensor_sectors", self._h, lab, sz, off)
            L = np.ctypeslib.as_array(lab)[: nb * N].reshape(nb, N) if nb else np.zeros((0, N), int)
            Z = np.ctypeslib.as_array(sz)[: nb * N].reshape(nb, N) if nb else np.zeros((0, N), int)
            O = np.ctypeslib.as_array(off)[:nb].copy() if nb else np.zeros(0, int)
            self._sect = ([tuple(int(x) for x in r) for r in L],
                          [tuple(int(x) for x in r) for r in Z], [int(o) for o in O])
        return self._sect

    def sectors(self):
        """Sector labels in reference order (src/symtensor.jl:87)."""
        return list(self._sector_table()[0])

    def block_sizes(self):
        return list(self._sector_table()[1])

    def offsets(self):
        return list(self._sector_table()[2])

    def isdiagonal(self) -> bool:
        d = C.c_int32()
        call("mpsg_tensor_is_diagonal", self._h, C.byref(d))
        return bool(d.value)

    # -- data movement -------------------------------------------------------------------
    def to_flat(self) -> np.ndarray:
        if self.is_meta:
            raise MPSGError(_lib.ERR_ARGUMENT, "structure-only tensor has no data")
        n = self.numel()
        out = np.empty(n, dtype=np.float64)
        call("mpsg_tensor_download", self._h, out.ctypes.data_as(_lib.PF64), n)
        return out

    def upload(self, flat):
        flat = np.ascontiguousarray(flat, dtype=np.float64)
        call("mpsg_tensor_upload", self._h, flat.ctypes.data_as(_lib.PF64), flat.size)
        return self

    @property
    def blocks(self):
        """Sector -> block (column-major numpy arrays), downloaded from the device."""
        flat = self.to_flat()
        out = {}
        for s, z, o in zip(*self._sector_table()):
            n = int(np.prod(z))
            out[s] = flat[o:o + n].reshape(z, order="F")
        return out

    def __getitem__(self, sector):
        return self.blocks[tuple(sector)]

    def device_ptr(self) -> int:
        p = C.c_void_p()
        call("mpsg_tensor_device_ptr", self._h, C.byref(p))
        return p.value or 0

    def issimilar(self, other) -> bool:
        return self.charge == other.charge and self.space == other.space

    # -- operators -----------------------------------------------------------------------
    def __mul__(self, other):
        if isinstance(other, SymTensor):
            return matmul(self, other)
        out = copy(self)
        rmul(out, float(other))
        return out

    __rmul__ = __mul__

    def __repr__(self):
        kind = "meta " if self.is_meta else ""
        return f"<{kind}SymTensor charge={self.charge} space={self.space} blocks={self.nblocks()}>"


def _wrap(h, ctx):
    if not h:
        return None
    return SymTensor(h, ctx)


def _ctx(ctx):
    return ctx if ctx is not None else get_context()


def zeros(charge, space, ctx=None) -> SymTensor:
    """Zero tensor holding every allowed sector (``fill(0.0, charge, space)``)."""
    ctx = _ctx(ctx)
    h = C.c_void_p()
    call("mpsg_tensor_create", ctx.handle, int(charge), *_space_args(space), C.byref(h))
    return SymTensor(h, ctx)


def fill(x, charge, space, ctx=None) -> SymTensor:
    """``fill(x, charge, space)`` (src/symtensor.jl:157-164)."""
    t = zeros(charge, space, ctx)
    if x != 0:
        call("mpsg_fill", t.ctx.handle, t.handle, float(x))
    return t


def fill_(A: SymTensor, x) -> SymTensor:
    """``fill!(A, x)`` (src/symtensor.jl:166-171)."""
    call("mpsg_fill", A.ctx.handle, A.handle, float(x))
    return A


def meta(charge, space) -> SymTensor:
    """Structure-only tensor: sector table without data (works without a GPU)."""
    h = C.c_void_p()
    call("mpsg_meta_create", int(charge), *_space_args(space), C.byref(h))
    return SymTensor(h, None)


def from_flat(charge, space, flat, ctx=None) -> SymTensor:
    t = zeros(charge, space, ctx)
    return t.upload(flat)


def device_checks(reset: bool = False, ctx=None):
    """Violations recorded by the device-checked library (``MPSG_LIBRARY=checked``): (count,
    first) with first = (kind, task, index, detail), kind 1 task lookup, 2 decode, 3 span.
    Raises MPSGError (status 5) with the normal library."""
    n = C.c_int64()
    first = (C.c_int64 * 4)()
    h = None if ctx is None and not checked_library() else _ctx(ctx).handle
    call("mpsg_device_checks", h, int(bool(reset)), C.byref(n), first)
    return n.value, tuple(first)


def checked_library() -> bool:
    """Whether the loaded library is the device-checked debug build."""
    return _lib.LIB_PATH.endswith("_checked.so")


class HostBuffer:
    """Page-locked host memory for ``n`` doubles (``mpsg_host_alloc``); ``array`` is a NumPy view
    of it that keeps the memory alive. Asynchronous copies overlap compute only from such
    memory."""

    def __init__(self, n: int):
        p = C.c_void_p()
        call("mpsg_host_alloc", int(n), C.byref(p))
        self._p = p
        self.n = int(n)

    @property
    def ptr(self):
        return self._p

    @property
    def array(self) -> np.ndarray:
        raw = (C.c_double * max(self.n, 1)).from_address(self._p.value)
        raw._owner = self  # the view's base holds the buffer
        return np.frombuffer(raw, dtype=np.float64, count=self.n)

    def __del__(self):
        try:
            if self._p:
                _lib.lib.mpsg_host_free(self._p)
                self._p = None
        except Exception:
            pass


class Copy:
    """A host<->device copy running on the context's copy stream (``mpsg_copy``). The library
    keeps the tensor's device memory until the copy has completed; this object keeps the host
    buffer, and releasing it first waits for the copy."""

    def __init__(self, h, ctx, host):
        self._h, self.ctx, self._host = h, ctx, host

    def wait(self):
        """Orders later work on the context stream after the copy (no host wait)."""
        call("mpsg_copy_wait", self.ctx.handle, self._h)

    def query(self) -> bool:
        d = C.c_int32()
        call("mpsg_copy_query", self._h, C.byref(d))
        return bool(d.value)

    def synchronize(self):
        call("mpsg_copy_synchronize", self._h)

    def __del__(self):
        try:
            if self._h:
                _lib.lib.mpsg_copy_free(self._h)
                self._h = None
        except Exception:
            pass


def download_async(t: SymTensor, host: HostBuffer) -> Copy:
    """Starts the copy of ``t``'s flat data into ``host.array[:t.numel()]`` after the work queued
    so far on ``t``'s context stream (``mpsg_tensor_download_async``)."""
    n = t.numel()
    if host.n < n:
        raise MPSGError(_lib.ERR_ARGUMENT, "download_async: host buffer too small")
    h = C.c_void_p()
    call("mpsg_tensor_download_async", t.ctx.handle, t.handle, host.ptr, n, C.byref(h))
    return Copy(h, t.ctx, host)


def upload_async(t: SymTensor, host: HostBuffer) -> Copy:
    """Starts the copy of ``host.array[:t.numel()]`` into ``t``; call ``wait()`` on the result
    before queueing work that reads ``t`` (``mpsg_tensor_upload_async``)."""
    n = t.numel()
    if host.n < n:
        raise MPSGError(_lib.ERR_ARGUMENT, "upload_async: host buffer too small")
    h = C.c_void_p()
    call("mpsg_tensor_upload_async", t.ctx.handle, t.handle, host.ptr, n, C.byref(h))
    return Copy(h, t.ctx, host)


def from_blocks(charge, space, blocks, ctx=None) -> SymTensor:
    """Upload a sector -> block mapping; every allowed sector must be present
    (the SymTensor constructor check, src/symtensor.jl:17-28)."""
    t = zeros(charge, space, ctx)
    sects, sizes, offs = t._sector_table()
    if len(blocks) != len(sects):
        raise SpaceMismatch(_lib.ERR_SPACE_MISMATCH,
                            f"SectorMismatch(): {len(blocks)} blocks vs {len(sects)} sectors")
    flat = np.empty(t.numel(), dtype=np.float64)
    for s, z, o in zip(sects, sizes, offs):
        if s not in blocks:
            raise SpaceMismatch(_lib.ERR_SPACE_MISMATCH, f"SectorMismatch(): missing {s}")
        b = np.asarray(blocks[s], dtype=np.float64)
        if tuple(b.shape) != tuple(z):
            raise SpaceMismatch(_lib.ERR_SPACE_MISMATCH, f"SizeMismatch() at {s}")
        flat[o:o + b.size] = b.ravel(order="F")
    return t.upload(flat)


def dual(x):
    """``dual`` of a space or of a tensor (src/vspace.jl:53, src/symtensor.jl:201-212)."""
    if isinstance(x, VectorSpace):
        return VectorSpace(x.sectors, not x.isdual)
    h = C.c_void_p()
    if x.is_meta:
        sp = tuple(VectorSpace(V.sectors, not V.isdual) for V in x.space)
        return meta(-x.charge, sp)
    call("mpsg_dual", x.ctx.handle, x.handle, C.byref(h))
    return SymTensor(h, x.ctx)


def copy(A: SymTensor, ctx=None) -> SymTensor:
    """A copy of A, on ``ctx`` (another context of the same device) when given: the copy is
    ordered on that context's stream, so A's producer must have finished."""
    ctx = ctx or A.ctx
    h = C.c_void_p()
    call("mpsg_tensor_copy", ctx.handle, A.handle, C.byref(h))
    return SymTensor(h, ctx)


def similar(A: SymTensor) -> SymTensor:
    """``similar(A)`` (src/symtensor.jl:252-255); contents are zero here."""
    return zeros(A.charge, A.space, A.ctx)


# ---------------------------------------------------------------------------------------------
# releg (src/symreleg.jl) and contraction (src/contract.jl)
# ---------------------------------------------------------------------------------------------
def permutelegs(A: SymTensor, perm) -> SymTensor:
    perm = [int(p) for p in perm]
    h = C.c_void_p()
    if A.is_meta:
        call("mpsg_plan_permutelegs", A.handle, i32arr(perm), C.byref(h))
    else:
        call("mpsg_permutelegs", A.ctx.handle, A.handle, i32arr(perm), C.byref(h))
    return SymTensor(h, A.ctx)


def fuselegs(A: SymTensor, l: int, n: int = 2, _dual: bool = False) -> SymTensor:
    h = C.c_void_p()
    if A.is_meta:
        call("mpsg_plan_fuselegs", A.handle, int(l), int(n), int(_dual), C.byref(h))
    else:
        call("mpsg_fuselegs", A.ctx.handle, A.handle, int(l), int(n), int(_dual), C.byref(h))
    return SymTensor(h, A.ctx)


def splitleg(A: SymTensor, l: int, space) -> SymTensor:
    if isinstance(space, VectorSpace):
        space = (space,)
    h = C.c_void_p()
    args = _space_args(space)
    if A.is_meta:
        call("mpsg_plan_splitleg", A.handle, int(l), *args, C.byref(h))
    else:
        call("mpsg_splitleg", A.ctx.handle, A.handle, int(l), *args, C.byref(h))
    return SymTensor(h, A.ctx)


def SymMatrix(A: SymTensor, rowidxs, colidxs) -> SymTensor:
    """Permute-fuse into a block-diagonal matrix (src/contract.jl:112-171)."""
    r = [int(x) for x in rowidxs]
    c_ = [int(x) for x in colidxs]
    h = C.c_void_p()
    if A.is_meta:
        call("mpsg_plan_symmatrix", A.handle, len(r), i32arr(r), len(c_), i32arr(c_), C.byref(h))
    else:
        call("mpsg_symmatrix", A.ctx.handle, A.handle, len(r), i32arr(r), len(c_), i32arr(c_),
             C.byref(h))
    return SymTensor(h, A.ctx)


def matmul(A: SymTensor, B: SymTensor, precision=None) -> SymTensor:
    """``A * B`` of two SymMatrix (src/contract.jl:234-298)."""
    h = C.c_void_p()
    if A.is_meta:
        f = C.c_double()
        call("mpsg_plan_matmul", A.handle, B.handle, C.byref(h), C.byref(f))
    else:
        call("mpsg_matmul", A.ctx.handle, A.handle, B.handle, _prec(precision), C.byref(h))
    return SymTensor(h, A.ctx)


def contract(A: SymTensor, idxA, B: SymTensor, idxB, precision=None):
    """``contract(A, idxA, B, idxB)`` with ncon-style index tuples (src/contract.jl:11-47).
    Returns a number when every leg is contracted."""
    ia, ib = i32arr(idxA), i32arr(idxB)
    if len(idxA) != A.rank or len(idxB) != B.rank:
        raise MPSGError(_lib.ERR_ARGUMENT, "index tuple length differs from tensor rank")
    h = C.c_void_p()
    if A.is_meta:
        f = C.c_double()
        call("mpsg_plan_contract", A.handle, ia, B.handle, ib, C.byref(h), C.byref(f))
        return _wrap(h.value, None)
    s = C.c_double()
    call("mpsg_contract", A.ctx.handle, A.handle, ia, B.handle, ib, _prec(precision), C.byref(h),
         C.byref(s))
    if not h.value:
        return s.value
    return SymTensor(h, A.ctx)


def contract_complex(Ar, Ai, sa, idxA, Br, Bi, sb, idxB, precision=None):
    """contract of (Ar + i sa Ai) with (Br + i sb Bi) in one library call (Ai / Bi may be None):
    returns (Cr, Ci) (Ci None for two real operands), or a Python complex when every leg is
    contracted."""
    if len(idxA) != Ar.rank or len(idxB) != Br.rank:
        raise MPSGError(_lib.ERR_ARGUMENT, "index tuple length differs from tensor rank")
    cr, ci = C.c_void_p(), C.c_void_p()
    sr, si = C.c_double(), C.c_double()
    call("mpsg_contract_complex", Ar.ctx.handle, Ar.handle, Ai.handle if Ai is not None else None,
         float(sa), i32arr(idxA), Br.handle, Bi.handle if Bi is not None else None, float(sb),
         i32arr(idxB), _prec(precision), C.byref(cr), C.byref(ci), C.byref(sr), C.byref(si))
    if not cr.value:
        return complex(sr.value, si.value)
    return SymTensor(cr, Ar.ctx), (SymTensor(ci, Ar.ctx) if ci.value else None)


def contract_flops(A: SymTensor, idxA, B: SymTensor, idxB) -> float:
    h = C.c_void_p()
    f = C.c_double()
    call("mpsg_plan_contract", A.handle, i32arr(idxA), B.handle, i32arr(idxB), C.byref(h),
         C.byref(f))
    _wrap(h.value, None)
    return f.value


# ---------------------------------------------------------------------------------------------
# effective Hamiltonian and environments (src/apply.jl)
# ---------------------------------------------------------------------------------------------
def applymps2site(v, envL, envR, W1, W2, precision=None) -> SymTensor:
    """``_applymps2site`` (src/apply.jl:93-105)."""
    h = C.c_void_p()
    call("mpsg_applymps2site", v.ctx.handle, v.handle, envL.handle, envR.handle, W1.handle,
         W2.handle, _prec(precision), C.byref(h))
    return SymTensor(h, v.ctx)


class Heff2:
    """The two-site effective Hamiltonian v -> _applymps2site(v, envL, envR, W1, W2)
    (src/apply.jl:93-105) prepared once and applied many times, as the Krylov solver does
    (src/dmrg.jl:77).  ``precision`` 0 = the reference's FP64 contractions; S >= 2 = W-folded
    split-precision tensor-core path."""

    def __init__(self, v_like, envL, envR, W1, W2, precision=None):
        h = C.c_void_p()
        call("mpsg_heff2_create", v_like.ctx.handle, v_like.handle, envL.handle, envR.handle,
             W1.handle, W2.handle, _prec(precision), C.byref(h))
        self._h = h
        self.ctx = v_like.ctx
        self._free = _lib.lib.mpsg_heff2_free

    @classmethod
    def prepare(cls, v_like, envL, envR, W1, W2, precision=4):
        """One chain's share of a ``HeffBatch`` prepared on that chain's context (plans and the
        FP64 W folds): usable only in ``HeffBatch.from_prepared``."""
        self = cls.__new__(cls)
        h = C.c_void_p()
        call("mpsg_heff2_prepare", v_like.ctx.handle, v_like.handle, envL.handle, envR.handle,
             W1.handle, W2.handle, int(precision), C.byref(h))
        self._h = h
        self.ctx = v_like.ctx
        self._free = _lib.lib.mpsg_heff2_free
        return self

    def __call__(self, v) -> SymTensor:
        h = C.c_void_p()
        call("mpsg_heff2_apply", self.ctx.handle, self._h, v.handle, C.byref(h))
        return SymTensor(h, self.ctx)

    def flops(self) -> float:
        f = C.c_double()
        call("mpsg_heff2_flops", self._h, C.byref(f))
        return f.value

    def traffic(self):
        """(copy bytes, packing bytes) per application: the algorithmic HBM traffic of the
        block-permute copies and of the operand packing (split-precision operators)."""
        c, p = C.c_double(), C.c_double()
        call("mpsg_heff2_traffic", self._h, C.byref(c), C.byref(p))
        return c.value, p.value

    def __del__(self):
        try:
            if self._h:
                self._free(self._h)
                self._h = None
        except Exception:
            pass


def _host_ptr(x, n):
    """Address of a float64 host buffer of n elements (a torch tensor or a numpy array)."""
    if hasattr(x, "data_ptr"):
        if x.numel() != n or x.element_size() != 8 or not x.is_contiguous():
            raise MPSGError(_lib.ERR_ARGUMENT, "host buffer: wrong size, type or layout")
        return x.data_ptr()
    a = np.asarray(x)
    if a.dtype != np.float64 or a.size != n or not a.flags.c_contiguous:
        raise MPSGError(_lib.ERR_ARGUMENT, "host buffer: wrong size, type or layout")
    return a.ctypes.data


def applymps2site_host(v, envL, envR, W1, W2, host_in, host_out, precision=None,
                       keep=False):
    """``_applymps2site`` from host buffers to a host buffer in one call: ``host_in`` holds the
    flat data of (v, envL, envR, W1, W2), copied into those device tensors while the operator
    is prepared; the result's flat data lands in ``host_out``. Returns the device result when
    ``keep``. Pinned buffers (e.g. torch ``pin_memory()``) make the copies asynchronous."""
    ts = (v, envL, envR, W1, W2)
    ptrs = [_host_ptr(h, t.numel()) for h, t in zip(host_in, ts)]
    optr = _host_ptr(host_out, v.numel())
    out = C.c_void_p()
    call("mpsg_applymps2site_host", v.ctx.handle, *[t.handle for t in ts], *ptrs,
         _prec(precision), optr, C.byref(out) if keep else None)
    return SymTensor(out, v.ctx) if keep else None


def applymps2site_flops(v, envL, envR, W1, W2) -> float:
    f = C.c_double()
    call("mpsg_applymps2site_flops", v.ctx.handle, v.handle, envL.handle, envR.handle,
         W1.handle, W2.handle, C.byref(f))
    return f.value


def mpsupdateleft(env, A, W, precision=None) -> SymTensor:
    """``_mpsupdateleft`` (src/apply.jl:49-58)."""
    h = C.c_void_p()
    call("mpsg_mpsupdateleft", env.ctx.handle, env.handle, A.handle, W.handle, _prec(precision),
         C.byref(h))
    return SymTensor(h, env.ctx)


def mpsupdateright(env, A, W, precision=None) -> SymTensor:
    """``_mpsupdateright`` (src/apply.jl:17-25)."""
    h = C.c_void_p()
    call("mpsg_mpsupdateright", env.ctx.handle, env.handle, A.handle, W.handle,
         _prec(precision), C.byref(h))
    return SymTensor(h, env.ctx)


# ---------------------------------------------------------------------------------------------
# factorisations and the Krylov solver (src/symtools.jl, src/mpsutils.jl, KrylovKit boundary)
# ---------------------------------------------------------------------------------------------
def _svd_(A: SymTensor):
    """Per-sector thin SVD of a rank-2 tensor (src/symtools.jl:1-35): (u, s, v)."""
    u, s, v = C.c_void_p(), C.c_void_p(), C.c_void_p()
    call("mpsg_svd", A.ctx.handle, A.handle, C.byref(u), C.byref(s), C.byref(v))
    return SymTensor(u, A.ctx), SymTensor(s, A.ctx), SymTensor(v, A.ctx)


SVD_METHODS = ("exact", "gram_left", "gram_right")


def svdtrunc(A: SymTensor, maxdim=None, tol: float = 1e-12, tieband: float = 0.0,
             method: str = "exact"):
    """``svdtrunc(A; maxdim, tol)`` (src/mpsutils.jl:116-179): absolute ``tol``, global greedy
    ``maxdim``; ``tieband`` > 0 widens ties (0 = the reference rule).

    ``method``: "exact" per-sector thin SVD; "gram_left" / "gram_right" the density-matrix
    truncation (eigen-decomposition of A A^T / A^T A): u (resp. v) orthonormal, and u*s*v the
    projection of A on the kept singular subspace."""
    if maxdim is None:
        maxdim = max(A.size())
    if method not in SVD_METHODS:
        raise MPSGError(_lib.ERR_ARGUMENT, f"unknown svd method {method!r}")
    u, s, v = C.c_void_p(), C.c_void_p(), C.c_void_p()
    if method == "exact":
        call("mpsg_svdtrunc", A.ctx.handle, A.handle, int(maxdim), float(tol), float(tieband),
             C.byref(u), C.byref(s), C.byref(v))
    else:
        call("mpsg_svdtrunc_gram", A.ctx.handle, A.handle, int(maxdim), float(tol),
             float(tieband), 0 if method == "gram_left" else 1, C.byref(u), C.byref(s),
             C.byref(v))
    return SymTensor(u, A.ctx), SymTensor(s, A.ctx), SymTensor(v, A.ctx)


def svd_complex(Are: SymTensor, Aim: SymTensor, maxdim=None, tol: float = 0.0,
                tieband: float = 0.0, truncate: bool = True):
    """Per-sector SVD of the complex matrix Are + i Aim: (u_re, u_im, s, v_re, v_im) with
    A = u s v per sector, u isometric, s real and v = V^H. ``truncate=False`` keeps every value
    (``_svd_``); otherwise the rule of ``svdtrunc``."""
    if maxdim is None:
        maxdim = max(Are.size())
    out = [C.c_void_p() for _ in range(5)]
    call("mpsg_svd_complex", Are.ctx.handle, Are.handle, Aim.handle, 1 if truncate else 0,
         int(maxdim), float(tol), float(tieband), *[C.byref(o) for o in out])
    return tuple(SymTensor(o, Are.ctx) for o in out)


def truncatedsizes(S, maxdim: int = 200, tol: float = 1e-14, tieband: float = 0.0):
    """``truncatedsizes`` (src/mpsutils.jl:89-112) of a list of descending value lists."""
    lens = [len(s) for s in S]
    vals = [float(x) for s in S for x in s]
    out = (C.c_int64 * len(S))()
    call("mpsg_truncatedsizes", len(S), i64arr(lens), (C.c_double * max(1, len(vals)))(*vals),
         int(maxdim), float(tol), float(tieband), out)
    return list(out)


def small_eigh(A):
    """Eigen-decomposition of a small symmetric matrix on the host (FP64 Jacobi), ascending."""
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    a = np.asfortranarray(A)
    w = np.empty(n)
    v = np.empty((n, n), order="F")
    call("mpsg_small_eigh", n, a.ctypes.data_as(_lib.PF64), w.ctypes.data_as(_lib.PF64),
         v.ctypes.data_as(_lib.PF64))
    return w, v


class EigInfo:
    """Convergence report of ``eigsolve`` (KrylovKit's ``info``: normres, numiter, numops)."""

    def __init__(self, normres, numiter, numops, converged):
        self.normres = normres
        self.numiter = numiter
        self.numops = numops
        self.converged = converged

    def __repr__(self):
        return (f"EigInfo(normres={self.normres:.3e}, numiter={self.numiter}, "
                f"numops={self.numops}, converged={self.converged})")


def _handles(ts):
    return (C.c_void_p * max(1, len(ts)))(*[t.handle for t in ts])


class HeffBatch:
    """The two-site H_eff of many independent chains prepared together (no counterpart in the
    reference, which runs one chain per process): ``ops[i] = (v_like, envL, envR, W1, W2)`` of
    chain i, any structures, one split precision S = 2..7. Every phase of an application is one
    launch over all chains (the split GEMMs one persistent grouped launch each, tile shape and
    order from the tuner), captured in a CUDA graph at its second use when ``graph``."""

    def __init__(self, ops, precision=4, graph=True, ctx=None):
        ops = list(ops)
        if not ops:
            raise MPSGError(_lib.ERR_ARGUMENT, "a batch needs at least one operator")
        # the batch's work runs on ``ctx``; operands may come from other contexts of the device
        # once their producers have finished
        self.ctx = ctx or ops[0][0].ctx
        self.n = len(ops)
        cols = [_handles([o[k] for o in ops]) for k in range(5)]
        h = C.c_void_p()
        call("mpsg_heff2_batch_create", self.ctx.handle, self.n, *cols, int(precision),
             int(bool(graph)), C.byref(h))
        self._h = h
        self._free = _lib.lib.mpsg_heff2_batch_free

    @classmethod
    def from_prepared(cls, ops, ctx, graph=True):
        """The batch of operators from ``Heff2.prepare`` (on any contexts of ``ctx``'s device,
        their contexts synchronised), assembled and run on ``ctx``; the operators may be
        released once this returns."""
        ops = list(ops)
        if not ops:
            raise MPSGError(_lib.ERR_ARGUMENT, "a batch needs at least one operator")
        self = cls.__new__(cls)
        self.ctx = ctx
        self.n = len(ops)
        h = C.c_void_p()
        call("mpsg_heff2_batch_from", ctx.handle, self.n,
             (C.c_void_p * self.n)(*[o._h for o in ops]), int(bool(graph)), C.byref(h))
        self._h = h
        self._free = _lib.lib.mpsg_heff2_batch_free
        return self

    def __call__(self, vs):
        """[H_eff_i(v_i)] in one batched application."""
        vs = list(vs)
        if len(vs) != self.n:
            raise MPSGError(_lib.ERR_ARGUMENT, "one tensor per chain")
        out = (C.c_void_p * self.n)()
        call("mpsg_heff2_batch_apply", self._h, _handles(vs), out)
        return [SymTensor(C.c_void_p(h), self.ctx) for h in out]

    def eigsolve(self, x0s, krylovdim=5, maxiter=8, tol=1e-7):
        """``eigsolve_heff2`` of every chain, the Lanczos recurrences in lock step: returns
        (eigenvalues, eigenvectors, infos)."""
        x0s = list(x0s)
        if len(x0s) != self.n:
            raise MPSGError(_lib.ERR_ARGUMENT, "one start vector per chain")
        n = self.n
        ev = (C.c_double * n)()
        vecs = (C.c_void_p * n)()
        nr = (C.c_double * n)()
        ni, no, cv = (C.c_int32 * n)(), (C.c_int32 * n)(), (C.c_int32 * n)()
        call("mpsg_heff2_batch_eigsolve", self._h, _handles(x0s), int(krylovdim), int(maxiter),
             float(tol), ev, vecs, nr, ni, no, cv)
        return (list(ev), [SymTensor(C.c_void_p(h), self.ctx) for h in vecs],
                [EigInfo(nr[i], ni[i], no[i], bool(cv[i])) for i in range(n)])

    def info(self):
        """dict: reference flops per application, kernels per graph replay (0 before the graph
        exists), applications so far, tuned (N tile, order) of both GEMM stages."""
        f, gk, ap = C.c_double(), C.c_int64(), C.c_int64()
        t = (C.c_int32 * 4)()
        call("mpsg_heff2_batch_info", self._h, C.byref(f), C.byref(gk), C.byref(ap), t)
        return {"ref_flops": f.value, "graph_kernels": gk.value, "applies": ap.value,
                "tuning": [(t[0], t[1]), (t[2], t[3])]}

    def __del__(self):
        try:
            if self._h:
                self._free(self._h)
                self._h = None
        except Exception:
            pass


def tuner(ctx, enable=None):
    """Split-GEMM tuner of a context: ``enable`` True / False switches tuning of single
    prepared operators; returns (shape classes timed, choices served from the table)."""
    r, h = C.c_int64(), C.c_int64()
    call("mpsg_ctx_tuner", ctx.handle, -1 if enable is None else int(bool(enable)), C.byref(r),
         C.byref(h))
    return r.value, h.value


def set_split_tuning(ctx, bn=None, order=0, splitk=0):
    """Fix the split-GEMM configuration of plans built from now on in ``ctx``: N tile ``bn``
    (64, 128 or 0 = default; None returns to the tuner / defaults), tile ``order`` (0 =
    decreasing K, 1 = problem by problem) and ``splitk`` (1: the longest tiles halved along K
    while there are fewer than two waves)."""
    call("mpsg_ctx_set_split_tuning", ctx.handle, -1 if bn is None else int(bn), int(order),
         int(splitk))


def eigsolve_heff2(x0, envL, envR, W1, W2, krylovdim=5, maxiter=8, tol=1e-7, precision=None):
    """``eigsolve(v -> _applymps2site(v, envL, envR, W1, W2), x0, 1, :SR, ishermitian=true)``
    (src/dmrg.jl:77-82): returns (eigenvalue, eigenvector, info)."""
    e = C.c_double()
    x = C.c_void_p()
    nr = C.c_double()
    ni, no, cv = C.c_int32(), C.c_int32(), C.c_int32()
    call("mpsg_eigsolve_heff2", x0.ctx.handle, x0.handle, envL.handle, envR.handle, W1.handle,
         W2.handle, int(krylovdim), int(maxiter), float(tol), _prec(precision), C.byref(e),
         C.byref(x), C.byref(nr), C.byref(ni), C.byref(no), C.byref(cv))
    return e.value, SymTensor(x, x0.ctx), EigInfo(nr.value, ni.value, no.value, bool(cv.value))


# ---------------------------------------------------------------------------------------------
# vector operations (src/symtensor.jl:266-323)
# ---------------------------------------------------------------------------------------------
def dots(As, Bs):
    """[dot(a, b) for a, b in zip(As, Bs)] in one library call (one synchronisation)."""
    n = len(As)
    if n != len(Bs):
        raise MPSGError(_lib.ERR_ARGUMENT, "dots: length mismatch")
    if n == 0:
        return []
    out = (C.c_double * n)()
    ha = (C.c_void_p * n)(*[a.handle for a in As])
    hb = (C.c_void_p * n)(*[b.handle for b in Bs])
    call("mpsg_dots", As[0].ctx.handle, n, ha, hb, out)
    return list(out)


def lincomb(coeffs, Xs, out):
    """out <- sum_i coeffs[i] * Xs[i] in one launch (out may be one of the Xs); returns out."""
    n = len(Xs)
    c = (C.c_double * max(n, 1))(*[float(x) for x in coeffs])
    hx = (C.c_void_p * max(n, 1))(*[x.handle for x in Xs])
    call("mpsg_lincomb", out.ctx.handle, n, c, hx, out.handle)
    return out


def dot(A, B) -> float:
    out = C.c_double()
    call("mpsg_dot", A.ctx.handle, A.handle, B.handle, C.byref(out))
    return out.value


def norm(A) -> float:
    out = C.c_double()
    call("mpsg_norm", A.ctx.handle, A.handle, C.byref(out))
    return out.value


def axpy(alpha, A, B):
    call("mpsg_axpy", A.ctx.handle, float(alpha), A.handle, B.handle)
    return B


def axpby(alpha, A, beta, B):
    call("mpsg_axpby", A.ctx.handle, float(alpha), A.handle, float(beta), B.handle)
    return B


def rmul(A, alpha):
    call("mpsg_rmul", A.ctx.handle, A.handle, float(alpha))
    return A


def mul(B, A, alpha):
    call("mpsg_mul", A.ctx.handle, B.handle, A.handle, float(alpha))
    return B
