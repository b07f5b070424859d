"""Complex block-sparse tensors over the real kernels, and the Krylov exponential.

Time evolution needs complex MPS (src/tdvp.jl:19: "TDVP only accepts complex MPSs"). A complex
SymTensor is held as two real SymTensors of identical structure, ``value = re + i*sign*im``
(``im`` None means a real tensor), so every complex operation is a handful of the library's real
block-sparse operations on the GPU:

* contract: (Ar + i Ai)(Br + i Bi) = (ArBr - AiBi) + i(ArBi + AiBr), up to four real
  contractions (two when one operand is real, e.g. an MPO tensor);
* the bra of a state is ``cdual(A)`` = conj(dual(A)): dual spaces and a flipped sign, no copy
  (the reference's ``dual`` does not conjugate, src/symtensor.jl:201-212, so its symmetric path is
  real only);
* complex factorisations go through ``svd_complex`` (cuSOLVER per sector, C ABI
  ``mpsg_svd_complex``).

``Ops`` names the real operations this layer uses, so the same host code runs on the GPU library
(``gpu_ops``) or, in tests, on any other implementation with the same interface.

``exponentiate`` computes exp(t f) x for a Hermitian map f (the role of KrylovKit.exponentiate at
src/tdvp.jl:27,40,52,68,78,122,139,153,172,184): Lanczos with full reorthogonalisation on the
GPU vectors; the host only holds the small tridiagonal matrix and its exponential.
"""
from __future__ import annotations

import numpy as np


class Ops:
    """Real block-sparse operations: contract (tensor, or float when fully contracted), dual,
    lincomb([(c, T), ...]) -> new tensor, dot, symmatrix, splitleg, matmul, space, and
    svd_complex(re, im, truncate, maxdim, tol, tieband) -> (ure, uim, s, vre, vim)."""

    def __init__(self, contract, dual, lincomb, dot, symmatrix, splitleg, matmul, space,
                 svd_complex, download, fill, from_blocks, dual_space, fuselegs, dots=None,
                 ccontract=None):
        self.contract = contract
        self.dual = dual
        self.lincomb = lincomb
        self.dot = dot
        self.symmatrix = symmatrix
        self.splitleg = splitleg
        self.matmul = matmul
        self.space = space
        self.svd_complex = svd_complex
        self.download = download
        self.fill = fill                # fill(x, charge, spaces)
        self.from_blocks = from_blocks  # from_blocks(charge, spaces, {sector: block})
        self.dual_space = dual_space
        self.fuselegs = fuselegs        # fuselegs(A, l, n)
        # dots([(a, b), ...]) -> [dot(a, b), ...] (one synchronisation when batched)
        self.dots = dots if dots is not None else (lambda pairs: [dot(a, b) for a, b in pairs])
        # optional one-call complex contraction: ccontract(ar, ai, sa, ia, br, bi, sb, ib)
        # -> (cr, ci) or a complex number
        self.ccontract = ccontract


def gpu_ops(precision: int = 0, ctx=None) -> Ops:
    """The GPU library's operations on context ``ctx`` (default: the current device's);
    ``precision`` selects the block-GEMM arithmetic of every contraction (0 = FP64)."""
    from . import symtensors as mg

    def lincomb(terms):
        out = mg.similar(terms[0][1])
        return mg.lincomb([c for c, _ in terms], [T for _, T in terms], out)

    def dots(pairs):
        return mg.dots([a for a, _ in pairs], [b for _, b in pairs])

    def ccon(ar, ai, sa, ia, br, bi, sb, ib):
        return mg.contract_complex(ar, ai, sa, ia, br, bi, sb, ib, precision=precision)

    def svdc(re, im, truncate, maxdim, tol, tieband):
        return mg.svd_complex(re, im, maxdim=maxdim, tol=tol, tieband=tieband,
                              truncate=truncate)

    return Ops(lambda A, ia, B, ib: mg.contract(A, ia, B, ib, precision=precision), mg.dual,
               lincomb, mg.dot, mg.SymMatrix, mg.splitleg,
               lambda A, B: mg.matmul(A, B, precision=0), lambda A: A.space, svdc,
               lambda A: A.to_flat(), lambda x, c, sp: mg.fill(x, c, sp, ctx),
               lambda c, sp, b: mg.from_blocks(c, sp, b, ctx), mg.dual, mg.fuselegs, dots,
               ccon)


class CTensor:
    """re + i*sign*im over real tensors of identical structure (im None: a real tensor)."""

    __slots__ = ("re", "im", "sign")

    def __init__(self, re, im=None, sign: float = 1.0):
        self.re = re
        self.im = im
        self.sign = float(sign)


def creal(A) -> CTensor:
    return A if isinstance(A, CTensor) else CTensor(A)


def cdual(ops: Ops, A: CTensor) -> CTensor:
    """The bra of A: conj(dual(A)) (dual spaces, negated charge, conjugated values)."""
    A = creal(A)
    return CTensor(ops.dual(A.re), None if A.im is None else ops.dual(A.im), -A.sign)


def cspace(ops: Ops, A: CTensor):
    return ops.space(creal(A).re)


def _combine(ops: Ops, terms):
    """Sum of (coefficient, real tensor or None) terms as a tensor (None when empty); a single
    term with coefficient +-1 is returned as is, with its sign."""
    terms = [(c, T) for c, T in terms if T is not None and c != 0.0]
    if not terms:
        return None, 1.0
    if len(terms) == 1 and abs(terms[0][0]) == 1.0:
        return terms[0][1], terms[0][0]
    return ops.lincomb(terms), 1.0


def ccontract(ops: Ops, A, ia, B, ib):
    """contract for complex operands (either may be real); a full contraction returns a
    Python complex."""
    A, B = creal(A), creal(B)
    if ops.ccontract is not None:
        r = ops.ccontract(A.re, A.im, A.sign, ia, B.re, B.im, B.sign, ib)
        return r if isinstance(r, complex) else CTensor(r[0], r[1])
    rr = ops.contract(A.re, ia, B.re, ib)
    ri = None if B.im is None else ops.contract(A.re, ia, B.im, ib)
    ir = None if A.im is None else ops.contract(A.im, ia, B.re, ib)
    ii = None if (A.im is None or B.im is None) else ops.contract(A.im, ia, B.im, ib)
    sA, sB = A.sign, B.sign
    if isinstance(rr, float):  # every leg contracted
        re = rr - sA * sB * (ii if ii is not None else 0.0)
        im = sB * (ri if ri is not None else 0.0) + sA * (ir if ir is not None else 0.0)
        return complex(re, im)
    re, sre = _combine(ops, [(1.0, rr), (-sA * sB, ii)])
    if sre != 1.0:
        re = ops.lincomb([(sre, re)])
    im, sim = _combine(ops, [(sB, ri), (sA, ir)])
    return CTensor(re, im, sim)


def clincomb(ops: Ops, terms) -> CTensor:
    """sum_k z_k X_k for complex coefficients z_k and complex tensors X_k."""
    rt, it = [], []
    for z, X in terms:
        X = creal(X)
        z = complex(z)
        rt.append((z.real, X.re))
        it.append((z.imag, X.re))
        if X.im is not None:
            rt.append((-z.imag * X.sign, X.im))
            it.append((z.real * X.sign, X.im))
    re, sre = _combine(ops, rt)
    if re is not None and sre != 1.0:
        re = ops.lincomb([(sre, re)])
    if re is None:  # keep the real part a tensor: 0 * X
        re = ops.lincomb([(0.0, creal(terms[0][1]).re)])
    im, sim = _combine(ops, it)
    return CTensor(re, im, sim)


def cdot(ops: Ops, A, B) -> complex:
    """<A|B> = sum conj(A) B."""
    return cdots(ops, [A], B)[0]


def cdots(ops: Ops, As, B):
    """[<A|B> for A in As] with every real dot product in one batched call."""
    B = creal(B)
    pairs, plan = [], []
    for A in As:
        A = creal(A)
        idx = []
        for (x, y, coef, part) in ((A.re, B.re, 1.0, 0), (A.im, B.im, A.sign * B.sign, 0),
                                   (A.re, B.im, B.sign, 1), (A.im, B.re, -A.sign, 1)):
            if x is None or y is None:
                continue
            idx.append((len(pairs), coef, part))
            pairs.append((x, y))
        plan.append(idx)
    vals = ops.dots(pairs) if pairs else []
    out = []
    for idx in plan:
        z = [0.0, 0.0]
        for k, coef, part in idx:
            z[part] += coef * vals[k]
        out.append(complex(z[0], z[1]))
    return out


def cnorm(ops: Ops, A) -> float:
    A = creal(A)
    pairs = [(A.re, A.re)] + ([] if A.im is None else [(A.im, A.im)])
    n2 = sum(ops.dots(pairs))
    return float(np.sqrt(max(n2, 0.0)))


def cscale(ops: Ops, A, z) -> CTensor:
    return clincomb(ops, [(z, A)])


def csymmatrix(ops: Ops, A, rows, cols) -> CTensor:
    A = creal(A)
    return CTensor(ops.symmatrix(A.re, rows, cols),
                   None if A.im is None else ops.symmatrix(A.im, rows, cols), A.sign)


def cfuselegs(ops: Ops, A, l, n) -> CTensor:
    A = creal(A)
    return CTensor(ops.fuselegs(A.re, l, n),
                   None if A.im is None else ops.fuselegs(A.im, l, n), A.sign)


def csplitleg(ops: Ops, A, l, spaces) -> CTensor:
    A = creal(A)
    return CTensor(ops.splitleg(A.re, l, spaces),
                   None if A.im is None else ops.splitleg(A.im, l, spaces), A.sign)


def cmatmul_real(ops: Ops, s, B) -> CTensor:
    """s * B for a real (diagonal) s and a complex B."""
    B = creal(B)
    return CTensor(ops.matmul(s, B.re), None if B.im is None else ops.matmul(s, B.im), B.sign)


def cmatmul_real_right(ops: Ops, A, s) -> CTensor:
    """A * s for a complex A and a real (diagonal) s."""
    A = creal(A)
    return CTensor(ops.matmul(A.re, s), None if A.im is None else ops.matmul(A.im, s), A.sign)


def csvd(ops: Ops, M, truncate: bool = False, maxdim=None, tol: float = 0.0,
         tieband: float = 0.0):
    """M = u s v per sector (u isometric, s real diagonal, v = V^H); the rule of svdtrunc when
    ``truncate``."""
    M = creal(M)
    im = M.im
    if im is None:
        im = ops.lincomb([(0.0, M.re)])
    elif M.sign != 1.0:
        im = ops.lincomb([(M.sign, im)])
    if maxdim is None:
        maxdim = 1 << 40
    ure, uim, s, vre, vim = ops.svd_complex(M.re, im, truncate, maxdim, tol, tieband)
    return CTensor(ure, uim), s, CTensor(vre, vim)


def cdownload(ops: Ops, A) -> np.ndarray:
    """Flat values (reference block order) as complex128."""
    A = creal(A)
    re = np.asarray(ops.download(A.re), dtype=np.float64)
    if A.im is None:
        return re.astype(np.complex128)
    return re + 1j * A.sign * np.asarray(ops.download(A.im), dtype=np.float64)


# ---------------------------------------------------------------------------------------------
# Krylov exponential
# ---------------------------------------------------------------------------------------------
class ExpInfo:
    def __init__(self, numops, numsteps, converged):
        self.numops = numops
        self.numsteps = numsteps
        self.converged = converged

    def __repr__(self):
        return f"ExpInfo(numops={self.numops}, numsteps={self.numsteps}, converged={self.converged})"


def _expT(alphas, betas, tau):
    """exp(tau T) e_1 for the real symmetric tridiagonal T(alphas, betas) (host, m <= krylovdim)."""
    m = len(alphas)
    T = np.diag(np.asarray(alphas, dtype=float))
    for i in range(m - 1):
        T[i, i + 1] = T[i + 1, i] = betas[i]
    w, Q = np.linalg.eigh(T)
    return Q @ (np.exp(tau * w) * Q[0, :])


def exponentiate(ops: Ops, f, t, x, krylovdim: int = 30, tol: float = 1e-12,
                 maxiter: int = 100):
    """exp(t f) x for a Hermitian map f on complex tensors, t complex: Lanczos with full
    reorthogonalisation (classical Gram-Schmidt, twice, with batched dot products); the Krylov
    dimension is the first m whose a-posteriori error
    beta_m |e_m^T exp(tau T_m) e_1| |x| is within tol for the remaining time tau; when the full
    basis cannot reach that, the step is halved until it can and the integration restarts from
    the new vector. Returns (y, ExpInfo)."""
    scale = cnorm(ops, x)
    if scale == 0.0:
        return x, ExpInfo(0, 0, True)
    v = cscale(ops, x, 1.0 / scale)
    left = 1.0
    numops = numsteps = 0
    converged = True
    while left > 0.0 and numsteps < maxiter:
        numsteps += 1
        V = [v]
        alphas, betas = [], []
        step, c = None, None
        for j in range(krylovdim):
            w = f(V[j])
            numops += 1
            # classical Gram-Schmidt against the whole basis, twice; the first pass's coefficient
            # on V[j] is the Lanczos alpha (the others vanish in exact arithmetic)
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
        y = clincomb(ops, [(complex(c[i]) * scale, V[i]) for i in range(len(c))])
        left = left - step if step < left else 0.0
        scale = cnorm(ops, y)
        v = cscale(ops, y, 1.0 / scale)
    if left > 0.0:
        converged = False
    return cscale(ops, v, scale), ExpInfo(numops, numsteps, converged)
