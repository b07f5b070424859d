"""Reverse-mode gradients through block-sparse contractions (the adjoint kernels of the
environment and effective-Hamiltonian networks).

The adjoint of a contraction is again a contraction. For C = contract(A, ia, B, ib):

    dA = contract(dC, ia', dual(B), ib')

where the legs of dC that came from A get output labels at their position in A, the legs of dC
that came from B and the open legs of B are paired by fresh negative labels, and the legs of B
that were contracted with A get A's positions. ``dual`` gives B's legs the dual spaces the
contraction needs (flipped arrows, same blocks, negated charge), so dA has A's charge and spaces
and every adjoint runs on the same planner and GPU kernels as the forward pass (and in the same
precision). A full contraction (a number) has dA = dS * permutelegs(dual(B), ...).

A ``Tape`` records contract / dual calls on any backend with the SymTensors vector interface
(``contract, dual, permutelegs, axpy, scaled`` and ``dot``): the GPU library (``mps_gb300``)
or the CPU oracle. ``mpo_expectation`` builds <psi|O|psi> by left environment updates
(src/apply.jl:49-58), keeping every environment (the checkpoints the backward pass reads), so
gradients of energies with respect to site tensors and MPO tensors (and through the MPO, to
Hamiltonian couplings such as the XXZ anisotropy) cost one backward sweep.
"""
from __future__ import annotations

_FRESH = 1000  # offset of the negative labels that pair legs in an adjoint contraction


class Backend:
    """The operations a tape needs, bound to a module (mps_gb300 or the CPU oracle)."""

    def __init__(self, contract, dual, permutelegs, axpy, scaled, dot):
        self.contract = contract
        self.dual = dual
        self.permutelegs = permutelegs
        self.axpy = axpy
        self.scaled = scaled
        self.dot = dot


def gpu_backend():
    from . import symtensors as mg

    def scaled(A, a):
        return mg.rmul(mg.copy(A), a)

    return Backend(lambda A, ia, B, ib: mg.contract(A, ia, B, ib, precision=0), mg.dual,
                   mg.permutelegs, mg.axpy, scaled, mg.dot)


def contract_vjp(be: Backend, A, ia, B, ib, dC):
    """(dA, dB) of C = contract(A, ia, B, ib) for the cotangent dC (a tensor, or a number when
    every leg is contracted)."""
    ia, ib = tuple(int(x) for x in ia), tuple(int(x) for x in ib)
    return _vjp_one(be, ia, B, ib, dC), _vjp_one(be, ib, A, ia, dC)


def _vjp_one(be: Backend, ix, Y, iy, dC):
    """Cotangent of the operand X (index tuple ix) of contract(X, ix, Y, iy)."""
    if not any(lab > 0 for lab in ix + iy):  # full contraction: dX = dC * Y in X's leg order
        pos = {lab: k for k, lab in enumerate(iy)}
        perm = [pos[lab] + 1 for lab in ix]
        return be.scaled(be.permutelegs(be.dual(Y), perm), float(dC))
    nC = sum(1 for lab in ix + iy if lab > 0)
    idx_dc = []
    for p in range(1, nC + 1):
        idx_dc.append(ix.index(p) + 1 if p in ix else -(_FRESH + p))
    idx_y = [-(_FRESH + lab) if lab > 0 else ix.index(lab) + 1 for lab in iy]
    return be.contract(dC, tuple(idx_dc), be.dual(Y), tuple(idx_y))


class Tape:
    """Records contractions and duals; ``backward`` propagates cotangents to every input."""

    def __init__(self, be: Backend):
        self.be = be
        self.ops = []

    def contract(self, A, ia, B, ib):
        C = self.be.contract(A, ia, B, ib)
        self.ops.append(("contract", A, tuple(ia), B, tuple(ib), C))
        return C

    def dual(self, A):
        D = self.be.dual(A)
        self.ops.append(("dual", A, D))
        return D

    def backward(self, out, seed):
        """Cotangents of every recorded input given d(out) = seed (``out`` is a recorded
        result: a tensor, or the number a full contraction returned); returns grad(x), None for
        objects the output does not depend on. Objects are matched by identity; the tape keeps
        every recorded object alive."""
        grads = {id(out): seed}

        def acc(x, g):
            k = id(x)
            if k in grads:  # sum into a fresh copy: a stored cotangent may share storage (dual)
                grads[k] = self.be.axpy(1.0, g, self.be.scaled(grads[k], 1.0))
            else:
                grads[k] = g

        for op in reversed(self.ops):
            if op[0] == "dual":
                _, A, D = op
                if id(D) in grads:
                    acc(A, self.be.dual(grads[id(D)]))
            else:
                _, A, ia, B, ib, C = op
                g = grads.get(id(C))
                if g is None:
                    continue
                dA, dB = contract_vjp(self.be, A, ia, B, ib, g)
                acc(A, dA)
                acc(B, dB)
        return lambda x: grads.get(id(x))


def energy_gradients(As, Ws):
    """<psi|H|psi> of a device MPS and MPO and the cotangent map of every site and MPO tensor
    (one forward and one backward sweep of FP64 contractions on the GPU)."""
    from . import symtensors as mg
    from .symtensors import dual as dsp
    tape = Tape(gpu_backend())
    ctx = As[0].ctx
    lVa, rVa = As[0].space[0], dsp(As[-1].space[2])
    lVw, rVw = Ws[0].space[0], dsp(Ws[-1].space[2])
    Lb = mg.fill(1.0, 0, (dsp(lVa), dsp(lVw), lVa), ctx)
    Rb = mg.fill(1.0, 0, (rVa, rVw, dsp(rVa)), ctx)
    E = mpo_expectation(tape, As, Ws, Lb, Rb)
    return float(E), tape.backward(E, 1.0)


def xxz_delta_derivative(g, Ws, lx):
    """dE/dDelta of the XXZ chain from the MPO cotangents: the MPO is linear in Delta, so
    dW/dDelta = W(Delta=1) - W(Delta=0) site by site (src/symmpo.jl:45-97); tensors shared by
    several sites carry the summed cotangent once."""
    from . import dmrg as gd
    from . import symtensors as mg
    W1, W0 = gd.xxz_u1mpo(lx, 1.0, ctx=Ws[0].ctx), gd.xxz_u1mpo(lx, 0.0, ctx=Ws[0].ctx)
    seen, total = set(), 0.0
    for W, a, b in zip(Ws, W1, W0):
        if id(W) in seen or g(W) is None:
            continue
        seen.add(id(W))
        total += mg.dot(g(W), mg.axpy(-1.0, b, mg.copy(a)))
    return total


def _left_update(contract, dual, L, A, W):
    """One left environment update (src/apply.jl:49-58) with the given contract / dual."""
    t = contract(L, (-1, 3, 4), A, (-1, 2, 1))
    t = contract(t, (1, -1, -2, 4), W, (-2, 2, 3, -1))
    return contract(t, (1, -1, 2, -2), dual(A), (-2, -1, 3))


def checkpointed_gradients(be: Backend, As, Ws, Lb, Rb, every: int | None = None):
    """<psi|O|psi> and the cotangent map of every site and MPO tensor, keeping only every
    ``every``-th left environment (default ceil(sqrt(L))) instead of all of them and every
    intermediate: the backward sweep recomputes one segment at a time from its checkpoint on a
    fresh tape and propagates the environment cotangent to the previous checkpoint. Memory is
    O(L / every + every) environments instead of O(3 L); the extra cost is one more forward
    sweep. Results equal ``mpo_expectation`` + ``Tape.backward`` (same contractions)."""
    import math
    lx = len(As)
    k = every if every else max(1, math.ceil(math.sqrt(lx)))
    ckpt = {0: Lb}
    L = Lb
    for x in range(lx):
        L = _left_update(be.contract, be.dual, L, As[x], Ws[x])
        if (x + 1) % k == 0 and x + 1 < lx:
            ckpt[x + 1] = L
    E = be.contract(L, (-1, -2, -3), Rb, (-1, -2, -3))
    dL = _vjp_one(be, (-1, -2, -3), Rb, (-1, -2, -3), 1.0)
    del L
    grads = {}

    def acc(x, g):
        if g is None:
            return
        k_ = id(x)
        grads[k_] = g if k_ not in grads else be.axpy(1.0, g, be.scaled(grads[k_], 1.0))

    end = lx
    for c in sorted(ckpt, reverse=True):
        tape = Tape(be)
        L = ckpt.pop(c)
        L0 = L
        for x in range(c, end):
            L = _left_update(tape.contract, tape.dual, L, As[x], Ws[x])
        g = tape.backward(L, dL)
        for x in range(c, end):
            if id(As[x]) not in {id(a) for a in As[x + 1:end]}:  # once per object per segment
                acc(As[x], g(As[x]))
        for W in {id(w): w for w in Ws[c:end]}.values():
            acc(W, g(W))
        dL = g(L0)
        end = c
    return float(E), lambda t: grads.get(id(t))


def energy_gradients_checkpointed(As, Ws, every: int | None = None):
    """``energy_gradients`` with checkpointed environments on the GPU library."""
    from . import symtensors as mg
    from .symtensors import dual as dsp
    ctx = As[0].ctx
    lVa, rVa = As[0].space[0], dsp(As[-1].space[2])
    lVw, rVw = Ws[0].space[0], dsp(Ws[-1].space[2])
    Lb = mg.fill(1.0, 0, (dsp(lVa), dsp(lVw), lVa), ctx)
    Rb = mg.fill(1.0, 0, (rVa, rVw, dsp(rVa)), ctx)
    return checkpointed_gradients(gpu_backend(), As, Ws, Lb, Rb, every)


def mpo_expectation(tape: Tape, As, Ws, Lb, Rb):
    """<psi|O|psi> for the MPS tensors As (legs (Vl, d, dual(Vr))) and the MPO Ws by left
    environment updates (src/apply.jl:49-58) from the boundary Lb, closed with Rb. Every
    environment is kept on the tape."""
    L = Lb
    for A, W in zip(As, Ws):
        L = _left_update(tape.contract, tape.dual, L, A, W)
    return tape.contract(L, (-1, -2, -3), Rb, (-1, -2, -3))
