"""Shared test helpers: conversion between oracle tensors and device tensors, random inputs."""
import numpy as np

import mps_gb300 as mg
from oracle import symtensors as st


def mg_space(V):
    return mg.VectorSpace(V.sectors, V.isdual)


def st_space(V):
    return st.VectorSpace(V.sectors, V.isdual)


def to_device(T, ctx=None):
    """Upload an oracle tensor (dense blocks expanded for SymDiagonal)."""
    if isinstance(T, st.SymDiagonal):
        T = T.as_dense()
    return mg.from_flat(T.charge, tuple(mg_space(V) for V in T.space),
                        st.flatten(T).astype(np.float64), ctx)


def to_oracle(t):
    return st.from_flat(t.charge, tuple(st_space(V) for V in t.space), t.to_flat())


def rand_tensor(charge, space, rng):
    sects, sizes = st.allsectorsandsizes(charge, space)
    return st.SymTensor(charge, space, {s: rng.standard_normal(z) for s, z in zip(sects, sizes)})


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def assert_tensor_close(dev, T, rtol=1e-12, exact=False):
    """Device tensor vs oracle tensor: same structure, values within rtol (relative Frobenius)."""
    assert dev.charge == T.charge
    assert dev.space == tuple(mg_space(V) for V in T.space)
    assert dev.sectors() == T.sectors()
    got = dev.to_flat()
    want = st.flatten(T)
    if exact:
        assert np.array_equal(got, want)
    else:
        assert relerr(got, want) <= rtol, relerr(got, want)


def oracle_ops():
    """The real operations of ``mps_gb300.ctensor`` implemented by the CPU oracle, so the
    complex / TDVP host logic can be checked without a GPU."""
    from mps_gb300.ctensor import Ops

    def lincomb(terms):
        c0, T0 = terms[0]
        out = st.scaled(T0, c0)
        for c, T in terms[1:]:
            st.axpy(c, T, out)
        return out

    def part(T, f):
        if isinstance(T, st.SymDiagonal):
            return st.SymDiagonal(T.charge, T.space, {k: f(b) for k, b in T.blocks.items()})
        return st.SymTensor(T.charge, T.space, {k: f(b) for k, b in T.blocks.items()},
                            check=False)

    def svdc(re, im, truncate, maxdim, tol, tieband):
        M = st.SymTensor(re.charge, re.space,
                         {s: re.blocks[s] + 1j * im.blocks[s] for s in re.blocks}, check=False)
        if truncate:
            u, s, v = st.svdtrunc(M, maxdim=maxdim, tol=tol, tieband=tieband)
        else:
            u, s, v = st.svd_(M)
        real = lambda b: np.ascontiguousarray(np.real(b))
        imag = lambda b: np.ascontiguousarray(np.imag(b))
        return part(u, real), part(u, imag), part(s, real), part(v, real), part(v, imag)

    def from_blocks(charge, space, blocks):
        return st.from_blocks(charge, space, {k: np.asarray(b, dtype=np.float64)
                                              for k, b in blocks.items()})

    return Ops(st.contract, st.dual, lincomb, lambda A, B: float(np.real(st.dot(A, B))),
               st.symmatrix, st.splitleg, st.matmul, lambda A: A.space, svdc, st.flatten,
               st.fill, from_blocks, st.dual_space, st.fuselegs)


def dense_site(ops, A):
    """Dense complex array of a CTensor site tensor (legs in charge order)."""
    from mps_gb300.ctensor import creal
    A = creal(A)
    re = A.re if not hasattr(A.re, "to_flat") else to_oracle(A.re)
    out = st.array(re).astype(complex)
    if A.im is not None:
        im = A.im if not hasattr(A.im, "to_flat") else to_oracle(A.im)
        out = out + 1j * A.sign * st.array(im)
    return out
