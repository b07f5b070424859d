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
