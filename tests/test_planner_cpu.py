"""CPU checks of the C-ABI library: it loads, exports every declared symbol, and its sector
planner reproduces the oracle's bookkeeping bit-exactly (sector lists, order, sizes, spaces and
dual flags) for every operation of the hot path.  No GPU is touched: structure-only tensors
carry sector tables without data."""
import itertools
import os
import re

import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import _lib
from oracle import symtensors as st
from oracle import mps as om

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            names.update(re.findall(r"\b(mpsg_\w+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    names = declared_symbols()
    assert len(names) > 30
    for n in names:
        assert hasattr(_lib.lib, n), n
    assert set(names) >= set(_lib.SIGNATURES)


def test_library_is_in_tree_and_built_for_sm103a():
    assert os.path.dirname(_lib.LIB_PATH) == os.path.join(ROOT, "mps_gb300")
    assert _lib.lib.mpsg_version() == 1


def to_mg_space(V):
    return mg.VectorSpace(V.sectors, V.isdual)


def mg_meta(T):
    return mg.meta(T.charge, tuple(to_mg_space(V) for V in T.space))


def assert_same_structure(m, T):
    """m: structure-only mps_gb300 tensor; T: oracle tensor."""
    assert m.charge == T.charge
    assert m.space == tuple(to_mg_space(V) for V in T.space)
    assert m.sectors() == T.sectors()
    assert m.block_sizes() == [tuple(np.shape(b)) for b in T.blocks.values()]


def rand_space(rng, lo=-2, hi=3, maxd=3, dual=None):
    ch = sorted(rng.choice(np.arange(lo, hi), size=rng.integers(1, hi - lo), replace=False))
    isd = bool(rng.integers(2)) if dual is None else dual
    return st.VectorSpace([(int(c), int(rng.integers(1, maxd + 1))) for c in ch], isd)


def rand_struct(rng, N, charge=None):
    for _ in range(100):
        sp = tuple(rand_space(rng) for _ in range(N))
        c = int(rng.integers(-1, 2)) if charge is None else charge
        sects, _ = st.allsectorsandsizes(c, sp)
        if sects:
            return st.fill(0.0, c, sp)
    raise RuntimeError("no non-empty random tensor")


@pytest.mark.parametrize("seed", range(12))
def test_allsectors_and_relegs_match_oracle(seed):
    rng = np.random.default_rng(seed)
    N = int(rng.integers(2, 6))
    T = rand_struct(rng, N)
    m = mg_meta(T)
    assert_same_structure(m, T)
    for perm in itertools.islice(itertools.permutations(range(1, N + 1)), 6):
        assert_same_structure(mg.permutelegs(m, perm), st.permutelegs(T, list(perm)))
    for l in range(1, N + 1):
        for n in range(1, N - l + 2):
            for d in (False, True):
                F = st.fuselegs(T, l, n, d)
                mf = mg.fuselegs(m, l, n, d)
                assert_same_structure(mf, F)
                if n >= 2:
                    back = st.splitleg(F, l, T.space[l - 1:l - 1 + n])
                    assert_same_structure(mg.splitleg(mf, l, [to_mg_space(V) for V in
                                                              T.space[l - 1:l - 1 + n]]), back)


@pytest.mark.parametrize("seed", range(10))
def test_symmatrix_and_contract_structure_match_oracle(seed):
    rng = np.random.default_rng(100 + seed)
    N = int(rng.integers(2, 5))
    T = rand_struct(rng, N)
    m = mg_meta(T)
    for k in range(1, N):
        perm = list(rng.permutation(range(1, N + 1)))
        rows, cols = [int(x) for x in perm[:k]], [int(x) for x in perm[k:]]
        assert_same_structure(mg.SymMatrix(m, rows, cols), st.symmatrix(T, rows, cols))
    # contract T with a partner built on the dual of some of its legs
    ncon = int(rng.integers(1, N))
    conlegs = sorted(rng.choice(range(N), size=ncon, replace=False))
    extra = [rand_space(rng) for _ in range(int(rng.integers(1, 3)))]
    Bspace = [st.dual_space(T.space[i]) for i in conlegs] + extra
    order = list(rng.permutation(len(Bspace)))
    Bspace = [Bspace[i] for i in order]
    for cB in (-1, 0, 1):
        if st.allsectorsandsizes(cB, Bspace)[0]:
            break
    else:
        pytest.skip("empty partner")
    B = st.fill(0.0, cB, Bspace)
    idxA, labels = [], {}
    free = N - ncon + len(extra)
    outs = list(rng.permutation(range(1, free + 1)))
    for i in range(N):
        if i in conlegs:
            lab = -(conlegs.index(i) + 1)
            idxA.append(lab)
            labels[i] = lab
        else:
            idxA.append(int(outs.pop()))
    idxB = []
    for j in order:
        if j < ncon:
            idxB.append(labels[conlegs[j]])
        else:
            idxB.append(int(outs.pop()))
    R = st.contract(T, idxA, B, idxB)
    mR = mg.contract(m, idxA, mg_meta(B), idxB)
    assert_same_structure(mR, R)


def test_contract_errors_like_reference():
    T = st.fill(0.0, 0, (st.U1Space((0, 2)), st.dual_space(st.U1Space((0, 3)))))
    m = mg_meta(T)
    with pytest.raises(mg.SpaceMismatch):
        mg.contract(m, (1, -1), m, (-1, 2))  # dims 3 vs 2 do not contract
    with pytest.raises(mg.MPSGError):
        mg.SymMatrix(m, [1, 1], [])


def binomial_space(chi, ncharges=25, offset=0):
    """Bond space of a chi-dimensional bond: largest-remainder rounding of chi*C(n-1,k)/2^(n-1)
    with a floor of 1 per charge (the binomial sector profile of the chi=2048 workload)."""
    from mps_gb300.dmrg import binomial_profile
    return mg.VectorSpace([(offset + k, d) for k, d in enumerate(binomial_profile(chi, ncharges))])


@pytest.mark.parametrize("chi,nq", [(64, 9), (2048, 25)])
def test_folded_heff_plans_self_check(chi, nq):
    """The tensor-core H_eff (W folded into the environments, intermediate never materialised):
    every copy/GEMM window in bounds, every element written once, and the composed copy of the
    intermediate equal to split-then-fuse, element by element."""
    from mps_gb300 import dmrg
    prob = dmrg.heff_problem(chi, meta_only=True, ncharges=nq)
    _lib.call("mpsg_plan_heff2_check", *[t.handle for t in prob])


def test_heff_chain_structure_at_chi2048():
    """The chi=2048 H_eff workload: v has 96 blocks and 1.8 M elements, and the planned flops
    of the four contractions add up to about 9.7 GFLOP."""
    from mps_gb300 import dmrg
    prob = dmrg.heff_problem(2048, meta_only=True)
    v, envL, envR, W1, W2 = prob
    assert v.nblocks() == 96
    assert 1_700_000 < v.numel() < 1_900_000
    f = dmrg.heff_flops_meta(*prob)
    assert 9.0e9 < f < 10.5e9


def test_empty_structures_match_oracle():
    """A charge no sector can carry gives a tensor without blocks; relegs, SymMatrix and
    contractions of it stay empty, as in the reference (SortedDicts without entries)."""
    Vo = st.VectorSpace([(0, 2), (1, 3)])
    W = st.VectorSpace([(-1, 1), (0, 2)])
    T = st.fill(0.0, 5, (Vo, Vo, W))
    m = mg_meta(T)
    assert m.sectors() == [] and m.numel() == 0
    assert_same_structure(m, T)
    assert_same_structure(mg.permutelegs(m, (3, 1, 2)), st.permutelegs(T, [3, 1, 2]))
    F = st.fuselegs(T, 1, 2)
    mf = mg.fuselegs(m, 1, 2)
    assert_same_structure(mf, F)
    assert_same_structure(mg.splitleg(mf, 1, [to_mg_space(Vo), to_mg_space(Vo)]),
                          st.splitleg(F, 1, (Vo, Vo)))
    assert_same_structure(mg.SymMatrix(m, [1, 3], [2]), st.symmatrix(T, [1, 3], [2]))
    B = st.fill(0.0, 0, (st.dual_space(W), Vo))
    assert_same_structure(mg.contract(m, (1, 2, -1), mg_meta(B), (-1, 3)),
                          st.contract(T, (1, 2, -1), B, (-1, 3)))
