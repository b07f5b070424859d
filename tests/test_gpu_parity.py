"""GPU parity of the C-ABI library against the oracle (FP64 path).

Data-movement operations (permutelegs, fuselegs, splitleg, SymMatrix, split) must be bit-exact;
contractions must agree within 1e-12 relative (Frobenius over the whole tensor), the bar of the
plain FP64 drop-in.  Every call goes through the C ABI of libmpsgb300.so.
"""
import itertools

import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from oracle import symtensors as st
from oracle import mps as om
from oracle.symtensors import U1Space, dual_space as dual

from helpers import to_device, to_oracle, rand_tensor, assert_tensor_close, relerr, mg_space

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def rand_space(rng, lo=-2, hi=3, maxd=4):
    ch = sorted(rng.choice(np.arange(lo, hi), size=rng.integers(1, hi - lo), replace=False))
    return st.VectorSpace([(int(c), int(rng.integers(1, maxd + 1))) for c in ch],
                          bool(rng.integers(2)))


def rand_nonempty(rng, N):
    for _ in range(200):
        sp = tuple(rand_space(rng) for _ in range(N))
        c = int(rng.integers(-1, 2))
        if st.allsectorsandsizes(c, sp)[0]:
            return rand_tensor(c, sp, rng)
    raise RuntimeError


@pytest.mark.parametrize("seed", range(8))
def test_releg_bit_exact(seed):
    rng = np.random.default_rng(seed)
    N = int(rng.integers(2, 6))
    T = rand_nonempty(rng, N)
    A = to_device(T)
    assert_tensor_close(A, T, exact=True)
    for perm in itertools.islice(itertools.permutations(range(1, N + 1)), 8):
        assert_tensor_close(mg.permutelegs(A, perm), st.permutelegs(T, list(perm)), exact=True)
    for l in range(1, N + 1):
        for n in range(1, N - l + 2):
            for d in (False, True):
                F = st.fuselegs(T, l, n, d)
                Fd = mg.fuselegs(A, l, n, d)
                assert_tensor_close(Fd, F, exact=True)
                if n >= 2:
                    sp = [mg_space(V) for V in T.space[l - 1:l - 1 + n]]
                    assert_tensor_close(mg.splitleg(Fd, l, sp), T, exact=True)
    for k in range(1, N):
        perm = [int(x) for x in rng.permutation(range(1, N + 1))]
        assert_tensor_close(mg.SymMatrix(A, perm[:k], perm[k:]),
                            st.symmatrix(T, perm[:k], perm[k:]), exact=True)


def test_reference_kats_on_device():
    """symtensortests.jl "fuse/split", "U1 unitary", "converts" and "matrices" through the GPU."""
    space = (U1Space((0, 2), (1, 3)), U1Space((0, 1), (1, 1)), dual(U1Space((0, 3), (1, 4))))
    blks = [np.arange(1, 7).reshape((2, 1, 3), order="F"),
            np.arange(7, 15).reshape((2, 1, 4), order="F"),
            np.arange(15, 27).reshape((3, 1, 4), order="F")]
    A0 = st.SymTensor(0, space, dict(zip([(0, 0, 0), (0, 1, 1), (1, 0, 1)], blks)))
    d0 = to_device(A0)
    sp = [mg_space(V) for V in space]
    assert np.array_equal(mg.splitleg(mg.fuselegs(d0, 1, 2), 1, sp[0:2]).to_flat(),
                          st.flatten(A0))
    assert np.array_equal(mg.splitleg(mg.fuselegs(d0, 2, 2, True), 2, sp[1:3]).to_flat(),
                          st.flatten(A0))

    E = st.eye(U1Space((0, 1), (1, 2), (2, 1)))
    E[(1, 1)] = np.array([[2.0, 3.0], [4.0, 5.0]])
    d = mg.U1Space((0, 1), (1, 1))
    B = mg.splitleg(mg.splitleg(to_device(E), 2, (mg.dual(d), mg.dual(d))), 1, (d, d))
    assert B.sectors() == sorted([(1, 1, 1, 1), (1, 0, 0, 1), (0, 1, 0, 1), (1, 0, 1, 0),
                                  (0, 1, 1, 0), (0, 0, 0, 0)], key=st.sector_key)
    assert list(B.to_flat()) == [1.0, 2.0, 4.0, 3.0, 5.0, 1.0]

    vlist = (U1Space((0, 2), (1, 3), (2, 4)), U1Space((-2, 4), (-1, 3), (0, 2), (1, 1)),
             U1Space((-1, 1), (0, 2), (1, 3), (2, 4)), U1Space((-2, 3), (-1, 2), (0, 1)))
    L = st.fill_linearindex(0, vlist)
    L = st.SymTensor(0, vlist, {s: b.astype(float) for s, b in L.blocks.items()})
    dl = to_device(L)
    M = mg.SymMatrix(dl, [1, 2], [3, 4]).to_flat()
    assert np.array_equal(M, mg.fuselegs(mg.fuselegs(dl, 3, 2, True), 1, 2).to_flat())

    vl = (U1Space((0, 2), (1, 3), (2, 4)), dual(U1Space((0, 4), (1, 2), (2, 2), (3, 3))),
          U1Space((0, 4), (1, 2), (2, 2), (3, 3)), dual(U1Space((0, 3), (1, 5), (2, 2))))
    Am = st.fill_linearindex(0, vl[0:2])
    Am = st.SymTensor(0, vl[0:2], {s: b.astype(float) for s, b in Am.blocks.items()})
    Bm = st.fill(1.0, 0, vl[2:4])
    C = mg.contract(to_device(Am), (1, -1), to_device(Bm), (-1, 2))
    assert np.array_equal(st.array(to_oracle(C)), st.array(Am) @ st.array(Bm))


@pytest.mark.parametrize("seed", range(10))
def test_contract_random_structures(seed):
    rng = np.random.default_rng(1000 + seed)
    N = int(rng.integers(2, 5))
    T = rand_nonempty(rng, N)
    ncon = int(rng.integers(1, N))
    conlegs = sorted(rng.choice(range(N), size=ncon, replace=False))
    extra = [rand_space(rng) for _ in range(int(rng.integers(1, 3)))]
    Bspace = [st.dual_space(T.space[i]) for i in conlegs] + extra
    order = list(rng.permutation(len(Bspace)))
    Bspace = [Bspace[i] for i in order]
    for cB in (0, 1, -1):
        if st.allsectorsandsizes(cB, Bspace)[0]:
            break
    else:
        pytest.skip("empty partner")
    B = rand_tensor(cB, Bspace, rng)
    idxA, labels = [], {}
    outs = list(rng.permutation(range(1, N - ncon + len(extra) + 1)))
    for i in range(N):
        if i in conlegs:
            labels[i] = -(conlegs.index(i) + 1)
            idxA.append(labels[i])
        else:
            idxA.append(int(outs.pop()))
    idxB = [labels[conlegs[j]] if j < ncon else int(outs.pop()) for j in order]
    R = st.contract(T, idxA, B, idxB)
    Rd = mg.contract(to_device(T), idxA, to_device(B), idxB)
    assert_tensor_close(Rd, R, rtol=RTOL)


def test_full_contraction_scalar():
    rng = np.random.default_rng(5)
    sp = (U1Space((0, 2), (1, 3)), dual(U1Space((0, 3), (1, 2))))
    A = rand_tensor(0, sp, rng)
    B = rand_tensor(0, tuple(st.dual_space(V) for V in sp), rng)
    want = st.contract(A, (-1, -2), B, (-1, -2))
    got = mg.contract(to_device(A), (-1, -2), to_device(B), (-1, -2))
    assert abs(got - want) <= 1e-12 * abs(want)


def heff_inputs(chi, ncharges=25, seed=1911, delta=0.5):
    (sv, sl, sr), flats = gd.heff_inputs_host(chi, delta, seed, ncharges)
    toO = lambda sp: tuple(st.VectorSpace(V.sectors, V.isdual) for V in sp)
    W = om.xxz_u1mpo(3, delta)[1]
    O = [st.from_flat(0, toO(s), f) for s, f in zip((sv, sl, sr), flats)] + [W, W]
    D = list(gd.heff_problem(chi, delta, seed, ncharges=ncharges))
    return O, D


@pytest.mark.parametrize("chi,nq", [(16, 5), (64, 9), (256, 13)])
def test_applymps2site_matches_oracle(chi, nq):
    O, D = heff_inputs(chi, nq)
    want = om.applymps2site(*O)
    got = mg.applymps2site(*D, precision=0)
    assert_tensor_close(got, want, rtol=RTOL)


def test_xxz_mpo_device_equals_oracle():
    for k, (Wd, Wo) in enumerate(zip(gd.xxz_u1mpo(5, 0.7), om.xxz_u1mpo(5, 0.7))):
        assert_tensor_close(Wd, Wo, exact=True)


@pytest.mark.parametrize("chi,nq", [(32, 7), (128, 11)])
def test_env_updates_match_oracle(chi, nq):
    rng = np.random.default_rng(chi)
    Vl = st.VectorSpace([(k, d) for k, d in enumerate(gd.binomial_profile(chi, nq))])
    Vr = st.VectorSpace([(k + 1, d) for k, d in enumerate(gd.binomial_profile(chi, nq))])
    d = U1Space((0, 1), (1, 1))
    Vw = U1Space((-1, 1), (0, 3), (1, 1))
    A = rand_tensor(0, (Vl, d, dual(Vr)), rng)
    W = om.xxz_u1mpo(3, 0.9)[1]
    envL = rand_tensor(0, (dual(Vl), dual(Vw), Vl), rng)
    envR = rand_tensor(0, (Vr, Vw, dual(Vr)), rng)
    assert_tensor_close(mg.mpsupdateleft(to_device(envL), to_device(A), to_device(W)),
                        om.mpsupdateleft(envL, A, W), rtol=RTOL)
    assert_tensor_close(mg.mpsupdateright(to_device(envR), to_device(A), to_device(W)),
                        om.mpsupdateright(envR, A, W), rtol=RTOL)


def test_vector_ops_match_oracle():
    rng = np.random.default_rng(9)
    sp = (U1Space((0, 20), (1, 30), (2, 40)), U1Space((0, 4), (-1, 2), (-2, 2)),
          dual(U1Space((0, 30), (1, 50))))
    A, B = rand_tensor(0, sp, rng), rand_tensor(0, sp, rng)
    dA, dB = to_device(A), to_device(B)
    assert abs(mg.dot(dA, dB) - st.dot(A, B)) <= 1e-12 * abs(st.dot(A, B)) + 1e-12
    assert abs(mg.norm(dA) - st.norm(A)) <= 1e-13 * st.norm(A)
    mg.axpby(0.3, dA, -1.7, dB)
    st.axpby(0.3, A, -1.7, B)
    assert_tensor_close(dB, B, rtol=1e-15)
    mg.axpy(2.5, dA, dB)
    st.axpy(2.5, A, B)
    assert_tensor_close(dB, B, rtol=1e-15)
    mg.rmul(dB, 0.125)
    st.rmul(B, 0.125)
    assert_tensor_close(dB, B, rtol=1e-15)
    before = dB.to_flat()
    mg.rmul(dB, 0.125)  # a power of two scales exactly
    assert np.array_equal(dB.to_flat(), before * 0.125)
    with pytest.raises(mg.SpaceMismatch):
        mg.dot(dA, to_device(rand_tensor(0, sp[:2] + (U1Space((0, 2)),), rng)))


def test_heff_linearity_full_size():
    """chi=2048 workload (the benchmark size): H(a x + b y) == a H x + b H y."""
    v, eL, eR, W1, W2 = gd.heff_problem(2048)
    rng = np.random.default_rng(3)
    y = mg.from_flat(v.charge, v.space, rng.standard_normal(v.numel()))
    z = mg.copy(v)
    mg.axpby(0.7, y, -1.3, z)  # z = 0.7 y - 1.3 v
    Hv = mg.applymps2site(v, eL, eR, W1, W2).to_flat()
    Hy = mg.applymps2site(y, eL, eR, W1, W2).to_flat()
    Hz = mg.applymps2site(z, eL, eR, W1, W2).to_flat()
    assert relerr(Hz, 0.7 * Hy - 1.3 * Hv) < 1e-12
