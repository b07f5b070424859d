"""GPU checks of the batched form: many chains' two-site H_eff in one grouped launch per phase
(``HeffBatch``), the lock-step Lanczos over them, the CUDA graph replay and the split-GEMM
tuner.  Every batched result is compared with the single-operator path of the same precision
(which the other GPU tests pin to the oracle) and, for the applications, with the FP64 oracle.
"""
import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from oracle import mps as om
from oracle import symtensors as st

from helpers import relerr

pytestmark = pytest.mark.gpu

# heterogeneous operators: (chi, charges, Philox seed)
SHAPES = [(64, 9, 3), (96, 11, 5), (48, 7, 7), (128, 13, 9), (64, 9, 11)]
TOL4 = 2e-8  # 4 slices: the slicing bound of one application


def _ops(ctx, shapes=SHAPES, delta=0.5):
    return [gd.heff_problem(chi, delta, seed, ctx=ctx, ncharges=nq) for chi, nq, seed in shapes]


def _oracle_apply(chi, nq, seed, delta=0.5):
    (sv, sl, sr), flats = gd.heff_inputs_host(chi, delta, seed, nq)
    conv = lambda sp: tuple(st.VectorSpace(V.sectors, V.isdual) for V in sp)
    O = [st.from_flat(0, conv(s), f) for s, f in zip((sv, sl, sr), flats)]
    W = om.xxz_u1mpo(3, delta)[1]
    return st.flatten(om.applymps2site(O[0], O[1], O[2], W, W))


@pytest.mark.parametrize("graph", [False, True])
def test_batch_apply_equals_single_operators(graph):
    ctx = mg.Context(0)
    ops = _ops(ctx)
    B = mg.HeffBatch(ops, precision=4, graph=graph)
    vs = [o[0] for o in ops]
    for rep in range(3):  # the second and third applications replay the graph
        got = B(vs)
        for (op, g, shp) in zip(ops, got, SHAPES):
            single = mg.Heff2(*op, precision=4)(op[0]).to_flat()
            assert relerr(g.to_flat(), single) < 1e-12, (rep, shp)
            assert relerr(g.to_flat(), _oracle_apply(*shp)) < TOL4, (rep, shp)
    info = B.info()
    assert info["applies"] == 3
    assert (info["graph_kernels"] > 0) == graph
    runs, hits = mg.tuner(ctx)
    assert runs + hits >= 2  # both GEMM stages went through the tuner


def test_batch_from_operators_prepared_on_other_contexts():
    """Each chain prepares its share on its own context; the batch is assembled and applied on a
    third context (the chains' operators released right after assembly)."""
    shapes = SHAPES[:3]
    ctxs = [mg.Context(0) for _ in shapes]
    ops = [_ops(c, [shp])[0] for c, shp in zip(ctxs, shapes)]
    prepared = [mg.Heff2.prepare(*op, precision=4) for op in ops]
    with pytest.raises(mg.MPSGError):
        prepared[0](ops[0][0])  # a prepared share cannot be applied alone
    for c in ctxs:
        c.synchronize()
    bctx = mg.Context(0)
    B = mg.HeffBatch.from_prepared(prepared, bctx)
    bctx.synchronize()
    del prepared
    for rep in range(3):
        got = B([op[0] for op in ops])
        bctx.synchronize()
        for op, g, shp in zip(ops, got, shapes):
            single = mg.Heff2(*op, precision=4)(op[0]).to_flat()
            assert relerr(g.to_flat(), single) < 1e-12, (rep, shp)


def test_batch_apply_on_new_inputs():
    """The graph reads the batch's input buffer: new vectors give new results."""
    ctx = mg.Context(0)
    ops = _ops(ctx, SHAPES[:3])
    B = mg.HeffBatch(ops, precision=5, graph=True)
    rng = np.random.default_rng(1)
    for rep in range(3):
        xs = [mg.from_flat(0, op[0].space, rng.standard_normal(op[0].numel()), ctx) for op in ops]
        got = B(xs)
        for op, x, g in zip(ops, xs, got):
            want = mg.Heff2(*op, precision=0)(x).to_flat()
            assert relerr(g.to_flat(), want) < 2e-10


def test_batch_eigsolve_matches_single_solves():
    ctx = mg.Context(0)
    ops = _ops(ctx)
    B = mg.HeffBatch(ops, precision=4)
    x0s = [o[0] for o in ops]
    vals, vecs, infos = B.eigsolve(x0s, krylovdim=6, maxiter=6, tol=1e-9)
    for op, val, vec, info in zip(ops, vals, vecs, infos):
        e1, v1, i1 = mg.eigsolve_heff2(op[0], *op[1:], krylovdim=6, maxiter=6, tol=1e-9,
                                       precision=4)
        assert abs(val - e1) <= 1e-10 * abs(e1)
        assert info.numops == i1.numops and info.numiter == i1.numiter
        assert info.converged == i1.converged
        a, b = vec.to_flat(), v1.to_flat()  # eigenvectors agree up to sign
        assert min(relerr(a, b), relerr(a, -b)) < 1e-7
        assert abs(np.linalg.norm(a) - 1.0) < 1e-12
    assert B.info()["graph_kernels"] > 0


def test_batch_rejects_what_it_cannot_do():
    ctx = mg.Context(0)
    ops = _ops(ctx, SHAPES[:2])
    with pytest.raises(mg.MPSGError):
        mg.HeffBatch(ops, precision=0)  # the batch is the split-precision path
    B = mg.HeffBatch(ops, precision=4)
    with pytest.raises(mg.MPSGError):
        B([ops[1][0], ops[0][0]])  # structures swapped
    with pytest.raises(mg.MPSGError):
        B.eigsolve([o[0] for o in ops], krylovdim=40)


def test_lockstep_chains_match_one_by_one():
    """Lock-step DMRG of independent chains (one batched eigensolve per step) against the same
    chains run one by one through the single-operator path: same sweeps, same energies."""
    specs = [(12, 0.4, 16), (16, 1.1, 24), (10, 0.0, 8), (14, 0.7, 32)]
    o = gd.SweepOptions(tol=1e-10, lanczostol=1e-9, krylovdim=5, krylovmaxiter=6, precision=4,
                        energy_precision=7, env_precision=7, svd="exact")
    stats = {}
    e_lock = gd.run_chains_lockstep(specs, 2, o, stats=stats)
    e_one = gd.run_chains(specs, 2, o, threads=1)
    for a, b in zip(e_lock, e_one):
        assert abs(a - b) <= 1e-10 * abs(b), (a, b)
    assert stats["batches"] >= 2 * (2 * 16 - 3)  # the longest chain: 2L - 3 eigensolves a sweep
    assert max(stats["chains_per_batch"]) == len(specs)
    # dynamic batching (whatever is waiting) gives the same energies
    e_dyn = gd.run_chains_lockstep(specs, 2, o, wait_all=False)
    for a, b in zip(e_dyn, e_one):
        assert abs(a - b) <= 1e-10 * abs(b), (a, b)
