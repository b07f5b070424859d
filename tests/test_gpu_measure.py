"""Measurements and checkpoints on the GPU: the library's transfers against the same host code
on the oracle's operations, and bit-exact checkpoint round trips of device MPS."""
import numpy as np
import pytest

import mps_gb300 as mg
from helpers import oracle_ops, rand_tensor, to_device
from mps_gb300 import checkpoint as cp
from mps_gb300 import ctensor as ct
from mps_gb300 import dmrg as gd
from mps_gb300 import measure as ms
from mps_gb300 import tdvp as td
from oracle import mps as om
from oracle import symtensors as st
from oracle.symtensors import U1Space, dual_space

pytestmark = pytest.mark.gpu

LX, M = 12, 6


def oracle_state(seed):
    rng = np.random.default_rng(seed)
    d = U1Space((0, 1), (1, 1))
    Vl = U1Space((0, 1))
    As = []
    for site in range(1, LX + 1):
        Vr = U1Space(*om.binomial_bond_dims(LX, site, M, 16))
        As.append(rand_tensor(0, (Vl, d, dual_space(Vr)), rng))
        Vl = Vr
    mps = om.center_at(om.MPState(As, 0), 1)
    mps.As[0] = st.scaled(mps.As[0], 1.0 / st.norm(mps.As[0]))
    return mps


def test_measurements_match_oracle_operations():
    og, oo = ct.gpu_ops(), oracle_ops()
    a, b = oracle_state(31), oracle_state(32)
    ga, gb = [to_device(A) for A in a.As], [to_device(A) for A in b.As]
    sz_g = td.site_operator(og, mg.VectorSpace(gd.SITE), {0: -0.5, 1: 0.5})
    sz_o = td.site_operator(oo, U1Space(*gd.SITE), {0: -0.5, 1: 0.5})
    loc_g, loc_o = ms.measure_site(ga, sz_g, ops=og), ms.measure_site(a.As, sz_o, ops=oo)
    assert max(abs(loc_g[x] - loc_o[x]) for x in loc_o) < 1e-13
    pg, po = ms.measure_pairs(ga, sz_g, sz_g, ops=og), ms.measure_pairs(a.As, sz_o, sz_o, ops=oo)
    assert len(pg) == LX * (LX - 1) // 2
    assert max(abs(pg[k] - po[k]) for k in po) < 1e-13
    eg = ms.measure_mpo(ga, gd.xxz_u1mpo(LX, 1.0), ops=og)[1]
    eo = ms.measure_mpo(a.As, om.xxz_u1mpo(LX, 1.0), ops=oo)[1]
    assert abs(eg - eo) < 1e-12 * max(1.0, abs(eo))
    assert abs(ms.overlap(ga, gb, ops=og) - ms.overlap(a.As, b.As, ops=oo)) < 1e-13
    assert ms.norm(ga, ops=og) == pytest.approx(1.0, abs=1e-13)
    for s_g, s_o in zip(ms.schmidtvalues(ga, ops=og), ms.schmidtvalues(a.As, ops=oo)):
        np.testing.assert_allclose(s_g, s_o, rtol=1e-10, atol=1e-14)


def test_checkpoint_round_trip_on_device(tmp_path):
    ops = ct.gpu_ops()
    mps = gd.mps_from_host(gd.random_mps_host(10, 5, 8, seed=4))
    gd.center_at(mps, 1)
    p = tmp_path / "real.mps"
    cp.save_mps(p, mps)
    back = cp.load_mps(p)
    assert back.center == mps.center
    for A, B in zip(mps.As, back.As):
        assert A.space == B.space and A.charge == B.charge
        np.testing.assert_array_equal(A.to_flat(), B.to_flat())
    # a complex state from time evolution
    Ws = gd.xxz_u1mpo(10, 0.5)
    As = [ct.CTensor(A) for A in mps.As]
    env = td.initialenv(ops, As, Ws)
    td.tdvp1sitesweep(ops, 0.05, As, Ws, env)
    state = gd.MPState(As, center=1)
    p = tmp_path / "complex.mps"
    cp.save_mps(p, state)
    back = cp.load_mps(p)
    for A, B in zip(As, back.As):
        np.testing.assert_array_equal(ct.cdownload(ops, A), ct.cdownload(ops, B))
