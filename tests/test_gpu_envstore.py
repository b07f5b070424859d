"""Asynchronous host copies of device tensors (mpsg_tensor_download_async / upload_async on the
context's copy stream) and the environment store built on them."""
import gc

import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from mps_gb300.envstore import AsyncTransfer, OffloadedEnvs, PinnedPool

pytestmark = pytest.mark.gpu


def test_async_round_trip_is_exact_and_holds_device_memory():
    v, eL, eR, W1, W2 = gd.heff_problem(256, 0.5, 7, ncharges=15)
    keep = mg.copy(eL)
    want = eL.to_flat()
    charge, space = eL.charge, eL.space
    host = mg.HostBuffer(eL.numel() + 5)  # a larger buffer is fine
    c = mg.download_async(eL, host)
    del eL  # the copy holds the device memory until it has finished
    gc.collect()
    # more work on the context stream while the copy runs
    y = mg.applymps2site(v, keep, eR, W1, W2, precision=0)
    c.synchronize()
    assert c.query()
    np.testing.assert_array_equal(host.array[:want.size], want)
    t = mg.zeros(charge, space)
    u = mg.upload_async(t, host)
    u.wait()  # the context stream waits for the upload; the host does not
    got = mg.copy(t).to_flat()  # a kernel on the context stream reads t
    np.testing.assert_array_equal(got, want)
    assert np.isfinite(y.to_flat()).all()


def test_async_copy_argument_errors():
    v, *_ = gd.heff_problem(64, 0.5, 1911, ncharges=9)
    small = mg.HostBuffer(v.numel() - 1)
    with pytest.raises(mg.MPSGError):
        mg.download_async(v, small)
    with pytest.raises(mg.MPSGError):
        mg.upload_async(v, small)
    ok = mg.HostBuffer(v.numel())  # the context keeps working
    c = mg.download_async(v, ok)
    c.synchronize()
    np.testing.assert_array_equal(ok.array, v.to_flat())


def test_store_round_trips_real_tensors_exactly():
    _, eL, eR, W1, W2 = gd.heff_problem(128, 0.5, 3, ncharges=11)
    envs = [mg.copy(eL), mg.copy(eR), mg.copy(W1), mg.copy(W2), mg.copy(eL)]
    want = [e.to_flat() for e in envs]
    st = OffloadedEnvs(envs, window=2, transfer=AsyncTransfer(pool=PinnedPool()))
    del envs
    for order in (range(5), reversed(range(5)), (0, 4, 1, 3, 2)):
        for i in order:
            st.prefetch((i + 1) % 5)
            np.testing.assert_array_equal(st[i].to_flat(), want[i])
    assert st.downloads >= 3 and st.uploads > 0 and st.prefetches > 0
    assert st.clean_evictions > 0
