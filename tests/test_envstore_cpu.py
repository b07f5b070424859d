"""Environment residency store: window, least-recently-used eviction to host copies, exact
round trips (host logic with stand-in tensors)."""
import numpy as np
import pytest

from mps_gb300.envstore import OffloadedEnvs


class Fake:
    def __init__(self, charge, space, flat):
        self.charge, self.space, self.flat = charge, space, np.array(flat)

    def to_flat(self):
        return self.flat.copy()


def load(charge, space, flat):
    return Fake(charge, space, flat)


def test_window_and_exact_round_trips():
    rng = np.random.default_rng(0)
    envs = [None] + [Fake(i, ("V", i), rng.standard_normal(5)) for i in range(1, 9)] + [None]
    want = {i: e.flat.copy() for i, e in enumerate(envs) if e is not None}
    st = OffloadedEnvs(envs, window=3, load=load)
    assert len(st) == 10 and len(st.resident()) == 3 and st.downloads == 5
    assert st[0] is None and st[9] is None
    # a sweep-like access pattern: every value comes back exactly, the window holds
    for i in list(range(1, 9)) + list(range(8, 0, -1)):
        e = st[i]
        np.testing.assert_array_equal(e.flat, want[i])
        assert e.charge == i and e.space == ("V", i)
        assert len(st.resident()) <= 3
    assert st.uploads > 0
    # writes replace host copies and count as most recent
    st[2] = Fake(2, ("V", 2), np.zeros(5))
    assert st.resident()[-1] == 2
    np.testing.assert_array_equal(st[2].flat, np.zeros(5))
    st[2] = None
    assert st[2] is None
    with pytest.raises(IndexError):
        st[10]
    with pytest.raises(ValueError):
        OffloadedEnvs(envs, window=0, load=load)
