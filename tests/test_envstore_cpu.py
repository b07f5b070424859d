"""Environment residency store: window, least-recently-used eviction to host copies, exact
round trips (host logic with stand-in tensors)."""
import os

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


# ---- asynchronous transfers: a fake copy stream whose copies finish when the test says so -----
class _Stream:
    def __init__(self):
        self.queue = []  # copies in issue order (one in-order copy stream)

    def complete(self, k=None):
        k = len(self.queue) if k is None else min(k, len(self.queue))
        for _ in range(k):
            self.queue.pop(0).run()

    def run_until(self, c):
        while c in self.queue:
            self.complete(1)


class _Buf:
    def __init__(self, n):
        self.n, self.data, self.users = n, np.full(max(n, 1), np.nan), 0


class _Copy:
    def __init__(self, stream, fn, buf):
        self.done, self.fn, self.buf = False, fn, buf
        buf.users += 1
        stream.queue.append(self)

    def run(self):
        self.fn()
        self.done = True
        self.buf.users -= 1


class _T:
    """Device tensor stand-in; ``space = (name, index, n)`` carries its size."""

    def __init__(self, charge, space, flat):
        self.charge, self.space, self.flat = charge, space, flat
        self.unordered = None  # upload the context stream is not yet ordered after
        self.after = None

    def numel(self):
        return self.space[2]


class _FakeAsync:
    def __init__(self, stream):
        from mps_gb300.envstore import PinnedPool
        self.stream = stream
        self.pool = PinnedPool(alloc=_Buf, keep=2)

    def download(self, t):
        buf = self.pool.take(t.numel())
        assert buf.users == 0, "pinned buffer reused while a copy still uses it"
        n = t.numel()
        c = _Copy(self.stream, lambda: buf.data.__setitem__(slice(0, n), t.flat), buf)
        return (t.charge, t.space, buf), c

    def upload(self, entry):
        charge, space, buf = entry
        n = space[2]
        t = _T(charge, space, np.full(n, np.nan))
        c = _Copy(self.stream, lambda: t.flat.__setitem__(slice(None), buf.data[:n]), buf)
        c.dst = t
        t.unordered = c
        return t, c

    def ready(self, c):
        return c.done

    def order(self, c):
        c.dst.unordered = None
        c.dst.after = c

    def release(self, entry):
        assert entry[2].users == 0, "host copy released while a copy still uses it"
        self.pool.give(entry[2])


def _read(stream, t):
    """What a kernel on the context stream sees when it reads t."""
    assert t.unordered is None, "read before the context stream was ordered after the upload"
    if t.after is not None:
        stream.run_until(t.after)
    return t.flat.copy()


@pytest.mark.parametrize("seed,lazy", [(0, False), (1, False), (2, True), (3, True)])
def test_async_transfers_in_a_sweep_pattern(seed, lazy):
    """lazy: copies finish only when a read needs them, so downloads are still running when
    their entries are overwritten or their buffers come up for reuse."""
    rng = np.random.default_rng(seed)
    lx = 12
    stream = _Stream()
    sizes = [int(rng.integers(3, 9)) for _ in range(lx + 2)]
    envs = [_T(0, ("E", i, sizes[i]), rng.standard_normal(sizes[i])) for i in range(lx + 2)]
    want = {i: e.flat.copy() for i, e in enumerate(envs)}
    st = OffloadedEnvs(envs, window=3, transfer=_FakeAsync(stream))

    def check(i):
        got = _read(stream, st[i])
        np.testing.assert_array_equal(got, want[i])
        return got

    def write(i, base):
        flat = base + 0.5 * i
        want[i] = flat.copy()
        st[i] = _T(0, ("E", i, flat.size), flat)

    for _ in range(2):  # two full sweeps, copies finishing at random points
        for l in range(1, lx - 1):
            st.prefetch(min(l + 3, lx + 1))
            stream.complete(0 if lazy else int(rng.integers(0, 3)))
            check(l + 2)
            write(l, np.resize(check(l - 1), sizes[l]))
            assert len(st.resident()) <= 4
        for l in range(lx - 1, 1, -1):
            st.prefetch(l - 2)
            stream.complete(0 if lazy else int(rng.integers(0, 3)))
            check(l - 1)
            write(l + 1, np.resize(check(l + 2), sizes[l + 1]))
    stream.complete()
    assert st.in_flight() == 0
    for i in range(lx + 2):
        check(i)
    assert st.prefetches > 0 and st.prefetch_hits > 0
    assert st.clean_evictions > 0 and st.downloads > 0 and st.uploads > 0


def test_overwrite_during_copies_defers_the_buffer():
    """An entry overwritten while its download (or a prefetched upload) is still running keeps
    its host buffer out of the pool until those copies finish."""
    stream = _Stream()
    tr = _FakeAsync(stream)
    a = _T(0, ("E", 0, 4), np.arange(4.0))
    b = _T(0, ("E", 1, 4), np.arange(4.0) + 10)
    st = OffloadedEnvs([a, b], window=1, transfer=tr)  # a's download is queued, not finished
    assert st.downloads == 1 and st.in_flight() == 1
    st[0] = _T(0, ("E", 0, 4), np.zeros(4))           # overwrite: the download still runs
    # (and 1 leaves the one-entry window: a second download)
    assert st.downloads == 2 and st.in_flight() == 2 and not tr.pool._free
    stream.complete()
    assert st.in_flight() == 0 and len(tr.pool._free) == 1
    # now 1 is on the host; prefetch it, then overwrite it before it is read
    assert st.prefetch(1)
    st[1] = _T(0, ("E", 1, 4), np.ones(4))
    assert st.in_flight() >= 1
    stream.complete()
    assert st.in_flight() == 0
    np.testing.assert_array_equal(_read(stream, st[1]), np.ones(4))
    np.testing.assert_array_equal(_read(stream, st[0]), np.zeros(4))


def test_pinned_pool_best_fit_and_bound():
    from mps_gb300.envstore import PinnedPool
    pool = PinnedPool(alloc=_Buf, keep=2)
    a, b, c = pool.take(10), pool.take(40), pool.take(15)
    assert pool.allocated == 3
    for x in (a, b, c):
        pool.give(x)
    assert len(pool._free) == 2            # the oldest free buffer was dropped
    assert pool.take(8) is c               # smallest free buffer within 2x
    assert pool.take(8) is not b           # b (40) is more than twice 8: a new buffer
    assert pool.allocated == 4
    assert pool.take(25) is b              # 40 <= 2 * 25


def test_file_transfer_round_trips_and_cleans_up(tmp_path):
    """Host copies in files (as the reference's environment I/O keeps them): exact round trips
    in a sweep-like pattern, and no file outlives its entry's overwrite."""
    from mps_gb300.envstore import FileTransfer
    rng = np.random.default_rng(4)
    envs = [Fake(i, ("V", i), rng.standard_normal(7)) for i in range(8)]
    want = {i: e.flat.copy() for i, e in enumerate(envs)}
    st = OffloadedEnvs(envs, window=2, transfer=FileTransfer(str(tmp_path), load))
    assert len(list(tmp_path.iterdir())) == 6
    for i in list(range(8)) + list(range(7, -1, -1)):
        np.testing.assert_array_equal(st[i].flat, want[i])
    for i in range(8):  # overwrite everything: the old files go
        st[i] = Fake(i, ("V", i), np.full(7, float(i)))
    for i in range(8):
        np.testing.assert_array_equal(st[i].flat, np.full(7, float(i)))
    # every file left belongs to a current host copy, one file each
    assert sorted(p.name for p in tmp_path.iterdir()) == sorted(
        os.path.basename(e[2]) for e in st._host.values())
    assert st.transfer.bytes_down > 0 and st.transfer.bytes_up > 0


def test_file_transfer_rejects_a_truncated_file(tmp_path):
    from mps_gb300.envstore import FileTransfer
    tr = FileTransfer(str(tmp_path), load)
    entry, _ = tr.download(Fake(0, ("V", 0), np.arange(6.0)))
    with open(entry[2], "r+b") as f:
        f.truncate(8 * 5)
    with pytest.raises(OSError):
        tr.upload(entry)
    tr.release(entry)
    assert not os.path.exists(entry[2])
    tr.release(entry)  # releasing twice is harmless


def test_byte_budget_bounds_the_resident_entries():
    sizes = [4, 40, 8, 16, 4, 64, 8]
    envs = [Fake(i, ("V", i), np.arange(float(n))) for i, n in enumerate(sizes)]
    want = {i: e.flat.copy() for i, e in enumerate(envs)}
    budget = 8 * 48
    st = OffloadedEnvs(envs, window=7, load=load, budget_bytes=budget)
    assert st.resident_bytes() <= budget
    for i in list(range(7)) + list(range(6, -1, -1)):
        np.testing.assert_array_equal(st[i].flat, want[i])
        # the entry just read stays even when it alone exceeds the budget (index 5: 64 doubles)
        assert st.resident()[-1] == i
        assert st.resident_bytes() <= max(budget, 8 * sizes[i])
    with pytest.raises(ValueError):
        OffloadedEnvs(envs, load=load, budget_bytes=0)


def test_byte_budget_keeps_the_entry_just_used_beside_pending_prefetches():
    """A budget below two entries while the only other resident entries are prefetches that the
    sweep has not read: eviction takes a prefetch, never the entry just read."""
    stream = _Stream()
    tr = _FakeAsync(stream)
    n = 6
    envs = [_T(0, ("E", i, 4), np.arange(4.0) + 10 * i) for i in range(n)]
    st = OffloadedEnvs(envs, window=n, transfer=tr, budget_bytes=8 * 4 + 8)
    stream.complete()
    assert st.resident() == [n - 1]
    assert st.prefetch(0)       # its upload is pending: the sweep has not read it yet
    assert st.resident()[-1] == 0 and 0 in st.resident()
    uploads = st.uploads
    got = _read(stream, st[2])  # a read while prefetch 0 is pending
    np.testing.assert_array_equal(got, np.arange(4.0) + 20)
    assert st.resident() == [2]  # the pending prefetch went, the entry just read stayed
    assert st.uploads == uploads + 1
    np.testing.assert_array_equal(_read(stream, st[2]), np.arange(4.0) + 20)
    assert st.uploads == uploads + 1  # read again without another upload
    stream.complete()
    for i in range(n):
        np.testing.assert_array_equal(_read(stream, st[i]), np.arange(4.0) + 10 * i)
        assert st.resident()[-1] == i
