"""Environment residency for long sweeps (the role of src/dmrg_envio.jl:5-261, which keeps every
environment in a file and moves it with ``@async`` tasks when the sweep reaches it).

``OffloadedEnvs`` stands in for the environment list of ``dmrg2sitesweep`` (which only indexes
it): at most ``window`` environments stay on the device and the least recently used ones move
to host memory. By default the copies run on the context's copy stream, between HBM and
page-locked host buffers, while the context stream computes:

* an evicted environment is downloaded asynchronously; its device memory is released when the
  copy has finished, and the host buffer is reused only after every copy that uses it is done;
* a host copy is uploaded asynchronously and the context stream is ordered after the upload
  (no host wait), either when the sweep reads the entry or earlier, through ``prefetch(i)``,
  which the sweep calls about one bond ahead so that the copy overlaps the eigensolve;
* a host copy stays valid until the entry is written again, so evicting an environment that
  was only read costs no copy at all.

The stored values are exact copies: a sweep gives bit-identical results with any window.
"""
from __future__ import annotations


def _nbytes(t):
    """Device bytes of a stored tensor (``numel()`` doubles; stand-ins without it: their flat
    data)."""
    n = getattr(t, "numel", None)
    return 8 * int(n()) if n is not None else int(t.to_flat().nbytes)


class SyncTransfer:
    """Blocking copies through NumPy arrays: ``to_flat()`` down, ``load(charge, space, flat)``
    up. Works with any tensor type that has ``charge``, ``space`` and ``to_flat()``."""

    def __init__(self, load):
        self.load = load
        self.bytes_down = self.bytes_up = 0

    def download(self, t):
        flat = t.to_flat()
        self.bytes_down += flat.nbytes
        return (t.charge, t.space, flat), None

    def upload(self, entry):
        charge, space, flat = entry
        self.bytes_up += flat.nbytes
        return self.load(charge, space, flat), None

    def ready(self, copy):
        return True

    def order(self, copy):
        pass

    def release(self, entry):
        pass


class FileTransfer:
    """Host copies in files, one per environment (what src/dmrg_envio.jl:5-39 does with JLD2
    files): ``to_flat()`` is written to ``directory`` as raw FP64 and read back through
    ``load(charge, space, flat)``; a file is deleted once its entry is overwritten."""

    def __init__(self, directory, load):
        import itertools
        import os
        os.makedirs(directory, exist_ok=True)
        self.directory = directory
        self.load = load
        self._ids = itertools.count()
        self.bytes_down = self.bytes_up = 0

    def download(self, t):
        import os

        import numpy as np
        flat = np.ascontiguousarray(t.to_flat(), dtype=np.float64)
        path = os.path.join(self.directory, f"env{next(self._ids)}.f64")
        flat.tofile(path)
        self.bytes_down += flat.nbytes
        return (t.charge, t.space, path, flat.size), None

    def upload(self, entry):
        import numpy as np
        charge, space, path, n = entry
        flat = np.fromfile(path, dtype=np.float64, count=n)
        if flat.size != n:
            raise OSError(f"environment file {path} is truncated")
        self.bytes_up += flat.nbytes
        return self.load(charge, space, flat), None

    def ready(self, copy):
        return True

    def order(self, copy):
        pass

    def release(self, entry):
        import os
        try:
            os.remove(entry[2])
        except FileNotFoundError:
            pass


class PinnedPool:
    """Reusable page-locked host buffers (``HostBuffer``): a request takes the smallest free
    buffer of at least ``n`` and at most ``2 n`` doubles, else a new one; at most ``keep``
    free buffers are held."""

    def __init__(self, alloc=None, keep: int = 8):
        if alloc is None:
            from .symtensors import HostBuffer as alloc
        self._alloc = alloc
        self._free = []
        self.keep = keep
        self.allocated = 0

    def take(self, n: int):
        best = None
        for b in self._free:
            if n <= b.n <= 2 * max(n, 1) and (best is None or b.n < best.n):
                best = b
        if best is not None:
            self._free.remove(best)
            return best
        self.allocated += 1
        return self._alloc(n)

    def give(self, b):
        self._free.append(b)
        if len(self._free) > self.keep:
            self._free.pop(0)


class AsyncTransfer:
    """Copies on the context's copy stream between device tensors and pinned host buffers
    (``download_async`` / ``upload_async``)."""

    def __init__(self, ctx=None, pool=None):
        self.ctx = ctx
        self.pool = pool if pool is not None else PinnedPool()
        self.bytes_down = self.bytes_up = 0

    def download(self, t):
        from . import symtensors as mg
        if self.ctx is None:
            self.ctx = t.ctx
        n = t.numel()
        buf = self.pool.take(n)
        self.bytes_down += 8 * n
        return (t.charge, t.space, buf), mg.download_async(t, buf)

    def upload(self, entry):
        from . import symtensors as mg
        charge, space, buf = entry
        t = mg.zeros(charge, space, self.ctx)
        self.bytes_up += 8 * t.numel()
        return t, mg.upload_async(t, buf)

    def ready(self, copy):
        return copy.query()

    def order(self, copy):
        copy.wait()

    def release(self, entry):
        self.pool.give(entry[2])


class OffloadedEnvs:
    """List-like store of environments with a device-resident window of ``window`` entries.

    ``transfer`` moves the data (default: ``AsyncTransfer`` on ``ctx``; ``load`` given instead
    selects blocking ``SyncTransfer`` copies with that loader; ``FileTransfer`` keeps the host
    copies in files). ``budget_bytes`` also bounds the device bytes of the resident entries
    (the most recently used entry always stays), for environments whose sizes vary along the
    chain."""

    def __init__(self, envs, window: int = 6, ctx=None, load=None, transfer=None,
                 budget_bytes=None):
        if window < 1:
            raise ValueError("window must be at least 1")
        if budget_bytes is not None and budget_bytes <= 0:
            raise ValueError("budget_bytes must be positive")
        if transfer is None:
            transfer = SyncTransfer(load) if load is not None else AsyncTransfer(ctx)
        self.transfer = transfer
        self.window = window
        self.budget_bytes = budget_bytes  # also evict while the resident entries hold more
        self._n = len(envs)
        self._size = {}      # index -> bytes of the device-resident entry
        self._dev = {}       # index -> device tensor
        self._host = {}      # index -> host entry (valid copy of the entry's current value)
        self._busy = {}      # index -> copies in flight that use the host entry's buffer
        self._pending = {}   # index -> upload not yet ordered before the context stream
        self._retired = []   # (copies, host entry) of overwritten entries, released when done
        self._order = []     # device-resident indices, least recently used first
        self.uploads = 0
        self.downloads = 0
        self.prefetches = 0
        self.prefetch_hits = 0
        self.clean_evictions = 0
        for i, e in enumerate(envs):
            if e is not None:
                self[i] = e

    def __len__(self):
        return self._n

    def _index(self, i):
        if i < 0:
            i += self._n
        if not 0 <= i < self._n:
            raise IndexError(i)
        return i

    def _touch(self, i):
        if i in self._order:
            self._order.remove(i)
        self._order.append(i)

    def _reap(self):
        ready = self.transfer.ready
        for i in list(self._busy):
            left = [c for c in self._busy[i] if not ready(c)]
            if left:
                self._busy[i] = left
            else:
                del self._busy[i]
        keep = []
        for copies, entry in self._retired:
            copies = [c for c in copies if not ready(c)]
            if copies:
                keep.append((copies, entry))
            else:
                self.transfer.release(entry)
        self._retired = keep

    def resident_bytes(self) -> int:
        return sum(self._size.values())

    def _over_budget(self):
        return (self.budget_bytes is not None and len(self._dev) > 1
                and self.resident_bytes() > self.budget_bytes)

    def _evict(self):
        while len(self._dev) > self.window or self._over_budget():
            # the entry just read, written or fetched (the last in the order) stays; among the
            # others, prefetched entries the sweep has not read yet go last
            others = self._order[:-1] if len(self._order) > 1 else self._order
            cand = [j for j in others if j not in self._pending] or others
            j = cand[0]
            self._order.remove(j)
            self._pending.pop(j, None)
            t = self._dev.pop(j)
            self._size.pop(j, None)
            if j in self._host:
                self.clean_evictions += 1
                continue
            entry, c = self.transfer.download(t)
            self._host[j] = entry
            if c is not None:
                self._busy.setdefault(j, []).append(c)
            self.downloads += 1

    def _fetch(self, i, order_now):
        t, c = self.transfer.upload(self._host[i])
        self.uploads += 1
        if c is not None:
            self._busy.setdefault(i, []).append(c)
            if order_now:
                self.transfer.order(c)
            else:
                self._pending[i] = c
        self._dev[i] = t
        self._size[i] = _nbytes(t)
        self._touch(i)
        self._evict()
        return t

    def __getitem__(self, i):
        i = self._index(i)
        self._reap()
        if i in self._dev:
            c = self._pending.pop(i, None)
            if c is not None:
                self.transfer.order(c)
                self.prefetch_hits += 1
            self._touch(i)
            return self._dev[i]
        if i in self._host:
            return self._fetch(i, order_now=True)
        return None

    def prefetch(self, i) -> bool:
        """Starts the upload of entry ``i`` if it lives only on the host; the context stream is
        ordered after it when the entry is read."""
        i = self._index(i)
        if i in self._dev or i not in self._host:
            return False
        self._reap()
        self._fetch(i, order_now=False)
        self.prefetches += 1
        return True

    def __setitem__(self, i, t):
        i = self._index(i)
        self._reap()
        if i in self._host:
            self._retired.append((self._busy.pop(i, []), self._host.pop(i)))
        self._pending.pop(i, None)
        if t is None:
            self._dev.pop(i, None)
            self._size.pop(i, None)
            if i in self._order:
                self._order.remove(i)
            return
        self._dev[i] = t
        self._size[i] = _nbytes(t)
        self._touch(i)
        self._evict()

    def resident(self):
        """Indices held on the device, least recently used first."""
        return list(self._order)

    def in_flight(self) -> int:
        """Copies not yet known to have completed."""
        self._reap()
        return sum(len(v) for v in self._busy.values()) + sum(len(c) for c, _ in self._retired)
