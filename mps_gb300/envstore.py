"""Environment residency for long sweeps (the role of src/dmrg_envio.jl:5-261, which keeps every
environment in a file and loads it when the sweep reaches it).

``OffloadedEnvs`` stands in for the environment list of ``dmrg2sitesweep`` (which only indexes
it): at most ``window`` environments stay on the device, least recently used ones move to host
memory (downloaded before their device memory is released) and come back when the sweep reads
them again. A sweep touches each environment a few times per bond, so with a window of a few
bonds the traffic is about one environment down and one up per bond, small next to the
contractions that produce them. The stored values are exact copies: a sweep gives bit-identical
results with any window.
"""
from __future__ import annotations


class OffloadedEnvs:
    """List-like store of environments with a device-resident window of ``window`` entries.

    ``load(charge, space, flat)`` rebuilds a device tensor from its host copy (default: the
    library's ``from_flat`` on ``ctx``); stored tensors need ``charge``, ``space`` and
    ``to_flat()``."""

    def __init__(self, envs, window: int = 6, ctx=None, load=None):
        if window < 1:
            raise ValueError("window must be at least 1")
        if load is None:
            from . import symtensors as mg

            def load(charge, space, flat):
                return mg.from_flat(charge, space, flat, ctx)

        self._load = load
        self.window = window
        self._n = len(envs)
        self._dev = {}
        self._host = {}
        self._order = []  # device-resident indices, least recently used first
        self.uploads = 0
        self.downloads = 0
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

    def _evict(self):
        while len(self._dev) > self.window:
            j = self._order.pop(0)
            t = self._dev.pop(j)
            self._host[j] = (t.charge, t.space, t.to_flat())
            self.downloads += 1

    def __getitem__(self, i):
        i = self._index(i)
        if i in self._dev:
            self._touch(i)
            return self._dev[i]
        if i in self._host:
            charge, space, flat = self._host.pop(i)
            t = self._load(charge, space, flat)
            self.uploads += 1
            self._dev[i] = t
            self._touch(i)
            self._evict()
            return t
        return None

    def __setitem__(self, i, t):
        i = self._index(i)
        self._host.pop(i, None)
        if t is None:
            self._dev.pop(i, None)
            if i in self._order:
                self._order.remove(i)
            return
        self._dev[i] = t
        self._touch(i)
        self._evict()

    def resident(self):
        """Indices held on the device, least recently used first."""
        return list(self._order)
