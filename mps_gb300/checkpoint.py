"""MPS checkpoints for resuming long runs (the role of the JLD2 ``@save``/``@load`` of an MPS in
the reference's drivers, e.g. run6leg.jl:36-42).

File layout (little-endian):

    8 bytes   magic b"MPSGB300"
    4 bytes   format version (uint32, = 1)
    8 bytes   header length H (uint64)
    H bytes   header, UTF-8 JSON: {"length": L, "center": c, "sites": [site, ...]}, where each
              site is {"charge": q, "spaces": [[[charge, dim], ...], isdual] per leg,
              "numel": n, "complex": bool}
    data      per site: n float64 values (blocks in reference sector order, each column-major:
              the flat layout of the C ABI), then n more for the imaginary part of a complex site

The header carries everything needed to rebuild the sector tables, so a file is independent of
the process and the device that wrote it.
"""
from __future__ import annotations

import json
import struct

import numpy as np

MAGIC = b"MPSGB300"
VERSION = 1


def save_sites(path, sites, center: int = 0):
    """Write host sites: a list of (charge, spaces, re_flat, im_flat or None) where spaces are
    objects with ``sectors`` and ``isdual`` (or ([(c, d), ...], isdual) pairs)."""
    meta, blobs = [], []
    for charge, spaces, re, im in sites:
        re = np.ascontiguousarray(re, dtype="<f8")
        sp = []
        for V in spaces:
            secs, isd = (V.sectors, V.isdual) if hasattr(V, "sectors") else V
            sp.append([[[int(c), int(d)] for c, d in secs], bool(isd)])
        meta.append({"charge": int(charge), "spaces": sp, "numel": int(re.size),
                     "complex": im is not None})
        blobs.append(re)
        if im is not None:
            im = np.ascontiguousarray(im, dtype="<f8")
            if im.size != re.size:
                raise ValueError("real and imaginary parts differ in size")
            blobs.append(im)
    header = json.dumps({"length": len(sites), "center": int(center), "sites": meta}).encode()
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<IQ", VERSION, len(header)))
        f.write(header)
        for b in blobs:
            f.write(b.tobytes())


def load_sites(path):
    """Read a checkpoint: (sites, center) with sites as (charge, spaces, re, im or None) and
    spaces as ([(charge, dim), ...], isdual) pairs."""
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError(f"{path}: not an MPS checkpoint")
        version, hlen = struct.unpack("<IQ", f.read(12))
        if version != VERSION:
            raise ValueError(f"{path}: unsupported checkpoint version {version}")
        header = json.loads(f.read(hlen).decode())
        sites = []
        for s in header["sites"]:
            n = s["numel"]
            re = np.frombuffer(f.read(8 * n), dtype="<f8")
            if re.size != n:
                raise ValueError(f"{path}: truncated data")
            im = None
            if s["complex"]:
                im = np.frombuffer(f.read(8 * n), dtype="<f8")
                if im.size != n:
                    raise ValueError(f"{path}: truncated data")
            spaces = [([tuple(p) for p in secs], isd) for secs, isd in s["spaces"]]
            sites.append((s["charge"], spaces, re.copy(), None if im is None else im.copy()))
        if f.read(1):
            raise ValueError(f"{path}: trailing bytes")
    if len(sites) != header["length"]:
        raise ValueError(f"{path}: header length mismatch")
    return sites, header["center"]


def save_mps(path, mps):
    """Save a device MPS (``dmrg.MPState``; sites real ``SymTensor``s or ``ctensor.CTensor``s)."""
    from .ctensor import CTensor
    sites = []
    for A in mps.As:
        if isinstance(A, CTensor):
            im = None if A.im is None else A.sign * A.im.to_flat()
            sites.append((A.re.charge, A.re.space, A.re.to_flat(), im))
        else:
            sites.append((A.charge, A.space, A.to_flat(), None))
    save_sites(path, sites, getattr(mps, "center", 0))


def load_mps(path, ctx=None):
    """Load a checkpoint onto the device: a ``dmrg.MPState`` whose sites are ``SymTensor``s
    (real files) or ``ctensor.CTensor``s (complex sites)."""
    from . import symtensors as mg
    from .ctensor import CTensor
    from .dmrg import MPState
    sites, center = load_sites(path)
    As = []
    for charge, spaces, re, im in sites:
        sp = tuple(mg.VectorSpace(secs, isd) for secs, isd in spaces)
        t = mg.from_flat(charge, sp, re, ctx)
        As.append(t if im is None else CTensor(t, mg.from_flat(charge, sp, im, ctx)))
    return MPState(As, center=center)
