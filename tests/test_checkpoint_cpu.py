"""MPS checkpoint format: host round trip (real and complex sites), rejection of foreign,
truncated and padded files."""
import numpy as np
import pytest

from mps_gb300 import checkpoint as cp
from mps_gb300 import dmrg as gd


def host_sites(seed=3):
    sites = gd.random_mps_host(10, 5, 8, seed=seed)
    rng = np.random.default_rng(seed)
    out = []
    for i, (charge, sp, flat) in enumerate(sites):
        im = rng.standard_normal(flat.size) if i % 3 == 1 else None
        out.append((charge, sp, flat, im))
    return out


def test_round_trip(tmp_path):
    sites = host_sites()
    p = tmp_path / "state.mps"
    cp.save_sites(p, sites, center=4)
    got, center = cp.load_sites(p)
    assert center == 4 and len(got) == len(sites)
    for (c0, sp0, re0, im0), (c1, sp1, re1, im1) in zip(sites, got):
        assert c0 == c1
        assert [(list(V.sectors), V.isdual) for V in sp0] == [(s, d) for s, d in sp1]
        np.testing.assert_array_equal(re0, re1)
        if im0 is None:
            assert im1 is None
        else:
            np.testing.assert_array_equal(im0, im1)


def test_rejects_bad_files(tmp_path):
    sites = host_sites()
    p = tmp_path / "state.mps"
    cp.save_sites(p, sites)
    raw = p.read_bytes()
    bad = tmp_path / "bad.mps"
    bad.write_bytes(b"NOTANMPS" + raw[8:])
    with pytest.raises(ValueError, match="not an MPS checkpoint"):
        cp.load_sites(bad)
    bad.write_bytes(raw[:-8])
    with pytest.raises(ValueError, match="truncated"):
        cp.load_sites(bad)
    bad.write_bytes(raw + b"\0")
    with pytest.raises(ValueError, match="trailing"):
        cp.load_sites(bad)
