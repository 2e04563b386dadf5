"""Host <-> device particle transfers through the C ABI.

Pinned host arrays (cudaHostAlloc / cudaHostRegister) are read and written by the
conversion kernels directly; pageable arrays go through the device staging
buffer.  Both routes must leave the same device state and return the same bits.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _particles(n, shape, seed):
    rng = np.random.default_rng(seed)
    p = {k: rng.uniform(0, shape[d], n) for d, k in enumerate(("x", "y", "z"))}
    p.update({k: rng.normal(0, 1.0, n) for k in ("vx", "vy", "vz")})
    return p


def _pinned_like(torch, a):
    t = torch.empty(len(a), dtype=torch.float64, pin_memory=True)
    v = t.numpy()
    v[:] = a
    return t, v


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pinned_and_pageable_transfers_agree(ohpic, precision):
    torch = pytest.importorskip("torch")
    P = ohpic
    n = (32, 16, 8)
    count = 300_001          # odd, and larger than one staging chunk of a small context
    p = _particles(count, n, 7)
    cfg = P.make_config(n=n, dt=0.1, b0=(0, 0, 0.5), qm=[-1.0], q=[-0.1], capacity=[count + 64],
                        precision=P.FP32 if precision == "fp32" else P.FP64, sort_every=0)
    keep = []
    pinned = {}
    for k, a in p.items():
        t, v = _pinned_like(torch, a)
        keep.append(t)
        pinned[k] = v
    with P.PicContext(cfg) as a, P.PicContext(cfg) as b:
        a.upload(0, p)           # pageable numpy arrays: staged
        b.upload(0, pinned)      # pinned arrays: direct
        ra = a.download(0)
        out = {}
        for k in ("x", "y", "z", "vx", "vy", "vz"):
            t = torch.empty(count + 64, dtype=torch.float64, pin_memory=True)
            keep.append(t)
            out[k] = t.numpy()
        got = b.download_into(0, out)
        assert got == count
        rb = {k: out[k][:count] for k in out}
        for k in ("x", "y", "z", "vx", "vy", "vz"):
            # download() orders by id; download_into() keeps device order, which is
            # upload order before any sort
            assert np.array_equal(ra[k], rb[k]), k
        if precision == "fp64":
            for k in p:
                assert np.array_equal(rb[k], p[k]), k
        else:
            for k in ("vx", "vy", "vz"):
                assert np.array_equal(rb[k], p[k].astype(np.float32).astype(np.float64)), k
            for k in ("x", "y", "z"):
                assert np.max(np.abs(rb[k] - p[k])) < 4e-6 * max(n), k
        a.step(0.1, 2)
        b.step(0.1, 2)
        fa, fb = a.field(P.RHO), b.field(P.RHO)
        assert np.array_equal(fa, fb)              # integer fixed-point deposit in both forms
