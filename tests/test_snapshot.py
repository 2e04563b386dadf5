"""Checkpoint and restart through ohpic_snapshot_save / ohpic_snapshot_load.

A run interrupted after 7 steps and restarted from its snapshot in a fresh
context must continue like the uninterrupted run, bit for bit in both forms
(their deposits are integer fixed point, so re-depositing the restored
particles gives the same sums whatever order the atomics land in).  Snapshots
of another grid, truncated or foreign bytes, and cells outside the grid are
refused with a status code.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("x", "y", "z", "vx", "vy", "vz")


def _setup(P, precision, n=(32, 16, 16), sort_every=5):
    ppc = 8
    qm = [-1.0, 0.01]
    q = [1.0 / qm[0] / ppc, 0.01 / qm[1] / ppc]
    cap = [ppc * n[0] * n[1] * n[2] + 64] * 2
    cfg = P.make_config(n=n, dt=0.1, b0=(0.0, 0.0, 0.5), qm=qm, q=q, capacity=cap, precision=precision,
                        sort_every=sort_every)
    return cfg, [P.species_init(ppc, 1.0), P.species_init(ppc, 0.1)]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_restart_continues_the_run(ohpic, precision):
    P = ohpic
    cfg, sp = _setup(P, P.FP32 if precision == "fp32" else P.FP64)
    with P.PicContext(cfg) as a:
        a.init_particles(sp, seed=(42, 52))
        a.step(0.1, 7)
        snap = a.snapshot()
        at_snap = [a.download(s) for s in range(2)]
        a.step(0.1, 6)
        ref = [a.download(s) for s in range(2)]
        ref_rho = a.field(P.RHO)
        ref_d = a.diagnostics()
    with P.PicContext(cfg) as b:
        b.restore(snap)
        restored = [b.download(s) for s in range(2)]
        for s in range(2):
            for k in KEYS:
                assert np.array_equal(restored[s][k], at_snap[s][k]), (s, k)
        b.step(0.1, 6)
        got = [b.download(s) for s in range(2)]
        rho = b.field(P.RHO)
        d = b.diagnostics()
    assert d["step"] == ref_d["step"] == 13
    assert d["count"] == ref_d["count"]
    assert np.array_equal(rho, ref_rho)
    for s in range(2):
        for k in KEYS:
            assert np.array_equal(got[s][k], ref[s][k]), (s, k)
    assert d["crossings"] == ref_d["crossings"]


def test_snapshot_mismatch_is_refused(ohpic):
    P = ohpic
    cfg, sp = _setup(P, P.FP32)
    other, _ = _setup(P, P.FP32, n=(16, 16, 16))
    with P.PicContext(cfg) as a:
        a.init_particles(sp, seed=(42, 52))
        snap = a.snapshot()
        with pytest.raises(P.OhpicError):
            a.restore(snap[: len(snap) // 2])               # truncated
        with pytest.raises(P.OhpicError):
            a.restore(b"\0" * len(snap))                     # not a snapshot
        with P.PicContext(other) as b:
            with pytest.raises(P.OhpicError):
                b.restore(snap)                              # another grid
        bad = bytearray(snap)
        bad[256:260] = b"\xff\xff\xff\xff"             # species 0, particle 0: cell out of the grid
        with pytest.raises(P.OhpicError):
            a.restore(bytes(bad))
        a.restore(snap)                                      # still usable
        a.step(0.1, 1)
