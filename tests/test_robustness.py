"""Error paths that must report a status and leave the context usable.

  * The bounded wait for a tile's TMA-staged E box: with the poll limit at 0
    every wait gives up at once.  The push then gathers from global memory, waits
    the copy out before the CTA finishes, and the next synchronising call returns
    OHPIC_ERR_TIMEOUT, while the particles and fields come out bit-identical to a
    run whose waits completed.  No copy is left unfinished and nothing faults.
  * Uploads of non-finite positions or velocities into the FP32 form (whose push
    does no per-particle checks) are refused with OHPIC_ERR_NONFINITE.
  * A restored FP32 snapshot with an offset outside [0, 1), or a non-finite
    offset or velocity, is refused.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("x", "y", "z", "vx", "vy", "vz")


def _config(P, n=(32, 32, 16), ppc=8, sort_every=5, precision=None):
    qm = [-1.0, 0.01]
    q = [1.0 / qm[0] / ppc, 0.01 / qm[1] / ppc]
    cap = [2 * ppc * n[0] * n[1] * n[2]] * 2
    cfg = P.make_config(n=n, dt=0.1, b0=(0.0, 0.0, 0.6), qm=qm, q=q, capacity=cap,
                        precision=P.FP32 if precision is None else precision, sort_every=sort_every)
    return cfg, [P.species_init(ppc, 1.4), P.species_init(ppc, 0.14)]


def _run(P, tuning, polls=None, steps=7):
    cfg, sp = _config(P)
    with P.PicContext(cfg) as ctx:
        if tuning:
            ctx.set_tuning(**tuning)
        if polls is not None:
            ctx.set_tma_wait_limit(polls)
        ctx.init_particles(sp, seed=(42, 321))
        ctx.step(0.1, steps)
        status = P.OK
        try:
            ctx.synchronize()
        except P.OhpicError as e:
            status = e.status
        parts = [ctx.download(s) for s in range(2)]
        fields = {w: ctx.field(w) for w in (P.RHO, P.EX, P.EY, P.EZ)}
        d = ctx.diagnostics()
    return status, parts, fields, d


@pytest.mark.parametrize("tuning", [{}, {"lane_particles": 2}, {"halo": 1, "tile": (8, 8, 8)}])
def test_tma_wait_timeout_is_reported_and_harmless(ohpic, tuning):
    """Seven steps with a sort every five: the record push after each sort and the
    array pushes all take the timeout path (four and two particles per lane)."""
    P = ohpic
    st_ref, p_ref, f_ref, d_ref = _run(P, tuning)
    assert st_ref == P.OK
    st, p, f, d = _run(P, tuning, polls=0)
    assert st == P.ERR_TIMEOUT
    for s in range(2):
        for k in KEYS:
            assert np.array_equal(p[s][k], p_ref[s][k]), (tuning, s, k)
    for w in f:
        assert np.array_equal(f[w], f_ref[w]), (tuning, w)
    assert d["crossings"] == d_ref["crossings"]
    # the limit back at its default: the same context runs clean again
    cfg, sp = _config(P)
    with P.PicContext(cfg) as ctx:
        ctx.set_tma_wait_limit(0)
        ctx.init_particles(sp, seed=(42, 321))
        ctx.step(0.1, 2)
        with pytest.raises(P.OhpicError) as e:
            ctx.synchronize()
        assert e.value.status == P.ERR_TIMEOUT
        ctx.set_tma_wait_limit(1 << 22)
        ctx.step(0.1, 2)
        ctx.synchronize()


def _particles(n, cells):
    rng = np.random.default_rng(7)
    p = {k: rng.uniform(0, c, n) for k, c in zip(("x", "y", "z"), cells)}
    p.update({k: rng.normal(0, 1, n) for k in ("vx", "vy", "vz")})
    return p


@pytest.mark.parametrize("key,value", [("x", np.nan), ("z", np.inf), ("vy", np.nan), ("vx", 1e300)])
def test_fp32_upload_refuses_nonfinite(ohpic, key, value):
    """1e300 is finite in FP64 but not in FP32, so the FP32 form refuses it too."""
    P = ohpic
    cfg, _ = _config(P)
    with P.PicContext(cfg) as ctx:
        p = _particles(1000, ctx.n)
        p[key][517] = value
        with pytest.raises(P.OhpicError) as e:
            ctx.upload(0, p)
        assert e.value.status == P.ERR_NONFINITE
        # the direct path: pinned host arrays read by the conversion kernel itself
        torch = pytest.importorskip("torch")
        pinned = {k: torch.tensor(v, dtype=torch.float64).pin_memory().numpy() for k, v in p.items()}
        with pytest.raises(P.OhpicError) as e:
            ctx.upload_n(0, pinned, 1000)
        assert e.value.status == P.ERR_NONFINITE
        good = _particles(1000, ctx.n)
        ctx.upload(0, good)
        ctx.step(0.1, 2)
        ctx.synchronize()


def test_restore_refuses_bad_offsets_and_velocities(ohpic):
    P = ohpic
    cfg, sp = _config(P, n=(16, 16, 16), ppc=4)
    with P.PicContext(cfg) as a:
        counts = a.init_particles(sp, seed=(42, 52))
        a.step(0.1, 3)
        snap = a.snapshot()
        n0 = counts[0]
        # species 0 after the 256-byte header: cell[n0], ox[n0], oy[n0], oz[n0], vx[n0], ...
        def poke(array, index, value):
            bad = bytearray(snap)
            off = 256 + 4 * n0 * array + 4 * index
            bad[off:off + 4] = np.array([value], dtype=np.float32).tobytes()
            return bytes(bad)
        for array, value in ((1, 1.5), (2, -0.25), (3, np.nan), (3, 1.0), (5, np.inf)):
            with pytest.raises(P.OhpicError) as e:
                a.restore(poke(array, 10, value))
            assert e.value.status == P.ERR_INVALID, (array, value)
        a.restore(snap)
        a.step(0.1, 1)
        a.synchronize()
