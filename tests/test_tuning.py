"""Launch-shape tuning and the autotuner.

The FP32 form deposits in integer fixed point and advances every particle on its
own, so every launch shape must give the same state bit for bit:
  - deposit reduction: runs, uniform, match or groups;
  - tile shape, halo, CTAs per tile;
  - sort cadence.
That is what lets the autotuner pick shapes freely.  CPU tests cover the
autotuner's candidate generation.
"""
import numpy as np
import pytest


def test_proxy_grid_and_candidate_tiles():
    from ohhelppic3d_gb300 import autotune as A
    assert A.proxy_grid((256, 256, 256)) == (128, 128, 64)
    assert A.proxy_grid((32, 32, 32)) == (32, 32, 32)
    assert A.proxy_grid((128, 128, 512)) == (128, 128, 64)
    for n in ((256, 256, 256), (24, 24, 24), (128, 128, 512), (48, 16, 8)):
        tiles = A._tiles(n)
        assert tiles and all(n[d] % t[d] == 0 for t in tiles for d in range(3))


def _run(P, tuning: dict, steps: int = 6, vth: float = 1.4):
    n = (32, 32, 16)
    ppc = 8
    qm = [-1.0, 0.01]
    q = [1.0 / qm[0] / ppc, 0.01 / qm[1] / ppc]
    sp = [P.species_init(ppc, vth), P.species_init(ppc, 0.1 * vth)]
    cap = [2 * ppc * n[0] * n[1] * n[2]] * 2
    cfg = P.make_config(n=n, dt=0.1, b0=(0.0, 0.0, 0.6), qm=qm, q=q, capacity=cap, precision=P.FP32, sort_every=10)
    with P.PicContext(cfg) as ctx:
        if tuning:
            ctx.set_tuning(**tuning)
        ctx.init_particles(sp, seed=(42, 123))
        ctx.step(0.1, steps)
        fields = {w: ctx.field(w) for w in (P.RHO, P.PHI, P.EX, P.EY, P.EZ)}
        parts = [ctx.download(s) for s in range(2)]
        d = ctx.diagnostics()
    return fields, parts, d


@pytest.mark.gpu
def test_fp32_state_identical_across_launch_shapes(ohpic):
    P = ohpic
    ref_f, ref_p, ref_d = _run(P, {})
    variants = [{"deposit": P.DEPOSIT_UNIFORM}, {"deposit": P.DEPOSIT_MATCH}, {"deposit": P.DEPOSIT_GROUPS},
                {"deposit": P.DEPOSIT_RUNS}, {"lane_particles": 2, "deposit": P.DEPOSIT_LANES},
                {"tile": (4, 4, 4)}, {"tile": (16, 8, 8)}, {"tile": (16, 8, 8), "deposit": P.DEPOSIT_GROUPS},
                {"sort_lead": 5}, {"sort_lead": 5, "tile": (16, 8, 8)}, {"sort_lead": 3, "lane_particles": 2},
                {"tile": (16, 8, 8), "halo": 1}, {"tile": (16, 8, 8), "halo": 1, "sort_lead": 5},
                {"halo": 1},
                {"halo": 3}, {"split": 3}, {"sort_every": 1}, {"sort_every": 100},
                {"lane_particles": 2}, {"lane_particles": 2, "deposit": P.DEPOSIT_UNIFORM},
                {"lane_particles": 2, "deposit": P.DEPOSIT_GROUPS, "tile": (4, 4, 4)},
                {"lane_particles": 2, "split": 2, "halo": 1}, {"lane_particles": 2, "sort_every": 1}]
    for v in variants:
        f, p, d = _run(P, v)
        for w in f:
            assert np.array_equal(f[w], ref_f[w]), (v, w)
        for s in range(2):
            for k in ("x", "y", "z", "vx", "vy", "vz"):
                assert np.array_equal(p[s][k], ref_p[s][k]), (v, s, k)
        assert d["crossings"] == ref_d["crossings"], v


@pytest.mark.gpu
def test_fp32_particles_outside_their_box_identical(ohpic):
    """Without a re-sort, fast particles drift far outside their tile's staged box
    and take the global-memory gather and deposit.  The four-per-lane and
    two-per-lane passes must then match a run that re-sorts before every step (no
    particle outside its box)."""
    P = ohpic
    base = {"tile": (8, 8, 8), "halo": 1}
    ref_f, ref_p, ref_d = _run(P, dict(base, sort_every=1), steps=24, vth=4.0)
    for v in (dict(base, sort_every=1000, lane_particles=4), dict(base, sort_every=1000, lane_particles=2),
              dict(sort_every=1000, lane_particles=4, tile=(16, 8, 8), halo=2),
              dict(base, sort_every=1000, lane_particles=4, deposit=P.DEPOSIT_MATCH)):
        f, p, d = _run(P, v, steps=24, vth=4.0)
        # the global path was exercised (a sorted run has only the few particles of the
        # four-particle groups that straddle a tile boundary outside)
        assert d["outside_tile"] > 1000 + 10 * ref_d["outside_tile"], (v, d["outside_tile"])
        for w in f:
            assert np.array_equal(f[w], ref_f[w]), (v, w)
        for s in range(2):
            for k in ("x", "y", "z", "vx", "vy", "vz"):
                assert np.array_equal(p[s][k], ref_p[s][k]), (v, s, k)
        assert d["crossings"] == ref_d["crossings"], v


@pytest.mark.gpu
def test_autotuner_returns_a_valid_shape(ohpic):
    from ohhelppic3d_gb300 import autotune as A
    P = ohpic
    ppc = 8
    sp = [P.species_init(ppc, 1.0), P.species_init(ppc, 0.1)]
    t = A.tune(n=(32, 32, 32), dt=0.1, b0=(0.0, 0.0, 0.5), qm=[-1.0, 0.01], q=[-1.0 / ppc, 1.0 / ppc],
               capacity_per_cell=[2 * ppc, 2 * ppc], species=sp, precision=P.FP32, steps=2, max_cadence=8)
    assert all(32 % t["tile"][d] == 0 for d in range(3))
    assert 0 <= t["halo"] <= 4 and t["split"] >= 1 and t["sort_every"] >= 1
    assert t["deposit"] in (P.DEPOSIT_RUNS, P.DEPOSIT_UNIFORM, P.DEPOSIT_MATCH, P.DEPOSIT_GROUPS, P.DEPOSIT_LANES)


@pytest.mark.gpu
@pytest.mark.parametrize("tuning", [{}, {"halo": 1, "split": 2}, {"deposit": "RUNS"}, {"tile": (16, 8, 8)},
                                    {"tile": (16, 8, 8), "sort_lead": 4}])
def test_push_from_sort_records_matches_arrays(ohpic, tuning):
    """The FP32 sort leaves its 32-byte records pending and the next push (four
    per lane, LANES deposit) reads them and writes the word arrays and ids
    itself.  Turning the records back into arrays first (here: a download between
    the sort and the push) must give the same bits: every particle (matched by
    id; the slot order across warps follows the sort's atomics), rho and the
    crossing counts.  Other shapes (RUNS) always push from the arrays."""
    P = ohpic
    if "deposit" in tuning:
        tuning = dict(tuning, deposit=getattr(P, "DEPOSIT_" + tuning["deposit"]))
    n = (32, 32, 16)
    ppc = 8
    qm = [-1.0, 0.01]
    q = [1.0 / qm[0] / ppc, 0.01 / qm[1] / ppc]
    sp = [P.species_init(ppc, 1.5), P.species_init(ppc, 0.15)]
    cap = [2 * ppc * n[0] * n[1] * n[2] + 3] * 2          # odd capacity: segments not multiples of 4
    cfg = P.make_config(n=n, dt=0.1, b0=(0.0, 0.0, 0.6), qm=qm, q=q, capacity=cap, precision=P.FP32, sort_every=0)
    out = []
    for materialise in (False, True):
        with P.PicContext(cfg) as ctx:
            if tuning:
                ctx.set_tuning(**tuning)
            ctx.init_particles(sp, seed=(42, 77))
            ctx.sort()
            ctx.step(0.1, 6)                               # drift, so the next sort moves particles
            ctx.sort()
            if materialise:
                ctx.download(0)
            ctx.step(0.1, 1)
            ctx.sort()
            ctx.step(0.1, 2)
            parts = [ctx.download(s) for s in range(2)]
            out.append((parts, ctx.field(P.RHO), ctx.diagnostics()))
    (pa, ra, da), (pb, rb, db) = out
    assert np.array_equal(ra, rb)
    assert da["crossings"] == db["crossings"] and da["count"] == db["count"]
    for s in range(2):
        for k in ("x", "y", "z", "vx", "vy", "vz", "ids"):
            assert np.array_equal(pa[s][k], pb[s][k]), (s, k)
        # every id once: the record push carried the ids with their particles
        assert np.array_equal(pa[s]["ids"], np.arange(len(pa[s]["ids"]), dtype=np.uint32))
