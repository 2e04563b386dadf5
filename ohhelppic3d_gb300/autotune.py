"""Autotuner for the launch shape of the particle kernels.

Picks, per grid size and plasma, the tile shape, the halo staged around a tile,
the CTAs per (species, tile), the FP32 particles per lane, warp-deposit
reduction and sort lead, and the cell-sort cadence.  It measures on a throwaway
context filled by the device injector with the same particles per cell and
physics as the run, so tuning never advances the caller's simulation.  The per-CTA work depends only on the tile and the plasma,
not on the grid size, so large grids are tuned on a proxy grid (by default at
most 128 x 128 x 64 cells) holding the same particles per cell; CTAs per tile
only matter when the grid has few tiles, where the proxy is the grid itself.

Search: from the library defaults, particles per lane, deposit reduction, sort
lead (FP32), every (tile shape, halo) pair, deposit reduction, sort lead and
particles per lane again, split -- each candidate timed as the mean fused-push
time over `steps` steps after a sort (a whole sort cycle ranks the shapes as a
long run sees them: particles drift out of their tiles between sorts, which
favours larger halos late in the cycle), and kept only when it beats the
current choice by more than the noise; then the sort cadence K minimising
(sort time + sum of push times over K steps) / K.
"""
from __future__ import annotations

import json
import os
import time

from . import (DEPOSIT_GROUPS, DEPOSIT_LANES, DEPOSIT_MATCH, DEPOSIT_RUNS, DEPOSIT_UNIFORM, FP32, OhpicError,
               PicContext, make_config)


def _divisors(n: int) -> list:
    return [t for t in (1, 2, 4, 8, 16, 32, 64) if n % t == 0]


def _tiles(n) -> list:
    """Candidate tile shapes: cubes and flat/tall boxes of power-of-two edges."""
    shapes = [(4, 4, 4), (8, 8, 8), (8, 8, 4), (8, 4, 4), (16, 8, 8), (16, 8, 4), (8, 8, 16), (4, 4, 8),
              (16, 16, 4), (32, 8, 8), (16, 16, 8), (32, 8, 4), (2, 2, 2)]
    out = []
    for s in shapes:
        if all(n[d] % s[d] == 0 for d in range(3)) and s not in out:
            out.append(s)
    return out or [tuple(max(_divisors(n[d])[-1:] or [1]) for d in range(3))]


def proxy_grid(n, limit=(128, 128, 64)) -> tuple:
    """The largest grid <= limit per axis that keeps every edge a multiple of 8 (when n is)."""
    out = []
    for d in range(3):
        m = min(n[d], limit[d])
        while n[d] % 8 == 0 and m % 8 != 0 and m > 8:
            m -= 1
        out.append(m)
    return tuple(out)


def _ctx(cfg_kw: dict, species: list, seed=(42, 4242)) -> PicContext:
    ctx = PicContext(make_config(**cfg_kw))
    ctx.init_particles(species, seed=seed)
    return ctx


def _push_ms(ctx: PicContext, dt: float, steps: int) -> float:
    ctx.sort()
    ctx.step(dt, 1)                      # first push after the sort (also re-solves)
    ctx.set_push_timing(True)
    ctx.step(dt, steps)
    st = ctx.stats()
    ctx.set_push_timing(False)
    return st["push_ms"] / max(st["push_launches"], 1)


def _sort_ms(ctx: PicContext) -> float:
    ctx.synchronize()
    t0 = time.perf_counter()
    ctx.sort()
    ctx.synchronize()
    return 1e3 * (time.perf_counter() - t0)


def tune(n, dt, b0, qm, q, capacity_per_cell, species, precision=FP32, weights=0, proxy=True,
         steps=3, max_cadence=40, log=None, proxy_limit=(128, 128, 64), keep=0.01) -> dict:
    """Returns the best tuning dict for a run on grid n.

    species: list of SpeciesInit (device injector parameters) of the run;
    capacity_per_cell: particles per cell to reserve per species (>= ppc);
    proxy_limit: the largest proxy grid.  A proxy with many tiles per SM ranks
    tile shapes as the full grid does; a small one favours small tiles.
    keep: the margin by which a candidate must beat the current choice."""
    grid = proxy_grid(n, proxy_limit) if proxy else tuple(n)
    ncell = grid[0] * grid[1] * grid[2]
    caps = [int(c * ncell) + 1024 for c in capacity_per_cell]
    cfg_kw = dict(n=grid, dt=dt, b0=b0, qm=qm, q=q, capacity=caps, precision=precision, weights=weights,
                  sort_every=0)
    ctx = _ctx(cfg_kw, species)
    best = ctx.get_tuning()
    trials = []

    def measure(**kw):
        try:
            ctx.set_tuning(**kw)
        except OhpicError:
            return None
        ms = _push_ms(ctx, dt, steps)
        trials.append({**ctx.get_tuning(), "push_ms": ms})
        if log:
            log(f"tune {grid} {kw} -> {ms:.3f} ms")
        return ms

    def joint(candidates):
        """Measures every candidate (a dict of tuning keys) on top of the current
        best.  A candidate replaces the current best only when it beats the current
        best's own time in this pass by more than `keep` (run-to-run noise of a few
        steps on the proxy is about 1%), so near-ties do not flip the choice."""
        nonlocal best
        base = dict(best)
        scores = []
        incumbent = None
        for cand in candidates:
            s = measure(**{**base, **cand})
            if s is None:
                continue
            scores.append((s, cand))
            if all(base.get(k) == v or (isinstance(v, (tuple, list)) and tuple(base.get(k, ())) == tuple(v))
                   for k, v in cand.items()):
                incumbent = s
        if scores:
            s, cand = min(scores, key=lambda x: x[0])
            if incumbent is None or s < incumbent * (1.0 - keep):
                best = {**base, **cand}
            ctx.set_tuning(**best)

    def descend(key, values):
        joint([{key: v} for v in values])

    # sort leads (FP32 form): none, a quarter and half of the measured cycle, so
    # that particles are filed where they are a quarter or half way through it
    leads = sorted({0, (steps + 1) // 4, (steps + 1) // 2})
    try:
        if precision == FP32:
            descend("lane_particles", [2, 4])
            descend("deposit", [DEPOSIT_LANES, DEPOSIT_RUNS, DEPOSIT_GROUPS, DEPOSIT_UNIFORM, DEPOSIT_MATCH])
            descend("sort_lead", leads)
        # tile and halo together: the halo's absolute width sets how far particles
        # drift before they leave the staged box, and with the tile it sets the
        # shared memory per CTA, so a small tile with a wide halo can beat both a
        # wide halo alone and a large tile alone
        # (with the LANES deposit too when the first pass chose another: the
        # LANES push of the common box shapes has kernels compiled for them)
        deps = [best["deposit"]]
        if precision == FP32 and best["deposit"] != DEPOSIT_LANES:
            deps.append(DEPOSIT_LANES)
        joint([{"tile": t, "halo": h, "deposit": d} for t in _tiles(grid) for h in (1, 2, 3) for d in deps])
        if precision == FP32:
            # again on the chosen box: the deposit reduction's cost depends on the
            # tile (particles per cell run, the shape's compiled kernels)
            descend("deposit", [DEPOSIT_LANES, DEPOSIT_RUNS, DEPOSIT_GROUPS, DEPOSIT_UNIFORM, DEPOSIT_MATCH])
            descend("sort_lead", leads)
            descend("lane_particles", [2, 4])
        if not proxy or grid == tuple(n):
            descend("split", [1, 2, 4, 8])
        # sort cadence: per-step push time grows as particles drift out of their tiles
        sort_ms = _sort_ms(ctx)
        ctx.set_push_timing(True)
        pushes = []
        for _ in range(max_cadence):
            before = ctx.stats()["push_ms"]
            ctx.step(dt, 1)
            pushes.append(ctx.stats()["push_ms"] - before)
        ctx.set_push_timing(False)
        acc, cadence, cost = 0.0, 1, float("inf")
        for k, p in enumerate(pushes, start=1):
            acc += p
            c = (sort_ms + acc) / k
            if c < cost:
                cost, cadence = c, k
        best = {**best, "sort_every": cadence}
    finally:
        ctx.close()
    best["grid_tuned_on"] = grid
    best["trials"] = trials
    best["sort_ms"] = sort_ms
    best["push_ms_by_step_since_sort"] = pushes
    return best


def apply(ctx: PicContext, tuning: dict, keep_sort_every: bool = False):
    """Sets a tuning on a context; keep_sort_every leaves the context's cadence as is."""
    cur = ctx.get_tuning()
    ctx.set_tuning(tile=tuning.get("tile", cur["tile"]), halo=tuning.get("halo", cur["halo"]),
                   split=tuning.get("split", cur["split"]), deposit=tuning.get("deposit", cur["deposit"]),
                   lane_particles=tuning.get("lane_particles", cur["lane_particles"]),
                   sort_lead=tuning.get("sort_lead", cur.get("sort_lead", 0)),
                   sort_every=cur["sort_every"] if keep_sort_every else tuning.get("sort_every", cur["sort_every"]))


def save(path: str, key: str, tuning: dict):
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    data[key] = {k: v for k, v in tuning.items() if k != "trials"}
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
