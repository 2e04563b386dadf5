"""The autotuner's search logic on the CPU, driven by a fake context.

The fake times each push from a fixed cost model of the launch shape and the
steps since the last sort, and refuses shapes the way the library does (an
OhpicError from set_tuning).  The tuner must then pick the model's best shape
among its candidates, skip refused shapes, and choose the sort cadence K that
minimises (sort time + the pushes of K steps) / K.
"""
import pytest

P = pytest.importorskip("ohhelppic3d_gb300")
from ohhelppic3d_gb300 import autotune as A  # noqa: E402

TILE_COST = {(16, 8, 8): 10.0, (8, 8, 8): 11.0, (16, 8, 4): 11.5, (32, 8, 8): 10.5}
HALO_COST = {1: 0.0, 2: 0.4, 3: 1.2}
DECAY = {1: 0.30, 2: 0.12, 3: 0.05}        # ms per step since the sort


def cost(t: dict, since_sort: int) -> float:
    c = TILE_COST.get(tuple(t["tile"]), 14.0) + HALO_COST[t["halo"]] + DECAY[t["halo"]] * since_sort
    c += 0.0 if t["deposit"] == P.DEPOSIT_LANES else 0.7
    c += 0.0 if t["lane_particles"] == 4 else 0.9
    c += 0.3 * (t["split"] - 1)
    return c


class FakeCtx:
    def __init__(self):
        self.t = {"tile": (8, 8, 8), "halo": 1, "split": 1, "deposit": P.DEPOSIT_RUNS, "lane_particles": 2,
                  "sort_every": 0}
        self.since = 0
        self.timing = False
        self.push_ms = 0.0
        self.push_launches = 0

    def get_tuning(self):
        return dict(self.t)

    def set_tuning(self, **kw):
        t = {**self.t, **kw}
        if tuple(t["tile"]) == (32, 8, 8) and t["halo"] == 3:
            raise P.OhpicError(-3, "tuning: the staged box does not fit")   # as the library refuses it
        self.t = t
        self.since = 0

    def sort(self):
        self.since = 0

    def step(self, dt, n=1):
        for _ in range(n):
            if self.timing:
                self.push_ms += cost(self.t, self.since)
                self.push_launches += 1
            self.since += 1

    def set_push_timing(self, on):
        self.timing = bool(on)
        self.push_ms, self.push_launches = 0.0, 0

    def stats(self):
        return {"push_ms": self.push_ms, "push_launches": self.push_launches, "launches": 0}

    def synchronize(self):
        pass

    def close(self):
        pass


def test_search_picks_the_model_best_and_the_cadence(monkeypatch):
    SORT_MS = 6.0
    monkeypatch.setattr(A, "_ctx", lambda cfg_kw, species, seed=(42, 4242): FakeCtx())
    monkeypatch.setattr(A, "_sort_ms", lambda ctx: (ctx.sort(), SORT_MS)[1])
    grid = (64, 32, 32)
    steps = 6
    best = A.tune(n=grid, dt=0.1, b0=(0, 0, 0.5), qm=[-1.0], q=[1.0], capacity_per_cell=[9.0],
                  species=[None], steps=steps, max_cadence=30)

    # the model's best among the tuner's candidates: mean push over steps 1..steps after a sort
    def mean_push(t):
        return sum(cost(t, s) for s in range(1, steps + 1)) / steps
    cands = [{"tile": tl, "halo": h} for tl in A._tiles(grid) for h in (1, 2, 3)
             if not (tl == (32, 8, 8) and h == 3)]
    base = {"split": 1, "deposit": P.DEPOSIT_LANES, "lane_particles": 4}
    want = min(cands, key=lambda c: mean_push({**base, **c}))
    assert tuple(best["tile"]) == want["tile"] and best["halo"] == want["halo"]
    assert best["deposit"] == P.DEPOSIT_LANES and best["lane_particles"] == 4 and best["split"] == 1
    # the refused shape was never measured
    assert not any(tuple(tr["tile"]) == (32, 8, 8) and tr["halo"] == 3 for tr in best["trials"])

    # cadence: pushes after the tuner's own sort, steps since the sort 0, 1, 2, ...
    t = {**base, **want}
    pushes = [cost(t, s) for s in range(30)]
    cad = min(range(1, 31), key=lambda k: (SORT_MS + sum(pushes[:k])) / k)
    assert best["sort_every"] == cad
    assert best["push_ms_by_step_since_sort"] == pytest.approx(pushes)


def test_search_keeps_the_defaults_when_every_candidate_is_refused(monkeypatch):
    class Refusing(FakeCtx):
        def set_tuning(self, **kw):
            raise P.OhpicError(-3, "refused")

    monkeypatch.setattr(A, "_ctx", lambda cfg_kw, species, seed=(42, 4242): Refusing())
    monkeypatch.setattr(A, "_sort_ms", lambda ctx: 1.0)
    best = A.tune(n=(32, 32, 32), dt=0.1, b0=(0, 0, 0), qm=[-1.0], q=[1.0], capacity_per_cell=[9.0],
                  species=[None], steps=2, max_cadence=5)
    assert best["trials"] == []
    assert tuple(best["tile"]) == (8, 8, 8) and best["halo"] == 1


def test_near_ties_keep_the_current_choice_and_deposit_is_retuned_on_the_box(monkeypatch):
    """RUNS is 0.5% faster than LANES on the default box (a near-tie: kept at
    LANES), and on the (16,8,8) box LANES is much faster than RUNS: whatever the
    first deposit pass picks, the tile pass (run with LANES as well) and the
    second deposit pass must end at (16,8,8) with LANES."""
    def cost2(t, since_sort):
        c = cost(t, since_sort)
        lanes = t["deposit"] == P.DEPOSIT_LANES
        if tuple(t["tile"]) == (16, 8, 8):
            c += 0.0 if lanes else 1.5
        else:
            c -= 0.7 if not lanes else 0.0       # undo the model's LANES advantage
            c += -0.05 if t["deposit"] == P.DEPOSIT_RUNS else 0.0
        return c

    class Ctx2(FakeCtx):
        def step(self, dt, n=1):
            for _ in range(n):
                if self.timing:
                    self.push_ms += cost2(self.t, self.since)
                    self.push_launches += 1
                self.since += 1

    def start():
        c = Ctx2()
        c.t["deposit"] = P.DEPOSIT_LANES
        return c

    monkeypatch.setattr(A, "_ctx", lambda cfg_kw, species, seed=(42, 4242): start())
    monkeypatch.setattr(A, "_sort_ms", lambda ctx: 1.0)
    best = A.tune(n=(64, 32, 32), dt=0.1, b0=(0, 0, 0.5), qm=[-1.0], q=[1.0], capacity_per_cell=[9.0],
                  species=[None], steps=4, max_cadence=5)
    assert tuple(best["tile"]) == (16, 8, 8)
    assert best["deposit"] == P.DEPOSIT_LANES
    # the first deposit pass (on the default (8,8,8) box) measured RUNS 0.5% faster
    # than LANES and kept LANES
    first = [tr for tr in best["trials"] if tuple(tr["tile"]) == (8, 8, 8)]
    assert any(tr["deposit"] == P.DEPOSIT_RUNS for tr in first)

    # with no margin, the near-tie flips the first pass to RUNS; the tile pass
    # still finds (16,8,8) with LANES
    monkeypatch.setattr(A, "_ctx", lambda cfg_kw, species, seed=(42, 4242): start())
    best0 = A.tune(n=(64, 32, 32), dt=0.1, b0=(0, 0, 0.5), qm=[-1.0], q=[1.0], capacity_per_cell=[9.0],
                   species=[None], steps=4, max_cadence=5, keep=0.0)
    assert tuple(best0["tile"]) == (16, 8, 8) and best0["deposit"] == P.DEPOSIT_LANES
    first0 = [tr for tr in best0["trials"] if tuple(tr["tile"]) == (8, 8, 8) and tr["halo"] == 1]
    assert min(first0, key=lambda tr: tr["push_ms"])["deposit"] == P.DEPOSIT_RUNS


def test_sort_lead_is_tuned_over_the_cycle(monkeypatch):
    """A model in which a push costs by how far its particles are from where the
    sort filed them: |steps since the sort - lead|.  Timed over a whole cycle
    after the sort, half the cycle is the best lead; the FP64 form never tries
    one (its sort files by the current cell only)."""
    steps = 11                                     # a 12-step cycle: leads 0, 3 and 6

    class LeadCtx(FakeCtx):
        def __init__(self):
            super().__init__()
            self.t["sort_lead"] = 0

        def step(self, dt, n=1):
            for _ in range(n):
                if self.timing:
                    self.push_ms += cost(self.t, 0) + 0.4 * abs(self.since - self.t["sort_lead"])
                    self.push_launches += 1
                self.since += 1

    monkeypatch.setattr(A, "_ctx", lambda cfg_kw, species, seed=(42, 4242): LeadCtx())
    monkeypatch.setattr(A, "_sort_ms", lambda ctx: (ctx.sort(), 1.0)[1])
    best = A.tune(n=(64, 32, 32), dt=0.1, b0=(0, 0, 0.5), qm=[-1.0], q=[1.0], capacity_per_cell=[9.0],
                  species=[None], steps=steps, max_cadence=5)
    assert best["sort_lead"] == 6
    assert sorted({tr["sort_lead"] for tr in best["trials"]}) == [0, 3, 6]
    best64 = A.tune(n=(64, 32, 32), dt=0.1, b0=(0, 0, 0.5), qm=[-1.0], q=[1.0], capacity_per_cell=[9.0],
                    species=[None], steps=steps, max_cadence=5, precision=P.FP64)
    assert best64["sort_lead"] == 0
    assert all(tr["sort_lead"] == 0 for tr in best64["trials"])
