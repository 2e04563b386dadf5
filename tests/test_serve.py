"""The continuous-batching server (include/ohpic_serve.h).

CPU: the header's functions are exported and bound; the request footprint is a
host computation; the request stream is deterministic and its pcg32 matches the
reference pcg-c vectors.  GPU: a run's final fields and particles are
bit-identical alone and mixed with other runs (and with the sort cadence or graph
replay changed), admission respects the HBM budget, runs that arrive while
others are on the GPU are admitted before those finish, and a served run agrees
with the same run on a single context.
"""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _serve_header_functions():
    with open(os.path.join(ROOT, "include", "ohpic_serve.h")) as f:
        text = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
    return sorted(set(re.findall(r"\b(ohpic_[a-z_0-9]+)\s*\(", text)))


def test_serve_symbols_exported_and_bound(ohpic):
    from ohhelppic3d_gb300 import serve as S
    L = C.CDLL(ohpic.LIB_PATH)
    names = _serve_header_functions()
    assert "ohpic_serve_submit" in names and "ohpic_serve_wait" in names
    assert [n for n in names if not hasattr(L, n)] == []
    assert sorted(S.SERVE_SIGNATURES) == names


def test_config_struct_matches_header():
    """The ctypes mirror of ohpic_serve_config has the header's fields, in order,
    with the same integer widths and array lengths."""
    from ohhelppic3d_gb300 import serve as S
    with open(os.path.join(ROOT, "include", "ohpic_serve.h")) as f:
        text = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
    body = re.search(r"typedef struct \{([^}]*)\}\s*ohpic_serve_config;", text).group(1)
    fields = re.findall(r"int(32|64)_t\s+(\w+)(?:\[(\d+)\])?;", body)
    ctypes_of = {"32": C.c_int32, "64": C.c_int64}
    mirror = S.ServeConfig._fields_
    assert [f[1] for f in fields] == [m[0] for m in mirror]
    for (bits, name, count), (mname, mtype) in zip(fields, mirror):
        want = ctypes_of[bits] * int(count) if count else ctypes_of[bits]
        assert C.sizeof(mtype) == C.sizeof(want), name


def test_footprint_is_host_side(ohpic):
    from ohhelppic3d_gb300 import serve as S
    cfg = S.config()
    req = S.thermal_request((24, 24, 24), 32, 10)
    fp = S.serve_lib().ohpic_serve_footprint(C.byref(cfg), C.byref(req.to_c()))
    n = req.particles()
    assert n == 2 * 32 * 24 ** 3
    # the FP32 particles (28 B), the sort's 32-byte record per slot, tile table and diagnostics
    assert 60 * n <= fp <= 60 * n + (1 << 20)
    keep = S.thermal_request((24, 24, 24), 32, 10, keep_fields=True, keep_particles=True)
    fp2 = S.serve_lib().ohpic_serve_footprint(C.byref(cfg), C.byref(keep.to_c()))
    assert fp2 >= fp + 4 * n + 8 * 5 * 24 ** 3 + 8 * 6 * n - (1 << 20)
    bad = S.thermal_request((24, 24, 24), 32, 0)      # no steps
    assert S.serve_lib().ohpic_serve_footprint(C.byref(cfg), C.byref(bad.to_c())) == -1
    bad = S.thermal_request((1, 24, 24), 32, 5)
    assert S.serve_lib().ohpic_serve_footprint(C.byref(cfg), C.byref(bad.to_c())) == -1


def test_stream_pcg32_matches_reference_vectors():
    from ohhelppic3d_gb300.serve import Pcg32
    with open(os.path.join(ROOT, "tests", "golden", "pcg32_reference.json")) as f:
        gold = json.load(f)
    for seq, key in ((52, "seed_42_52_u32"), (1000, "seed_42_1000_u32")):
        g = Pcg32(42, seq)
        assert [g.next() for _ in range(len(gold[key]))] == gold[key]
    g = Pcg32(42, 52)
    assert [repr(g.double()) for _ in range(3)] == gold["seed_42_52_doubles"][:3]


def test_ensemble_stream_deterministic_and_in_range():
    from ohhelppic3d_gb300.serve import GRIDS, PPCS, ensemble_stream
    a = ensemble_stream(64, rate=10.0)
    b = ensemble_stream(64, rate=10.0)
    assert [r.meta for r in a] == [r.meta for r in b]
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert all(x.arrival <= y.arrival for x, y in zip(a, a[1:]))
    for i, r in enumerate(a):
        assert r.meta["grid"] in GRIDS and r.meta["ppc"] in PPCS
        assert 0.0 <= r.meta["wce"] < 1.0 and 0.5 <= r.meta["vth_e"] < 2.0
        assert 200 <= r.meta["steps_drawn"] <= 2000
        assert r.seed == (42, 52 + i)
        assert r.b0 == (0.0, 0.0, r.meta["wce"])
    s = ensemble_stream(64, step_scale=0.1)
    assert all(x.nsteps == max(1, round(0.1 * y.nsteps)) for x, y in zip(s, ensemble_stream(64)))


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _probe(n, steps, seed, **kw):
    from ohhelppic3d_gb300.serve import thermal_request
    return thermal_request(n, 8, steps, wce=0.7, vth_e=1.3, seed=seed, keep_fields=True, keep_particles=True, **kw)


def _others():
    from ohhelppic3d_gb300.serve import thermal_request
    return [thermal_request((16, 16, 16), 16, 7, wce=0.2, vth_e=0.8, seed=(42, 60)),
            thermal_request((24, 24, 24), 8, 30, wce=0.9, vth_e=1.9, seed=(42, 61)),
            thermal_request((32, 32, 32), 8, 12, wce=0.5, vth_e=1.0, seed=(42, 62)),
            thermal_request((16, 16, 16), 8, 25, wce=0.1, vth_e=0.6, seed=(42, 63)),
            thermal_request((24, 24, 16), 16, 5, wce=0.3, vth_e=1.5, seed=(42, 64))]


def _serve(reqs, **cfg):
    from ohhelppic3d_gb300.serve import Server
    with Server(**cfg) as s:
        ids = [s.submit(r) for r in reqs]
        s.wait(120.0)
        out = [s.result(i, r) for i, r in zip(ids, reqs)]
        st = s.stats()
    for o in out:
        assert o["status"] == 0 and o["done"]
    return out, st


def _same_state(a, b):
    for k in ("rho", "phi", "ex", "ey", "ez"):
        assert np.array_equal(a["fields"][k], b["fields"][k]), k
    for pa, pb in zip(a["particles_by_species"], b["particles_by_species"]):
        for k in ("x", "y", "z", "vx", "vy", "vz"):
            assert np.array_equal(pa[k], pb[k]), k
    assert a["count"] == b["count"] and a["crossings"] == b["crossings"]
    for k in ("total_charge", "field_energy", "kinetic_energy"):
        # FP64 atomic sums: order-dependent in the last bits
        assert abs(a[k] - b[k]) <= 1e-12 * max(abs(a[k]), abs(b[k]), 1e-300), k


@pytest.mark.gpu
def test_run_identical_alone_and_in_the_mix(ohpic):
    probe = _probe((24, 24, 24), 23, (42, 77))
    alone, _ = _serve([probe])
    # the same run submitted between others of the same and other grid sizes,
    # some finishing before it and some after
    others = _others()
    mixed, st = _serve(others[:2] + [probe] + others[2:])
    assert st["completed"] == 6 and st["pools"] >= 3
    _same_state(alone[0], mixed[2])
    assert alone[0]["steps"] == 23 and alone[0]["fields"]["rho"].shape == (24, 24, 24)
    # charge of the final deposit: sum of q over particles (neutral plasma)
    assert abs(alone[0]["total_charge"]) < 1e-6 * abs(probe.q[0]) * probe.particles()


@pytest.mark.gpu
def test_result_independent_of_sort_cadence_and_graphs(ohpic):
    probe = _probe((16, 16, 32), 17, (42, 78))
    ref, _ = _serve([probe], sort_every=10, use_graphs=1)
    for kw in ({"sort_every": 1}, {"sort_every": 100}, {"use_graphs": 0}, {"sort_lead": 0},
               {"sort_lead": 7, "sort_every": 3}):
        got, st = _serve([probe], **kw)
        _same_state(ref[0], got[0])
        if kw.get("use_graphs") == 0:
            assert st["graph_launches"] == 0
    assert ref[0]["outside_tile"] >= 0


@pytest.mark.gpu
def test_result_independent_of_launch_shape(ohpic):
    """Tile edges (cubic, or longer in x), deposit combination and particles per
    lane change only how the work is cut: the integer deposit makes the state
    bit-identical."""
    P = ohpic
    probe = _probe((32, 16, 16), 11, (42, 81))
    ref, _ = _serve([probe])
    for kw in ({"tile_x": 8}, {"tile": 4}, {"deposit": P.DEPOSIT_RUNS}, {"lane_particles": 2},
               {"tile_x": 32, "halo": 2}):
        got, _ = _serve([probe], **kw)
        _same_state(ref[0], got[0])


@pytest.mark.gpu
def test_admission_by_hbm_budget(ohpic):
    from ohhelppic3d_gb300.serve import Server, thermal_request
    reqs = [thermal_request((32, 32, 32), 16, 15, seed=(42, 90 + i)) for i in range(6)]
    with Server() as s0:
        one = s0.footprint(reqs[0])
    # room for two runs and one 32^3 pool of 4 slots (a few MB), not for three runs
    budget = 2 * one + one // 2
    with Server(hbm_budget=budget, slots_per_pool=4) as s:
        ids = [s.submit(r) for r in reqs]
        s.wait(120.0)
        res = [s.result(i) for i in ids]
        st = s.stats()
        # a run that alone exceeds the budget is refused at submit
        big = thermal_request((64, 64, 64), 64, 5)
        with pytest.raises(ohpic.OhpicError) as e:
            s.submit(big)
        assert e.value.status == ohpic.ERR_CAPACITY
    assert all(r["status"] == 0 and r["steps"] == 15 for r in res)
    assert st["bytes_peak"] <= budget
    # at most two runs fit at once, so the six are served in at least three waves
    admits = sorted(r["admit_s"] for r in res)
    finishes = sorted(r["finish_s"] for r in res)
    assert admits[2] >= finishes[0] - 1e-6


@pytest.mark.gpu
def test_continuous_batching_overlaps_runs(ohpic):
    import time
    from ohhelppic3d_gb300.serve import Server, thermal_request
    with Server() as s:
        long_id = s.submit(thermal_request((48, 48, 48), 16, 400, seed=(42, 100)))
        time.sleep(0.05)
        short = [s.submit(thermal_request((16, 16, 16), 8, 20, seed=(42, 101 + i))) for i in range(4)]
        s.wait(300.0)
        lr = s.result(long_id)
        sr = [s.result(i) for i in short]
        st = s.stats()
        polled = s.poll()
    assert sorted(polled) == sorted([long_id] + short)
    # the short runs were admitted and finished while the long one was on the GPU
    assert all(r["admit_s"] < lr["finish_s"] and r["finish_s"] < lr["finish_s"] for r in sr)
    assert st["graph_captures"] >= 2 and st["ticks"] >= 400
    assert st["particle_steps"] == lr["particles"] * 400 + sum(r["particles"] * 20 for r in sr)


@pytest.mark.gpu
def test_served_run_matches_single_context(ohpic):
    """The same run on a single FP32 context: identical particle counts and
    crossings, fields within 1e-5 relative L2 after 8 steps (the served solve uses
    a batched cuFFT plan, the context a single-transform plan)."""
    P = ohpic
    probe = _probe((32, 32, 16), 8, (42, 79))
    served, _ = _serve([probe], sort_every=10)
    cfg = P.make_config(n=probe.n, dt=probe.dt, b0=probe.b0, qm=probe.qm, q=probe.q,
                        capacity=[c + 64 for c in served[0]["count"][:2]], precision=P.FP32, sort_every=10)
    with P.PicContext(cfg) as ctx:
        ctx.init_particles(probe.species, seed=probe.seed)
        ctx.step(probe.dt, probe.nsteps)
        ref = {"rho": ctx.field(P.RHO), "phi": ctx.field(P.PHI), "ex": ctx.field(P.EX),
               "ey": ctx.field(P.EY), "ez": ctx.field(P.EZ)}
        d = ctx.diagnostics()
    assert served[0]["count"][:2] == list(d["count"][:2])
    for k, v in ref.items():
        got = served[0]["fields"][k]
        assert np.linalg.norm(got - v) <= 1e-5 * np.linalg.norm(v), k
