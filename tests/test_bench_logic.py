"""CPU tests of bench.py's host logic: the CPU-path sample, the error metrics of
the accuracy block, and the reference arm's JSON line (run on the 32^3
configuration, one step)."""
import io
import json
from contextlib import redirect_stdout

import numpy as np

import bench
from ohhelppic3d_gb300.workloads import c1, c2, c4


def test_cpu_sample_is_a_slab_of_the_same_plasma():
    s = bench.cpu_sample_workload(c2())
    assert s.n == (256, 256, 16)
    assert s.nparticles == 2 * 32 * 256 * 256 * 16 <= bench.CPU_SAMPLE_PARTICLES
    assert [sp.ppc for sp in s.species] == [sp.ppc for sp in c2().species]
    s4 = bench.cpu_sample_workload(c4())
    assert s4.n == (128, 128, 64) and s4.nparticles <= bench.CPU_SAMPLE_PARTICLES
    assert [sp.q for sp in s4.species] == [sp.q for sp in c4().species]
    assert bench.cpu_sample_workload(c1()).n == (32, 32, 32)


def _cap(scale=1.0, we=2.0, ke=10.0):
    rng = np.random.default_rng(3)
    f = {k: rng.normal(size=(4, 5, 6)) for k in ("rho", "phi", "ex", "ey", "ez")}
    return {"fields": {k: v * scale for k, v in f.items()},
            "diag": {"field_energy": we, "kinetic_energy": ke}}


def test_compare_and_energy_drift():
    ref = _cap()
    got = _cap(scale=1.0 + 1e-6, we=2.0 * (1 + 3e-6))
    e = bench.compare(got, ref)
    for k in ("rho", "phi", "ex", "ey", "ez", "e"):
        assert abs(e[k] - 1e-6) < 1e-9, k
    assert abs(e["field_energy_rel_diff"] - 3e-6) < 1e-12
    caps = {0: _cap(we=2.0, ke=10.0), 1: _cap(we=2.5, ke=9.6), 10: _cap(we=2.0, ke=10.0)}
    d = bench.energy_drift(caps)
    assert set(d) == {"1", "10"} and abs(d["1"] - 0.1 / 12.0) < 1e-15 and d["10"] == 0.0
    acc = bench.accuracy_block({1: got, 10: got, 100: got, 0: got}, {1: ref, 10: ref, 100: ref, 0: ref}, 1)
    assert acc["meets_bar"] and acc["e_rel_l2_after_100"] < bench.E_ERROR_BAR
    assert acc["weights"] == "standard CIC"


def test_reference_arm_line(monkeypatch):
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    out = io.StringIO()
    with redirect_stdout(out):
        rc = bench.main(["--impl", "reference", "--workload", "c1", "--steps", "1", "--warmup", "0"])
    assert rc == 0
    line = json.loads(out.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 1
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["weights"] == "standard CIC"
    # measured directly: ms_per_step x steps is the measured time of 1,048,576 particles
    assert abs(line["value"] * line["ms_per_step"] / 1e3 - 1048576) < 1e-6 * 1048576


def test_tuning_block_keeps_the_sort_lead(monkeypatch):
    """The bench carries the autotuner's sort lead into the applied tuning, and
    counts the record pushes of a run the same way with or without a lead."""
    from types import SimpleNamespace

    import ohhelppic3d_gb300 as P
    from ohhelppic3d_gb300 import autotune

    seen = {}

    def fake_tune(**kw):
        seen.update(kw)
        return {"tile": (16, 8, 8), "halo": 2, "split": 1, "deposit": P.DEPOSIT_LANES, "lane_particles": 4,
                "sort_lead": 10, "sort_every": 19, "grid_tuned_on": (256, 128, 64), "trials": [{}] * 3}

    monkeypatch.setattr(autotune, "tune", fake_tune)
    args = SimpleNamespace(tuning=None, no_tune=False)
    t = bench.tune_form(P, c2(), "fp32", args, 1)
    assert t["sort_lead"] == 10 and t["tile"] == (16, 8, 8) and t["trials"] == 3
    assert seen["steps"] == c2().sort_every - 1 and seen["precision"] == P.FP32
    applied = {"lane_particles": 4, "deposit": P.DEPOSIT_LANES, "sort_lead": 10}
    assert bench.record_pushes("fp32", applied, 20, 20, P.DEPOSIT_LANES) == 1
    assert bench.record_pushes("fp32", dict(applied, sort_lead=0), 40, 20, P.DEPOSIT_LANES) == 2
    assert bench.record_pushes("fp64", applied, 20, 20, P.DEPOSIT_LANES) == 0
