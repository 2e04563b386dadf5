"""The synthetic workloads the bench and the parity tests use, against their
stated sizes and charges (charge per macro-particle wp^2 / qm / ppc,
parameters.f90:147-148; the clustered case neutral in total)."""
import pytest

from ohhelppic3d_gb300 import workloads as W


def test_c1_thermal_pair():
    w = W.c1()
    assert w.n == (32, 32, 32) and w.dt == 0.1 and w.b0 == (0.0, 0.0, 0.5) and w.steps == 100
    assert w.counts() == [524288, 524288] and w.nparticles == 1048576
    e, i = w.species
    assert (e.qm, e.q, e.vth) == (-1.0, -1.0 / 16, 1.0)
    assert (i.qm, i.vth) == (0.01, 0.1) and i.q == pytest.approx(1.0 / 16, rel=1e-15)


def test_c2_is_the_bench_workload():
    w = W.c2()
    assert w.n == (256, 256, 256) and w.sort_every == 20
    assert w.nparticles == 1073741824
    assert [s.q for s in w.species] == pytest.approx([-1.0 / 32, 1.0 / 32], rel=1e-15)


def test_c4_clustered_two_stream_is_neutral():
    w = W.c4()
    bg, beam, ion = w.species
    assert w.n == (128, 128, 512) and w.b0 == (0.0, 0.0, 0.0) and w.steps == 500
    assert bg.count(w.n) == 134217728 and ion.count(w.n) == 268435456
    assert beam.count(w.n) == 12079595            # 16 ppc over the central 30% of x and y
    assert w.nparticles == 414732779
    assert beam.drift == (0.0, 0.0, 5.0) and beam.vth == 0.5
    total = sum(s.q * s.count(w.n) for s in w.species)
    assert abs(total) <= 1e-9 * abs(bg.q) * bg.count(w.n)
