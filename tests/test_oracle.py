"""CPU tests of the oracle: pinned against the reference's pcg-c output and
against analytic known answers for every step of the particle path."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _pcg_golden():
    with open(os.path.join(GOLDEN, "pcg32_reference.json")) as f:
        return json.load(f)


def _render_check_pcg32(O) -> str:
    """Re-renders lib/pcg-c/test-high/check-base.c's output for pcg32 (seed 42/54)
    from the oracle's PCG: raw draws, the advance(-6) rewind, bounded draws for
    coins, dice and a card shuffle."""
    draws = O.pcg32_draws(42, 54, 20000)
    pos = [0]

    def rnd():
        v = int(draws[pos[0]])
        pos[0] += 1
        return v

    def bounded(bound):
        threshold = ((1 << 32) - bound) % bound
        while True:
            r = rnd()
            if r >= threshold:
                return r % bound

    out = ["pcg32_random_r:",
           "      -  result:      32-bit unsigned int (uint32_t)",
           "      -  period:      2^64   (* 2^63 streams)",
           "      -  state type:  pcg32_random_t (16 bytes)",
           "      -  output func: XSH-RR", "", ""]
    number = "A23456789TJQK"
    suit = "hcds"
    lines = []
    for rnd_i in range(1, 6):
        lines.append(f"Round {rnd_i}:")
        start = pos[0]
        vals = [rnd() for _ in range(6)]
        lines.append("  32bit:" + "".join(f" 0x{v:08x}" for v in vals))
        # advance(-6) rewinds the stream; the oracle's advance is checked separately.
        pos[0] = start
        again = [rnd() for _ in range(6)]
        lines.append("  Again:" + "".join(f" 0x{v:08x}" for v in again))
        lines.append("  Coins: " + "".join("H" if bounded(2) else "T" for _ in range(65)))
        lines.append("  Rolls:" + "".join(f" {bounded(6) + 1}" for _ in range(33)))
        cards = list(range(52))
        for i in range(52, 1, -1):
            ch = bounded(i)
            cards[ch], cards[i - 1] = cards[i - 1], cards[ch]
        txt = "  Cards:"
        for i, cval in enumerate(cards):
            txt += f" {number[cval // 4]}{suit[cval % 4]}"
            if (i + 1) % 22 == 0:
                txt += "\n\t"
        lines.append(txt)
        lines.append("")
    return "\n".join(out[:5]) + "\n\n" + "\n".join(lines) + "\n"


def test_pcg32_known_answer_matches_reference_pcg_c(oracle_mod):
    """The oracle's PCG reproduces check-pcg32 of the reference's pcg-c byte for byte."""
    assert _render_check_pcg32(oracle_mod) == _pcg_golden()["check_pcg32_out"]


def test_pcg32_advance_rewind(oracle_mod):
    O = oracle_mod
    a = O.pcg32_draws(42, 54, 12)
    b = O.pcg32_draws(42, 54, 6, advance=6)
    assert np.array_equal(a[6:], b)
    # advance by 2^64 - 6 rewinds 6 steps
    c = O.pcg32_draws(42, 54, 6, advance=(1 << 64) - 6 + 6)
    assert np.array_equal(a[:6], c)


def test_pcg32_reference_binding_vectors(oracle_mod):
    """Draws of the reference's RNG binding (pcg64.f90:10-32) for the driver's seeds."""
    O = oracle_mod
    g = _pcg_golden()
    u = O.pcg32_draws(42, 52, 64)
    assert u.tolist() == g["seed_42_52_u32"]
    d = [math.ldexp(int(v), -32) for v in u[:32]]
    assert [repr(v) for v in d] == g["seed_42_52_doubles"]
    assert O.pcg32_draws(42, 52, 16, advance=100000000).tolist() == g["seed_42_52_advance_1e8_u32"]
    assert O.pcg32_draws(42, 52, 16, advance=300000000).tolist() == g["seed_42_52_advance_3e8_u32"]
    assert O.pcg32_draws(42, 1000, 16).tolist() == g["seed_42_1000_u32"]


@pytest.mark.parametrize("shape", [(4, 6, 8), (3, 5, 7), (16, 12, 9)])
def test_fft_matches_numpy(oracle_mod, shape):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    fwd = oracle_mod.fft3d(a, -1)
    ref = np.fft.fftn(a)
    assert np.max(np.abs(fwd - ref)) < 1e-12 * np.max(np.abs(ref))
    back = oracle_mod.fft3d(fwd, +1) / a.size
    assert np.max(np.abs(back - a)) < 1e-13


def _setup(O, n=(8, 8, 8), species=None, weights=0, b0=(0.0, 0.0, 0.5), dt=0.1):
    if species is None:
        species = [O.SpeciesInit(ppc=2, vth=1.0, qm=-1.0, wp=1.0),
                   O.SpeciesInit(ppc=2, vth=0.1, qm=0.01, wp=0.1)]
    return O.Setup(n=n, dt=dt, b0=b0, species=species, weights=weights)


@pytest.mark.parametrize("k", [(1, 0, 0), (0, 2, 0), (1, 1, 3), (3, 2, 1)])
def test_poisson_single_mode(oracle_mod, k):
    """phi = rho / sum_d (2 sin(pi k_d/n_d))^2 for a single Fourier mode
    (poisson_solver3d.f90:104-117 with the truncated pi)."""
    O = oracle_mod
    n = (8, 12, 16)
    o = O.Oracle(_setup(O, n=n))
    z, y, x = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    rho = np.cos(2 * np.pi * (k[0] * x / n[0] + k[1] * y / n[1] + k[2] * z / n[2]))
    o.set_field(O.RHO, rho)
    o.solve()
    pi_ref = 3.14159265358979
    wn = sum((2 * math.sin(pi_ref * kk / nn)) ** 2 for kk, nn in zip(k, n))
    assert np.max(np.abs(o.get_field(O.PHI) - rho / wn)) < 1e-13
    assert abs(O.green(*k, *n) - 1.0 / wn) < 1e-15 / wn
    assert O.green(0, 0, 0, *n) == 0.0
    # E = 0.5*(phi[i-1] - phi[i+1]) along x for this mode
    phi = o.get_field(O.PHI)
    ex = 0.5 * (np.roll(phi, 1, axis=2) - np.roll(phi, -1, axis=2))
    assert np.max(np.abs(o.get_field(O.EX) - ex)) < 1e-14


def test_boris_gyration(oracle_mod):
    """E = 0, uniform B: |v| is conserved and each step rotates v by
    2*atan(qm*B*dt/2) (the Boris rotation, particle_mover_boris.f90:42-56)."""
    O = oracle_mod
    qm, b, dt = -1.0, 0.5, 0.1
    pos, vel = np.zeros(3), np.array([1.0, 0.0, 0.3])
    theta = 2 * math.atan(qm * b * dt / 2)
    ang0 = math.atan2(vel[1], vel[0])
    for step in range(1, 200):
        pos, vel = O.boris_one(qm, [0, 0, 0], [0, 0, b], dt, pos, vel)
        assert abs(np.hypot(vel[0], vel[1]) - 1.0) < 1e-13
        assert vel[2] == 0.3
        ang = math.atan2(vel[1], vel[0])
        d = (ang - ang0 + step * theta + math.pi) % (2 * math.pi) - math.pi
        assert abs(d) < 1e-11
    # E only: v += qm*E*dt exactly as two half kicks
    p2, v2 = O.boris_one(2.0, [1.0, -2.0, 0.5], [0, 0, 0], 0.25, [0, 0, 0], [0, 0, 0])
    assert np.allclose(v2, [0.5, -1.0, 0.25], rtol=0, atol=0)
    assert np.allclose(p2, v2 * 0.25, rtol=0, atol=0)


def test_wrap_edge_cases(oracle_mod):
    """apply_periodic twice (periodic_particle_boundary.f90:42-53)."""
    O = oracle_mod

    def twice(n, p):
        return O.wrap(n, O.wrap(n, p))

    assert twice(8, -1e-17) == 0.0          # n + p rounds to n, the second call maps it to 0
    assert twice(8, 8.0) == 0.0
    assert twice(8, -0.5) == 7.5
    assert twice(8, 8.25) == 0.25
    assert twice(8, 7.999999999999999) == 7.999999999999999
    assert twice(8, 0.0) == 0.0


@pytest.mark.parametrize("weights", [0, 1])
def test_cic_charge_conservation(oracle_mod, weights):
    """Each particle's 8 weights sum to 1, so sum(rho) = sum_s q_s N_s."""
    O = oracle_mod
    s = _setup(O, weights=weights)
    o = O.Oracle(s)
    o.init_particles()
    o.deposit()
    rho = o.get_field(O.RHO)
    expect = sum(s.charge(sp) * o.count(i) for i, sp in enumerate(s.species))
    assert abs(rho.sum() - expect) < 1e-10
    # single particle: weights of the swapped (reference) convention
    s1 = _setup(O, weights=weights, species=[O.SpeciesInit(ppc=1, vth=0, qm=-1.0, q=1.0)])
    o1 = O.Oracle(s1, capacity=[1])
    o1.set_particles(0, {"x": [2.25], "y": [3.5], "z": [7.75], "vx": [0], "vy": [0], "vz": [0]})
    o1.deposit()
    r = o1.get_field(O.RHO)
    wx = (0.25, 0.75) if weights == 0 else (0.75, 0.25)
    wy = (0.5, 0.5)
    wz = (0.75, 0.25) if weights == 0 else (0.25, 0.75)
    for i in range(2):
        for j in range(2):
            for k in range(2):
                assert r[(7 + k) % 8, 3 + j, 2 + i] == wx[i] * wy[j] * wz[k]


@pytest.mark.parametrize("weights", [0, 1])
def test_self_force_symmetric_points(oracle_mod, weights):
    """A lone particle at a cell centre feels no force from its own charge."""
    O = oracle_mod
    s = _setup(O, n=(8, 8, 8), weights=weights, species=[O.SpeciesInit(ppc=1, vth=0, qm=-1.0, q=1.0)])
    o = O.Oracle(s, capacity=[1])
    o.set_particles(0, {"x": [3.5], "y": [4.5], "z": [2.5], "vx": [0], "vy": [0], "vz": [0]})
    o.deposit()
    o.solve()
    assert np.max(np.abs(o.interp(3.5, 4.5, 2.5))) < 1e-15
    # and the force points away from the charge at a neighbour cell centre
    e = o.interp(4.5, 4.5, 2.5)
    assert e[0] > 0 and abs(e[1]) < 1e-15 and abs(e[2]) < 1e-15


def test_oracle_matches_frozen_run(oracle_mod):
    """Regression: the oracle reproduces its committed 8^3 run bit for bit."""
    O = oracle_mod
    g = np.load(os.path.join(GOLDEN, "oracle_small_run.npz"))
    setup = O.Setup(n=(8, 8, 8), dt=0.1, b0=(0.0, 0.0, 0.5),
                    species=[O.SpeciesInit(ppc=1, vth=1.0, qm=-1.0, wp=1.0),
                             O.SpeciesInit(ppc=1, vth=0.1, qm=0.01, wp=0.1)])
    o = O.Oracle(setup)
    o.init_particles()

    def check(tag):
        o.deposit()
        o.solve()
        for s in range(2):
            p = o.get_particles(s)
            for k, v in p.items():
                np.testing.assert_array_equal(v, g[f"{tag}_s{s}_{k}"])
        for name, w in (("rho", O.RHO), ("phi", O.PHI), ("ex", O.EX), ("ey", O.EY), ("ez", O.EZ)):
            np.testing.assert_array_equal(o.get_field(w), g[f"{tag}_{name}"])

    check("step0")
    o.step(1)
    check("step1")
    o.step(9)
    check("step10")


def test_init_threads_bit_identical(oracle_mod):
    """Jump-ahead init on several threads equals the sequential draw order."""
    O = oracle_mod
    s = _setup(O)
    a = O.Oracle(s, threads=1)
    a.init_particles()
    b = O.Oracle(s, threads=4)
    b.init_particles()
    for sp in range(2):
        pa, pb = a.get_particles(sp), b.get_particles(sp)
        for k in pa:
            np.testing.assert_array_equal(pa[k], pb[k])
    # first particle follows the documented draw order: 1 random_fix draw, then x, y, z
    u = [math.ldexp(int(v), -32) for v in O.pcg32_draws(42, 52, 8)]
    p0 = a.get_particles(0)
    assert p0["x"][0] == u[1] * 8 and p0["y"][0] == u[2] * 8 and p0["z"][0] == u[3] * 8
    r1, r2 = u[4], u[5]
    vx = 1.0 * math.sqrt(-2.0 * math.log(r1)) * math.cos(2.0 * 3.14159265358979 * r2)
    assert abs(p0["vx"][0] - vx) < 1e-15


def test_threaded_step_close_to_sequential(oracle_mod):
    O = oracle_mod
    s = _setup(O)
    a = O.Oracle(s, threads=1)
    b = O.Oracle(s, threads=4)
    for o in (a, b):
        o.init_particles()
        o.step(3)
    for sp in range(2):
        pa, pb = a.get_particles(sp), b.get_particles(sp)
        for k in pa:
            assert np.max(np.abs(pa[k] - pb[k])) < 1e-11


def test_energy_conservation_small(oracle_mod):
    O = oracle_mod
    s = _setup(O, n=(16, 16, 16), species=[O.SpeciesInit(ppc=4, vth=1.0, qm=-1.0, wp=1.0),
                                           O.SpeciesInit(ppc=4, vth=0.1, qm=0.01, wp=0.1)], weights=1)
    o = O.Oracle(s, threads=4)
    o.init_particles()
    o.deposit()
    o.solve()
    d0 = o.diagnostics()
    o.step(30)
    o.deposit()
    o.solve()
    d1 = o.diagnostics()
    e0 = d0["field_energy"] + d0["kinetic_energy"]
    e1 = d1["field_energy"] + d1["kinetic_energy"]
    assert abs(e1 - e0) / e0 < 5e-3
    assert abs(d1["total_charge"]) < 1e-9
