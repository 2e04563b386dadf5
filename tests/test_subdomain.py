"""A periodic box cut into OhHelp subdomains, one device-resident Subdomain per
rank (all on cuda:0, driven one after another by the host), against the oracle's
single-domain mainstep (deposit, solve, push: src/ohhelppic3d.f90:311-358).

* With the oracle's own E, one decomposed mainstep moves every particle to the
  same bits as the oracle's push, and the blocks' rho, reduced over the ranks,
  is the oracle's deposit within the fixed-point rounding.
* Ten decomposed mainsteps with the GPU's periodic solve keep every particle in
  the oracle's cell, on the rank that owns it, within the FP64 step tolerances.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PID_STRIDE = 1_000_000_000


def _setup(O, n=(16, 12, 20), ppc=2, weights=0):
    return O.Setup(n=n, dt=0.1, b0=(0.0, 0.0, 0.5), weights=weights,
                   species=[O.SpeciesInit(ppc=ppc, vth=1.0, qm=-1.0, wp=1.0),
                            O.SpeciesInit(ppc=ppc, vth=0.1, qm=0.01, wp=0.1)])


def _config(P, O, setup, caps):
    return P.make_config(n=setup.n, dt=setup.dt, b0=setup.b0, qm=[sp.qm for sp in setup.species],
                         q=[setup.charge(sp) for sp in setup.species], capacity=caps, precision=P.FP64,
                         weights=setup.weights, sort_every=0)


def _decompose(P, S, O, o, setup, cuts):
    blocks = S.Blocks(setup.n, cuts)
    caps = [o.count(s) for s in range(len(setup.species))]
    cfg = _config(P, O, setup, caps)
    ranks = {r: S.Subdomain(cfg, *blocks.block(r)) for r in range(blocks.nranks)}
    for s in range(len(setup.species)):
        p = o.get_particles(s)
        recs = S.records(p["x"], p["y"], p["z"], p["vx"], p["vy"], p["vz"],
                         s * PID_STRIDE + np.arange(len(p["x"])), s + 1)
        dest = blocks.rank_of(p["x"], p["y"], p["z"])
        for r, sd in ranks.items():
            sd.append(recs[dest == r])
    return blocks, ranks


def _gather(S, blocks, ranks, nspecies):
    """Every rank's particles of each species, by pid; checks each is on its owner."""
    out = []
    for s in range(nspecies):
        parts = []
        for r, sd in ranks.items():
            d = sd.download(s)
            assert np.all(blocks.rank_of(d["x"], d["y"], d["z"]) == r)
            parts.append(d)
        allp = np.concatenate(parts)
        allp = allp[np.argsort(allp["pid"])]
        assert np.array_equal(allp["pid"], s * PID_STRIDE + np.arange(len(allp)))
        out.append(allp)
    return out


@pytest.mark.parametrize("cuts", [([0, 8], [0, 5], [0, 10]), ([0], [0], [0, 3, 11, 17])])
def test_one_mainstep_matches_oracle_bits(ohpic, oracle_mod, cuts):
    from ohhelppic3d_gb300 import subdomain as S
    P, O = ohpic, oracle_mod
    setup = _setup(O)
    o = O.Oracle(setup)
    o.init_particles()
    blocks, ranks = _decompose(P, S, O, o, setup, cuts)
    o.deposit()
    rho_o = o.get_field(O.RHO)
    o.solve()
    e_o = np.stack([o.get_field(w) for w in (O.EX, O.EY, O.EZ)])
    seen = {}

    def solve(rho):
        seen["rho"] = rho.copy()
        return e_o

    S.mainstep(ranks, blocks, S.LocalComm(), solve, setup.dt)
    o.push()
    scale = float(np.max(np.abs(rho_o)))
    assert float(np.max(np.abs(seen["rho"] - rho_o))) <= 1e-13 * scale
    got = _gather(S, blocks, ranks, len(setup.species))
    for s in range(len(setup.species)):
        ref = o.get_particles(s)
        for k in ("x", "y", "z", "vx", "vy", "vz"):
            assert np.array_equal(got[s][k], ref[k]), (s, k)
    for sd in ranks.values():
        sd.close()
    o.close()


def test_ten_mainsteps_with_the_device_solve(ohpic, oracle_mod):
    from ohhelppic3d_gb300 import subdomain as S
    P, O = ohpic, oracle_mod
    setup = _setup(O, n=(16, 16, 16), ppc=4)
    o = O.Oracle(setup)
    o.init_particles()
    blocks, ranks = _decompose(P, S, O, o, setup, ([0, 6], [0, 8], [0, 4, 9]))
    solver = P.PicContext(_config(P, O, setup, [64, 64]))

    def solve(rho):
        solver.set_field(P.RHO, rho)
        solver.solve()
        return np.stack([solver.field(w) for w in (P.EX, P.EY, P.EZ)])

    moved = 0
    for _ in range(10):
        left = S.mainstep(ranks, blocks, S.LocalComm(), solve, setup.dt)
        moved += sum(left.values())
        o.deposit()
        o.solve()
        o.push()
    assert moved > 0   # particles did cross between ranks
    got = _gather(S, blocks, ranks, len(setup.species))
    for s in range(len(setup.species)):
        ref = o.get_particles(s)
        for k in ("x", "y", "z"):
            assert np.array_equal(np.floor(got[s][k]), np.floor(ref[k])), (s, k)
            assert float(np.max(np.abs(got[s][k] - ref[k]))) <= 1e-11
        for k in ("vx", "vy", "vz"):
            assert float(np.max(np.abs(got[s][k] - ref[k]))) <= 1e-11
    solver.close()
    for sd in ranks.values():
        sd.close()
    o.close()


def test_append_refuses_records_it_cannot_hold(ohpic, oracle_mod):
    from ohhelppic3d_gb300 import subdomain as S
    P, O = ohpic, oracle_mod
    setup = _setup(O, n=(8, 8, 8))
    sd = S.Subdomain(_config(P, O, setup, [8, 8]), (0, 0, 4), (8, 8, 4))
    good = S.records([1.0], [2.0], [5.5], [0.1], [0.0], [0.0], [7], 1)
    sd.append(good)
    for bad, status in ((S.records([1.0], [2.0], [3.5], [0.0], [0.0], [0.0], [8], 1), P.ERR_BOUNDS),
                        (S.records([1.0], [2.0], [np.nan], [0.0], [0.0], [0.0], [9], 2), P.ERR_NONFINITE),
                        (S.records([1.0], [2.0], [5.0], [0.0], [0.0], [0.0], [10], 3), P.ERR_INVALID)):
        with pytest.raises(P.OhpicError) as e:
            sd.append(bad)
        assert e.value.status == status
    assert sd.count(0) == 1 and sd.count(1) == 0
    d = sd.download(0)
    assert d["pid"][0] == 7 and d["z"][0] == 5.5 and d["spec"][0] == 1 and d["nid"][0] == 13
    sd.close()
