"""The allocation-free deposit, ohpic_scatter_noalloc, called through the C ABI.

Some callers cannot let a library allocate GPU memory (they size all device
memory once through their own pool); this entry point deposits into the
caller's rho using only a static device array as scratch.  The test compares it
with the context entry point (ohpic_scatter on an FP64 context) within the FP32
deposit tolerance used by test_gpu_parity (2e-6 of max|rho|), on two rounds of
calls in a row, so the second round also checks that each call leaves the shared
scratch cleared.  The file name sorts last so a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_scatter_noalloc_matches_context_scatter(ohpic, oracle_mod):
    torch = pytest.importorskip("torch")
    P, O = ohpic, oracle_mod
    n = (32, 24, 16)
    setup = O.Setup(n=n, dt=0.1, b0=(0.0, 0.0, 0.5), weights=0,
                    species=[O.SpeciesInit(ppc=8, vth=1.0, qm=-1.0, wp=1.0),
                             O.SpeciesInit(ppc=8, vth=0.1, qm=0.01, wp=0.1)])
    o = O.Oracle(setup, threads=8)
    o.init_particles()
    parts = [o.get_particles(s) for s in range(2)]
    charges = [setup.charge(sp) for sp in setup.species]

    cfg = P.make_config(n=n, dt=0.1, b0=(0, 0, 0.5), qm=[-1.0, 0.01], q=charges,
                        capacity=[len(p["x"]) + 64 for p in parts], precision=P.FP64, sort_every=0)
    ctx = P.PicContext(cfg)
    for s in range(2):
        ctx.upload(s, parts[s])
    ctx.scatter()
    ref = ctx.field(P.RHO)
    ctx.close()

    dev = torch.device("cuda", 0)
    xs = [{k: torch.tensor(p[k], dtype=torch.float64, device=dev) for k in ("x", "y", "z")} for p in parts]
    stream = torch.cuda.current_stream(dev)
    L = P.lib()
    for _ in range(2):
        rho = torch.zeros(n[2], n[1], n[0], dtype=torch.float64, device=dev)
        for s in range(2):
            rc = L.ohpic_scatter_noalloc(C.c_void_p(xs[s]["x"].data_ptr()), C.c_void_p(xs[s]["y"].data_ptr()),
                                         C.c_void_p(xs[s]["z"].data_ptr()), len(parts[s]["x"]), charges[s],
                                         n[0], n[1], n[2], 0, C.c_void_p(rho.data_ptr()),
                                         C.c_void_p(stream.cuda_stream))
            assert rc == P.OK
        stream.synchronize()
        got = rho.cpu().numpy()
        assert np.max(np.abs(got - ref)) <= 2e-6 * np.max(np.abs(ref))
        assert abs(got.sum() - ref.sum()) <= 1e-9 * np.abs(ref).sum()

    # a grid beyond the static scratch is refused without touching memory
    rc = L.ohpic_scatter_noalloc(None, None, None, 0, 1.0, 256, 256, 64, 0,
                                 C.c_void_p(rho.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == P.ERR_CAPACITY


@pytest.mark.parametrize("weights", [0, 1])
def test_scatter_noalloc_wraps_skips_and_matches_oracle(ohpic, oracle_mod, weights):
    """Both weight conventions, positions many periods outside the grid on either
    side (wrapped by fmod like the oracle's periodic wrap), and non-finite
    positions (deposit nothing).  Checked directly against the oracle's deposit of
    the wrapped finite particles, twice in a row on the shared scratch."""
    torch = pytest.importorskip("torch")
    P, O = ohpic, oracle_mod
    n = (16, 24, 8)
    rng = np.random.default_rng(11 + weights)
    m = 20000
    pos = {k: rng.uniform(0, c, m) for k, c in zip(("x", "y", "z"), n)}
    shift = rng.integers(-1000, 1000, size=(3, m))
    raw = {k: pos[k] + shift[d] * n[d] for d, k in enumerate(("x", "y", "z"))}
    raw["x"][::97] = np.nan
    raw["y"][5::131] = np.inf
    raw["z"][7::173] = -np.inf
    finite = np.isfinite(raw["x"]) & np.isfinite(raw["y"]) & np.isfinite(raw["z"])
    wrapped = {}
    for d, k in enumerate(("x", "y", "z")):
        w = np.mod(raw[k][finite], n[d])
        w[w >= n[d]] = 0.0
        wrapped[k] = w
    charge = -0.0625
    setup = O.Setup(n=n, dt=0.1, b0=(0.0, 0.0, 0.0), weights=weights,
                    species=[O.SpeciesInit(ppc=1, vth=1.0, qm=-1.0, q=charge)])
    o = O.Oracle(setup, capacity=[m])
    k = int(finite.sum())
    o.set_particles(0, {**wrapped, "vx": np.zeros(k), "vy": np.zeros(k), "vz": np.zeros(k)})
    o.deposit()
    ref = o.get_field(O.RHO)
    o.close()

    dev = torch.device("cuda", 0)
    xs = {kk: torch.tensor(raw[kk], dtype=torch.float64, device=dev) for kk in ("x", "y", "z")}
    stream = torch.cuda.current_stream(dev)
    L = P.lib()
    for _ in range(2):
        rho = torch.zeros(n[2], n[1], n[0], dtype=torch.float64, device=dev)
        rc = L.ohpic_scatter_noalloc(C.c_void_p(xs["x"].data_ptr()), C.c_void_p(xs["y"].data_ptr()),
                                     C.c_void_p(xs["z"].data_ptr()), m, charge, n[0], n[1], n[2], weights,
                                     C.c_void_p(rho.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == P.OK
        stream.synchronize()
        got = rho.cpu().numpy()
        assert np.max(np.abs(got - ref)) <= 2e-6 * np.max(np.abs(ref))
        assert abs(got.sum() - charge * k) <= 1e-9 * abs(charge) * k
