"""The bounded-domain field solve (ohpic_poisson_*, non-periodic kinds) against the
oracle's restatement of the reference's r2r solve.

The GPU builds every DCT/DST from a complex DFT of a symmetric extension
(cuFFT) with its own twiddle kernels; the oracle evaluates FFTW's defining sums
directly.  Bar: max |phi - phi_oracle| <= 1e-11 max |phi_oracle| (and the same
for E), for every kind on every axis, both tables (as written and corrected),
non-zero boundary values, odd and even sizes.  The all-periodic case also
matches the context's periodic solve.
"""
import ctypes as C

import numpy as np
import pytest

COMBOS = [(1, 1, 1), (2, 2, 2), (3, 4, 0), (4, 3, 1), (0, 2, 3), (1, 0, 2), (2, 4, 3), (0, 0, 0), (3, 3, 4)]


def test_create_rejects_bad_arguments_without_a_device(ohpic):
    """Argument checks come before any CUDA call, so they hold on any host."""
    P = ohpic
    L = P.lib()
    out = C.c_void_p()
    for n, kinds, table in (((8, 8, 8), (5, 0, 0), 0), ((8, 8, 8), (0, 0, 0), 2), ((1, 8, 8), (1, 0, 0), 0),
                            ((0, 8, 8), (0, 0, 0), 0), ((8, 8, 5000), (0, 0, 0), 0)):
        rc = L.ohpic_poisson_create((C.c_int32 * 3)(*n), (C.c_int32 * 3)(*kinds), None, table, 0, C.byref(out))
        assert rc == P.ERR_INVALID, (n, kinds, table)
    bad_bv = np.array([0, 0, np.nan, 0, 0, 0], dtype=np.float64)
    rc = L.ohpic_poisson_create((C.c_int32 * 3)(8, 8, 8), (C.c_int32 * 3)(1, 1, 1),
                                bad_bv.ctypes.data_as(C.POINTER(C.c_double)), 0, 0, C.byref(out))
    assert rc == P.ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("table", [0, 1])
@pytest.mark.parametrize("kinds", COMBOS)
def test_bounded_solve_matches_oracle(ohpic, oracle_mod, kinds, table):
    P, O = ohpic, oracle_mod
    n = (12, 9, 10)
    rng = np.random.default_rng(sum(kinds) * 7 + table)
    rho = rng.normal(size=(n[2] + 1, n[1] + 1, n[0] + 1))
    bv = rng.normal(size=6)
    phi_o, e_o = O.poisson_bc(rho, kinds, bv, corrected=bool(table))
    with P.PoissonSolver(n, kinds, bv, table=table) as s:
        phi, e = s.solve(rho)
        again = s.solve(rho, with_e=False)
    scale = np.max(np.abs(phi_o))
    assert np.max(np.abs(phi - phi_o)) <= 1e-11 * scale, (kinds, table)
    assert np.max(np.abs(e - e_o)) <= 1e-11 * max(np.max(np.abs(e_o)), 1e-300), (kinds, table)
    assert np.array_equal(again, phi)


@pytest.mark.gpu
def test_all_periodic_matches_the_context_solve(ohpic):
    P = ohpic
    n = (16, 12, 8)
    cfg = P.make_config(n=n, dt=0.1, b0=(0, 0, 0.5), qm=[-1.0, 0.01], q=[-0.25, 0.25], capacity=[4096, 4096],
                        sort_every=0)
    rng = np.random.default_rng(5)
    rho = rng.normal(size=(n[2], n[1], n[0]))
    rho -= rho.mean()
    with P.PicContext(cfg) as ctx:
        ctx.set_field(P.RHO, rho)
        ctx.solve()
        phi_c = ctx.field(P.PHI)
        e_c = [ctx.field(w) for w in (P.EX, P.EY, P.EZ)]
    block = np.pad(rho, ((0, 1), (0, 1), (0, 1)), mode="wrap")
    for table in (0, 1):
        with P.PoissonSolver(n, (0, 0, 0), table=table) as s:
            phi, e = s.solve(block)
        scale = np.max(np.abs(phi_c))
        assert np.max(np.abs(phi[:-1, :-1, :-1] - phi_c)) <= 1e-12 * scale
        for d in range(3):
            assert np.max(np.abs(e[d][:-1, :-1, :-1] - e_c[d])) <= 1e-12 * scale


@pytest.mark.gpu
def test_device_entry_point_on_caller_stream(ohpic, oracle_mod):
    torch = pytest.importorskip("torch")
    P, O = ohpic, oracle_mod
    n, kinds = (24, 16, 20), (1, 3, 2)
    rng = np.random.default_rng(9)
    rho = rng.normal(size=(n[2] + 1, n[1] + 1, n[0] + 1))
    phi_o, e_o = O.poisson_bc(rho, kinds, corrected=True)
    dev = torch.device("cuda", 0)
    r = torch.tensor(rho, device=dev)
    phi = torch.full_like(r, float("nan"))
    e = torch.full((3,) + tuple(r.shape), float("nan"), dtype=torch.float64, device=dev)
    side = torch.cuda.Stream(dev)                 # a non-default stream: the solve must follow it
    side.wait_stream(torch.cuda.current_stream(dev))
    with P.PoissonSolver(n, kinds, table=P.TABLE_CORRECTED) as s:
        for _ in range(2):
            s.solve_device(r.data_ptr(), phi.data_ptr(), e.data_ptr(), side.cuda_stream)
        side.synchronize()
    assert np.max(np.abs(phi.cpu().numpy() - phi_o)) <= 1e-11 * np.max(np.abs(phi_o))
    assert np.max(np.abs(e.cpu().numpy() - e_o)) <= 1e-11 * np.max(np.abs(e_o))
