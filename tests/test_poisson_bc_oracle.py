"""The oracle's bounded-domain field solve (non-periodic kinds), pinned on the CPU.

  * Its one-dimensional r2r transforms, written as their defining sums, against
    scipy.fft's DCT/DST types I-III and numpy's real FFT (FFTW's conventions,
    unnormalised), and each forward/backward pair of the reference's kinds
    against its normaliser (mpi_fftw3_solver.f90:166-206).
  * Single eigenmodes per kind: with the corrected table phi = rho / mu exactly;
    as written, phi = rho / (the squared wave number at the mode's global node),
    which is what poisson_solver3d.f90:62-78 divides by.
  * All-periodic kinds against the oracle's periodic solve.
"""
import numpy as np
import pytest

REF_PI = 3.14159265358979


@pytest.fixture(scope="module")
def O():
    import oracle
    oracle.build()
    return oracle


@pytest.mark.parametrize("n", [5, 8, 13])
def test_r2r_against_scipy_and_numpy(O, n):
    sf = pytest.importorskip("scipy.fft")
    x = np.random.default_rng(n).normal(size=n)
    np.testing.assert_allclose(O.r2r_1d(O.REDFT00, x), sf.dct(x, type=1), atol=1e-12)
    np.testing.assert_allclose(O.r2r_1d(O.REDFT10, x), sf.dct(x, type=2), atol=1e-12)
    np.testing.assert_allclose(O.r2r_1d(O.REDFT01, x), sf.dct(x, type=3), atol=1e-12)
    np.testing.assert_allclose(O.r2r_1d(O.RODFT00, x), sf.dst(x, type=1), atol=1e-12)
    np.testing.assert_allclose(O.r2r_1d(O.RODFT10, x), sf.dst(x, type=2), atol=1e-12)
    np.testing.assert_allclose(O.r2r_1d(O.RODFT01, x), sf.dst(x, type=3), atol=1e-12)
    z = np.fft.rfft(x)
    hc = np.empty(n)
    hc[: n // 2 + 1] = z.real
    for k in range(1, (n + 1) // 2):
        hc[n - k] = z[k].imag
    np.testing.assert_allclose(O.r2r_1d(O.R2HC, x), hc, atol=1e-12)
    # forward/backward pairs of the reference's kinds and their normalisers
    for f, b, norm in ((O.R2HC, O.HC2R, n), (O.RODFT00, O.RODFT00, 2 * (n + 1)), (O.REDFT00, O.REDFT00, 2 * (n - 1)),
                       (O.RODFT01, O.RODFT10, 2 * n), (O.REDFT01, O.REDFT10, 2 * n)):
        np.testing.assert_allclose(O.r2r_1d(b, O.r2r_1d(f, x)) / norm, x, atol=1e-12)


def _mode(kind, n, m):
    """Eigenmode m of the 1-D Laplacian with the kind's walls on nodes 0..n, its
    corrected eigenvalue, and the global node whose table entry the reference
    divides it by."""
    i = np.arange(n + 1)
    if kind == 0:
        return np.cos(2 * np.pi * m * i / n), (2 * np.sin(REF_PI * m / n)) ** 2, m
    if kind == 1:
        return np.sin(np.pi * m * i / n), 2 - 2 * np.cos(REF_PI * m / n), m
    if kind == 2:
        return np.cos(np.pi * m * i / n), 2 - 2 * np.cos(REF_PI * m / n), m
    if kind == 3:
        return np.sin(np.pi * (m + 0.5) * i / n), 2 - 2 * np.cos(REF_PI * (m + 0.5) / n), m + 1
    return np.cos(np.pi * (m + 0.5) * i / n), 2 - 2 * np.cos(REF_PI * (m + 0.5) / n), m


def _wave_number(k, n, kind):
    if kind == 0:
        return 2 * np.sin(REF_PI * (k if k <= n // 2 else n - k) / n)
    if kind == 1:
        return 2 * (np.cos(REF_PI * (k + 1) / (n + 1)) - 1)
    if kind == 2:
        return 2 * (np.cos(REF_PI * k / n) - 1)
    return 2 * (np.cos(REF_PI * (k + 0.5) / (n + 1)) - 1)


@pytest.mark.parametrize("kind", [1, 2, 3, 4])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_single_mode_known_answers(O, kind, axis):
    n = [6, 6, 6]
    n[axis] = 10
    m = 3
    f, mu, g = _mode(kind, n[axis], m)
    shape = [1, 1, 1]
    shape[2 - axis] = n[axis] + 1
    rho = np.broadcast_to(f.reshape(shape), (n[2] + 1, n[1] + 1, n[0] + 1)).copy()
    kinds = [0, 0, 0]
    kinds[axis] = kind
    phi = O.poisson_bc(rho, kinds, corrected=True, with_e=False)
    inner = [slice(0, n[2]), slice(0, n[1]), slice(0, n[0])]     # periodic axes: drop the image node
    inner[2 - axis] = slice(0, n[axis] + 1)
    np.testing.assert_allclose(phi[tuple(inner)], rho[tuple(inner)] / mu, atol=1e-12)
    # as written: divided by the squared wave number at the mode's global node
    phi_ref = O.poisson_bc(rho, kinds, corrected=False, with_e=False)
    wn2 = _wave_number(g, n[axis], kind) ** 2
    sel = [slice(0, n[2]), slice(0, n[1]), slice(0, n[0])]
    lo = 1 if kind in (1, 3) else 0
    hi = n[axis] - 1 if kind in (1, 4) else n[axis]
    sel[2 - axis] = slice(lo, hi + 1)
    np.testing.assert_allclose(phi_ref[tuple(sel)], rho[tuple(sel)] / wn2, rtol=1e-11, atol=1e-12)


def test_all_periodic_matches_the_periodic_solve(O):
    n = (8, 6, 10)
    setup = O.Setup(n=n, dt=0.1, b0=(0, 0, 0.5), species=[O.SpeciesInit(ppc=2, vth=1.0, qm=-1.0, wp=1.0),
                                                          O.SpeciesInit(ppc=2, vth=0.1, qm=0.01, wp=0.1)])
    o = O.Oracle(setup)
    o.init_particles()
    o.deposit()
    o.solve()
    rho = o.get_field(O.RHO)
    block = np.pad(rho, ((0, 1), (0, 1), (0, 1)), mode="wrap")
    for corrected in (False, True):
        phi, e = O.poisson_bc(block, [0, 0, 0], corrected=corrected)
        scale = np.max(np.abs(o.get_field(O.PHI)))
        np.testing.assert_allclose(phi[:-1, :-1, :-1], o.get_field(O.PHI), atol=1e-12 * scale)
        for d, w in enumerate((O.EX, O.EY, O.EZ)):
            np.testing.assert_allclose(e[d][:-1, :-1, :-1], o.get_field(w), atol=1e-12 * scale)
        np.testing.assert_array_equal(phi[-1], phi[0])      # node n is the image of node 0
    o.close()


def test_dirichlet_wall_values_in_the_corrected_form(O):
    """A linear potential between two Dirichlet walls with no charge: phi(x) =
    V0 + (V1 - V0) x / n, constant along the periodic axes; E = -(V1 - V0)/n."""
    n = (12, 4, 4)
    rho = np.zeros((n[2] + 1, n[1] + 1, n[0] + 1))
    phi, e = O.poisson_bc(rho, [1, 0, 0], bv=(2.0, -1.0, 0, 0, 0, 0), corrected=True)
    x = np.arange(n[0] + 1)
    np.testing.assert_allclose(phi, np.broadcast_to(2.0 - 3.0 * x / n[0], phi.shape), atol=1e-12)
    np.testing.assert_allclose(e[0], 3.0 / n[0], atol=1e-12)
    np.testing.assert_allclose(e[1:], 0.0, atol=1e-12)
    # as written the wall terms land on the wall nodes, outside the transform
    phi_ref = O.poisson_bc(rho, [1, 0, 0], bv=(2.0, -1.0, 0, 0, 0, 0), corrected=False, with_e=False)
    np.testing.assert_allclose(phi_ref, 0.0, atol=1e-14)


def test_bad_arguments(O):
    with pytest.raises(ValueError):
        O.poisson_bc(np.zeros((3, 3, 1)), [2, 0, 0])       # n = 0 along x
    with pytest.raises(ValueError):
        O.poisson_bc(np.zeros((3, 3, 3)), [7, 0, 0])
