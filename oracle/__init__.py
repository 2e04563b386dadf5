"""ctypes binding of the oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: the CPU restatement of the reference's particle path
that the test suite, the smoke check and the benchmark's CPU-baseline leg use
as the checker.  The GPU library never imports this module.

The C sources cite the reference file:line each function follows; the
Python side only marshals arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

MAX_SPECIES = 8
WEIGHTS_REFERENCE = 0
WEIGHTS_STANDARD = 1
RHO, PHI, EX, EY, EZ = range(5)


class _Config(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("nspecies", C.c_int32), ("weights", C.c_int32), ("pad0", C.c_int32),
        ("dt", C.c_double), ("b0", C.c_double * 3),
        ("qm", C.c_double * MAX_SPECIES), ("q", C.c_double * MAX_SPECIES),
        ("capacity", C.c_int64 * MAX_SPECIES),
    ]


class _SpeciesInit(C.Structure):
    _fields_ = [
        ("ppc", C.c_double), ("vth", C.c_double), ("drift", C.c_double * 3),
        ("lo", C.c_double * 3), ("hi", C.c_double * 3),
    ]


class _Diag(C.Structure):
    _fields_ = [
        ("count", C.c_int64 * MAX_SPECIES), ("crossings", C.c_int64 * 3),
        ("total_charge", C.c_double), ("field_energy", C.c_double),
        ("kinetic_energy", C.c_double), ("momentum", C.c_double * 3),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, OpenMP)."""
    src = os.path.join(HERE, "ohpic_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def build_ref(reference_root: str) -> bool:
    """Compile pcg-c from the reference tree into oracle/_ref (when the tree exists)."""
    if not os.path.isdir(os.path.join(reference_root, "lib", "pcg-c")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={reference_root}"], check=True)
    return True


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        p = C.c_void_p
        dp = C.POINTER(C.c_double)
        L.orc_create.restype = p
        L.orc_create.argtypes = [C.POINTER(_Config)]
        L.orc_destroy.argtypes = [p]
        L.orc_set_threads.argtypes = [p, C.c_int]
        L.orc_max_threads.restype = C.c_int
        L.orc_init_particles.restype = C.c_int
        L.orc_init_particles.argtypes = [p, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(_SpeciesInit)]
        L.orc_set_particles.restype = C.c_int
        L.orc_set_particles.argtypes = [p, C.c_int] + [dp] * 6 + [C.c_int64]
        L.orc_get_particles.restype = C.c_int64
        L.orc_get_particles.argtypes = [p, C.c_int] + [dp] * 6
        L.orc_count.restype = C.c_int64
        L.orc_count.argtypes = [p, C.c_int]
        L.orc_get_field.argtypes = [p, C.c_int, dp]
        L.orc_set_field.argtypes = [p, C.c_int, dp]
        for fn in ("orc_deposit", "orc_solve", "orc_push"):
            getattr(L, fn).argtypes = [p]
        L.orc_step.argtypes = [p, C.c_int]
        L.orc_diagnostics.argtypes = [p, C.POINTER(_Diag)]
        L.orc_interp_one.argtypes = [p, C.c_double, C.c_double, C.c_double, dp]
        L.orc_boris_one.argtypes = [C.c_double, dp, dp, C.c_double, dp, dp]
        L.orc_wrap.argtypes = [C.c_int, dp]
        L.orc_fft3d.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_green.restype = C.c_double
        L.orc_green.argtypes = [C.c_int] * 6
        L.orc_pcg32_fill.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint32), C.c_int64]
        L.orc_poisson_bc.restype = C.c_int
        L.orc_poisson_bc.argtypes = [C.POINTER(C.c_int)] * 2 + [dp, C.c_int, dp, dp, dp]
        L.orc_r2r_1d.argtypes = [C.c_int, dp, dp, C.c_int]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass
class SpeciesInit:
    """Injector parameters of one species (reference injector + D3/D7)."""
    ppc: float
    vth: float
    qm: float
    wp: float = 1.0
    drift: tuple = (0.0, 0.0, 0.0)
    lo: tuple | None = None
    hi: tuple | None = None
    q: float | None = None  # overrides wp^2/qm/ppc (parameters.f90:147-148)


@dataclass
class Setup:
    """A periodic run: grid, time step, uniform B0 and the species list."""
    n: tuple
    dt: float
    b0: tuple
    species: list
    weights: int = WEIGHTS_REFERENCE
    seed: tuple = (42, 52)
    rank_advance: int = 0
    extra_capacity: int = 16
    counts: list = field(default_factory=list)

    def charge(self, sp: SpeciesInit) -> float:
        if sp.q is not None:
            return sp.q
        return sp.wp * sp.wp / sp.qm / sp.ppc

    def range_of(self, sp: SpeciesInit):
        lo = sp.lo if sp.lo is not None else (0.0, 0.0, 0.0)
        hi = sp.hi if sp.hi is not None else tuple(float(v) for v in self.n)
        return lo, hi

    def expected_count(self, sp: SpeciesInit) -> int:
        lo, hi = self.range_of(sp)
        vol = 1.0
        for d in range(3):
            vol *= max(min(hi[d], self.n[d]) - max(lo[d], 0.0), 0.0)
        return int(sp.ppc * vol)


BC_PERIODIC, BC_DIRICHLET, BC_NEUMANN, BC_DIRICHLET_NEUMANN, BC_NEUMANN_DIRICHLET = range(5)
R2HC, HC2R, RODFT00, REDFT00, RODFT01, RODFT10, REDFT01, REDFT10 = range(8)


def r2r_1d(kind: int, x) -> np.ndarray:
    """One unnormalised FFTW-convention real transform by its defining sum."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    lib().orc_r2r_1d(kind, _dp(x), _dp(y), len(x))
    return y


def poisson_bc(rho: np.ndarray, kinds, bv=(0.0,) * 6, corrected: bool = False, with_e: bool = True):
    """The bounded-domain field solve on a (nz+1, ny+1, nx+1) block of nodes
    (x fastest): returns phi (and E as (3, nz+1, ny+1, nx+1))."""
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    n = (C.c_int * 3)(rho.shape[2] - 1, rho.shape[1] - 1, rho.shape[0] - 1)
    k = (C.c_int * 3)(*[int(v) for v in kinds])
    b = np.ascontiguousarray(bv, dtype=np.float64)
    phi = np.empty_like(rho)
    e = np.empty((3,) + rho.shape) if with_e else None
    rc = lib().orc_poisson_bc(n, k, _dp(b), int(bool(corrected)), _dp(rho), _dp(phi),
                              _dp(e) if e is not None else None)
    if rc != 0:
        raise ValueError("orc_poisson_bc: bad grid or kinds")
    return (phi, e) if with_e else phi


def pcg32_draws(initstate: int, initseq: int, n: int, advance: int = 0) -> np.ndarray:
    out = np.empty(n, dtype=np.uint32)
    lib().orc_pcg32_fill(initstate, initseq, advance % (1 << 64), out.ctypes.data_as(C.POINTER(C.c_uint32)), n)
    return out


def green(kx, ky, kz, nx, ny, nz) -> float:
    return lib().orc_green(kx, ky, kz, nx, ny, nz)


def fft3d(data: np.ndarray, sign: int) -> np.ndarray:
    """Unnormalised complex 3-D DFT of a (nz, ny, nx) array (x fastest)."""
    a = np.ascontiguousarray(data, dtype=np.complex128).copy()
    nz, ny, nx = a.shape
    lib().orc_fft3d(a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)), nx, ny, nz, sign)
    return a


def boris_one(qm, e, b, dt, pos, vel):
    e = np.ascontiguousarray(e, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    pos = np.array(pos, dtype=np.float64)
    vel = np.array(vel, dtype=np.float64)
    lib().orc_boris_one(qm, _dp(e), _dp(b), dt, _dp(pos), _dp(vel))
    return pos, vel


def wrap(n: int, p: float) -> float:
    v = np.array([p], dtype=np.float64)
    lib().orc_wrap(n, _dp(v))
    return float(v[0])


class Oracle:
    """One periodic simulation held by the C oracle."""

    def __init__(self, setup: Setup, capacity: list | None = None, threads: int = 1):
        L = lib()
        self.setup = setup
        cfg = _Config()
        cfg.nx, cfg.ny, cfg.nz = setup.n
        cfg.nspecies = len(setup.species)
        cfg.weights = setup.weights
        cfg.dt = setup.dt
        for d in range(3):
            cfg.b0[d] = setup.b0[d]
        for i, sp in enumerate(setup.species):
            cfg.qm[i] = sp.qm
            cfg.q[i] = setup.charge(sp)
            cap = capacity[i] if capacity else setup.expected_count(sp) + setup.extra_capacity
            cfg.capacity[i] = cap
        self.cfg = cfg
        self.ptr = L.orc_create(C.byref(cfg))
        if not self.ptr:
            raise RuntimeError("orc_create failed")
        L.orc_set_threads(self.ptr, threads)

    def close(self):
        if self.ptr:
            lib().orc_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ncell(self) -> int:
        nx, ny, nz = self.setup.n
        return nx * ny * nz

    def set_threads(self, t: int):
        lib().orc_set_threads(self.ptr, t)

    def init_particles(self):
        arr = (_SpeciesInit * MAX_SPECIES)()
        for i, sp in enumerate(self.setup.species):
            lo, hi = self.setup.range_of(sp)
            arr[i].ppc = sp.ppc
            arr[i].vth = sp.vth
            for d in range(3):
                arr[i].drift[d] = sp.drift[d]
                arr[i].lo[d] = lo[d]
                arr[i].hi[d] = hi[d]
        rc = lib().orc_init_particles(self.ptr, self.setup.seed[0], self.setup.seed[1],
                                      self.setup.rank_advance % (1 << 64), arr)
        if rc != 0:
            raise RuntimeError("orc_init_particles: capacity exceeded")

    def count(self, sp: int) -> int:
        return lib().orc_count(self.ptr, sp)

    def get_particles(self, sp: int) -> dict:
        n = self.count(sp)
        out = {k: np.empty(n, dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
        lib().orc_get_particles(self.ptr, sp, *[_dp(out[k]) for k in ("x", "y", "z", "vx", "vy", "vz")])
        return out

    def set_particles(self, sp: int, p: dict):
        arrs = [np.ascontiguousarray(p[k], dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")]
        rc = lib().orc_set_particles(self.ptr, sp, *[_dp(a) for a in arrs], len(arrs[0]))
        if rc != 0:
            raise RuntimeError("orc_set_particles failed")

    def get_field(self, which: int) -> np.ndarray:
        nx, ny, nz = self.setup.n
        out = np.empty((nz, ny, nx), dtype=np.float64)
        lib().orc_get_field(self.ptr, which, _dp(out))
        return out

    def set_field(self, which: int, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        lib().orc_set_field(self.ptr, which, _dp(a))

    def deposit(self):
        lib().orc_deposit(self.ptr)

    def solve(self):
        lib().orc_solve(self.ptr)

    def push(self):
        lib().orc_push(self.ptr)

    def step(self, nsteps: int = 1):
        lib().orc_step(self.ptr, nsteps)

    def interp(self, x, y, z) -> np.ndarray:
        e = np.empty(3, dtype=np.float64)
        lib().orc_interp_one(self.ptr, x, y, z, _dp(e))
        return e

    def diagnostics(self) -> dict:
        d = _Diag()
        lib().orc_diagnostics(self.ptr, C.byref(d))
        ns = len(self.setup.species)
        return {
            "count": [d.count[i] for i in range(ns)],
            "crossings": [d.crossings[i] for i in range(3)],
            "total_charge": d.total_charge,
            "field_energy": d.field_energy,
            "kinetic_energy": d.kinetic_energy,
            "momentum": [d.momentum[i] for i in range(3)],
        }
