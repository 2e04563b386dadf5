"""ohhelppic3d_gb300 -- GB300 (sm_103a) particle hot path of ohhelppic3d.

The compute lives in libohpic.so (CUDA kernels + the C ABI of
include/ohpic.h).  This module binds that ABI with ctypes and mirrors the
reference's Fortran module API for the path, batched over all particles:

  reference (per particle)                         here (all particles, device-resident)
  t_Scatter%scatter       scatter.f90:15-24        Scatter.scatter_all()
  t_FieldSolver%solve     field_solver.f90:15-25   FieldSolver.solve()
  t_Interpolator%interp   interpolator.f90:16-25   Interpolator.interp_all(species)
  t_ParticleMover%move    particle_mover.f90:16-24 ParticleMover.move_all(dt)
  + t_ParticleBoundaries%apply x2                  (inside move_all / push)
  mainstep loops          ohhelppic3d.f90:311-358  PicContext.step(dt, nsteps)

There is no CPU fallback: if libohpic.so is missing or no GPU is visible,
every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libohpic.so")

MAX_SPECIES = 8
FP64, FP32 = 0, 1
WEIGHTS_REFERENCE, WEIGHTS_STANDARD = 0, 1
RHO, PHI, EX, EY, EZ = range(5)

OK = 0
ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_BOUNDS, ERR_TIMEOUT = 1, 2, 3, 4, 5
ERR_CAPACITY, ERR_UNSUPPORTED, ERR_NONFINITE, ERR_REJECTED = 6, 7, 8, 9


class Config(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("nspecies", C.c_int32), ("precision", C.c_int32), ("weights", C.c_int32),
        ("sort_every", C.c_int32), ("tile", C.c_int32 * 3), ("track_ids", C.c_int32),
        ("device", C.c_int32), ("dt", C.c_double), ("b0", C.c_double * 3),
        ("qm", C.c_double * MAX_SPECIES), ("q", C.c_double * MAX_SPECIES),
        ("capacity", C.c_int64 * MAX_SPECIES),
    ]


class Diag(C.Structure):
    _fields_ = [
        ("count", C.c_int64 * MAX_SPECIES), ("crossings", C.c_int64 * 3),
        ("outside_tile", C.c_int64), ("step", C.c_int64),
        ("total_charge", C.c_double), ("field_energy", C.c_double),
        ("kinetic_energy", C.c_double), ("momentum", C.c_double * 3),
    ]


class SpeciesInit(C.Structure):
    _fields_ = [
        ("ppc", C.c_double), ("vth", C.c_double), ("drift", C.c_double * 3),
        ("lo", C.c_double * 3), ("hi", C.c_double * 3),
    ]


def species_init(ppc, vth, drift=(0.0, 0.0, 0.0), lo=(0.0, 0.0, 0.0), hi=(1e30, 1e30, 1e30)) -> SpeciesInit:
    s = SpeciesInit()
    s.ppc, s.vth = float(ppc), float(vth)
    for d in range(3):
        s.drift[d], s.lo[d], s.hi[d] = float(drift[d]), float(lo[d]), float(hi[d])
    return s


class Tuning(C.Structure):
    _fields_ = [
        ("tile", C.c_int32 * 3), ("halo", C.c_int32), ("split", C.c_int32),
        ("deposit", C.c_int32), ("sort_every", C.c_int32), ("lane_particles", C.c_int32),
        ("sort_lead", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {"tile": tuple(self.tile), "halo": self.halo, "split": self.split,
                "deposit": self.deposit, "sort_every": self.sort_every, "lane_particles": self.lane_particles,
                "sort_lead": self.sort_lead}


DEPOSIT_RUNS, DEPOSIT_UNIFORM, DEPOSIT_MATCH, DEPOSIT_GROUPS, DEPOSIT_LANES = 0, 1, 2, 3, 4


class OhpicError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"ohpic status {status}: {message}")
        self.status = status


_lib = None

# Every symbol include/ohpic.h declares, with its ctypes signature.
_P = C.c_void_p
_DP = C.POINTER(C.c_double)
SIGNATURES = {
    "ohpic_config_default": (None, [C.POINTER(Config)]),
    "ohpic_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
    "ohpic_destroy": (C.c_int, [_P]),
    "ohpic_init_particles": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(SpeciesInit),
                                       C.POINTER(C.c_int64)]),
    "ohpic_upload_particles": (C.c_int, [_P, C.c_int, _P, C.c_int64, C.c_int64]),
    "ohpic_upload_particles_soa": (C.c_int, [_P, C.c_int] + [_DP] * 6 + [C.c_int64]),
    "ohpic_download_particles_soa": (C.c_int, [_P, C.c_int] + [_DP] * 6 +
                                     [C.POINTER(C.c_uint32), C.c_int64, C.POINTER(C.c_int64)]),
    "ohpic_download_particles": (C.c_int, [_P, C.c_int, _P, C.c_int64, C.c_int64, C.POINTER(C.c_int64)]),
    "ohpic_scatter": (C.c_int, [_P]),
    "ohpic_solve": (C.c_int, [_P]),
    "ohpic_interp": (C.c_int, [_P, C.c_int, _DP, C.c_int64, C.POINTER(C.c_int64)]),
    "ohpic_move": (C.c_int, [_P, C.c_double]),
    "ohpic_push": (C.c_int, [_P, C.c_double]),
    "ohpic_step": (C.c_int, [_P, C.c_double, C.c_int]),
    "ohpic_sort": (C.c_int, [_P]),
    "ohpic_snapshot_size": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "ohpic_snapshot_save": (C.c_int, [_P, C.c_void_p, C.c_int64]),
    "ohpic_snapshot_load": (C.c_int, [_P, C.c_void_p, C.c_int64]),
    "ohpic_download_field": (C.c_int, [_P, C.c_int, _DP]),
    "ohpic_upload_field": (C.c_int, [_P, C.c_int, _DP]),
    "ohpic_download_field_ohfield": (C.c_int, [_P, C.c_int, _DP, C.c_int,
                                               C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ohpic_diagnostics": (C.c_int, [_P, C.POINTER(Diag)]),
    "ohpic_set_energy_tracking": (C.c_int, [_P, C.c_int]),
    "ohpic_set_tma_wait_limit": (C.c_int, [_P, C.c_uint32]),
    "ohpic_move_one": (C.c_int, [_P, _DP, C.c_double, _DP, C.c_double]),
    "ohpic_scatter_one": (C.c_int, [_P, _DP, C.c_double, C.c_int]),
    "ohpic_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "ohpic_status_string": (C.c_char_p, [C.c_int]),
    "ohpic_synchronize": (C.c_int, [_P]),
    "ohpic_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "ohpic_set_push_timing": (C.c_int, [_P, C.c_int]),
    "ohpic_stats": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "ohpic_memory": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "ohpic_get_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "ohpic_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "ohpic_scatter_noalloc": (C.c_int, [_P, _P, _P, C.c_int64, C.c_double, C.c_int32, C.c_int32, C.c_int32,
                                        C.c_int32, _P, _P]),
    "ohpic_poisson_create": (C.c_int, [C.POINTER(C.c_int32), C.POINTER(C.c_int32), _DP, C.c_int32, C.c_int32,
                                       C.POINTER(_P)]),
    "ohpic_poisson_destroy": (C.c_int, [_P]),
    "ohpic_poisson_solve": (C.c_int, [_P, _DP, _DP, _DP]),
    "ohpic_poisson_solve_device": (C.c_int, [_P, _P, _P, _P, _P]),
    "ohpic_poisson_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
}

BC_PERIODIC, BC_DIRICHLET, BC_NEUMANN, BC_DIRICHLET_NEUMANN, BC_NEUMANN_DIRICHLET = range(5)
TABLE_AS_WRITTEN, TABLE_CORRECTED = 0, 1


def build(force: bool = False) -> str:
    from . import buildlib
    return buildlib.build(force=force)


def lib():
    """Loads libohpic.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OhpicError(ERR_CUDA, f"{LIB_PATH} is missing: run ohhelppic3d_gb300.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def default_config() -> Config:
    cfg = Config()
    lib().ohpic_config_default(C.byref(cfg))
    return cfg


def make_config(n, dt, b0, qm, q, capacity, precision=FP64, weights=WEIGHTS_REFERENCE,
                sort_every=20, tile=(0, 0, 0), track_ids=1, device=0) -> Config:
    cfg = default_config()
    cfg.nx, cfg.ny, cfg.nz = (int(v) for v in n)
    cfg.nspecies = len(qm)
    cfg.precision = precision
    cfg.weights = weights
    cfg.sort_every = sort_every
    for d in range(3):
        cfg.tile[d] = int(tile[d])
        cfg.b0[d] = float(b0[d])
    cfg.track_ids = track_ids
    cfg.device = device
    cfg.dt = float(dt)
    for s in range(len(qm)):
        cfg.qm[s] = float(qm[s])
        cfg.q[s] = float(q[s])
        cfg.capacity[s] = int(capacity[s])
    return cfg


class PicContext:
    """One device-resident run (owns particles, fields and a CUDA stream)."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        ptr = _P()
        rc = lib().ohpic_create(C.byref(cfg), C.byref(ptr))
        if rc != OK:
            raise OhpicError(rc, lib().ohpic_status_string(rc).decode())
        self.ptr = ptr
        self.nspecies = cfg.nspecies
        self.n = (cfg.nx, cfg.ny, cfg.nz)

    # -- plumbing -------------------------------------------------------
    def _check(self, rc: int):
        if rc != OK:
            buf = C.create_string_buffer(512)
            lib().ohpic_last_error(self.ptr, buf, 512)
            raise OhpicError(rc, buf.value.decode(errors="replace"))

    def close(self):
        if getattr(self, "ptr", None):
            lib().ohpic_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        s = _P()
        self._check(lib().ohpic_get_stream(self.ptr, C.byref(s)))
        return s.value or 0

    # -- particles --------------------------------------------------------
    def init_particles(self, species: list, seed=(42, 52), advance: int = 0) -> list:
        """Device-side injector (reference streams); species: list of SpeciesInit."""
        arr = (SpeciesInit * max(len(species), 1))(*species)
        counts = (C.c_int64 * MAX_SPECIES)()
        self._check(lib().ohpic_init_particles(self.ptr, seed[0], seed[1], advance % (1 << 64), arr, counts))
        return [counts[i] for i in range(self.nspecies)]

    def upload(self, species: int, p: dict):
        arrs = [np.ascontiguousarray(p[k], dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")]
        self._check(lib().ohpic_upload_particles_soa(self.ptr, species, *[_dp(a) for a in arrs], len(arrs[0])))

    def upload_aos(self, species: int, pbuf: np.ndarray):
        """pbuf: (n, k) float64 records, k >= 6 (x, y, z, vx, vy, vz first)."""
        pbuf = np.ascontiguousarray(pbuf, dtype=np.float64)
        self._check(lib().ohpic_upload_particles(self.ptr, species, pbuf.ctypes.data_as(_P),
                                                 pbuf.shape[0], pbuf.shape[1] * 8))

    def count(self, species: int) -> int:
        return self.diagnostics()["count"][species]

    def download(self, species: int, capacity: int | None = None, order: bool = True) -> dict:
        """Particles of one species; with order=True they are returned in upload order."""
        cap = capacity if capacity is not None else int(self.cfg.capacity[species])
        out = {k: np.empty(cap, dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
        ids = np.empty(cap, dtype=np.uint32) if self.cfg.track_ids else None
        n = C.c_int64()
        self._check(lib().ohpic_download_particles_soa(
            self.ptr, species, *[_dp(out[k]) for k in ("x", "y", "z", "vx", "vy", "vz")],
            ids.ctypes.data_as(C.POINTER(C.c_uint32)) if ids is not None else None, cap, C.byref(n)))
        m = n.value
        res = {k: v[:m] for k, v in out.items()}
        if ids is not None:
            res["ids"] = ids[:m]
            if order:
                perm = np.argsort(res["ids"], kind="stable")
                res = {k: v[perm] for k, v in res.items()}
        return res

    # -- checkpoint / restart ------------------------------------------------
    def snapshot(self) -> bytes:
        """The particle state and step counters as a byte image (ohpic_snapshot_save)."""
        n = C.c_int64()
        self._check(lib().ohpic_snapshot_size(self.ptr, C.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        self._check(lib().ohpic_snapshot_save(self.ptr, buf.ctypes.data_as(C.c_void_p), n.value))
        return buf.tobytes()

    def restore(self, snap: bytes):
        """Replaces the particle state with a snapshot (ohpic_snapshot_load)."""
        arr = np.frombuffer(snap, dtype=np.uint8)
        self._check(lib().ohpic_snapshot_load(self.ptr, arr.ctypes.data_as(C.c_void_p), arr.size))

    def download_into(self, species: int, out: dict, ids: np.ndarray | None = None) -> int:
        """Device-order download into caller-provided float64 arrays (e.g. pinned host memory)."""
        cap = min(len(out[k]) for k in ("x", "y", "z", "vx", "vy", "vz"))
        n = C.c_int64()
        self._check(lib().ohpic_download_particles_soa(
            self.ptr, species, *[_dp(out[k]) for k in ("x", "y", "z", "vx", "vy", "vz")],
            ids.ctypes.data_as(C.POINTER(C.c_uint32)) if ids is not None else None, cap, C.byref(n)))
        return n.value

    def upload_n(self, species: int, p: dict, n: int):
        """Upload the first n particles of caller-provided float64 arrays (no copy on the host)."""
        self._check(lib().ohpic_upload_particles_soa(
            self.ptr, species, *[_dp(p[k]) for k in ("x", "y", "z", "vx", "vy", "vz")], n))

    def download_aos(self, species: int, width: int = 6) -> np.ndarray:
        cap = int(self.cfg.capacity[species])
        buf = np.zeros((cap, width), dtype=np.float64)
        n = C.c_int64()
        self._check(lib().ohpic_download_particles(self.ptr, species, buf.ctypes.data_as(_P), cap, width * 8,
                                                   C.byref(n)))
        return buf[: n.value]

    # -- the reference's operations, batched ---------------------------------
    def scatter(self):
        self._check(lib().ohpic_scatter(self.ptr))

    def solve(self):
        self._check(lib().ohpic_solve(self.ptr))

    def interp(self, species: int) -> np.ndarray:
        cap = int(self.cfg.capacity[species])
        out = np.empty(3 * max(cap, 1), dtype=np.float64)
        n = C.c_int64()
        self._check(lib().ohpic_interp(self.ptr, species, _dp(out), out.size, C.byref(n)))
        return out[: 3 * n.value].reshape(-1, 3)

    def move(self, dt: float):
        self._check(lib().ohpic_move(self.ptr, dt))

    def push(self, dt: float):
        self._check(lib().ohpic_push(self.ptr, dt))

    def step(self, dt: float, nsteps: int = 1):
        self._check(lib().ohpic_step(self.ptr, dt, nsteps))

    def sort(self):
        self._check(lib().ohpic_sort(self.ptr))

    def synchronize(self):
        self._check(lib().ohpic_synchronize(self.ptr))

    # -- fields -------------------------------------------------------------
    def field(self, which: int) -> np.ndarray:
        nx, ny, nz = self.n
        out = np.empty((nz, ny, nx), dtype=np.float64)
        self._check(lib().ohpic_download_field(self.ptr, which, _dp(out)))
        return out

    def set_field(self, which: int, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self._check(lib().ohpic_upload_field(self.ptr, which, _dp(a)))

    def field_ohfield(self, which: int, lo, hi, nelem: int) -> np.ndarray:
        lo_a = (C.c_int32 * 3)(*lo)
        hi_a = (C.c_int32 * 3)(*hi)
        ext = [hi[d] - lo[d] + 1 for d in range(3)]
        out = np.zeros(nelem * ext[0] * ext[1] * ext[2], dtype=np.float64)
        self._check(lib().ohpic_download_field_ohfield(self.ptr, which, _dp(out), nelem, lo_a, hi_a))
        return out.reshape(ext[2], ext[1], ext[0], nelem)

    def diagnostics(self) -> dict:
        d = Diag()
        self._check(lib().ohpic_diagnostics(self.ptr, C.byref(d)))
        return {
            "count": [d.count[i] for i in range(self.nspecies)],
            "crossings": [d.crossings[i] for i in range(3)],
            "outside_tile": d.outside_tile,
            "step": d.step,
            "total_charge": d.total_charge,
            "field_energy": d.field_energy,
            "kinetic_energy": d.kinetic_energy,
            "momentum": [d.momentum[i] for i in range(3)],
        }

    def set_energy_tracking(self, on: bool):
        self._check(lib().ohpic_set_energy_tracking(self.ptr, 1 if on else 0))

    def set_tma_wait_limit(self, polls: int):
        """Polls allowed for each tile's staged E box (0: every wait gives up at once)."""
        self._check(lib().ohpic_set_tma_wait_limit(self.ptr, int(polls)))

    # -- instrumentation ------------------------------------------------------
    def set_push_timing(self, on: bool):
        self._check(lib().ohpic_set_push_timing(self.ptr, 1 if on else 0))

    def stats(self) -> dict:
        a, b, ms = C.c_int64(), C.c_int64(), C.c_double()
        self._check(lib().ohpic_stats(self.ptr, C.byref(a), C.byref(b), C.byref(ms)))
        return {"launches": a.value, "push_launches": b.value, "push_ms": ms.value}

    def get_tuning(self) -> dict:
        t = Tuning()
        self._check(lib().ohpic_get_tuning(self.ptr, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw):
        cur = self.get_tuning()
        cur.update(kw)
        t = Tuning()
        for d in range(3):
            t.tile[d] = int(cur["tile"][d])
        t.halo, t.split = int(cur["halo"]), int(cur["split"])
        t.deposit, t.sort_every = int(cur["deposit"]), int(cur["sort_every"])
        t.lane_particles = int(cur.get("lane_particles", 4))
        t.sort_lead = int(cur.get("sort_lead", 0))
        self._check(lib().ohpic_set_tuning(self.ptr, C.byref(t)))

    def memory(self) -> int:
        v = C.c_int64()
        self._check(lib().ohpic_memory(self.ptr, C.byref(v)))
        return v.value


class PoissonSolver:
    """The field solve on a bounded block (ohpic_poisson_*): t_PoissonFieldSolver
    with a boundary kind per axis (poisson_field_solver.f90:34-175).  Arrays are
    (nz+1, ny+1, nx+1) blocks of nodes, x fastest."""

    def __init__(self, n, kinds, boundary_values=(0.0,) * 6, table=TABLE_AS_WRITTEN, device=0):
        self.n = tuple(int(v) for v in n)
        na = (C.c_int32 * 3)(*self.n)
        ka = (C.c_int32 * 3)(*[int(k) for k in kinds])
        bv = np.ascontiguousarray(boundary_values, dtype=np.float64)
        ptr = _P()
        rc = lib().ohpic_poisson_create(na, ka, _dp(bv), int(table), int(device), C.byref(ptr))
        if rc != OK:
            raise OhpicError(rc, lib().ohpic_status_string(rc).decode())
        self.ptr = ptr

    def _check(self, rc: int):
        if rc != OK:
            buf = C.create_string_buffer(512)
            lib().ohpic_poisson_last_error(self.ptr, buf, 512)
            raise OhpicError(rc, buf.value.decode(errors="replace"))

    def solve(self, rho: np.ndarray, with_e: bool = True):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        shape = (self.n[2] + 1, self.n[1] + 1, self.n[0] + 1)
        if rho.shape != shape:
            raise OhpicError(ERR_INVALID, f"rho must have shape {shape}")
        phi = np.empty_like(rho)
        e = np.empty((3,) + shape) if with_e else None
        self._check(lib().ohpic_poisson_solve(self.ptr, _dp(rho), _dp(phi), _dp(e) if e is not None else None))
        return (phi, e) if with_e else phi

    def solve_device(self, rho_ptr: int, phi_ptr: int, e_ptr: int | None = None, stream: int = 0):
        """Device arrays, ordered on `stream` (a cudaStream_t handle; 0 = the default stream)."""
        self._check(lib().ohpic_poisson_solve_device(self.ptr, _P(rho_ptr), _P(phi_ptr),
                                                     _P(e_ptr) if e_ptr else None, _P(stream)))

    def close(self):
        if getattr(self, "ptr", None):
            lib().ohpic_poisson_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Mirror of the reference's module API for the path (batched, device-resident).
# ---------------------------------------------------------------------------
class Scatter:
    """t_LinearScatter (linear_scatter.f90) over every particle of the run."""

    def __init__(self, ctx: PicContext):
        self.ctx = ctx

    def scatter_all(self):
        self.ctx.scatter()


class FieldSolver:
    """t_PoissonFieldSolver (poisson_field_solver.f90) on the device."""

    def __init__(self, ctx: PicContext):
        self.ctx = ctx

    def solve(self):
        self.ctx.solve()


class Interpolator:
    """t_LinearInterpolator (linear_interpolator.f90), all particles of a species."""

    def __init__(self, ctx: PicContext):
        self.ctx = ctx

    def interp_all(self, species: int) -> np.ndarray:
        return self.ctx.interp(species)


class ParticleMover:
    """t_ParticleMoverBoris + t_ParticleBoundaries (periodic, applied twice)."""

    def __init__(self, ctx: PicContext):
        self.ctx = ctx

    def move_all(self, dt: float):
        self.ctx.move(dt)


def create_particle_mover(name: str, ctx: PicContext) -> ParticleMover:
    """Factory mirroring particle_mover_factory.f90:20-31 ('boris' only);
    an unknown name raises instead of leaving the result unallocated."""
    if name != "boris":
        raise OhpicError(ERR_INVALID, f"unknown particle mover '{name}'")
    return ParticleMover(ctx)
