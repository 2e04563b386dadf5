"""Continuous batching of many small periodic runs: the Python side of include/ohpic_serve.h.

A `Server` owns one worker thread on one GPU.  `submit` queues a run described by
`Request`.  The worker admits runs by HBM footprint as memory and slots free up,
and advances every admitted run one step per tick:
  - one batched field solve per grid size;
  - one persistent multi-run push over every run's tiles;
  - a periodic cell sort of all runs together.
The tick is replayed from a captured CUDA graph.  `wait`, `poll` and `result`
give each run's time to completion and its final diagnostics.  A run can also
keep its final fields and particles.

`ensemble_stream` draws the serving workload: runs with grids from
{16,24,32,48,64}^3, ppc per species from {8,16,32,64}, wce/wpe ~ U[0,1],
vth_e ~ U[0.5,2], mass ratio 100, dt = 0.1, steps ~ U{200..2000} and Poisson
arrivals.  The draws come from a pcg32 stream seeded (42, 1000); run i's
injector uses (42, 52 + i).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import (DEPOSIT_RUNS, ERR_CUDA, MAX_SPECIES, OK, WEIGHTS_REFERENCE, Diag, OhpicError, SpeciesInit, lib,
               species_init)


class ServeConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_active", C.c_int32), ("hbm_budget", C.c_int64),
                ("slots_per_pool", C.c_int32), ("sort_every", C.c_int32), ("use_graphs", C.c_int32),
                ("weights", C.c_int32), ("tile", C.c_int32), ("halo", C.c_int32), ("deposit", C.c_int32),
                ("max_species", C.c_int32), ("lane_particles", C.c_int32), ("tile_x", C.c_int32),
                ("sort_lead", C.c_int32), ("reserved", C.c_int32 * 3)]


class RunRequest(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("nspecies", C.c_int32),
                ("dt", C.c_double), ("b0", C.c_double * 3), ("qm", C.c_double * MAX_SPECIES),
                ("q", C.c_double * MAX_SPECIES), ("species", SpeciesInit * MAX_SPECIES),
                ("seed_state", C.c_uint64), ("seed_seq", C.c_uint64), ("nsteps", C.c_int64),
                ("keep_fields", C.c_int32), ("keep_particles", C.c_int32)]


class RunResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("done", C.c_int32), ("steps", C.c_int64),
                ("particles", C.c_int64), ("submit_s", C.c_double), ("admit_s", C.c_double),
                ("finish_s", C.c_double), ("diag", Diag)]


class ServeStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "admitted", "completed", "failed", "active", "pending",
                                         "ticks", "sort_ticks", "particle_steps", "graph_captures",
                                         "graph_launches", "launches", "bytes_in_use", "bytes_peak", "budget")]
    _fields_ += [("pools", C.c_int32), ("reserved", C.c_int32)]


_P = C.c_void_p
_DP = C.POINTER(C.c_double)
SERVE_SIGNATURES = {
    "ohpic_serve_config_default": (None, [C.POINTER(ServeConfig)]),
    "ohpic_run_request_default": (None, [C.POINTER(RunRequest)]),
    "ohpic_serve_create": (C.c_int, [C.POINTER(ServeConfig), C.POINTER(_P)]),
    "ohpic_serve_destroy": (C.c_int, [_P]),
    "ohpic_serve_submit": (C.c_int, [_P, C.POINTER(RunRequest), C.POINTER(C.c_int64)]),
    "ohpic_serve_poll": (C.c_int, [_P, C.POINTER(C.c_int64), C.c_int32, C.POINTER(C.c_int32)]),
    "ohpic_serve_wait": (C.c_int, [_P, C.c_double]),
    "ohpic_serve_result": (C.c_int, [_P, C.c_int64, C.POINTER(RunResult), _DP, _DP]),
    "ohpic_serve_release": (C.c_int, [_P, C.c_int64]),
    "ohpic_serve_stats_get": (C.c_int, [_P, C.POINTER(ServeStats)]),
    "ohpic_serve_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "ohpic_serve_footprint": (C.c_int64, [C.POINTER(ServeConfig), C.POINTER(RunRequest)]),
}

_bound = False


def serve_lib():
    """libohpic.so with the server's signatures set."""
    global _bound
    L = lib()
    if not _bound:
        for name, (res, args) in SERVE_SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _bound = True
    return L


def config(**kw) -> ServeConfig:
    cfg = ServeConfig()
    serve_lib().ohpic_serve_config_default(C.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


@dataclass
class Request:
    """One periodic run: grid, species (qm, q, injector), B0, dt, steps, seed."""
    n: tuple
    nsteps: int
    qm: list
    q: list
    species: list                      # SpeciesInit per species
    dt: float = 0.1
    b0: tuple = (0.0, 0.0, 0.0)
    seed: tuple = (42, 52)
    keep_fields: bool = False
    keep_particles: bool = False
    arrival: float = 0.0               # seconds after the stream starts
    meta: dict = field(default_factory=dict)

    def particles(self) -> int:
        tot = 0
        for sp in self.species:
            vol = 1.0
            for d in range(3):
                vol *= max(min(sp.hi[d], self.n[d]) - max(sp.lo[d], 0.0), 0.0)
            tot += int(sp.ppc * vol)
        return tot

    def to_c(self) -> RunRequest:
        r = RunRequest()
        serve_lib().ohpic_run_request_default(C.byref(r))
        r.nx, r.ny, r.nz = (int(v) for v in self.n)
        r.nspecies = len(self.species)
        r.dt = self.dt
        for d in range(3):
            r.b0[d] = self.b0[d]
        for s, sp in enumerate(self.species):
            r.qm[s] = self.qm[s]
            r.q[s] = self.q[s]
            r.species[s] = sp
        r.seed_state, r.seed_seq = int(self.seed[0]), int(self.seed[1])
        r.nsteps = int(self.nsteps)
        r.keep_fields = int(bool(self.keep_fields))
        r.keep_particles = int(bool(self.keep_particles))
        return r


def thermal_request(n, ppc, nsteps, wce=0.5, vth_e=1.0, seed=(42, 52), dt=0.1, **kw) -> Request:
    """Electrons (qm -1, wp 1) and ions (qm +0.01, wp 0.1, vth_e/10) at ppc per species,
    charge per macro-particle wp^2/qm/ppc (parameters.f90:147-148), B0 along z."""
    qm = [-1.0, 0.01]
    q = [1.0 / qm[0] / ppc, 0.01 / qm[1] / ppc]
    sp = [species_init(ppc, vth_e), species_init(ppc, vth_e / 10.0)]
    return Request(n=tuple(n), nsteps=int(nsteps), qm=qm, q=q, species=sp, dt=dt,
                   b0=(0.0, 0.0, wce), seed=tuple(seed), **kw)


class Pcg32:
    """The published PCG32 (XSH RR) generator, for the parameter stream only."""
    MULT = 6364136223846793005
    MASK = (1 << 64) - 1

    def __init__(self, initstate: int, initseq: int):
        self.inc = ((initseq << 1) | 1) & self.MASK
        self.state = 0
        self.next()
        self.state = (self.state + initstate) & self.MASK
        self.next()

    def next(self) -> int:
        old = self.state
        self.state = (old * self.MULT + self.inc) & self.MASK
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF

    def double(self) -> float:
        return self.next() * 2.0 ** -32


GRIDS = (16, 24, 32, 48, 64)
PPCS = (8, 16, 32, 64)


def ensemble_stream(runs: int = 512, rate: float | None = None, step_scale: float = 1.0,
                    seed: tuple = (42, 1000)) -> list:
    """The serving workload: `runs` requests with their parameters and Poisson
    arrival times (rate in runs/s; None = all at time 0).  Per run the stream
    draws, in order: grid, ppc, wce/wpe, vth_e, steps, inter-arrival gap.
    step_scale < 1 shortens every run (the steps drawn from [200, 2000] times
    step_scale, at least 1) for a bounded sample of the same mix."""
    g = Pcg32(*seed)
    out, t = [], 0.0
    for i in range(runs):
        n = GRIDS[min(int(g.double() * len(GRIDS)), len(GRIDS) - 1)]
        ppc = PPCS[min(int(g.double() * len(PPCS)), len(PPCS) - 1)]
        wce = g.double()
        vth_e = 0.5 + 1.5 * g.double()
        steps = 200 + min(int(g.double() * 1801), 1800)
        gap = -math.log(1.0 - g.double())
        if rate:
            t += gap / rate
        nsteps = max(1, int(round(steps * step_scale)))
        req = thermal_request((n, n, n), ppc, nsteps, wce=wce, vth_e=vth_e, seed=(42, 52 + i))
        req.arrival = t if rate else 0.0
        req.meta = {"index": i, "grid": n, "ppc": ppc, "wce": wce, "vth_e": vth_e, "steps_drawn": steps}
        out.append(req)
    return out


class Server:
    """A continuous-batching server on one GPU (ohpic_serve_create)."""

    def __init__(self, cfg: ServeConfig | None = None, **kw):
        self.L = serve_lib()
        self.cfg = cfg if cfg is not None else config(**kw)
        h = C.c_void_p()
        rc = self.L.ohpic_serve_create(C.byref(self.cfg), C.byref(h))
        if rc != OK:
            raise OhpicError(rc, "ohpic_serve_create failed")
        self.h = h

    def _check(self, rc: int, what: str):
        if rc != OK:
            buf = C.create_string_buffer(512)
            self.L.ohpic_serve_last_error(self.h, buf, 512)
            raise OhpicError(rc, f"{what}: {buf.value.decode(errors='replace')}")

    def close(self):
        if getattr(self, "h", None):
            self.L.ohpic_serve_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def footprint(self, req: Request) -> int:
        return int(self.L.ohpic_serve_footprint(C.byref(self.cfg), C.byref(req.to_c())))

    def submit(self, req: Request) -> int:
        rid = C.c_int64()
        self._check(self.L.ohpic_serve_submit(self.h, C.byref(req.to_c()), C.byref(rid)), "submit")
        return rid.value

    def poll(self, cap: int = 4096) -> list:
        ids = (C.c_int64 * cap)()
        n = C.c_int32()
        self._check(self.L.ohpic_serve_poll(self.h, ids, cap, C.byref(n)), "poll")
        return list(ids[:n.value])

    def wait(self, timeout: float = 0.0):
        self._check(self.L.ohpic_serve_wait(self.h, float(timeout)), "wait")

    def result(self, rid: int, req: Request | None = None) -> dict:
        res = RunResult()
        fields = parts = None
        fp = pp = None
        if req is not None and req.keep_fields:
            fields = np.empty(5 * int(np.prod(req.n)), dtype=np.float64)
            fp = fields.ctypes.data_as(_DP)
        if req is not None and req.keep_particles:
            parts = np.empty(6 * req.particles(), dtype=np.float64)
            pp = parts.ctypes.data_as(_DP)
        self._check(self.L.ohpic_serve_result(self.h, rid, C.byref(res), fp, pp), "result")
        d = res.diag
        out = {"id": res.id, "status": res.status, "done": bool(res.done), "steps": res.steps,
               "particles": res.particles, "submit_s": res.submit_s, "admit_s": res.admit_s,
               "finish_s": res.finish_s, "ttc_s": res.finish_s - res.submit_s,
               "count": list(d.count), "crossings": list(d.crossings), "outside_tile": d.outside_tile,
               "total_charge": d.total_charge, "field_energy": d.field_energy,
               "kinetic_energy": d.kinetic_energy, "momentum": list(d.momentum)}
        if fields is not None and res.done:
            nc = int(np.prod(req.n))
            shape = (req.n[2], req.n[1], req.n[0])
            out["fields"] = {name: fields[k * nc:(k + 1) * nc].reshape(shape)
                             for k, name in enumerate(("rho", "phi", "ex", "ey", "ez"))}
        if parts is not None and res.done:
            ps, off = [], 0
            for s in range(len(req.species)):
                c = int(d.count[s])
                blk = parts[off:off + 6 * c].reshape(6, c)
                ps.append({k: blk[j] for j, k in enumerate(("x", "y", "z", "vx", "vy", "vz"))})
                off += 6 * c
            out["particles_by_species"] = ps
        return out

    def release(self, rid: int):
        self._check(self.L.ohpic_serve_release(self.h, rid), "release")

    def stats(self) -> dict:
        st = ServeStats()
        self._check(self.L.ohpic_serve_stats_get(self.h, C.byref(st)), "stats")
        return {k: getattr(st, k) for k, _ in ServeStats._fields_ if k != "reserved"}


def run_stream(server: Server, reqs: list, poll_s: float = 0.0005) -> dict:
    """Submits each request at its arrival time (relative to now), waits for all,
    and returns per-run times to completion and the aggregate throughput."""
    t0 = time.perf_counter()
    ids = []
    for r in sorted(reqs, key=lambda r: r.arrival):
        while True:
            dt = r.arrival - (time.perf_counter() - t0)
            if dt <= 0:
                break
            time.sleep(min(dt, poll_s) if dt < 0.002 else dt - 0.001)
        ids.append((server.submit(r), r))
    server.wait()
    wall = time.perf_counter() - t0
    res = [server.result(i, r) for i, r in ids]
    bad = [x for x in res if x["status"] != OK]
    if bad:
        raise OhpicError(bad[0]["status"] or ERR_CUDA, f"{len(bad)} runs failed")
    ttc = np.array([x["ttc_s"] for x in res])
    work = sum(x["particles"] * x["steps"] for x in res)
    first = min(x["submit_s"] for x in res)
    last = max(x["finish_s"] for x in res)
    return {"runs": len(res), "particle_steps": work, "wall_s": wall, "span_s": last - first,
            "throughput": work / (last - first), "p50_s": float(np.percentile(ttc, 50)),
            "p99_s": float(np.percentile(ttc, 99)), "mean_s": float(ttc.mean()), "results": res}
