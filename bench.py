"""Benchmark of the particle hot path: particle-steps/s on one GB300 (or N replicas).

Default workload: the 256^3 configuration (2 species x 32 ppc = 1,073,741,824
particles).  The headline `value` is the FP32 precision form with standard CIC
weights, the convention in which it meets the error bar; `fp64_form` is the
plain FP64 form on the same workload.  A step is one mainstep: spectral field
solve, then the fused gather + Boris + periodic wrap + deposit over every
particle, with the cell sort before every step whose index is a multiple of 20.

Each (form, convention) is one run from the injector: whole sort cycles of
warm-up, the K timed steps, then on to step 100.  Fields are captured after
steps 1, 10 and 100, outside the timed window, and the FP32 run's captures are
compared with the FP64 run's from the same seeds (`accuracy`).  The FP32 form in
the reference's own swapped-weight convention is run the same way beside it,
with its own error.  Also in the line: the 32^3 configuration's errors against
the oracle itself (`c3_vs_oracle`), the clustered two-stream workload (`c4`),
the bounded-domain field solve at 256^3 (`poisson_bounded`), both forms end to
end through the C ABI (`e2e`), the oracle on the host cores (`cpu_baseline`)
and the serving ensemble (`serving`).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c2|c1|c4] [--forms fp32,fp64] [--weights 1|0] [--no-e2e] ...

For N > 1 (launched with torch.distributed.run) every rank advances its own
replica of the workload (different random streams); there is no collective on
the data path ("replicas only"), only a barrier and a max-reduction of the
timings.  `--impl reference` times the reference's CPU path (the C restatement
in oracle/, since the Fortran reference cannot be built) on the host cores, on
a slab of the workload with the same plasma.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (1 GB300, %HBM peak), FP32 vs FP64; ensemble p50/p99 latency"
UNIT = "particle-steps/s"
# Algorithmic bytes of the fused push kernel per particle (one read + one write of
# the record) and per grid node (E read + rho write), by form.
PUSH_BYTES_PER_PARTICLE = {"fp32": 2 * (4 + 12 + 12), "fp64": 2 * 48}
# The FP32 push right after a sort reads the sort's 32-byte records and writes the
# 28 bytes of arrays plus the 4-byte id: 8 bytes per particle more than a push.
REC_PUSH_EXTRA_BYTES = 8
PUSH_BYTES_PER_NODE = {"fp32": 12 + 4, "fp64": 24 + 8}
# Whole-step grid term: rho write, R2C read, spectrum write, scale r/w, C2R read,
# phi write, stencil read, E write, gather read (per node).
STEP_BYTES_PER_NODE = {"fp32": 72, "fp64": 144}
# DRAM traffic of one push launch over its algorithmic bytes, from one ncu capture of
# the push one step after a sort (dram__bytes_read.sum + dram__bytes_write.sum) at
# 128x128x64 with the same tuned tile, halo and particle density: 3.801 / 3.775 GB
# (FP32) and 6.812 / 6.476 GB (FP64, two steps after a sort).  Both terms scale with
# the grid at fixed density, so the ratio carries to 256^3.
PUSH_TRAFFIC_RATIO = {"fp32": 3.801085 / 3.774873600, "fp64": 6.812251 / 6.476005376}
PUSH_TRAFFIC_SOURCE = {
    "fp32": "ncu DRAM bytes of one push launch at 128x128x64 (same tile, halo and density), scaled by particles",
    "fp64": "ncu DRAM bytes of one push launch at 128x128x64 (same tile, halo and density), scaled by particles",
}
# The precision form's accuracy target: E-field relative L2 error against the FP64
# run after 100 steps.
E_ERROR_BAR = 1e-5


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during timed regions."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50", "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            time.sleep(0.12)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)
            self.proc = None

    def summary(self) -> dict:
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = sorted(x for x in (num(r[1]) for r in self.rows) if x is not None)
        mx = [x for x in (num(r[2]) for r in self.rows) if x is not None]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i - 5] for r in self.rows for i in range(5, 9) if r[i].lower().startswith("active")})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------------------
# Distributed plumbing (replicas only)
# ---------------------------------------------------------------------------
class Dist:
    """Replicas only: every rank runs its own copy of the workload; the ranks meet
    only in barriers and in max/sum reductions of host timings and counts."""

    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = False
        self.device = "cuda"

    def init(self, backend: str = "nccl"):
        import torch
        import torch.distributed as dist
        if self.world > 1 and not dist.is_initialized():
            if backend == "nccl":
                dist.init_process_group("nccl", device_id=torch.device("cuda", self.local))
            else:
                dist.init_process_group(backend)
                self.device = "cpu"
            self.pg = True

    def barrier(self):
        if self.pg:
            import torch.distributed as dist
            dist.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        import torch.distributed as dist
        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        import torch.distributed as dist
        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            import torch.distributed as dist
            dist.destroy_process_group()


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
CHECKPOINTS = (1, 10, 100)


def make_context(P, wl, form: str, weights: int, device: int):
    caps = [c + 1024 for c in wl.counts()]
    cfg = P.make_config(n=wl.n, dt=wl.dt, b0=wl.b0, qm=[s.qm for s in wl.species], q=[s.q for s in wl.species],
                        capacity=caps, precision=P.FP32 if form == "fp32" else P.FP64, weights=weights,
                        sort_every=0, device=device)
    return P.PicContext(cfg)


def species_inits(P, wl):
    return [P.species_init(s.ppc, s.vth, s.drift, s.lo, s.hi if s.hi is not None else (1e30, 1e30, 1e30))
            for s in wl.species]


def tune_form(P, wl, form, args, weights) -> dict | None:
    """Launch shape for this workload from the autotuner, measured on a proxy grid
    of at most 256 x 128 x 64 cells with the same particles per cell and physics,
    each candidate ranked by its mean push over one sort cycle (the sort cadence
    stays the workload's).  The weight convention does not change the kernels'
    work, so one tuning serves both conventions."""
    if args.tuning:
        return dict(json.loads(args.tuning), tuned_on="given on the command line")
    if args.no_tune:
        return None
    from ohhelppic3d_gb300 import autotune
    t0 = time.perf_counter()
    t = autotune.tune(n=wl.n, dt=wl.dt, b0=wl.b0, qm=[s.qm for s in wl.species], q=[s.q for s in wl.species],
                      capacity_per_cell=[s.ppc * 1.02 + 1 for s in wl.species], species=species_inits(P, wl),
                      precision=P.FP32 if form == "fp32" else P.FP64, weights=weights,
                      steps=max(4, wl.sort_every - 1) if form == "fp32" else 4,
                      max_cadence=40, proxy_limit=(256, 128, 64))
    keep = ("tile", "halo", "split", "deposit", "lane_particles", "sort_lead")
    return {**{k: t[k] for k in keep}, "sort_every_suggested": t["sort_every"],
            "tuned_on": list(t["grid_tuned_on"]), "trials": len(t["trials"]),
            "seconds": round(time.perf_counter() - t0, 2)}


def record_pushes(form: str, applied: dict, steps: int, sort_every: int, lanes: int) -> int:
    """Pushes among `steps` timed steps that read the sort's records: the first
    push after each sort (the course sorts at every multiple of sort_every), in
    the FP32 form with four particles per lane and the LANES deposit."""
    if form != "fp32" or not sort_every or applied["lane_particles"] != 4 or applied["deposit"] != lanes:
        return 0
    return sum(1 for i in range(steps) if i % sort_every == 0)


def capture(P, ctx) -> dict:
    """The state at the current step: rho, phi and E (FP64 host copies, solved
    from the particles' current charge) and the diagnostics."""
    ctx.solve()
    f = {name: ctx.field(w) for name, w in (("rho", P.RHO), ("phi", P.PHI), ("ex", P.EX), ("ey", P.EY),
                                             ("ez", P.EZ))}
    return {"fields": f, "diag": ctx.diagnostics()}


def _rel_l2(a, b) -> float:
    import numpy as np
    return float(np.linalg.norm(a - b) / max(float(np.linalg.norm(b)), 1e-300))


def compare(got: dict, ref: dict) -> dict:
    """Relative L2 errors of rho, phi, each E component and E as a whole, and the
    relative difference of the field energy, of `got` against `ref`."""
    import numpy as np
    g, r = got["fields"], ref["fields"]
    out = {k: _rel_l2(g[k], r[k]) for k in ("rho", "phi", "ex", "ey", "ez")}
    num = sum(float(np.linalg.norm(g[k] - r[k])) ** 2 for k in ("ex", "ey", "ez"))
    den = sum(float(np.linalg.norm(r[k])) ** 2 for k in ("ex", "ey", "ez"))
    out["e"] = (num / max(den, 1e-300)) ** 0.5
    wr = ref["diag"]["field_energy"]
    out["field_energy_rel_diff"] = (got["diag"]["field_energy"] - wr) / wr if wr else None
    return out


def energy_drift(caps: dict) -> dict:
    """Total (kinetic + field) energy at each checkpoint relative to step 0."""
    e0 = caps[0]["diag"]["kinetic_energy"] + caps[0]["diag"]["field_energy"]
    return {str(k): (v["diag"]["kinetic_energy"] + v["diag"]["field_energy"] - e0) / e0
            for k, v in sorted(caps.items()) if k}


def run_course(P, torch, dist, wl, form, weights, args, sampler, peak, tuning, checkpoints=()):
    """One run of the workload from the injector: whole sort cycles of warm-up (at
    least --warmup steps), the K timed steps, then on to the last checkpoint.  The
    cell sort runs before every step whose index is a multiple of sort_every, so
    the timed window's first sort meets particles that drifted for a full cycle,
    as every sort of a long run does.  `checkpoints` are steps after which the
    fields are captured (outside the timed window; step 0 is always captured
    when any is asked for).  Returns the context, the per-species counts, the
    timing result and the captures."""
    ctx = make_context(P, wl, form, weights, dist.local)
    if tuning:
        from ohhelppic3d_gb300 import autotune
        autotune.apply(ctx, tuning, keep_sort_every=True)
    counts = ctx.init_particles(species_inits(P, wl), seed=(42, 52 + dist.rank))
    n_local = sum(counts)
    se = wl.sort_every
    warm = -(-args.warmup // se) * se if se else args.warmup
    t_end = warm + args.steps
    inside = [c for c in checkpoints if warm < c <= t_end]
    if inside:
        raise ValueError(f"checkpoints {inside} fall inside the timed window ({warm}, {t_end}]")
    caps = {0: capture(P, ctx)} if checkpoints else {}
    step = 0

    def advance(target, on_step=None):
        nonlocal step
        while step < target:
            if se and step % se == 0:
                ctx.sort()
            elif not se and step == 0:
                ctx.sort()
            ctx.step(wl.dt, 1)
            step += 1
            if on_step is not None:
                on_step()
            if step in checkpoints:
                caps[step] = capture(P, ctx)

    advance(warm)
    ctx.synchronize()
    ctx.set_push_timing(True)
    launches0 = ctx.stats()["launches"]
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    e0.record(stream)
    advance(t_end)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    sampler.stop()
    dist.barrier()
    ms = e0.elapsed_time(e1)
    st = ctx.stats()
    ctx.set_push_timing(False)
    launches = st["launches"] - launches0
    advance(max([t_end] + list(checkpoints)))
    ms_max = dist.max(ms)
    n_total = dist.sum(float(n_local))
    value = n_total * args.steps / (ms_max / 1e3)
    avg_push_ms = st["push_ms"] / max(st["push_launches"], 1)
    push_bytes = n_local * PUSH_BYTES_PER_PARTICLE[form] + wl.ncell * PUSH_BYTES_PER_NODE[form]
    rec_pushes = record_pushes(form, ctx.get_tuning(), args.steps, se, P.DEPOSIT_LANES)
    push_bytes += rec_pushes * n_local * REC_PUSH_EXTRA_BYTES / max(st["push_launches"], 1)
    achieved = push_bytes / (avg_push_ms / 1e3) / 1e9
    step_bytes = n_local * PUSH_BYTES_PER_PARTICLE[form] + wl.ncell * STEP_BYTES_PER_NODE[form]
    out = {
        "value": value, "ms_per_step": ms_max / args.steps, "particles": int(n_total),
        "roofline": {"bound": "hbm", "kernel": f"tiled_{'f32' if form == 'fp32' else 'f64'}<MODE_PUSH> (fused push)",
                     "achieved": achieved, "peak": peak[0], "unit": "GB/s", "frac": achieved / peak[0],
                     "traffic": PUSH_TRAFFIC_RATIO[form] * push_bytes, "bytes_per_launch": push_bytes,
                     "avg_launch_ms": avg_push_ms, "record_pushes": rec_pushes,
                     "peak_source": f"{peak[1]} (MEASURED_PEAKS.json hbm_gbs: copy bandwidth)",
                     "traffic_source": PUSH_TRAFFIC_SOURCE[form]},
        "step_hbm_frac": step_bytes / (ms_max / args.steps / 1e3) / 1e9 / peak[0],
        "push_share": st["push_ms"] / ms if ms > 0 else None,
        "gpu_launches": launches,
        "tuning": dict(tuning or {}, applied=ctx.get_tuning()),
        "sort_every": se,
        "warmup_steps_run": warm,
        "timed_steps": [warm, t_end],
        "weights": _wname(weights),
    }
    return ctx, counts, out, caps


def pinned_host_arrays(torch, wl) -> list:
    """Pinned FP64 host arrays (x, y, z, vx, vy, vz) per species, with room for the
    injector's counts; allocated once and shared by the e2e runs of both forms."""
    return [{k: torch.empty(c + 1024, dtype=torch.float64, pin_memory=True).numpy()
             for k in ("x", "y", "z", "vx", "vy", "vz")} for c in wl.counts()]


def run_e2e(P, torch, dist, wl, args, ctx, counts, host):
    """The same K steps through the C ABI with host buffers: upload every particle
    from pinned host memory, K steps each followed by a diagnostics read (the
    step's result: charge and energies), and a download of every particle."""
    import numpy as np
    for s, n in enumerate(counts):
        ctx.download_into(s, host[s])
    ctx.set_energy_tracking(True)
    ctx.synchronize()
    se = wl.sort_every
    dist.barrier()
    t0 = time.perf_counter()
    for s, n in enumerate(counts):
        ctx.upload_n(s, host[s], n)
    for i in range(args.steps):
        if (se and i % se == 0) or (not se and i == 0):
            ctx.sort()
        ctx.step(wl.dt, 1)
        ctx.diagnostics()
    for s in range(len(counts)):
        ctx.download_into(s, host[s])
    ctx.synchronize()
    t1 = time.perf_counter()
    dist.barrier()
    sec = dist.max(t1 - t0)
    n_total = dist.sum(float(sum(counts)))
    moved = 48 * sum(counts)
    finite = bool(np.isfinite(host[0]["x"][:1000]).all())
    return {"value": n_total * args.steps / sec, "unit": UNIT,
            "h2d_bytes_per_step": moved / args.steps,
            "d2h_bytes_per_step": (moved + args.steps * 160) / args.steps,
            "seconds": sec, "finite": finite,
            "how": ("job through the C ABI: ohpic_upload_particles_soa from pinned FP64 host arrays, "
                    "K x (ohpic_sort every sort_every steps + ohpic_step + ohpic_diagnostics), "
                    "ohpic_download_particles_soa")}


def c3_vs_oracle(P, weights_list, threads: int) -> dict:
    """The precision form (and the plain form) of the 32^3 configuration against
    the oracle itself: the same initial particles uploaded to the GPU and to the
    oracle, 100 steps with a sort every 20, fields compared after 1, 10 and 100
    steps.  The FP32 form meets the 1e-5 bar only with the continuous (standard)
    CIC weights; the reference's swapped weights are discontinuous at cell faces."""
    import oracle as O
    from ohhelppic3d_gb300.workloads import c1
    wl = c1()
    out = {"workload": wl.description, "threads": threads}
    for w in weights_list:
        setup = O.Setup(n=wl.n, dt=wl.dt, b0=wl.b0, weights=w,
                        species=[O.SpeciesInit(ppc=s.ppc, vth=s.vth, qm=s.qm, q=s.q) for s in wl.species])
        o = O.Oracle(setup, threads=threads)
        o.init_particles()
        parts = [o.get_particles(s) for s in range(len(wl.species))]
        ref = {}
        done = 0
        for step in CHECKPOINTS:
            o.step(step - done)
            done = step
            o.deposit()
            o.solve()
            ref[step] = {"fields": {k: o.get_field(getattr(O, k.upper())) for k in ("rho", "phi", "ex", "ey", "ez")},
                         "diag": o.diagnostics()}
        o.close()
        for form in ("fp32", "fp64"):
            caps = [len(p["x"]) + 64 for p in parts]
            cfg = P.make_config(n=wl.n, dt=wl.dt, b0=wl.b0, qm=[s.qm for s in wl.species],
                                q=[s.q for s in wl.species], capacity=caps,
                                precision=P.FP32 if form == "fp32" else P.FP64, weights=w, sort_every=20)
            with P.PicContext(cfg) as ctx:
                for s, p in enumerate(parts):
                    ctx.upload(s, p)
                errs, done = {}, 0
                for step in CHECKPOINTS:
                    ctx.step(wl.dt, step - done)
                    done = step
                    errs[str(step)] = compare(capture(P, ctx), ref[step])
            out[f"{form}_{'standard' if w else 'reference'}_weights"] = errs
    return out


def run_poisson_bc(P, torch, peak, n=(256, 256, 256), reps: int = 10) -> dict:
    """The bounded-domain field solve (non-periodic kinds) at 256^3, FP64, on
    device arrays: CUDA-event time per solve (after 3 untimed) for all-Dirichlet
    walls and for a mixed set, with the algorithmic bytes rho read + phi write + E
    write = 40 B per node (the transforms' internal passes count against it)."""
    out = {"grid": list(n), "bytes_per_node": 40, "reps": reps}
    dev = torch.device("cuda", torch.cuda.current_device())
    shape = (n[2] + 1, n[1] + 1, n[0] + 1)
    g = torch.Generator(device=dev).manual_seed(3)
    rho = torch.randn(shape, dtype=torch.float64, device=dev, generator=g)
    phi = torch.empty_like(rho)
    e = torch.empty((3,) + shape, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    nodes = shape[0] * shape[1] * shape[2]
    for name, kinds in (("dirichlet_xyz", (P.BC_DIRICHLET,) * 3),
                        ("dirichlet_neumann_periodic", (P.BC_DIRICHLET, P.BC_NEUMANN, P.BC_PERIODIC))):
        with P.PoissonSolver(n, kinds, table=P.TABLE_CORRECTED) as s:
            for _ in range(3):
                s.solve_device(rho.data_ptr(), phi.data_ptr(), e.data_ptr(), stream.cuda_stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                s.solve_device(rho.data_ptr(), phi.data_ptr(), e.data_ptr(), stream.cuda_stream)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / reps
        gbs = 40.0 * nodes / (ms / 1e3) / 1e9
        out[name] = {"kinds": list(kinds), "ms_per_solve": ms, "achieved_gbs": gbs, "frac": gbs / peak[0]}
    del rho, phi, e
    torch.cuda.empty_cache()
    return out


def accuracy_block(caps32: dict, caps64: dict, weights: int) -> dict:
    steps = {str(k): compare(caps32[k], caps64[k]) for k in CHECKPOINTS}
    e100 = steps[str(CHECKPOINTS[-1])]["e"]
    return {"against": ("the plain FP64 form on the GPU from the same injector seeds and weight convention "
                        "(oracle-checked on the 32^3 configuration: cell indices and crossings exact, "
                        "fields within 2e-12 after 100 steps)"),
            "weights": _wname(weights), "steps": steps, "e_rel_l2_after_100": e100,
            "bar": E_ERROR_BAR, "meets_bar": e100 <= E_ERROR_BAR,
            "energy_drift": {"fp32": energy_drift(caps32), "fp64": energy_drift(caps64)}}


# ---------------------------------------------------------------------------
# Serving: the ensemble of small runs through the continuous-batching server
# ---------------------------------------------------------------------------
def sequential_runs(P, reqs, sort_every: int, sort_lead: int, weights: int, halo: int = 1) -> dict:
    """One run at a time on the single-context API: create, draw, step, read the
    diagnostics, destroy.  Times with and without the per-run set-up.  The runs
    get the server's launch shape, cadence and sort lead."""
    import torch
    total = steps_only = 0.0
    work = 0
    for r in reqs:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        caps = [c + 64 for c in _req_counts(r)]
        cfg = P.make_config(n=r.n, dt=r.dt, b0=r.b0, qm=r.qm, q=r.q, capacity=caps, precision=P.FP32,
                            weights=weights, sort_every=sort_every)
        with P.PicContext(cfg) as ctx:
            # the server's launch shape: its halo, tile edges up to 16 in x and 8 in y, z
            tile = tuple(max(t for t in (1, 2, 4, 8, 16) if t <= want and n % t == 0)
                         for n, want in zip(r.n, (16, 8, 8)))
            ctx.set_tuning(halo=halo, tile=tile, sort_lead=sort_lead)
            counts = ctx.init_particles(r.species, seed=r.seed)
            ctx.synchronize()
            t1 = time.perf_counter()
            ctx.step(r.dt, r.nsteps)
            ctx.diagnostics()
            t2 = time.perf_counter()
        total += time.perf_counter() - t0
        steps_only += t2 - t1
        work += sum(counts) * r.nsteps
    return {"runs": len(reqs), "particle_steps": work, "seconds": total, "throughput": work / total,
            "throughput_steps_only": work / steps_only}


def _req_counts(r) -> list:
    out = []
    for sp in r.species:
        vol = 1.0
        for d in range(3):
            vol *= max(min(sp.hi[d], r.n[d]) - max(sp.lo[d], 0.0), 0.0)
        out.append(int(sp.ppc * vol) + 1)
    return out


def run_serving(P, args) -> dict:
    """The ensemble workload: runs drawn from {16,24,32,48,64}^3 grids, {8,16,32,64}
    ppc per species, wce/wpe ~ U[0,1], vth_e ~ U[0.5,2], mass ratio 100, dt 0.1,
    steps ~ U{200..2000} x step_scale.  First all runs at once (the batched
    capacity C), then Poisson arrivals at 0.8 C / E[work] for the p50/p99 time to
    completion, then a sample of the same runs one at a time."""
    from ohhelppic3d_gb300 import serve as S
    n_runs, scale = args.serve_runs, args.serve_step_scale
    sat_reqs = S.ensemble_stream(n_runs, rate=None, step_scale=scale)
    lead = args.serve_sort_every // 2 if args.serve_sort_lead < 0 else args.serve_sort_lead
    with S.Server(sort_every=args.serve_sort_every, sort_lead=lead, halo=args.serve_halo,
                  weights=args.weights) as srv:
        sat = S.run_stream(srv, sat_reqs)
        sat_stats = srv.stats()
    mean_work = sat["particle_steps"] / n_runs
    rate = 0.8 * sat["throughput"] / mean_work
    reqs = S.ensemble_stream(n_runs, rate=rate, step_scale=scale)
    with S.Server(sort_every=args.serve_sort_every, sort_lead=lead, halo=args.serve_halo,
                  weights=args.weights) as srv:
        poi = S.run_stream(srv, reqs)
        poi_stats = srv.stats()
    k = min(args.serve_sequential, n_runs)
    seq = sequential_runs(P, sat_reqs[:k], args.serve_sort_every, lead, args.weights, args.serve_halo)
    keep = ("ticks", "sort_ticks", "graph_captures", "graph_launches", "launches", "bytes_peak", "pools")
    return {
        "workload": (f"{n_runs} periodic FP32 runs: grids {{16,24,32,48,64}}^3, ppc per species {{8,16,32,64}}, "
                     f"wce/wpe~U[0,1], vth_e~U[0.5,2], vth_i=vth_e/10, mass ratio 100, dt=0.1, "
                     f"steps~U{{200..2000}} x {scale}; parameter stream pcg32 (42, 1000), run i seeded (42, 52+i)"),
        "runs": n_runs, "step_scale": scale, "weights": _wname(args.weights), "particle_steps": sat["particle_steps"],
        "sort_every": args.serve_sort_every, "sort_lead": lead, "halo": args.serve_halo,
        "saturated": {"throughput": sat["throughput"], "span_s": sat["span_s"], "p50_s": sat["p50_s"],
                      "p99_s": sat["p99_s"], "stats": {k2: sat_stats[k2] for k2 in keep}},
        "poisson_80": {"rate_runs_per_s": rate, "throughput": poi["throughput"], "span_s": poi["span_s"],
                       "p50_s": poi["p50_s"], "p99_s": poi["p99_s"], "mean_s": poi["mean_s"],
                       "stats": {k2: poi_stats[k2] for k2 in keep}},
        "sequential": dict(seq, how=f"the first {k} runs of the stream, one at a time on ohpic_create/"
                                    f"ohpic_init_particles/ohpic_step/ohpic_diagnostics/ohpic_destroy"),
        "batched_over_sequential": sat["throughput"] / seq["throughput"],
        "unit": UNIT,
    }


# ---------------------------------------------------------------------------
# CPU path (oracle): the reference's algorithm on the host cores
# ---------------------------------------------------------------------------
CPU_SAMPLE_PARTICLES = 6.8e7


def cpu_sample_workload(wl):
    """A bounded sample of the workload for the CPU path: the same plasma (density,
    species, physics) on a slab of the box, the z extent cut to the largest power
    of two that keeps about 6.8e7 particles.  Every per-particle and per-node cost
    is the workload's own, measured directly rather than scaled."""
    import copy
    if wl.nparticles <= CPU_SAMPLE_PARTICLES:
        return wl
    nz = wl.n[2]
    while nz > 1 and wl.nparticles * nz / wl.n[2] > CPU_SAMPLE_PARTICLES:
        nz //= 2
    s = copy.deepcopy(wl)
    s.n = (wl.n[0], wl.n[1], nz)
    s.description = f"{wl.n[0]}x{wl.n[1]}x{nz} slab of: {wl.description}"
    return s


def oracle_course(wl, threads: int, weights: int, steps: int, warmup: int):
    """`warmup` untimed then `steps` timed mainsteps (deposit + FFT solve + push) of
    the oracle on the workload; returns the per-step seconds and the particle count."""
    import oracle as O
    species = [O.SpeciesInit(ppc=s.ppc, vth=s.vth, qm=s.qm, q=s.q, drift=s.drift, lo=s.lo, hi=s.hi)
               for s in wl.species]
    setup = O.Setup(n=wl.n, dt=wl.dt, b0=wl.b0, species=species, weights=weights)
    o = O.Oracle(setup, threads=threads)
    o.init_particles()
    n = sum(o.count(i) for i in range(len(species)))
    for _ in range(warmup):
        o.step(1)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        o.step(1)
        times.append(time.perf_counter() - t0)
    o.close()
    return times, n


def run_reference(args, wl):
    dist = Dist()
    if dist.rank != 0:
        return 0
    threads = os.cpu_count() or 1
    sample = cpu_sample_workload(wl)
    times, n_sample = oracle_course(sample, threads, args.weights, args.steps, min(args.warmup, 2))
    sec = sum(times)
    value = n_sample * args.steps / sec
    what = (f"{args.steps} timed mainsteps (deposit + FFT solve + push, after {min(args.warmup, 2)} untimed) of "
            f"the oracle with {threads} OpenMP threads on {n_sample} particles: {sample.description}; "
            f"throughput measured on that sample, not scaled")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic: pcg32 seeds (42, 52), the reference injector's draw order",
        "config": {"workload": wl.description, "sample": sample.description,
                   "form": "reference CPU path (FP64; the oracle restatement, the Fortran reference cannot be built)",
                   "weights": _wname(args.weights)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": what},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _wname(w: int) -> str:
    return "reference (swapped CIC, linear_scatter.f90:41-52)" if w == 0 else "standard CIC"


def _short(res: dict, keys=("value", "ms_per_step", "particles", "roofline", "step_hbm_frac", "push_share",
                             "gpu_launches", "tuning", "sort_every", "weights")) -> dict:
    return {k: res[k] for k in keys if k in res}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c4"])
    ap.add_argument("--forms", default="fp32,fp64")
    ap.add_argument("--weights", type=int, default=1,
                    help="CIC convention of the headline: 1 standard (default), 0 the reference's swapped weights")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the error checkpoints against the FP64 form")
    ap.add_argument("--no-other-weights", action="store_true",
                    help="skip the FP32 run in the other CIC convention")
    ap.add_argument("--no-c3", action="store_true", help="skip the 32^3 errors against the oracle")
    ap.add_argument("--no-c4", action="store_true", help="skip the clustered two-stream block")
    ap.add_argument("--no-bounded", action="store_true", help="skip the bounded-domain field solve timing")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n", default=None, help="grid override nx,ny,nz (same physics and ppc; for profiling)")
    ap.add_argument("--no-serve", action="store_true", help="skip the ensemble serving measurement")
    ap.add_argument("--no-tune", action="store_true", help="library default launch shape instead of the autotuner's")
    ap.add_argument("--tuning", default=None,
                    help='fixed launch shape instead of the autotuner, e.g. \'{"tile": [16, 8, 8], "halo": 1}\'')
    ap.add_argument("--serve-only", action="store_true", help="only the ensemble serving measurement")
    ap.add_argument("--serve-runs", type=int, default=512)
    ap.add_argument("--serve-step-scale", type=float, default=1.0)
    ap.add_argument("--serve-sort-every", type=int, default=8)
    ap.add_argument("--serve-halo", type=int, default=1, help="staged halo of the served and one-at-a-time runs")
    ap.add_argument("--serve-sort-lead", type=int, default=-1,
                    help="sort lead of the served and one-at-a-time runs (-1: half the cadence)")
    ap.add_argument("--serve-sequential", type=int, default=32, help="runs timed one at a time")
    args = ap.parse_args(argv)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3

    from ohhelppic3d_gb300.workloads import WORKLOADS
    wl = WORKLOADS[args.workload]()
    if args.n:
        wl.n = tuple(int(v) for v in args.n.split(","))
        wl.description += f" [grid overridden to {wl.n[0]}x{wl.n[1]}x{wl.n[2]}]"
    if args.impl == "reference":
        return run_reference(args, wl)

    import torch

    import ohhelppic3d_gb300 as P
    dist = Dist()
    torch.cuda.set_device(dist.local)
    dist.init()
    peak = _peaks()
    forms = [f.strip() for f in args.forms.split(",") if f.strip()]
    sampler = ClockSampler(dist.local)
    solo = dist.rank == 0 and dist.world == 1
    if args.serve_only:
        sampler.start()
        serving = run_serving(P, args)
        sampler.stop()
        if dist.rank == 0:
            print(json.dumps({"metric": METRIC, "serving": serving, "clocks": sampler.summary()}), flush=True)
        dist.close()
        return 0

    accuracy = not args.no_accuracy and "fp32" in forms and "fp64" in forms
    checkpoints = CHECKPOINTS if accuracy else ()
    other_w = 1 - args.weights
    tunings = {f: tune_form(P, wl, f, args, args.weights) for f in forms}
    results, caps, e2e = {}, {}, {}
    host = None if args.no_e2e else pinned_host_arrays(torch, wl)
    # the plain FP64 form first, so its captures are at hand when the FP32 run ends
    for form in sorted(forms, key=lambda f: f != "fp64"):
        ctx, counts, res, cp = run_course(P, torch, dist, wl, form, args.weights, args, sampler, peak,
                                          tunings[form], checkpoints)
        if not args.no_e2e:
            e2e[form] = run_e2e(P, torch, dist, wl, args, ctx, counts, host)
        ctx.close()
        torch.cuda.empty_cache()
        results[form], caps[form] = res, cp
    acc = accuracy_block(caps["fp32"], caps["fp64"], args.weights) if accuracy else None
    caps.clear()
    host = None

    other = None
    if "fp32" in forms and not args.no_other_weights:
        cp64 = cp32 = {}
        if accuracy:
            ctx, _, _, cp64 = run_course(P, torch, dist, wl, "fp64", other_w, args, sampler, peak,
                                         tunings.get("fp64"), checkpoints)
            ctx.close()
            torch.cuda.empty_cache()
        ctx, _, res, cp32 = run_course(P, torch, dist, wl, "fp32", other_w, args, sampler, peak,
                                       tunings["fp32"], checkpoints)
        ctx.close()
        torch.cuda.empty_cache()
        other = _short(res)
        if accuracy:
            other["accuracy"] = accuracy_block(cp32, cp64, other_w)
        del cp64, cp32

    c3 = None
    if solo and not args.no_c3:
        c3 = c3_vs_oracle(P, (args.weights, other_w), os.cpu_count() or 1)

    c4 = None
    if args.workload == "c2" and not args.no_c4 and not args.n:
        from ohhelppic3d_gb300.workloads import c4 as c4_workload
        w4 = c4_workload()
        t4 = tune_form(P, w4, "fp32", args, args.weights)
        ctx, _, res, _ = run_course(P, torch, dist, w4, "fp32", args.weights, args, sampler, peak, t4)
        ctx.close()
        torch.cuda.empty_cache()
        c4 = dict(_short(res), workload=w4.description)

    bounded = None
    if args.workload == "c2" and not args.no_bounded and not args.n:
        bounded = run_poisson_bc(P, torch, peak)

    cpu = None
    if solo and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = cpu_sample_workload(wl)
        times, n_sample = oracle_course(sample, threads, args.weights, 1, 1)
        cpu = {"value": n_sample / times[-1], "unit": UNIT, "cores": threads, "kind": "port",
               "sample": (f"1 timed mainstep (after 1 untimed) of the oracle with {threads} OpenMP threads on "
                          f"{n_sample} particles: {sample.description}; measured on that sample, not scaled")}

    serving = None
    if not args.no_serve and dist.world == 1:
        serving = run_serving(P, args)

    head = forms[0]
    r = results[head]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if head == "fp32" else "f64",
        "data": "synthetic: device-side pcg32 injector, seeds (42, 52 + rank), Maxwellian velocities",
        "config": {"workload": wl.description, "form": {"fp32": "FP32 precision form (int32 cell + FP32 offset)",
                                                        "fp64": "plain FP64 form"}[head],
                   "weights": _wname(args.weights), "particles": r["particles"], "sort_every": r["sort_every"],
                   "warmup_steps_run": r["warmup_steps_run"], "timed_steps": r["timed_steps"],
                   "l2": (f"inputs larger than L2: {r['particles'] * (28 if head == 'fp32' else 48) / 1e9:.1f} GB "
                          f"of particle state per GPU against a 129 MB L2"),
                   "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "single GPU"},
        "roofline": r["roofline"],
        "accuracy": acc if head == "fp32" else None,
        "tuning": r["tuning"],
        "step_hbm_frac": r["step_hbm_frac"],
        "gpu_launches": r["gpu_launches"],
        "clocks": sampler.summary(),
        "e2e": e2e.get(head),
        "cpu_baseline": cpu,
    }
    for form, res in results.items():
        if form != head:
            line[f"{form}_form"] = dict(_short(res), dtype="f64" if form == "fp64" else "f32", e2e=e2e.get(form))
    if "fp64" in results and head == "fp32":
        line["fp32_over_fp64"] = results["fp32"]["value"] / results["fp64"]["value"]
    if other is not None:
        line[f"fp32_{'reference' if other_w == 0 else 'standard'}_weights"] = other
    if c3 is not None:
        line["c3_vs_oracle"] = c3
    if c4 is not None:
        line["c4"] = c4
    if bounded is not None:
        line["poisson_bounded"] = bounded
    if serving is not None:
        line["serving"] = serving
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
