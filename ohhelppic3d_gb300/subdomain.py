"""One MPI rank's OhHelp subdomain on its GPU, and the host side of a decomposed
mainstep.

`Subdomain` mirrors include/ohpic_subdomain.h (the device half of a rank).
`Blocks`, `mainstep` and the two communicators are the host half that OhHelp and
MPI do in the reference (src/ohhelppic3d.f90:286-381, src/ohhelp/ohhelp.f90:299-337):
the blocks' rho are reduced into the global charge (oh3_reduce_field and the
border exchange), the global field solve runs once, each block receives its E
nodes, the particles move on their GPUs, and the ones that left a block go to
the rank that owns their new position (transbound).  The global reduction here
sums whole grids, where OhHelp exchanges only border planes; the particle
routing and the per-rank device work are the same.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import OK, OhpicError, _P, lib

# oh_particle as OhHelp moves it between ranks (include/ohpic_subdomain.h).
PARTICLE = np.dtype([("x", "f8"), ("y", "f8"), ("z", "f8"), ("vx", "f8"), ("vy", "f8"), ("vz", "f8"),
                     ("pid", "i8"), ("nid", "i4"), ("spec", "i4")])
assert PARTICLE.itemsize == 64

_I32x3 = C.c_int32 * 3
# Every symbol include/ohpic_subdomain.h declares, with its ctypes signature.
SIGNATURES = {
    "ohpic_sub_create": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(_P)]),
    "ohpic_sub_destroy": (C.c_int, [_P]),
    "ohpic_sub_append": (C.c_int, [_P, _P, C.c_int64]),
    "ohpic_sub_count": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int64)]),
    "ohpic_sub_download": (C.c_int, [_P, C.c_int, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "ohpic_sub_scatter": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "ohpic_sub_set_e": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "ohpic_sub_move": (C.c_int, [_P, C.c_double, C.POINTER(C.c_int64)]),
    "ohpic_sub_take_emigrants": (C.c_int, [_P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "ohpic_sub_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
}

_bound = False


def sublib():
    global _bound
    L = lib()
    if not _bound:
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _bound = True
    return L


def records(x, y, z, vx, vy, vz, pid, spec) -> np.ndarray:
    """oh_particle records from columns (spec 1-based, nid 13)."""
    r = np.zeros(len(x), dtype=PARTICLE)
    for k, v in (("x", x), ("y", y), ("z", z), ("vx", vx), ("vy", vy), ("vz", vz), ("pid", pid), ("spec", spec)):
        r[k] = v
    r["nid"] = 13
    return r


class Subdomain:
    """A rank's block lo .. lo + m - 1 of the periodic grid cfg.n (FP64 form)."""

    def __init__(self, cfg, lo, m):
        self.cfg = cfg
        self.lo = tuple(int(v) for v in lo)
        self.m = tuple(int(v) for v in m)
        self.nspecies = cfg.nspecies
        ptr = _P()
        rc = sublib().ohpic_sub_create(C.byref(cfg), _I32x3(*self.lo), _I32x3(*self.m), C.byref(ptr))
        if rc != OK:
            raise OhpicError(rc, sublib().ohpic_status_string(rc).decode())
        self.ptr = ptr

    def _check(self, rc: int):
        if rc != OK:
            buf = C.create_string_buffer(512)
            sublib().ohpic_sub_last_error(self.ptr, buf, 512)
            raise OhpicError(rc, buf.value.decode(errors="replace"))

    def close(self):
        if getattr(self, "ptr", None):
            sublib().ohpic_sub_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def node_shape(self):
        return (self.m[2] + 1, self.m[1] + 1, self.m[0] + 1)

    def append(self, recs: np.ndarray):
        recs = np.ascontiguousarray(recs, dtype=PARTICLE)
        if len(recs):
            self._check(sublib().ohpic_sub_append(self.ptr, recs.ctypes.data_as(_P), len(recs)))

    def count(self, species: int) -> int:
        n = C.c_int64()
        self._check(sublib().ohpic_sub_count(self.ptr, species, C.byref(n)))
        return n.value

    def download(self, species: int) -> np.ndarray:
        n = self.count(species)
        out = np.zeros(max(n, 1), dtype=PARTICLE)
        got = C.c_int64()
        self._check(sublib().ohpic_sub_download(self.ptr, species, out.ctypes.data_as(_P), len(out), C.byref(got)))
        return out[: got.value]

    def scatter(self) -> np.ndarray:
        rho = np.empty(self.node_shape, dtype=np.float64)
        self._check(sublib().ohpic_sub_scatter(self.ptr, rho.ctypes.data_as(C.POINTER(C.c_double))))
        return rho

    def set_e(self, e: np.ndarray):
        e = np.ascontiguousarray(e, dtype=np.float64)
        assert e.shape == (3,) + self.node_shape
        self._check(sublib().ohpic_sub_set_e(self.ptr, e.ctypes.data_as(C.POINTER(C.c_double))))

    def move(self, dt: float) -> list:
        left = (C.c_int64 * max(self.nspecies, 1))()
        self._check(sublib().ohpic_sub_move(self.ptr, dt, left))
        return [left[i] for i in range(self.nspecies)]

    def take_emigrants(self) -> np.ndarray:
        n = C.c_int64()
        self._check(sublib().ohpic_sub_take_emigrants(self.ptr, None, 0, C.byref(n)))
        out = np.zeros(max(n.value, 1), dtype=PARTICLE)
        if n.value:
            self._check(sublib().ohpic_sub_take_emigrants(self.ptr, out.ctypes.data_as(_P), len(out), C.byref(n)))
        return out[: n.value]


class Blocks:
    """A periodic grid n cut into rank blocks: cuts[d] lists the first cell of
    every block along axis d (starting with 0).  Rank r = bx + px (by + py bz)."""

    def __init__(self, n, cuts):
        self.n = tuple(int(v) for v in n)
        self.cuts = [np.asarray(sorted(set(int(c) for c in cuts[d]) | {0}), dtype=np.int64) for d in range(3)]
        for d in range(3):
            if self.cuts[d][-1] >= self.n[d] or self.cuts[d][0] != 0:
                raise ValueError("cuts must lie in [0, n)")
        self.p = tuple(len(c) for c in self.cuts)
        self.nranks = self.p[0] * self.p[1] * self.p[2]

    def block(self, r: int):
        """(lo, m) of rank r."""
        b = (r % self.p[0], (r // self.p[0]) % self.p[1], r // (self.p[0] * self.p[1]))
        lo, m = [], []
        for d in range(3):
            c = self.cuts[d]
            lo.append(int(c[b[d]]))
            m.append(int((c[b[d] + 1] if b[d] + 1 < len(c) else self.n[d]) - c[b[d]]))
        return tuple(lo), tuple(m)

    def rank_of(self, x, y, z) -> np.ndarray:
        """Rank owning each position (oh3_map_particle_to_subdomain)."""
        b = [np.searchsorted(self.cuts[d], np.floor(v).astype(np.int64), side="right") - 1
             for d, v in enumerate((x, y, z))]
        return b[0] + self.p[0] * (b[1] + self.p[1] * b[2])

    def _index(self, lo, m):
        return np.ix_(*[(lo[d] + np.arange(m[d] + 1)) % self.n[d] for d in (2, 1, 0)])

    def add_block(self, rho: np.ndarray, blk: np.ndarray, r: int):
        """Adds a block's rho (nodes lo .. lo + m) into the global (nz, ny, nx) array,
        the ghost planes onto their periodic images."""
        lo, m = self.block(r)
        np.add.at(rho, self._index(lo, m), blk)

    def cut_e(self, e: np.ndarray, r: int) -> np.ndarray:
        """Block r's E nodes lo .. lo + m from the global (3, nz, ny, nx) field."""
        lo, m = self.block(r)
        idx = self._index(lo, m)
        return np.stack([e[c][idx] for c in range(3)])


class LocalComm:
    """Every rank in this process (a single-process decomposition)."""

    def allreduce_sum(self, a: np.ndarray) -> np.ndarray:
        return a

    def exchange(self, sends: dict, local_ranks) -> dict:
        out = {r: [] for r in local_ranks}
        for (src, dst), recs in sends.items():
            out[dst].append(recs)
        return {r: (np.concatenate(v) if v else np.zeros(0, dtype=PARTICLE)) for r, v in out.items()}


class TorchComm:
    """One rank per process over torch.distributed (gloo on CPU, NCCL on GPUs)."""

    def __init__(self, dist):
        self.dist = dist

    def allreduce_sum(self, a: np.ndarray) -> np.ndarray:
        import torch
        t = torch.from_numpy(np.ascontiguousarray(a))
        self.dist.all_reduce(t)
        return t.numpy()

    def exchange(self, sends: dict, local_ranks) -> dict:
        gathered = [None] * self.dist.get_world_size()
        self.dist.all_gather_object(gathered, {k: v.tobytes() for k, v in sends.items()})
        out = {r: [] for r in local_ranks}
        for part in gathered:
            for (src, dst), buf in part.items():
                if dst in out:
                    out[dst].append(np.frombuffer(buf, dtype=PARTICLE))
        return {r: (np.concatenate(v) if v else np.zeros(0, dtype=PARTICLE)) for r, v in out.items()}


def mainstep(local: dict, blocks: Blocks, comm, solve, dt: float) -> dict:
    """One mainstep of every rank held in `local` (rank -> Subdomain or an object
    with the same methods).  solve(rho) -> E (3, nz, ny, nx) is the global field
    solve.  Returns per rank the number of particles that left it."""
    n = blocks.n
    rho = np.zeros((n[2], n[1], n[0]))
    for r, sd in local.items():                 # scatter (ohhelppic3d.f90:311-320)
        blocks.add_block(rho, sd.scatter(), r)
    rho = comm.allreduce_sum(rho)               # reduce_field / exchange_borders
    e = solve(rho)                              # field_solver%solve (:323)
    sends, left = {}, {}
    for r, sd in local.items():                 # interp + move + boundaries (:334-358)
        sd.set_e(blocks.cut_e(e, r))
        sd.move(dt)
        em = sd.take_emigrants()                # correct_particle: the new owner
        left[r] = len(em)
        if len(em):
            dest = blocks.rank_of(em["x"], em["y"], em["z"])
            for d in np.unique(dest):
                sends[(r, int(d))] = em[dest == d]
    arrived = comm.exchange(sends, list(local))  # transbound (ohhelp.f90:323-337)
    for r, recs in arrived.items():
        local[r].append(recs)
    return left
