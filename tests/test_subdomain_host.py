"""CPU tests of the subdomain path's host half (no GPU): the C ABI of
include/ohpic_subdomain.h is exported and bound, the block decomposition maps
positions and node planes as OhHelp does, and a decomposed mainstep over two
gloo ranks routes every particle to the rank that owns it.

The gloo test drives ohhelppic3d_gb300.subdomain.mainstep with a stand-in for
the device half (plain numpy: a CIC deposit into the block's nodes and a
force-free move), so it checks the exchange logic itself: charge reduction over
ranks, the E blocks each rank receives, and transbound.
"""
import ctypes as C
import os
import re
import socket
import sys

import numpy as np
import pytest

from conftest import ROOT


def _header_functions():
    with open(os.path.join(ROOT, "include", "ohpic_subdomain.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ohpic_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_subdomain_symbol(ohpic):
    from ohhelppic3d_gb300 import subdomain as S
    L = C.CDLL(ohpic.LIB_PATH)
    names = _header_functions()
    assert "ohpic_sub_move" in names and "ohpic_sub_take_emigrants" in names
    assert not [n for n in names if not hasattr(L, n)]
    assert sorted(S.SIGNATURES) == names
    S.sublib()


def test_create_rejects_bad_blocks_before_the_device(ohpic):
    from ohhelppic3d_gb300 import subdomain as S
    cfg = ohpic.make_config(n=(8, 8, 8), dt=0.1, b0=(0, 0, 0), qm=[-1.0], q=[-0.1], capacity=[16])
    for lo, m in (((0, 0, 0), (9, 8, 8)), ((4, 0, 0), (5, 8, 8)), ((0, 0, 0), (0, 8, 8)), ((-1, 0, 0), (4, 8, 8))):
        with pytest.raises(ohpic.OhpicError) as e:
            S.Subdomain(cfg, lo, m)
        assert e.value.status == ohpic.ERR_INVALID
    cfg32 = ohpic.make_config(n=(8, 8, 8), dt=0.1, b0=(0, 0, 0), qm=[-1.0], q=[-0.1], capacity=[16],
                              precision=ohpic.FP32)
    with pytest.raises(ohpic.OhpicError):
        S.Subdomain(cfg32, (0, 0, 0), (8, 8, 8))


def test_blocks_map_positions_and_planes():
    from ohhelppic3d_gb300 import subdomain as S
    b = S.Blocks((8, 6, 10), ([0, 3], [0], [0, 4, 7]))
    assert b.nranks == 6
    assert b.block(0) == ((0, 0, 0), (3, 6, 4))
    assert b.block(5) == ((3, 0, 7), (5, 6, 3))
    x = np.array([0.0, 2.999, 3.0, 7.99])
    z = np.array([0.5, 4.0, 6.99, 9.5])
    assert list(b.rank_of(x, np.zeros(4), z)) == [0, 2, 3, 5]
    # every node receives one count from the block interiors plus the ghost planes
    rho = np.zeros((10, 6, 8))
    for r in range(b.nranks):
        lo, m = b.block(r)
        b.add_block(rho, np.ones((m[2] + 1, m[1] + 1, m[0] + 1)), r)
    cuts = [{0, 3}, {0}, {0, 4, 7}]
    for (k, j, i), v in np.ndenumerate(rho):
        want = 1
        for d, c in zip((i, j, k), (0, 1, 2)):
            want *= 2 if d in cuts[c] else 1
        assert v == want
    e = np.random.default_rng(1).random((3, 10, 6, 8))
    blk = b.cut_e(e, 5)
    assert blk.shape == (3, 4, 7, 6)
    assert blk[1, 3, 6, 5] == e[1, 0, 0, 0]   # the upper ghost nodes are the periodic images


# ---- a decomposed run over two gloo ranks, device half stood in by numpy ----

class _NumpyBlock:
    """The device half of a rank in numpy: records, a CIC deposit into the
    block's nodes (reference weights) and a force-free move with the periodic
    wrap applied twice.  Test double only."""

    def __init__(self, blocks, r, q):
        self.blocks, self.r, self.q = blocks, r, q
        self.lo, self.m = blocks.block(r)
        self.recs = None
        self.out = None

    def append(self, recs):
        assert np.all(self.blocks.rank_of(recs["x"], recs["y"], recs["z"]) == self.r)
        self.recs = recs.copy() if self.recs is None else np.concatenate([self.recs, recs])

    def scatter(self):
        m = self.m
        rho = np.zeros((m[2] + 1, m[1] + 1, m[0] + 1))
        loc = [self.recs[k] - self.lo[d] for d, k in enumerate(("x", "y", "z"))]
        c = [np.floor(v).astype(np.int64) for v in loc]
        f = [v - ci for v, ci in zip(loc, c)]
        q = np.asarray(self.q)[self.recs["spec"] - 1]
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    w = q.copy()
                    for fd, dd in zip(f, (dx, dy, dz)):
                        w = w * (fd if dd == 0 else 1.0 - fd)
                    np.add.at(rho, (c[2] + dz, c[1] + dy, c[0] + dx), w)
        return rho

    def set_e(self, e):
        assert e.shape == (3, self.m[2] + 1, self.m[1] + 1, self.m[0] + 1)

    def move(self, dt):
        n = self.blocks.n
        for d, k in enumerate(("x", "y", "z")):
            p = self.recs[k] + self.recs["v" + k] * dt
            for _ in range(2):
                p = np.where(p < 0, n[d] + p, p)
                p = np.where(p >= n[d], p - n[d], p)
            self.recs[k] = p
        home = self.blocks.rank_of(self.recs["x"], self.recs["y"], self.recs["z"]) == self.r
        self.out = self.recs[~home]
        self.recs = self.recs[home]

    def take_emigrants(self):
        out, self.out = self.out, None
        return out


def _all_particles(seed=5, n=(8, 6, 4), count=400):
    from ohhelppic3d_gb300 import subdomain as S
    g = np.random.default_rng(seed)
    pos = [g.random(count) * n[d] for d in range(3)]
    vel = [g.uniform(-0.9, 0.9, count) for _ in range(3)]
    return S.records(*pos, *vel, np.arange(count), 1 + (np.arange(count) % 2))


def _direct_cic(recs, n, q):
    rho = np.zeros((n[2], n[1], n[0]))
    c = [np.floor(recs[k]).astype(np.int64) for k in ("x", "y", "z")]
    f = [recs[k] - ci for k, ci in zip(("x", "y", "z"), c)]
    qq = np.asarray(q)[recs["spec"] - 1]
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = qq.copy()
                for fd, dd in zip(f, (dx, dy, dz)):
                    w = w * (fd if dd == 0 else 1.0 - fd)
                np.add.at(rho, ((c[2] + dz) % n[2], (c[1] + dy) % n[1], (c[0] + dx) % n[0]), w)
    return rho


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from ohhelppic3d_gb300 import subdomain as S
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n, charges, dt = (8, 6, 4), (-0.5, 0.25), 0.5
    blocks = S.Blocks(n, ([0, 5], [0], [0]))
    me = _NumpyBlock(blocks, rank, charges)
    allp = _all_particles(n=n)
    me.append(allp[blocks.rank_of(allp["x"], allp["y"], allp["z"]) == rank])
    rhos, moved = [], 0

    def solve(rho):
        rhos.append(rho.copy())
        return np.zeros((3,) + rho.shape)

    for _ in range(6):
        left = S.mainstep({rank: me}, blocks, S.TorchComm(dist), solve, dt)
        moved += left[rank]
    mine = me.recs
    gathered = [None] * world
    dist.all_gather_object(gathered, mine.tobytes())
    dist.destroy_process_group()
    q.put((rank, moved, [r.tolist() for r in rhos], gathered))


def test_decomposed_mainstep_over_gloo():
    import torch.multiprocessing as mp

    from ohhelppic3d_gb300 import subdomain as S
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    n, charges, dt = (8, 6, 4), (-0.5, 0.25), 0.5
    blocks = S.Blocks(n, ([0, 5], [0], [0]))
    ref = _all_particles(n=n)
    assert out[0][1] + out[1][1] > 0   # particles crossed between the ranks
    for step in range(6):
        # the charge both ranks solve for is the direct deposit of every particle
        want = _direct_cic(ref, n, charges)
        for rank in (0, 1):
            np.testing.assert_allclose(np.array(out[rank][2][step]), want, rtol=0, atol=1e-12)
        for d, k in enumerate(("x", "y", "z")):
            p = ref[k] + ref["v" + k] * dt
            for _ in range(2):
                p = np.where(p < 0, n[d] + p, p)
                p = np.where(p >= n[d], p - n[d], p)
            ref[k] = p
    final = [np.frombuffer(b, dtype=S.PARTICLE) for b in out[0][3]]
    for rank, recs in enumerate(final):
        assert np.all(blocks.rank_of(recs["x"], recs["y"], recs["z"]) == rank)
    allp = np.concatenate(final)
    allp = allp[np.argsort(allp["pid"])]
    assert np.array_equal(allp["pid"], ref["pid"])
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.array_equal(allp[k], ref[k])
