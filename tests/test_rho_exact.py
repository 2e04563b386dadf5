"""FP32 form: rho from the fixed-point weight sums, rounded once and exactly.

rho(node) = sum_s q_s * W_s * 2^-24, where W_s is a species' integer weight sum
(units of 2^-24).  The kernels (k_wsum_to_rho, k_pool_rho in fields.cu) write
each charge as an integer mantissa times a power of two, form the sum exactly in
128-bit integer arithmetic, and round it once to FP32 (nearest, ties to even).
Charges whose exponents lie more than 12 apart, and sums outside the normal FP32
range, take the FP64 expression instead.

The CPU tests check a Python restatement of that integer algorithm against
exact rational arithmetic; the GPU test checks the kernels on nodes whose weight
sums are known exactly (particles placed on grid nodes).
"""
import struct
from fractions import Fraction

import numpy as np
import pytest

MAX_SHIFT = 12


def _decompose(q: float):
    """q * 2^-24 as (m, k) with m * 2^k exact; None for subnormal, inf or nan."""
    b = struct.unpack("<Q", struct.pack("<d", q))[0]
    e = (b >> 52) & 0x7FF
    mant = b & ((1 << 52) - 1)
    if e == 0:
        return (0, 0) if mant == 0 else None
    if e == 0x7FF:
        return None
    m = mant | (1 << 52)
    return (-m if b >> 63 else m), e - 1075 - 24


def _to_float_rne(acc: int, K: int):
    """acc * 2^K rounded to FP32 (nearest, ties to even); None outside the normal range."""
    if acc == 0:
        return np.float32(0.0)
    neg = acc < 0
    a = -acc if neg else acc
    msb = a.bit_length() - 1
    if msb <= 23:
        mant = a << (23 - msb)
    else:
        sh = msb - 23
        mant = a >> sh
        rem = a & ((1 << sh) - 1)
        half = 1 << (sh - 1)
        if rem > half or (rem == half and mant & 1):
            mant += 1
            if mant == 1 << 24:
                mant >>= 1
                msb += 1
    be = msb + K + 127
    if be < 1 or be > 254:
        return None
    bits = (0x80000000 if neg else 0) | (be << 23) | (mant & 0x7FFFFF)
    return np.frombuffer(struct.pack("<I", bits), dtype=np.float32)[0]


def exact_rho_model(W, q):
    """The kernels' integer path; None where they fall back to FP64."""
    parts = [_decompose(x) for x in q]
    if any(p is None for p in parts):
        return None
    ks = [k for (m, k) in parts if m != 0]
    if not ks:
        return np.float32(0.0)
    K = min(ks)
    if max(ks) - K > MAX_SHIFT:
        return None
    acc = sum(m * w << (k - K) for (m, k), w in zip(parts, W) if m != 0)
    return _to_float_rne(acc, K)


def _nearest_f32(x: Fraction) -> np.float32:
    """Correctly rounded FP32 of an exact rational (nearest, ties to even)."""
    f = np.float32(float(x))
    best = None
    for c in (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))):
        d = abs(Fraction(float(c)) - x)
        mant_even = (struct.unpack("<I", struct.pack("<f", c))[0] & 1) == 0
        key = (d, not mant_even)
        if best is None or key < best[0]:
            best = (key, c)
    return best[1]


def _exact(W, q) -> Fraction:
    return sum(Fraction(x) * w for x, w in zip(q, W)) / (1 << 24)


def test_model_rounds_exactly_on_random_sums():
    rng = np.random.default_rng(7)
    n = 0
    for _ in range(4000):
        nsp = int(rng.integers(1, 5))
        scale = float(rng.choice([1e-3, 0.03125, 1.0, 7.0]))
        q = [float(rng.uniform(-1, 1) * scale * 2.0 ** int(rng.integers(-6, 7))) for _ in range(nsp)]
        W = [int(rng.integers(0, 1 << int(rng.integers(1, 50)))) for _ in range(nsp)]
        got = exact_rho_model(W, q)
        if got is None:
            continue
        n += 1
        want = _nearest_f32(_exact(W, q))
        assert got.tobytes() == want.tobytes(), (W, q, got, want)
    assert n > 3000


def test_model_on_cancelling_charges_and_ties():
    # a quasi-neutral node: the species terms nearly cancel
    q = [-1.0 / 32, 1.0 / 32]
    for we, wi in ((5 << 24, (5 << 24) + 1), (123456789, 123456788), (1 << 40, (1 << 40) - 3)):
        got = exact_rho_model([we, wi], q)
        assert got.tobytes() == _nearest_f32(_exact([we, wi], q)).tobytes()
    # an exact tie between two FP32 values rounds to the even mantissa
    q = [1.0]
    w = ((1 << 24) + 1) << 24          # (2^24 + 1) * 2^24 units = 2^24 + 1, halfway between FP32 values
    assert exact_rho_model([w], q) == np.float32(16777216.0)
    w = ((1 << 24) + 3) << 24          # 2^24 + 3 rounds up to 2^24 + 4
    assert exact_rho_model([w], q) == np.float32(16777220.0)


def test_model_falls_back_when_exponents_are_far_apart():
    assert exact_rho_model([1, 1], [1.0, 2.0 ** -20]) is None
    assert exact_rho_model([1, 1], [1.0, 2.0 ** -12]) is not None
    assert exact_rho_model([5, 7], [0.0, 0.0]) == np.float32(0.0)
    assert exact_rho_model([3], [5e-324]) is None      # subnormal charge


@pytest.mark.gpu
@pytest.mark.parametrize("weights", [0, 1])
def test_rho_on_nodes_is_exactly_rounded(ohpic, weights):
    """Particles placed on grid nodes put whole units (2^24) on one node each, so
    every node's weight sums are known exactly: rho must be the correctly rounded
    FP32 of sum_s q_s n_s(node)."""
    P = ohpic
    n = (8, 8, 8)
    q = [-1.0 / 3.0, 0.7, 0.1]
    rng = np.random.default_rng(5)
    counts = [rng.integers(0, 5, size=n[::-1]) for _ in q]   # particles per cell, [z][y][x]
    caps = [int(c.sum()) + 64 for c in counts]
    cfg = P.make_config(n=n, dt=0.1, b0=(0.0, 0.0, 0.0), qm=[-1.0, 0.01, 0.02], q=q, capacity=caps,
                        precision=P.FP32, sort_every=0, weights=weights)
    with P.PicContext(cfg) as ctx:
        for s, c in enumerate(counts):
            zz, yy, xx = np.nonzero(c)
            reps = c[zz, yy, xx]
            x = np.repeat(xx, reps).astype(np.float64)
            y = np.repeat(yy, reps).astype(np.float64)
            z = np.repeat(zz, reps).astype(np.float64)
            zero = np.zeros_like(x)
            ctx.upload(s, {"x": x, "y": y, "z": z, "vx": zero, "vy": zero, "vz": zero})
        ctx.scatter()
        rho = ctx.field(P.RHO)
    # where each on-node particle's unit weight lands: its own node, or (the
    # reference's swapped weights, offset 0 -> weight 1 on the upper node) the
    # node +1 along every axis
    shift = 0 if weights == P.WEIGHTS_STANDARD else 1
    node_counts = [np.roll(c, (shift, shift, shift), axis=(0, 1, 2)) for c in counts]
    want = np.empty(n[::-1], dtype=np.float32)
    for idx in np.ndindex(*n[::-1]):
        want[idx] = _nearest_f32(sum(Fraction(qs) * int(nc[idx]) for qs, nc in zip(q, node_counts)))
    got = np.asarray(rho, dtype=np.float32).reshape(n[::-1])
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
