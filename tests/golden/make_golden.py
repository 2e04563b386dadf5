"""Regenerates the golden fixtures in tests/golden/.

Run from the repository root where the reference checkout is available:

    python tests/golden/make_golden.py /path/to/reference

1. pcg32_reference.json -- output of the reference's own pcg-c known-answer
   program (lib/pcg-c/test-high/check-pcg32.c) and raw draws of the reference's
   RNG binding (pcg_setseq_64_srandom_r / pcg32_random_double_r /
   pcg_setseq_64_advance_r, bound at src/radom/pcg/pcg64.f90:10-32), both built
   from the reference tree by `make -C oracle ref`.  The script checks the
   known-answer output against lib/pcg-c/test-high/expected/check-pcg32.out
   before writing anything.
2. oracle_small_run.npz -- a frozen run of the oracle (8x8x8 cells, two
   species, 10 steps) used as a regression fixture for the oracle itself.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402


class _PcgState(C.Structure):
    _fields_ = [("state", C.c_uint64), ("inc", C.c_uint64)]


def reference_pcg(ref_root: str) -> dict:
    if not O.build_ref(ref_root):
        raise SystemExit(f"no pcg-c under {ref_root}")
    kat = subprocess.run([os.path.join(O.REF_DIR, "check-pcg32")], capture_output=True, text=True,
                         check=True).stdout
    expected_path = os.path.join(ref_root, "lib", "pcg-c", "test-high", "expected", "check-pcg32.out")
    with open(expected_path) as f:
        expected = f.read()
    if kat != expected:
        raise SystemExit("check-pcg32 built from the reference does not match its expected output")

    L = C.CDLL(os.path.join(O.REF_DIR, "libpcg_ref.so"))
    L.pcg_setseq_64_srandom_r.argtypes = [C.POINTER(_PcgState), C.c_uint64, C.c_uint64]
    L.pcg_setseq_64_advance_r.argtypes = [C.POINTER(_PcgState), C.c_uint64]
    L.pcg_setseq_64_xsh_rr_32_random_r.restype = C.c_uint32
    L.pcg_setseq_64_xsh_rr_32_random_r.argtypes = [C.POINTER(_PcgState)]
    L.pcg32_random_double_r.restype = C.c_double
    L.pcg32_random_double_r.argtypes = [C.POINTER(_PcgState)]

    def draws(seed, seq, advance, n, doubles):
        st = _PcgState()
        L.pcg_setseq_64_srandom_r(C.byref(st), seed, seq)
        if advance:
            L.pcg_setseq_64_advance_r(C.byref(st), advance % (1 << 64))
        f = L.pcg32_random_double_r if doubles else L.pcg_setseq_64_xsh_rr_32_random_r
        return [f(C.byref(st)) for _ in range(n)]

    return {
        "source": "reference lib/pcg-c compiled by oracle/Makefile (target ref)",
        "check_pcg32_out": kat,
        # The driver's seed (src/ohhelppic3d.f90:111) and the first ranks' jump-ahead (:112).
        "seed_42_52_doubles": [repr(v) for v in draws(42, 52, 0, 32, True)],
        "seed_42_52_u32": draws(42, 52, 0, 64, False),
        "seed_42_52_advance_1e8_u32": draws(42, 52, 100000000, 16, False),
        "seed_42_52_advance_3e8_u32": draws(42, 52, 300000000, 16, False),
        "seed_42_1000_u32": draws(42, 1000, 0, 16, False),
    }


def small_run() -> dict:
    setup = O.Setup(n=(8, 8, 8), dt=0.1, b0=(0.0, 0.0, 0.5),
                    species=[O.SpeciesInit(ppc=1, vth=1.0, qm=-1.0, wp=1.0),
                             O.SpeciesInit(ppc=1, vth=0.1, qm=0.01, wp=0.1)])
    o = O.Oracle(setup)
    o.init_particles()
    out = {}

    def snap(tag):
        o.deposit()
        o.solve()
        for s in range(2):
            p = o.get_particles(s)
            for k, v in p.items():
                out[f"{tag}_s{s}_{k}"] = v
        for name, w in (("rho", O.RHO), ("phi", O.PHI), ("ex", O.EX), ("ey", O.EY), ("ez", O.EZ)):
            out[f"{tag}_{name}"] = o.get_field(w)

    snap("step0")
    o.step(1)
    snap("step1")
    o.step(9)
    snap("step10")
    return out


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <path of the reference checkout>")
    ref_root = sys.argv[1]
    pcg = reference_pcg(ref_root)
    with open(os.path.join(HERE, "pcg32_reference.json"), "w") as f:
        json.dump(pcg, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "oracle_small_run.npz"), **small_run())
    print("wrote pcg32_reference.json and oracle_small_run.npz")


if __name__ == "__main__":
    main()
