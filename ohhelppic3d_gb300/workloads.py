"""The synthetic plasmas the path is measured and tested on.

All are periodic boxes with dx = 1 and Debye length 1 for the electrons.  Charge
per macro-particle follows parameters.f90:147-148 (wp^2 / qm / ppc) unless a
neutralising charge is set explicitly.
"""
from __future__ import annotations

from dataclasses import dataclass, field


@dataclass
class Species:
    name: str
    qm: float
    q: float
    ppc: float
    vth: float
    drift: tuple = (0.0, 0.0, 0.0)
    lo: tuple = (0.0, 0.0, 0.0)
    hi: tuple | None = None      # None: the whole box

    def count(self, n) -> int:
        hi = self.hi if self.hi is not None else tuple(float(v) for v in n)
        vol = 1.0
        for d in range(3):
            vol *= max(min(hi[d], n[d]) - max(self.lo[d], 0.0), 0.0)
        return int(self.ppc * vol)


@dataclass
class Workload:
    name: str
    n: tuple
    dt: float
    b0: tuple
    steps: int
    sort_every: int
    species: list = field(default_factory=list)
    description: str = ""

    @property
    def ncell(self) -> int:
        return self.n[0] * self.n[1] * self.n[2]

    def counts(self) -> list:
        return [s.count(self.n) for s in self.species]

    @property
    def nparticles(self) -> int:
        return sum(self.counts())


def _thermal_pair(ppc: int, wce: float = 0.5) -> list:
    # electrons: qm = -1, wp = 1; ions: qm = +0.01 (mass ratio 100), wp = 0.1
    return [Species("electron", -1.0, 1.0 * 1.0 / -1.0 / ppc, ppc, 1.0),
            Species("ion", 0.01, 0.1 * 0.1 / 0.01 / ppc, ppc, 0.1)]


def c1() -> Workload:
    return Workload("C1", (32, 32, 32), 0.1, (0.0, 0.0, 0.5), 100, 20, _thermal_pair(16),
                    "32^3 periodic, 2 species x 16 ppc (1,048,576 particles), vth_e=1, vth_i=0.1, "
                    "mass ratio 100, B0z=0.5 (wce/wpe=0.5), dt=0.1, 100 steps")


def c2() -> Workload:
    return Workload("C2", (256, 256, 256), 0.1, (0.0, 0.0, 0.5), 100, 20, _thermal_pair(32),
                    "256^3 periodic, 2 species x 32 ppc (1,073,741,824 particles), vth_e=1, vth_i=0.1, "
                    "mass ratio 100, B0z=0.5, dt=0.1, cell sort every 20 steps")


def c4() -> Workload:
    n = (128, 128, 512)
    lo, hi = (0.35 * n[0], 0.35 * n[1], 0.0), (0.65 * n[0], 0.65 * n[1], float(n[2]))
    bg = Species("electron", -1.0, -1.0 / 16, 16, 1.0)
    beam = Species("beam", -1.0, -1.0 / 16, 16, 0.5, drift=(0.0, 0.0, 5.0), lo=lo, hi=hi)
    ion = Species("ion", 0.01, 0.0, 32, 0.1)
    ne = bg.count(n) + beam.count(n)
    ion.q = ne / 16.0 / ion.count(n)        # neutral in total
    return Workload("C4", n, 0.1, (0.0, 0.0, 0.0), 500, 20, [bg, beam, ion],
                    "128x128x512 clustered two-stream: background e- 16 ppc vth 1, beam e- 16 ppc "
                    "drift +5 z vth 0.5 in the central 30% of x,y, ions 32 ppc vth 0.1, B=0, dt=0.1")


WORKLOADS = {"c1": c1, "c2": c2, "c4": c4}
