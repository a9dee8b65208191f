"""Scheme description shared by the host API, the workloads and the tests.

A ``Scheme`` names the same choices a Mara2 driver makes when it wires a
``MethodOfLinesTVD`` together (src/Problems.cpp:153-209): the conservation
law, the intercell flux scheme (reconstruction + Riemann solver), the
boundary condition, the Runge-Kutta order, the mesh and the gamma-law
index.  ``plm_theta`` and the gamma-law index have no getters on the
reference classes (src/Reconstruction.hpp:45, src/ConservationLaws.hpp:38),
so they are carried here explicitly.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

LAWS = ("hydro", "mhd", "rmhd")
RECONS = ("pcm", "plm", "weno5")
RIEMANNS = ("hlle", "hllc")
BCS = ("periodic", "outflow", "reflecting")
WENO_IS = ("js96", "borges08", "shenzha10")
NFIELDS = {"hydro": 5, "mhd": 8, "rmhd": 8}
STENCIL = {"pcm": 1, "plm": 2, "weno5": 3}


@dataclass
class Scheme:
    law: str = "hydro"
    recon: str = "plm"
    riemann: str = "hlle"
    bc: str = "outflow"
    rk_order: int = 2
    shape: tuple = (64, 1, 1)
    lower: tuple = (0.0, 0.0, 0.0)
    upper: tuple = (1.0, 1.0, 1.0)
    gamma: float = 5.0 / 3
    plm_theta: float = 1.5
    weno_is: str = "shenzha10"
    shenzha_A: float = 50.0
    pressure_floor: float = -1.0
    disable_ct: bool = False
    cooling_rate: float = -1.0        # NewtonianMHD::setCoolingRate: > 0 adds an auxiliary field
    guard: int | None = None          # guard width; default = stencil size
    # driver parameters (not part of advance(), used by run loops)
    cfl: float = 0.4
    t_final: float | None = None
    steps: int | None = None
    extra: dict = field(default_factory=dict)

    def __post_init__(self):
        self.shape = tuple(int(n) for n in self.shape)
        if self.law not in LAWS or self.recon not in RECONS or self.riemann not in RIEMANNS \
                or self.bc not in BCS or self.weno_is not in WENO_IS:
            raise ValueError(f"unknown scheme choice in {self}")

    @property
    def aux(self) -> int:
        """Auxiliary fields (NewtonianMHD with cooling, ConservationLaws.cpp:355-358)."""
        return 1 if self.law == "mhd" and self.cooling_rate > 0.0 else 0

    @property
    def nq(self) -> int:
        return NFIELDS[self.law] + self.aux

    @property
    def stencil(self) -> int:
        return STENCIL[self.recon]

    @property
    def ng(self) -> tuple:
        g = self.stencil if self.guard is None else self.guard
        return tuple(g if n > 1 else 0 for n in self.shape)

    @property
    def full_shape(self) -> tuple:
        return tuple(self.shape[a] + 2 * self.ng[a] for a in range(3)) + (self.nq,)

    @property
    def dims(self) -> int:
        return sum(1 for n in self.shape if n > 1)

    @property
    def zones(self) -> int:
        return self.shape[0] * self.shape[1] * self.shape[2]

    def interior(self):
        g = self.ng
        return tuple(slice(g[a], g[a] + self.shape[a]) for a in range(3))

    def with_(self, **kw) -> "Scheme":
        return replace(self, **kw)
