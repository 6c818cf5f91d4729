"""Physical <-> lattice units (host).  Restates src/core/units.js:52-261."""
from __future__ import annotations

import math

from .lattice import CS2, nu_from_omega, omega_from_nu

AR = {"rho": 1.204, "mu": 1.813e-5, "nu": 1.506e-5, "c": 343.2}
OMEGA_MAX = 1.90
OMEGA_MAX_PISO_PARADO = 1.90
NU_MIN = nu_from_omega(OMEGA_MAX)
U_LB_PADRAO = 0.05
U_LB_MAX = 0.1


class Units:
    """Scales fixed by body length in cells, lattice speed and the viscosity
    ceiling omega_max = 1.90 (src/core/units.js:110-171)."""

    def __init__(self, lengthM, speedMs, cellsPerLength, uLb=U_LB_PADRAO, rollingRoad=True,
                 fluid=None, lesCs=0.1):
        if not (lengthM > 0):
            raise ValueError("lengthM deve ser positivo")
        if not (speedMs > 0):
            raise ValueError("speedMs deve ser positivo")
        if not (cellsPerLength >= 8):
            raise ValueError(f"cellsPerLength = {cellsPerLength}: abaixo de ~8 células o corpo não tem forma")
        if not (0 < uLb <= U_LB_MAX):
            raise ValueError(f"uLb = {uLb} fora de (0, {U_LB_MAX}]")
        self.fluid = dict(fluid or AR)
        self.lengthM = lengthM
        self.speedMs = speedMs
        self.cellsPerLength = int(math.floor(cellsPerLength + 0.5))
        self.uLb = uLb
        self.rollingRoad = bool(rollingRoad)
        self.lesCs = lesCs
        self.dx = lengthM / self.cellsPerLength
        self.dt = uLb * self.dx / speedMs
        self.rePhysical = speedMs * lengthM / self.fluid["nu"]
        self.nuLbExact = uLb * self.cellsPerLength / self.rePhysical
        self.omegaMax = OMEGA_MAX if self.rollingRoad else OMEGA_MAX_PISO_PARADO
        self.nuLbMin = nu_from_omega(self.omegaMax)
        self.nuLb = max(self.nuLbExact, self.nuLbMin)
        self.omegaPlus = omega_from_nu(self.nuLb)
        self.reLattice = uLb * self.cellsPerLength / self.nuLb
        self.machLattice = uLb / math.sqrt(CS2)
        self.machPhysical = speedMs / self.fluid["c"]

    @property
    def resolved(self):
        return self.nuLbExact >= self.nuLbMin

    @property
    def reRatio(self):
        return self.rePhysical / self.reLattice

    def velToLb(self, v):
        return v * self.uLb / self.speedMs

    def velToSi(self, v):
        return v * self.speedMs / self.uLb

    def forceToSi(self, f):
        return f * self.fluid["rho"] * self.dx ** 4 / self.dt ** 2

    def pressureToSi(self, delta):
        return CS2 * delta * self.fluid["rho"] * (self.dx / self.dt) ** 2

    @property
    def dynamicPressure(self):
        return 0.5 * self.fluid["rho"] * self.speedMs ** 2


class LatticeUnits:
    """Minimal units object for runs specified directly in lattice units
    (the validation cases override Units the same way, tests/validacao.html:210-216)."""

    def __init__(self, uLb):
        self.uLb = uLb


def stepsForFlowthrough(units, n=1):
    return math.ceil(n * units.cellsPerLength / units.uLb)
