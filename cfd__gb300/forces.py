"""From lattice force to published coefficients (host, fp64).

Restates src/core/forces.js: ``maskell`` (:39-43), ``coeficientes`` (:55-95),
``JanelaCd`` (:106-137) and ``strouhal`` (:151-177).
"""
from __future__ import annotations

import math


def _finite(v) -> bool:
    return isinstance(v, (int, float)) and math.isfinite(v)


def maskell(cdMedido, bloqueio, theta=2.5):
    """Maskell blockage correction; Cd <= 0 or non-finite passes through."""
    if not (bloqueio > 0) or not _finite(cdMedido):
        return cdMedido
    if cdMedido <= 0:
        return cdMedido
    return cdMedido / (1 + theta * cdMedido * bloqueio)


def coeficientes(forcaLb, units, areaFrontalCelulas, grade, corrigirBloqueio=True, theta=2.5):
    fx, fy, fz = forcaLb
    q = 0.5 * units.uLb * units.uLb
    denom = max(q * areaFrontalCelulas, 1e-30)
    cdBruto = fx / denom
    bloqueio = areaFrontalCelulas / (grade["ny"] * grade["nz"])
    cd = maskell(cdBruto, bloqueio, theta) if corrigirBloqueio else cdBruto
    out = {
        "cd": cd, "cdBruto": cdBruto, "cl": fz / denom, "cs": fy / denom,
        "bloqueio": bloqueio, "theta": theta, "corrigido": bool(corrigirBloqueio and cdBruto > 0),
    }
    if hasattr(units, "forceToSi"):
        out["forcaN"] = [units.forceToSi(fx), units.forceToSi(fy), units.forceToSi(fz)]
        out["areaFrontalM2"] = areaFrontalCelulas * units.dx * units.dx
        out["arrastoN"] = cd * units.dynamicPressure * areaFrontalCelulas * units.dx * units.dx
    return out


class JanelaCd:
    """Sliding window of coefficients: mean and sample std (n - 1)."""

    def __init__(self, capacidade=600):
        self.capacidade = capacidade
        self.buf = []
        self.i = 0

    def adicionar(self, v):
        if not _finite(v):
            return
        if len(self.buf) < self.capacidade:
            self.buf.append(v)
        else:
            self.buf[self.i] = v
            self.i = (self.i + 1) % self.capacidade

    def limpar(self):
        self.buf = []
        self.i = 0

    @property
    def n(self):
        return len(self.buf)

    @property
    def media(self):
        if not self.buf:
            return math.nan
        s = 0.0
        for b in self.buf:
            s += b
        return s / len(self.buf)

    @property
    def desvio(self):
        n = len(self.buf)
        if n < 2:
            return math.nan
        m = self.media
        s = 0.0
        for b in self.buf:
            s += (b - m) ** 2
        return math.sqrt(s / (n - 1))

    @property
    def madura(self):
        return len(self.buf) >= self.capacidade


def strouhal(serie, passosPorAmostra, dCelulas, uLb):
    """St from thresholded zero crossings of the oscillating part."""
    n = len(serie)
    if n < 32:
        return {"st": math.nan, "motivo": "série curta demais"}
    m = 0.0
    for v in serie:
        m += v
    m /= n
    osc = [v - m for v in serie]
    s2 = 0.0
    for b in osc:
        s2 += b * b
    amp = math.sqrt(s2 / n)
    if amp < 1e-6:
        return {"st": 0, "motivo": "sem oscilação: esteira estacionária"}
    limiar = 0.25 * amp
    cruz, ultimo = 0, 0
    for v in osc:
        s = 1 if v > limiar else (-1 if v < -limiar else 0)
        if s != 0 and ultimo != 0 and s != ultimo:
            cruz += 1
        if s != 0:
            ultimo = s
    if cruz < 4:
        return {"st": math.nan, "motivo": f"só {cruz} cruzamentos; simule mais"}
    periodos = cruz / 2
    freq = periodos / (n * passosPorAmostra)
    return {"st": freq * dCelulas / uLb, "periodos": periodos, "freqLb": freq, "amplitude": amp}
