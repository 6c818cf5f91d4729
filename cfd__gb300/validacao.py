"""Validation correlations and cases (host).  Restates src/core/validacao.js."""
from __future__ import annotations

import math


def esferaCd(re):
    """Clift-Gauvin sphere drag (src/core/validacao.js:26-31)."""
    if not (re > 0):
        return math.inf
    if re < 0.1:
        return 24 / re
    return (24 / re) * (1 + 0.15 * re ** 0.687) + 0.42 / (1 + 4.25e4 * re ** -1.16)


def cilindroCd(re):
    """Cylinder drag (src/core/validacao.js:40-45)."""
    if not (re > 0):
        return math.inf
    if re < 1:
        return 8 * math.pi / (re * (2.002 - math.log(re)))
    if re < 2e5:
        return 1.0 + 10 * re ** (-2 / 3)
    return 0.35


def cilindroStrouhal(re):
    """src/core/validacao.js:56-61."""
    if re < 47:
        return 0
    if re < 300:
        return 0.2684 - 1.0356 / math.sqrt(re)
    if re < 2e5:
        return 0.198 * (1 - 19.7 / re)
    return 0.21


def poiseuille(y, H):
    s = 2 * y / H - 1
    return max(0.0, 1 - s * s)


def classificar(medido, referencia):
    """src/core/validacao.js:86-101."""
    if not (math.isfinite(medido) and math.isfinite(referencia)) or referencia == 0:
        return {"erro": math.nan, "pct": math.nan, "nivel": "indefinido", "ok": False}
    erro = (medido - referencia) / referencia
    a = abs(erro) * 100
    if a <= 5:
        return {"erro": erro, "pct": a, "nivel": "excelente", "ok": True}
    if a <= 15:
        return {"erro": erro, "pct": a, "nivel": "aceitável", "ok": True}
    if a <= 30:
        return {"erro": erro, "pct": a, "nivel": "qualitativo", "ok": False}
    return {"erro": erro, "pct": a, "nivel": "discordante", "ok": False}


def uLbParaOmega(re, dCelulas, omegaAlvo=1.90, uLbMax=0.1):
    """src/core/validacao.js:126-129."""
    nu = (1 / 3) * (1 / omegaAlvo - 0.5)
    return min(nu * re / dCelulas, uLbMax)


CASOS = [
    {"id": "esfera-re50", "nome": "Esfera, Re = 50", "forma": "esfera", "re": 50, "diametroCelulas": 24,
     "grade": {"nx": 240, "ny": 120, "nz": 96}, "referencia": lambda: esferaCd(50),
     "travessiasTransiente": 2.0, "travessiasMedida": 1.0},
    {"id": "esfera-re100", "nome": "Esfera, Re = 100", "forma": "esfera", "re": 100, "diametroCelulas": 24,
     "grade": {"nx": 240, "ny": 120, "nz": 96}, "referencia": lambda: esferaCd(100),
     "travessiasTransiente": 2.0, "travessiasMedida": 1.5},
    {"id": "cilindro-re100", "nome": "Cilindro, Re = 100", "forma": "cilindro", "re": 100, "diametroCelulas": 16,
     "grade": {"nx": 480, "ny": 8, "nz": 320}, "referencia": lambda: cilindroCd(100),
     "referenciaSt": lambda: cilindroStrouhal(100),
     "perturbacao": {"grausGuinada": 2.0, "passos": 600},
     "travessiasTransiente": 2.5, "travessiasMedida": 4.0},
    {"id": "esfera-re200", "nome": "Esfera, Re = 200", "forma": "esfera", "re": 200, "diametroCelulas": 40,
     "grade": {"nx": 480, "ny": 240, "nz": 192}, "referencia": lambda: esferaCd(200),
     "travessiasTransiente": 2.0, "travessiasMedida": 1.5, "profundo": True},
]

# Published results of the reference's WebGPU run (README.md:100-105).
PUBLICADOS = {
    "esfera-re50": {"cd": 1.480},
    "esfera-re100": {"cd": 1.070},
    "cilindro-re100": {"cd": 1.285, "st": 0.1663},
}
