"""Shared case builders for the parity tests (seeded, small enough for the
CPU oracle)."""
import math

import numpy as np

from cfd__gb300 import lattice as L
from cfd__gb300.tunel import corpoAnalitico, montarTipos


def js_round(v):
    return int(math.floor(v + 0.5))


def default_sponge(nx):
    return {"inicio": js_round(nx * 0.82), "comprimento": max(4, js_round(nx * 0.18))}


def sphere_tunnel(nx, ny, nz, r, cx=None, esteira=False, floor_mirror=True):
    """Sphere in a tunnel the way tests/validacao.html:219-231 builds it."""
    grade = {"nx": nx, "ny": ny, "nz": nz}
    corpo = corpoAnalitico(grade, {"tipo": "esfera", "cx": cx if cx is not None else nx * 0.30,
                                   "cy": ny * 0.5, "cz": nz * 0.5, "raio": r})
    mt = montarTipos(grade, corpo=corpo, esteira=esteira)
    tipo = mt["tipo"]
    if floor_mirror:
        t = tipo.reshape(nz, ny, nx)
        t[0, :, 1:nx - 1] = 6
    return grade, corpo, tipo, mt["esponja"]


def random_state(N, seed, amp=1e-3, u=(0.04, 0.0, 0.0)):
    """A perturbed equilibrium state, 19 x N fp64."""
    rng = np.random.default_rng(seed)
    delta = rng.normal(0.0, amp, N)
    uu = np.tile(np.asarray(u, np.float64), (N, 1)) + rng.normal(0.0, amp * 5, (N, 3))
    g = L.equilibrium(delta, uu) + rng.normal(0.0, amp * 0.1, (N, 19))
    return np.ascontiguousarray(g.T)


def all_types_tunnel(nx=40, ny=24, nz=20, seed=7):
    """Every cell class present: body (SOLIDO), belt floor (SOLIDO_MOVEL),
    inlet, outlet, y/z mirrors, plus a PAREDE block touching the body."""
    grade, corpo, tipo, esp = sphere_tunnel(nx, ny, nz, r=4.5, esteira=True, floor_mirror=False)
    t = tipo.reshape(nz, ny, nx)
    t[2:5, 3:6, 20:24] = 7          # a static wall block near the floor
    t[7:9, 10:14, int(nx * 0.3) + 4] = 7   # PAREDE touching the sphere's lee side
    return grade, tipo, esp
