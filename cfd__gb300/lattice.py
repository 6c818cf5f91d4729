"""D3Q19 velocity set and shifted distributions, host side (fp64).

Restates src/core/lattice.js: the tables (:48-89), the TRT magic parameters
(:111-116), the viscosity relations (:121-139), the shifted equilibrium and
moments used by the validation suite and by ``definirCampo`` (:150-174), and
the invariants checked at import (:184-231).  The hot path is the CUDA step;
this module serves the host (initial fields, unit conversion, tests).
"""
from __future__ import annotations

import numpy as np

Q = 19
CS2 = 1.0 / 3.0
INV_CS2 = 3.0
INV_CS4 = 9.0

# opposite pairs adjacent: (0), (1,2), (3,4), ...
C = np.array([
    (0, 0, 0),
    (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
    (1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0),
    (1, 0, 1), (-1, 0, -1), (1, 0, -1), (-1, 0, 1),
    (0, 1, 1), (0, -1, -1), (0, 1, -1), (0, -1, 1),
], dtype=np.int64)

W = np.array([1.0 / 3.0] + [1.0 / 18.0] * 6 + [1.0 / 36.0] * 12, dtype=np.float64)

OPP = np.array([0] + [((k) ^ 1) + 1 for k in range(Q - 1)], dtype=np.int64)

MAGIC = {"WALL": 3.0 / 16.0, "STABLE": 1.0 / 4.0, "THIRD_ORDER": 1.0 / 12.0, "FOURTH_ORDER": 1.0 / 6.0}


def omega_from_nu(nu):
    """omegaFromNu, src/core/lattice.js:121-123."""
    return 1.0 / (nu / CS2 + 0.5)


def nu_from_omega(omega):
    """nuFromOmega, src/core/lattice.js:126-128."""
    return CS2 * (1.0 / omega - 0.5)


def omega_minus_from_lambda(omega_plus, lam):
    """omegaMinusFromLambda, src/core/lattice.js:131-134."""
    return 1.0 / (lam / (1.0 / omega_plus - 0.5) + 0.5)


def lambda_from_omegas(omega_plus, omega_minus):
    return (1.0 / omega_plus - 0.5) * (1.0 / omega_minus - 0.5)


def equilibrium(delta, u, out=None):
    """Shifted equilibrium g_i^eq = w_i (delta + rho (3cu + 4.5cu^2 - 1.5uu)).

    Vectorised form of src/core/lattice.js:150-160: ``delta`` has shape (...),
    ``u`` shape (..., 3); returns (..., 19) in fp64 with the same operation
    order per element as the JS loop.
    """
    delta = np.asarray(delta, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    rho = 1.0 + delta
    uu = u[..., 0] * u[..., 0] + u[..., 1] * u[..., 1] + u[..., 2] * u[..., 2]
    g = np.empty(delta.shape + (Q,), dtype=np.float64) if out is None else out
    for i in range(Q):
        c = C[i]
        cu = c[0] * u[..., 0] + c[1] * u[..., 1] + c[2] * u[..., 2]
        g[..., i] = W[i] * (delta + rho * (3 * cu + 4.5 * cu * cu - 1.5 * uu))
    return g


def moments(g):
    """moments, src/core/lattice.js:163-174: returns (delta, u)."""
    g = np.asarray(g, dtype=np.float64)
    delta = np.zeros(g.shape[:-1])
    m = np.zeros(g.shape[:-1] + (3,))
    for i in range(Q):
        delta = delta + g[..., i]
        for a in range(3):
            m[..., a] = m[..., a] + g[..., i] * C[i][a]
    inv = 1.0 / (1.0 + delta)
    return delta, m * inv[..., None]


def espelhar_idx(i: int, eixo: int) -> int:
    """Specular reflection index (espelharIdx, src/core/emit/ir.js:86-93)."""
    c = C[i].copy()
    c[eixo] = -c[eixo]
    for j in range(Q):
        if (C[j] == c).all():
            return j
    raise ValueError(f"no mirror for {i} on axis {eixo}")


def self_check() -> bool:
    """Invariants of the velocity set (src/core/lattice.js:184-231)."""
    if not (len(C) == Q and len(W) == Q and len(OPP) == Q):
        raise AssertionError("table sizes")
    if abs(W.sum() - 1) > 1e-15:
        raise AssertionError(f"sum(w) = {W.sum()}")
    for a in range(3):
        s = sum(W[i] * C[i][a] for i in range(Q))
        if abs(s) > 1e-15:
            raise AssertionError(f"sum(w c)[{a}] = {s}")
    for a in range(3):
        for b in range(3):
            s = sum(W[i] * C[i][a] * C[i][b] for i in range(Q))
            if abs(s - (CS2 if a == b else 0.0)) > 1e-15:
                raise AssertionError(f"sum(w c c)[{a}][{b}] = {s}")
    for i in range(Q):
        if OPP[OPP[i]] != i or (C[OPP[i]] != -C[i]).any() or W[OPP[i]] != W[i]:
            raise AssertionError(f"opposite of {i}")
    g0 = equilibrium(0.0, [0.0, 0.0, 0.0])
    if (g0 != 0).any():
        raise AssertionError("rest equilibrium is not zero")
    d, u = 1e-4, [0.05, -0.02, 0.01]
    dm, um = moments(equilibrium(d, u))
    if abs(dm - d) > 1e-15 or np.abs(um - u).max() > 1e-15:
        raise AssertionError("moment round trip")
    return True


self_check()
