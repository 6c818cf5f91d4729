"""Seeded synthetic bodies for the mesh-voxelizer workloads.

The reference voxelizes vehicle meshes (examples/*.glb, *.stl) that are not in
its checkout; these generators stand in for them with a closed, jittered
superellipsoid triangle mesh:

    |x/a|^p + |y/b|^p + |z/c|^q = 1

tessellated from a latitude/longitude grid (each grid direction scaled onto
the surface), every vertex jittered by N(0, sigma^2) cells per axis
(numpy PCG64 with a fixed seed), stored as float32 in lattice units.
"""
from __future__ import annotations

import numpy as np


def _radius(d, a, b, c, p, q):
    """s > 0 with |s dx/a|^p + |s dy/b|^p + |s dz/c|^q = 1 (bisection)."""
    lo = np.zeros(d.shape[0])
    hi = np.full(d.shape[0], 4.0 * max(a, b, c))
    for _ in range(80):
        s = 0.5 * (lo + hi)
        f = np.abs(s * d[:, 0] / a) ** p + np.abs(s * d[:, 1] / b) ** p + np.abs(s * d[:, 2] / c) ** q
        out = f > 1.0
        hi = np.where(out, s, hi)
        lo = np.where(out, lo, s)
    return 0.5 * (lo + hi)


def superelipsoide(a=48.0, b=20.0, c=14.0, p=2.5, q=3.0, n_tri=20000, jitter=0.3, seed=2026):
    """Closed triangle mesh centred at the origin: (positions float32 [V,3],
    indices uint32 [T,3]) with about n_tri triangles."""
    # triangles = 2 * S * R for R latitude rings and S = 2R segments
    R = max(3, int(round(np.sqrt(n_tri / 4.0))))
    S = 2 * R
    rng = np.random.Generator(np.random.PCG64(seed))
    theta = np.pi * (np.arange(1, R + 1) / (R + 1))             # latitudes, poles excluded
    theta = theta + rng.uniform(-0.2, 0.2, R) * (np.pi / (R + 1))
    phi0 = 2 * np.pi * np.arange(S) / S
    dirs = []
    for t in theta:
        ph = phi0 + rng.uniform(-0.2, 0.2, S) * (2 * np.pi / S)
        dirs.append(np.stack([np.sin(t) * np.cos(ph), np.sin(t) * np.sin(ph), np.full(S, np.cos(t))], 1))
    dirs = np.concatenate([np.array([[0, 0, 1.0]]), np.concatenate(dirs), np.array([[0, 0, -1.0]])])
    # the body's long axis is x: rotate z-pole grid so poles sit on +-x
    dirs = dirs[:, [2, 1, 0]] * np.array([1.0, 1.0, -1.0])
    pos = dirs * _radius(dirs, a, b, c, p, q)[:, None]
    pos = pos + rng.normal(0.0, jitter, pos.shape)
    top, bot = 0, 1 + R * S
    tris = []
    ring = lambda r, s: 1 + r * S + (s % S)
    for s in range(S):
        tris.append((top, ring(0, s), ring(0, s + 1)))
    for r in range(R - 1):
        for s in range(S):
            a0, a1, b0, b1 = ring(r, s), ring(r, s + 1), ring(r + 1, s), ring(r + 1, s + 1)
            tris.append((a0, b0, a1))
            tris.append((a1, b0, b1))
    for s in range(S):
        tris.append((bot, ring(R - 1, s + 1), ring(R - 1, s)))
    return pos.astype(np.float32), np.asarray(tris, dtype=np.uint32)


def colocar(pos, grade, nariz=0.28, folga_piso=2.0):
    """Lattice placement: nose (min x) at nariz * nx, centred in y, lowest
    vertex folga_piso cells above the top of the floor row (z = 1)."""
    p = pos.astype(np.float64).copy()
    p[:, 0] += nariz * grade["nx"] - p[:, 0].min()
    p[:, 1] += 0.5 * grade["ny"] - 0.5 * (p[:, 1].min() + p[:, 1].max())
    p[:, 2] += 1.0 + folga_piso - p[:, 2].min()
    return p.astype(np.float32)


def corpo_config2(grade=None, seed=2026):
    """Mesh of the 320x160x128 mesh-body workload: semi-axes 48x20x14 cells,
    exponents 2.5/2.5/3, ~20k triangles, 0.3-cell jitter."""
    grade = grade or {"nx": 320, "ny": 160, "nz": 128}
    pos, idx = superelipsoide(48.0, 20.0, 14.0, 2.5, 3.0, 20000, 0.3, seed)
    return colocar(pos, grade), idx


def corpo_config3(grade=None, seed=2027):
    """512x256x192 precision workload: semi-axes 80x32x22."""
    grade = grade or {"nx": 512, "ny": 256, "nz": 192}
    pos, idx = superelipsoide(80.0, 32.0, 22.0, 2.5, 3.0, 20000, 0.3, seed)
    return colocar(pos, grade), idx


def mascara_analitica(grade, a, b, c, p, q, centro):
    """Voxel-centre inside test of the same superellipsoid (no mesh); used only
    where a mesh is not needed."""
    nx, ny, nz = grade["nx"], grade["ny"], grade["nz"]
    z, y, x = np.meshgrid(np.arange(nz) + 0.5, np.arange(ny) + 0.5, np.arange(nx) + 0.5, indexing="ij")
    f = (np.abs((x - centro[0]) / a) ** p + np.abs((y - centro[1]) / b) ** p + np.abs((z - centro[2]) / c) ** q)
    return np.where(f <= 1.0, 2, 0).astype(np.uint8).reshape(-1)
