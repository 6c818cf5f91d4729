"""Seeded meshes for the voxelizer parity tests."""
import json
import os

import numpy as np

from cfd__gb300.geometry import colocar, corpo_config2, superelipsoide

GOLD = os.path.join(os.path.dirname(__file__), "golden", "cube_example.json")


def cube_example(scale=24.0, grade=None):
    """The reference's example cube (tests/golden/cube_example.json) scaled to
    `scale` cells and placed as the tunnel places a body."""
    d = json.load(open(GOLD))
    p = np.array(d["positions"], np.float64) * scale
    grade = grade or {"nx": 240, "ny": 120, "nz": 96}
    return colocar(p.astype(np.float32), grade), np.array(d["indices"], np.uint32), grade


def aligned_cube(grade, lo=(10, 8, 6), size=16):
    """Cube with faces exactly on voxel faces: every shell decision is a tie
    for the fp32 filter and goes to the fp64 path."""
    d = json.load(open(GOLD))
    p = np.array(d["positions"], np.float64) * size + np.array(lo, np.float64)
    return p.astype(np.float32), np.array(d["indices"], np.uint32), grade


def sphere_mesh(grade, r=10.0, center=None, n_tri=3000, seed=5, jitter=0.0, hole=None):
    """Sphere mesh; hole=(ring, rings, segment, segments) removes that patch
    of the latitude/longitude grid (1 x 2 quads leak a flood unless sealed)."""
    pos, idx = superelipsoide(r, r, r, 2.0, 2.0, n_tri, jitter, seed)
    c = center or (grade["nx"] / 2, grade["ny"] / 2, grade["nz"] / 2)
    pos = pos + np.array(c, np.float32)
    if hole:
        R = max(3, int(round(np.sqrt(n_tri / 4.0))))
        S = 2 * R
        ring = lambda a, b: 1 + a * S + (b % S)
        r0, h, s0, w = hole
        bad = set()
        for a in range(r0, r0 + h):
            for b in range(s0, s0 + w):
                bad.add((ring(a, b), ring(a + 1, b), ring(a, b + 1)))
                bad.add((ring(a, b + 1), ring(a + 1, b), ring(a + 1, b + 1)))
        idx = np.array([t for t in idx.tolist() if tuple(t) not in bad], np.uint32)
    return pos.astype(np.float32), idx, grade


def soup(grade, n=2000, seed=9):
    """Random triangles of 0.05 to 8 cells, slivers, a few non-finite and a
    few outside the grid."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = grade["nx"], grade["ny"], grade["nz"]
    c = rng.uniform(-2, [nx + 2, ny + 2, nz + 2], (n, 3))
    size = np.exp(rng.uniform(np.log(0.05), np.log(8.0), (n, 1)))
    v = c[:, None, :] + rng.normal(0, 1, (n, 3, 3)) * size[:, :, None]
    sl = rng.random(n) < 0.1                      # slivers: third vertex on the first edge
    t = rng.random(n)[:, None]
    v[sl, 2] = v[sl, 0] + t[sl] * (v[sl, 1] - v[sl, 0])
    v[rng.random(n) < 0.01, 1, 0] = np.inf
    v[rng.random(n) < 0.01, 2, 1] = np.nan
    v[rng.random(n) < 0.02] += 1e4                # far outside
    pos = v.reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    return pos, idx, grade


def plate(grade):
    """An open, zero-thickness quad (a wing): a one-voxel wall."""
    nx, ny, nz = grade["nx"], grade["ny"], grade["nz"]
    p = np.array([[nx * 0.3, ny * 0.2, nz * 0.4], [nx * 0.7, ny * 0.25, nz * 0.45],
                  [nx * 0.7, ny * 0.8, nz * 0.6], [nx * 0.3, ny * 0.75, nz * 0.55]], np.float32)
    return p, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), grade


def config2():
    g = {"nx": 320, "ny": 160, "nz": 128}
    p, i = corpo_config2(g)
    return p, i, g
