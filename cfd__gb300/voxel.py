"""Triangle mesh -> lattice solid field, on the GPU (include/vox.h).

``voxelizar`` mirrors the reference's voxelizar (src/geom/voxel.js:376-433):
same arguments, same outputs ({tipo, sdf, stats}), classes VOXEL.FLUIDO 0,
CASCA 1, DENTRO 2.  ``areaFrontal`` restates src/geom/voxel.js:443-457.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat

VOXEL = {"FLUIDO": 0, "CASCA": 1, "DENTRO": 2}


def voxelizar(positions, indices, g, banda=1.5, selarFrestas=True, sdf=True):
    """positions: float32 (V*3) in lattice units (cell = 1); indices: uint32
    (T*3); g: {nx, ny, nz}.  Returns {"tipo": uint8[N], "sdf": float32[N] or
    None, "stats": dict}."""
    lib = nat.load()
    pos = np.ascontiguousarray(np.asarray(positions, dtype=np.float32).reshape(-1))
    idx = np.ascontiguousarray(np.asarray(indices, dtype=np.uint32).reshape(-1))
    if pos.size % 3 or idx.size % 3:
        raise ValueError("positions and indices must hold triples")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    N = nx * ny * nz
    tipo = np.empty(N, dtype=np.uint8)
    out_sdf = np.empty(N, dtype=np.float32) if sdf else None
    st = nat.VoxStats()
    dims = nat.Dims(nx, ny, nz)
    nat.check(lib.vox_voxelize(nat.ptr(pos), pos.size // 3, nat.ptr(idx), idx.size // 3, C.byref(dims),
                               float(banda), 1 if selarFrestas else 0, nat.ptr(tipo), nat.ptr(out_sdf), C.byref(st)))
    stats = {
        "nCelulas": int(st.n_cells), "nCasca": int(st.n_casca), "nDentro": int(st.n_dentro),
        "nSolido": int(st.n_solido), "fracaoSolida": st.n_solido / N, "trianguloFora": int(st.triangulo_fora),
        "ocoSuspeito": bool(st.oco_suspeito), "msRasterizacao": float(st.ms_raster),
        "msInundacao": float(st.ms_flood), "msTotal": float(st.ms_total),
        "passesInundacao": int(st.flood_iterations), "pares": int(st.n_pairs), "paresFp64": int(st.n_deferred),
    }
    return {"tipo": tipo, "sdf": out_sdf, "stats": stats}


def areaFrontal(tipo, g) -> int:
    """YZ shadow of every non-fluid voxel (src/geom/voxel.js:443-457)."""
    nx, ny, nz = g["nx"], g["ny"], g["nz"]
    t = np.asarray(tipo).reshape(nz, ny, nx)
    return int((t != VOXEL["FLUIDO"]).any(axis=2).sum())
