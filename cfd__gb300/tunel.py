"""Cell-type field of the tunnel: body plus tunnel walls (host, numpy).

Restates src/core/tunel.js: ``montarTipos`` (:39-108), ``areaFrontalCorpo``
(:118-133) and ``corpoAnalitico`` (:144-168).  Codes are the CELULA classes
(src/core/emit/ir.js:71-80) and the VOXEL codes (src/geom/voxel.js:155-159).
"""
from __future__ import annotations

import math

import numpy as np

CELULA = {"FLUIDO": 0, "SOLIDO": 1, "ENTRADA": 2, "SAIDA": 3, "SOLIDO_MOVEL": 4,
          "ESPELHO_Y": 5, "ESPELHO_Z": 6, "PAREDE": 7}
VOXEL = {"FLUIDO": 0, "CASCA": 1, "DENTRO": 2}


def montarTipos(grade, corpo=None, esteira=True, fracaoEsponja=0.18):
    """Body first, walls over it, inlet/outlet win the corners.

    Returns ``{"tipo": uint32[N], "esponja": {"inicio", "comprimento"},
    "contagem": {...}}`` like the reference.
    """
    nx, ny, nz = grade["nx"], grade["ny"], grade["nz"]
    N = nx * ny * nz
    if corpo is not None:
        corpo = np.asarray(corpo).reshape(-1)
        if corpo.size != N:
            raise ValueError(f"campo do corpo com {corpo.size}, esperado {N}")
        tipo = np.where(corpo != VOXEL["FLUIDO"], CELULA["SOLIDO"], CELULA["FLUIDO"]).astype(np.uint32)
    else:
        tipo = np.zeros(N, dtype=np.uint32)
    t = tipo.reshape(nz, ny, nx)
    piso = CELULA["SOLIDO_MOVEL"] if esteira else CELULA["PAREDE"]
    t[:, :, 0] = CELULA["ENTRADA"]
    t[:, :, nx - 1] = CELULA["SAIDA"]
    t[:, 0, :] = CELULA["ESPELHO_Y"]
    t[:, ny - 1, :] = CELULA["ESPELHO_Y"]
    t[0, :, :] = piso
    t[nz - 1, :, :] = CELULA["ESPELHO_Z"]
    t[:, :, 0] = CELULA["ENTRADA"]
    t[:, :, nx - 1] = CELULA["SAIDA"]
    comprimento = max(4, int(math.floor(nx * fracaoEsponja + 0.5)))
    esponja = {"inicio": nx - 1 - comprimento, "comprimento": comprimento}
    contagem = {
        "fluido": int((tipo == 0).sum()), "solido": int((tipo == 1).sum()),
        "solidoMovel": int((tipo == 4).sum()), "entrada": int((tipo == 2).sum()),
        "saida": int((tipo == 3).sum()),
    }
    contagem["espelho"] = N - sum(contagem.values())
    return {"tipo": tipo, "esponja": esponja, "contagem": contagem}


def areaFrontalCorpo(corpo, grade) -> int:
    """YZ shadow of the body over x, y, z in [1, n-2] (the floor row excluded)."""
    nx, ny, nz = grade["nx"], grade["ny"], grade["nz"]
    c = np.asarray(corpo).reshape(nz, ny, nx)
    inner = c[1:nz - 1, 1:ny - 1, 1:nx - 1] != VOXEL["FLUIDO"]
    return int(inner.any(axis=2).sum())


def corpoAnalitico(grade, forma):
    """Sphere, or cylinder along y, sampled at voxel centres (+0.5)."""
    nx, ny, nz = grade["nx"], grade["ny"], grade["nz"]
    f, cx, cy, cz, raio = forma["tipo"], forma["cx"], forma["cy"], forma["cz"], forma["raio"]
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    dx, dy, dz = x + 0.5 - cx, y + 0.5 - cy, z + 0.5 - cz
    if f == "esfera":
        dentro = dx * dx + dy * dy + dz * dz <= raio * raio
    elif f == "cilindro":
        dentro = dx * dx + dz * dz <= raio * raio
    else:
        raise ValueError(f"forma desconhecida: {f}")
    return np.where(dentro, VOXEL["DENTRO"], VOXEL["FLUIDO"]).astype(np.uint8).reshape(-1)
