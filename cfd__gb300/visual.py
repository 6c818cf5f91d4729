"""Visualisation compute of the tunnel on the GPU (include/lbm_vis.h): the
smoke volume (src/render/fumaca.js) and the streak particles
(src/render/renderer.js), as headless device buffers over a SolverCUDA's
macros field.  Names follow the reference's layers: Fumaca, Esteiras."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat


class Rake(C.Structure):
    _fields_ = [("x", C.c_float), ("passo_y", C.c_float), ("passo_z", C.c_float), ("raio", C.c_float),
                ("y0", C.c_float), ("y1", C.c_float), ("z0", C.c_float), ("z1", C.c_float)]


class Fumo(C.Structure):
    _fields_ = [("dt", C.c_float), ("dissipacao", C.c_float), ("taxa", C.c_float), ("avanco", C.c_float)]


class Part(C.Structure):
    _fields_ = [("pos", C.c_float * 4), ("ant", C.c_float * 4)]


def posicionar_rake(ny, nz, extentos, colunas=7, linhas=5):
    """VolumeFumaca.posicionarRake + _recalcularGrade (src/render/fumaca.js:539-590):
    the rake in front of the body, covering it with margin; filament spacing
    from the counts, radius 0.3 of the spacing within [0.7, 2.8]."""
    mn, tam, centro = extentos["min"], extentos["tamanho"], extentos["centro"]
    largura = max(tam[1], 4)
    altura = max(tam[2], 4)
    r = {"x": max(3, mn[0] - max(10, tam[0] * 0.55)),
         "y0": max(1, centro[1] - largura * 1.15), "y1": min(ny - 2, centro[1] + largura * 1.15),
         "z0": 1, "z1": min(nz - 2, altura * 2.3)}
    r["passo_y"] = (r["y1"] - r["y0"]) / max(colunas, 1)
    r["passo_z"] = (r["z1"] - r["z0"]) / max(linhas, 1)
    r["raio"] = min(2.8, max(0.7, 0.3 * min(r["passo_y"], r["passo_z"])))
    return r


class Fumaca:
    """The smoke volume of one solver (three fp16 volumes of its grid)."""

    def __init__(self, solver):
        self._lib = nat.load()
        self.solver = solver
        h = C.c_void_p()
        nat.check(self._lib.vis_fumaca_create(solver._h, C.byref(h)))
        self._h = h
        self.shape = (solver.nz, solver.ny, solver.nx)

    def limpar(self):
        nat.check(self._lib.vis_fumaca_limpar(self._h))

    def passo(self, rake, dt=17.0, dissipacao=0.999, taxa=2.4, avanco=None):
        """One advection step; avanco defaults to dt * 0.05 as in the reference."""
        R = Rake(**{k: float(rake[k]) for k in ("x", "passo_y", "passo_z", "raio", "y0", "y1", "z0", "z1")})
        F = Fumo(float(dt), float(dissipacao), float(taxa), float(dt * 0.05 if avanco is None else avanco))
        nat.check(self._lib.vis_fumaca_passo(self._h, C.byref(R), C.byref(F)))

    def ler(self):
        out = np.empty(int(np.prod(self.shape)), np.float16)
        nat.check(self._lib.vis_fumaca_ler(self._h, nat.ptr(out), out.size))
        return out.reshape(self.shape)

    def definir(self, dens):
        a = np.ascontiguousarray(dens, np.float16).reshape(-1)
        nat.check(self._lib.vis_fumaca_definir(self._h, nat.ptr(a), a.size))

    def destruir(self):
        if getattr(self, "_h", None):
            nat.check(self._lib.vis_fumaca_destroy(self._h))
            self._h = None


class Esteiras:
    """Streak particles of one solver: n records (pos xyzw, ant xyzw)."""

    def __init__(self, solver, n):
        self._lib = nat.load()
        self.n = int(n)
        h = C.c_void_p()
        nat.check(self._lib.vis_esteiras_create(solver._h, self.n, C.byref(h)))
        self._h = h

    def definir(self, parts):
        a = np.ascontiguousarray(parts, np.float32).reshape(self.n, 8)
        nat.check(self._lib.vis_esteiras_definir(self._h, nat.ptr(a), self.n))

    def ler(self):
        out = np.empty((self.n, 8), np.float32)
        nat.check(self._lib.vis_esteiras_ler(self._h, nat.ptr(out), self.n))
        return out

    def passo(self, dt_quadro, subpassos=1, quadro=0):
        nat.check(self._lib.vis_esteiras_passo(self._h, float(dt_quadro), int(subpassos), int(quadro) & 0xFFFFFFFF))

    def destruir(self):
        if getattr(self, "_h", None):
            nat.check(self._lib.vis_esteiras_destroy(self._h))
            self._h = None

