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


class Camera(C.Structure):
    _fields_ = [("inv_view_proj", C.c_float * 16), ("olho", C.c_float * 3), ("densidade", C.c_float),
                ("g", C.c_float), ("passos", C.c_int32), ("passos_luz", C.c_int32), ("luz", C.c_float * 4),
                ("quadro", C.c_float), ("largura", C.c_int32), ("altura", C.c_int32)]


def camera_orbita(nx, ny, nz, azimute=0.6, elevacao=0.35, distancia=2.6, fov=0.8, aspecto=16 / 9):
    """A view-projection looking at the middle of the tunnel floor from an
    orbit (world = lattice scaled by 2/nx, origin at the floor's centre, z up;
    src/render/comum.js:56-71), depth mapped to [0, 1] as WebGPU does.
    Returns (inv_view_proj column-major, eye)."""
    k = 2.0 / nx
    alvo = np.array([0.0, 0.0, nz * k * 0.35])
    olho = alvo + distancia * np.array([np.cos(elevacao) * np.cos(azimute), np.cos(elevacao) * np.sin(azimute),
                                        np.sin(elevacao)])
    f = alvo - olho
    f = f / np.linalg.norm(f)
    up = np.array([0.0, 0.0, 1.0])
    r = np.cross(f, up)
    r = r / np.linalg.norm(r)
    u = np.cross(r, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = r, u, -f
    view[:3, 3] = -view[:3, :3] @ olho
    near, far = 0.05, 50.0
    t = 1.0 / np.tan(fov / 2)
    proj = np.zeros((4, 4))
    proj[0, 0] = t / aspecto
    proj[1, 1] = t
    proj[2, 2] = far / (near - far)
    proj[2, 3] = near * far / (near - far)
    proj[3, 2] = -1.0
    inv = np.linalg.inv(proj @ view)
    return inv.T.reshape(-1).astype(np.float32), olho.astype(np.float32)


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

    def render(self, inv_view_proj, olho, largura=320, altura=180, densidade=70.0, g=0.45, passos=96,
               passos_luz=5, luz=(-0.35, 0.55, 0.76), intensidade=1.0, quadro=0):
        """Ray-march of the volume into an (altura, largura, 4) float32 image
        (premultiplied radiance, 1 - transmittance; row 0 at the top)."""
        cam = Camera()
        for i in range(16):
            cam.inv_view_proj[i] = float(inv_view_proj[i])
        for i in range(3):
            cam.olho[i] = float(olho[i])
        cam.densidade, cam.g, cam.passos, cam.passos_luz = float(densidade), float(g), int(passos), int(passos_luz)
        for i in range(3):
            cam.luz[i] = float(luz[i])
        cam.luz[3] = float(intensidade)
        cam.quadro, cam.largura, cam.altura = float(quadro), int(largura), int(altura)
        out = np.empty((int(altura), int(largura), 4), np.float32)
        nat.check(self._lib.vis_fumaca_render(self._h, C.byref(cam), nat.ptr(out), out.size))
        return out

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

    def passo_rasantes(self, dt_quadro, subpassos=1, quadro=0, altura=6.0):
        """The ground-streak frame (src/render/rasante.js:95-149) on the same records."""
        nat.check(self._lib.vis_rasantes_passo(self._h, float(dt_quadro), int(subpassos), int(quadro) & 0xFFFFFFFF,
                                               float(altura)))

    def destruir(self):
        if getattr(self, "_h", None):
            nat.check(self._lib.vis_esteiras_destroy(self._h))
            self._h = None


def cp_superficie(solver, pos, idx, u_ref):
    """Surface Cp per triangle of a mesh in lattice coordinates (the body
    shader's sample, src/render/renderer.js:168-180, at each centroid), from
    the solver's current macros."""
    lib = nat.load()
    p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(idx, np.uint32).reshape(-1, 3)
    out = np.empty(t.shape[0], np.float32)
    nat.check(lib.vis_cp_triangulos(solver._h, nat.ptr(p), p.shape[0], nat.ptr(t), t.shape[0], float(u_ref),
                                    nat.ptr(out)))
    return out
