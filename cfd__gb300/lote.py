"""LoteCUDA — many tunnels of uneven sizes stepped together (include/lbm_batch.h).

Each tunnel is configured like a SolverCUDA (configurar / definirTipos with
the reference's arguments, src/backend/webgpu/solver.js:277-301); passo(n)
advances all of them with one launch per step (mode 1), replayed from a
CUDA graph.  Per-tunnel results equal what separate SolverCUDA objects give.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from .lattice import MAGIC, Q
from .solver import STORAGE, js_round


class LoteCUDA:
    def __init__(self, grades, storage="f32", estrito=False):
        self._lib = nat.load()
        self.grades = [dict(g) for g in grades]
        self.T = len(self.grades)
        arr = (nat.Dims * self.T)(*[nat.Dims(g["nx"], g["ny"], g["nz"]) for g in self.grades])
        h = C.c_void_p()
        nat.check(self._lib.lbm_batch_create(C.cast(arr, C.c_void_p), self.T, STORAGE[storage],
                                             nat.FLAG_STRICT if estrito else 0, C.byref(h)))
        self._h = h
        self.passos = 0

    def configurar(self, k, omegaPlus, magic=MAGIC["WALL"], lesCs=0.1, inletU=(0, 0, 0), beltU=(0, 0, 0),
                   esponja=None, espessuraCL=0):
        g = self.grades[k]
        esp = esponja if esponja is not None else {
            "inicio": js_round(g["nx"] * 0.82), "comprimento": max(4, js_round(g["nx"] * 0.18))}
        p = nat.Params()
        p.omega_plus, p.magic, p.les_cs = omegaPlus, magic, lesCs
        for a in range(3):
            p.belt_u[a] = beltU[a]
            p.inlet_u[a] = inletU[a]
        p.sponge_start, p.sponge_len, p.bl_thickness, p.closure = esp["inicio"], esp["comprimento"], espessuraCL, 0
        nat.check(self._lib.lbm_batch_configure(self._h, int(k), C.byref(p)))

    def definirTipos(self, k, tipos):
        t = np.ascontiguousarray(np.asarray(tipos), dtype=np.uint32).reshape(-1)
        nat.check(self._lib.lbm_batch_set_types(self._h, int(k), nat.ptr(t), t.size))

    def inicializar(self):
        nat.check(self._lib.lbm_batch_init_equilibrium(self._h))
        self.passos = 0

    def passo(self, n=1):
        nat.check(self._lib.lbm_batch_step(self._h, int(n)))
        self.passos += n

    def lerPopulacoes(self, k):
        g = self.grades[k]
        N = g["nx"] * g["ny"] * g["nz"]
        out = np.empty(Q * N, dtype=np.float64)
        nat.check(self._lib.lbm_batch_get_populations(self._h, int(k), nat.ptr(out), out.size))
        return out.reshape(Q, N)

    def medirForcas(self):
        f = np.empty(3 * self.T, dtype=np.float64)
        nat.check(self._lib.lbm_batch_forces(self._h, nat.ptr(f)))
        return f.reshape(self.T, 3)

    def definirLadrilho(self, k, tile_x):
        nat.check(self._lib.lbm_batch_set_tile(self._h, int(k), int(tile_x)))

    def definirModo(self, modo):
        """0: graph of per-tunnel chains (default); 1: one launch per step whose CTAs walk all tunnels' tiles."""
        nat.check(self._lib.lbm_batch_set_mode(self._h, int(modo)))

    def ladrilho(self, k):
        """Tile width along x of tunnel k in the mode-1 launch."""
        t = C.c_int()
        nat.check(self._lib.lbm_batch_get_tile(self._h, int(k), C.byref(t)))
        return t.value

    def autoajustar(self, passos=64):
        """Measured choice of mode, register cap and per-size-class tile
        width (lbm_batch_autotune); the states are kept."""
        m, mb, ms = C.c_int(), C.c_int(), C.c_float()
        nat.check(self._lib.lbm_batch_autotune(self._h, int(passos), C.byref(m), C.byref(mb), C.byref(ms)))
        return {"mode": m.value, "resident_ctas_per_sm": mb.value, "ms_per_step": ms.value,
                "tiles": [self.ladrilho(k) for k in range(self.T)]}

    def definirStream(self, ptr):
        nat.check(self._lib.lbm_batch_set_stream(self._h, C.c_void_p(ptr)))

    @property
    def celulas(self):
        c, b = C.c_int64(), C.c_int64()
        nat.check(self._lib.lbm_batch_info(self._h, C.byref(c), C.byref(b)))
        return int(c.value)

    def destruir(self):
        if getattr(self, "_h", None):
            nat.check(self._lib.lbm_batch_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.destruir()
        except Exception:
            pass


def sorteio_lote(n=64, seed=2026, nx_min=96, nx_max=256):
    """The batched workload: n tunnels drawn from a seed.  Grid nx from
    {96, 112, ..., 256} with ny = nz = nx/2; a sphere or an ellipsoid of
    diameter 8-24 cells at (0.3 nx, ny/2, nz/2); Re log-uniform in [50, 400];
    u_in uniform in [0.03, 0.08]; nu = u_in D / Re; free-slip walls.
    Returns [(grade, tipo uint32, cfg dict, info dict)]."""
    from .tunel import montarTipos
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.choice(np.arange(nx_min, nx_max + 1, 16)))
        g = {"nx": nx, "ny": nx // 2, "nz": nx // 2}
        D = float(rng.uniform(8, 24))
        elip = bool(rng.random() < 0.5)
        ax = np.array([D, D, D]) / 2 if not elip else np.array([D / 2, D / 2 * rng.uniform(0.5, 1.0),
                                                               D / 2 * rng.uniform(0.5, 1.0)])
        re = float(np.exp(rng.uniform(np.log(50), np.log(400))))
        u = float(rng.uniform(0.03, 0.08))
        nu = u * D / re
        omega = 1.0 / (3.0 * nu + 0.5)
        z, y, x = np.meshgrid(np.arange(g["nz"]) + 0.5, np.arange(g["ny"]) + 0.5, np.arange(nx) + 0.5, indexing="ij")
        c = (0.3 * nx, g["ny"] / 2, g["nz"] / 2)
        dentro = ((x - c[0]) / ax[0]) ** 2 + ((y - c[1]) / ax[1]) ** 2 + ((z - c[2]) / ax[2]) ** 2 <= 1.0
        corpo = np.where(dentro, 2, 0).astype(np.uint8).reshape(-1)
        mt = montarTipos(g, corpo=corpo, esteira=False)
        t = mt["tipo"].reshape(g["nz"], g["ny"], nx)
        t[0, :, 1:nx - 1] = 6
        cfg = dict(omegaPlus=omega, lesCs=0.1, inletU=[u, 0.0, 0.0], esponja=mt["esponja"])
        out.append((g, mt["tipo"], cfg, {"D": D, "Re": re, "u": u, "omega": omega, "flag_omega": omega > 1.95,
                                          "ellipsoid": elip}))
    return out
