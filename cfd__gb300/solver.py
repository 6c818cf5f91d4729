"""SolverCUDA — the reference's solver class API over the sm_103a library.

Mirrors SolverWebGPU (src/backend/webgpu/solver.js:36-528) member by member,
with the same names, argument meaning and error behaviour, so a caller written
against the WebGPU/WebGL2 backends (index.html, tests/*.html) reads the same
here.  JavaScript promises become plain synchronous calls; the ones that
synchronise in the reference (lerMacros, medirForcas, calibrarRepouso)
synchronise here.

Everything runs in the CUDA library; this class holds host-side state only
(ramp, rest-force offset, configuration) exactly where the reference holds it
in JavaScript.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as nat
from .lattice import MAGIC, Q
from .lattice import equilibrium as _equilibrium

STORAGE = {"f32": nat.F32, "f16s": nat.F16S, "bf16s": nat.BF16S, "f64": nat.F64, "f16sr": nat.F16SR,
           "bf16sr": nat.BF16SR}


def js_round(v: float) -> int:
    """JavaScript Math.round: floor(v + 0.5)."""
    return int(math.floor(v + 0.5))


class SolverCUDA:
    """A D3Q19 TRT/LES wind tunnel on one GB300, one CUDA stream per solver."""

    def __init__(self, grade, storage="f32", escrever_macros=True, pingpong=False, estrito=False, soa=None):
        """storage: "f32" | "f16s" | "bf16s" | "f64" | "f16sr" | "bf16sr" (the
        16-bit forms with stochastically rounded stores); pingpong: the reference's
        two-set A/B layout instead of the in-place one; estrito: the shader's
        arithmetic read literally (no fused multiply-add) instead of the FAST
        restatement; soa: True keeps the in-place set in the SoA layout,
        False asks for the AoSoA layout where it applies, None (default)
        takes the library's choice (autotuneLayout's measurement, else AoSoA
        where it applies: blocks of 32 cells for f32, 64 for the 16-bit
        forms, rows padded to a multiple of the block); info()["layout"]
        says which is in use (0 SoA, 1 ping-pong, 2 AoSoA in blocks of 32
        cells, 3 in blocks of 64)."""
        self._lib = nat.load()
        self.nx, self.ny, self.nz = int(grade["nx"]), int(grade["ny"]), int(grade["nz"])
        self.N = self.nx * self.ny * self.nz
        self.storage = storage
        self.passos = 0
        self._frente = "A"
        self.cfg = None
        self.offsetForca = None
        self._rampa = None
        self.fontes = {"passo": "cfd__gb300/csrc/lbm_kernels.cuh:k_step_inplace"}
        flags = (nat.FLAG_WRITE_MACROS if escrever_macros else 0) | (nat.FLAG_PINGPONG if pingpong else 0) | \
            (nat.FLAG_STRICT if estrito else 0) | (0 if soa is None else (nat.FLAG_SOA if soa else nat.FLAG_AOS))
        dims = nat.Dims(self.nx, self.ny, self.nz)
        h = C.c_void_p()
        nat.check(self._lib.lbm_create(C.byref(dims), STORAGE[storage], flags, C.byref(h)))
        self._h = h

    # -------------------------------------------------------- construction
    @staticmethod
    def criarDevice(adapter=None):
        """The device is the process's current CUDA device; nothing to create
        (src/backend/webgpu/solver.js:61-82 creates one per page)."""
        return 0

    @classmethod
    def criar(cls, device, grade, **kw):
        """SolverWebGPU.criar (src/backend/webgpu/solver.js:93-124): allocates;
        raises with the size in GB when the device refuses."""
        return cls(grade, **kw)

    @property
    def bytesTotais(self) -> int:
        info = nat.Info()
        nat.check(self._lib.lbm_get_info(self._h, C.byref(info)))
        return int(info.device_bytes)

    # ------------------------------------------------------- configuration
    def configurar(self, omegaPlus, magic=MAGIC["WALL"], lesCs=0.1, inletU=(0, 0, 0),
                   beltU=(0, 0, 0), esponja=None, espessuraCL=0, closure=0):
        """SolverWebGPU.configurar (src/backend/webgpu/solver.js:277-293)."""
        esp = esponja if esponja is not None else {
            "inicio": js_round(self.nx * 0.82),
            "comprimento": max(4, js_round(self.nx * 0.18)),
        }
        p = nat.Params()
        p.omega_plus, p.magic, p.les_cs = omegaPlus, magic, lesCs
        for a in range(3):
            p.belt_u[a] = beltU[a]
            p.inlet_u[a] = inletU[a]
        p.sponge_start = esp["inicio"]
        p.sponge_len = esp["comprimento"]
        p.bl_thickness = espessuraCL
        p.closure = closure
        nat.check(self._lib.lbm_configure(self._h, C.byref(p)))
        self.cfg = {"omegaPlus": omegaPlus, "magic": magic, "lesCs": lesCs, "inletU": list(inletU),
                    "beltU": list(beltU), "esponja": esp, "espessuraCL": espessuraCL}

    def definirTipos(self, tipos):
        """SolverWebGPU.definirTipos (src/backend/webgpu/solver.js:296-301)."""
        t = np.ascontiguousarray(np.asarray(tipos), dtype=np.uint32).reshape(-1)
        if t.size != self.N:
            raise ValueError(f"campo de tipos com {t.size}, esperado {self.N}")
        nat.check(self._lib.lbm_set_types(self._h, nat.ptr(t), t.size))

    # ---------------------------------------------------------------- ramp
    def rampa(self, passos, aplicarVelocidade):
        """SolverWebGPU.rampa (src/backend/webgpu/solver.js:323-325)."""
        self._rampa = {"passos": passos, "aplicar": aplicarVelocidade, "atual": 0}

    @property
    def fatorRampa(self) -> float:
        """Smoothstep factor (src/backend/webgpu/solver.js:328-335)."""
        r = self._rampa
        if not r or r["atual"] >= r["passos"]:
            return 1.0
        t = r["atual"] / r["passos"]
        return t * t * (3 - 2 * t)

    # ---------------------------------------------------------------- state
    def inicializar(self):
        """SolverWebGPU.inicializar (src/backend/webgpu/solver.js:338-349)."""
        nat.check(self._lib.lbm_init_equilibrium(self._h))
        self._frente = "B"
        self.passos = 0
        if self._rampa:
            self._rampa["atual"] = 0

    @property
    def frente(self):
        """Which set holds the state in the reference's A/B scheme; with the
        in-place layout it is bookkeeping only (written by tests/nucleo.html:149)."""
        return self._frente

    @frente.setter
    def frente(self, v):
        self._frente = v

    def definirCampo(self, fn, equilibrium=_equilibrium):
        """SolverWebGPU.definirCampo (src/backend/webgpu/solver.js:363-389).

        ``fn(x, y, z)`` returns ``{"delta": d, "u": [ux, uy, uz]}``; it is called
        once with broadcast integer arrays (numpy), so an expression such as
        ``A0 * np.sin(k * y)`` fills the whole field in one call.  The
        equilibrium is evaluated in fp64 on the host and rounded to the storage
        type on upload, as the reference writes it into a Float32Array.
        """
        z, y, x = np.meshgrid(np.arange(self.nz), np.arange(self.ny), np.arange(self.nx), indexing="ij")
        r = fn(x, y, z) or {}
        delta = np.broadcast_to(np.asarray(r.get("delta", 0.0), dtype=np.float64), x.shape)
        u_in = r.get("u", [0.0, 0.0, 0.0])
        u = np.stack([np.broadcast_to(np.asarray(c, dtype=np.float64), x.shape) for c in u_in], axis=-1)
        g = equilibrium(delta, u)                              # (nz, ny, nx, 19)
        soa = np.ascontiguousarray(np.moveaxis(g, -1, 0).reshape(Q, -1))
        self.definirPopulacoes(soa)

    def definirPopulacoes(self, g_soa):
        """Upload a 19 x N fp64 state (direction-major), rounded to storage."""
        g = np.ascontiguousarray(np.asarray(g_soa, dtype=np.float64).reshape(-1))
        nat.check(self._lib.lbm_set_populations(self._h, nat.ptr(g), g.size))
        self.passos = 0

    def lerPopulacoes(self):
        """The current post-collision state as 19 x N fp64 (direction-major)."""
        g = np.empty(Q * self.N, dtype=np.float64)
        nat.check(self._lib.lbm_get_populations(self._h, nat.ptr(g), g.size))
        return g.reshape(Q, self.N)

    # ------------------------------------------------------------------ loop
    def passo(self, n=1):
        """SolverWebGPU.passo (src/backend/webgpu/solver.js:395-415): the ramp
        advances and re-applies before the n steps are enqueued."""
        r = self._rampa
        if r and r["atual"] < r["passos"]:
            r["atual"] += n
            if r["aplicar"]:
                r["aplicar"](self.fatorRampa)
        nat.check(self._lib.lbm_step(self._h, int(n)))
        self.passos += n
        if n % 2:   # the reference swaps its A/B sets once per dispatched step
            self._frente = "B" if self._frente == "A" else "A"

    def passoComForcas(self, n):
        """n steps that also return the force of the state each step streams
        from (n x 3, fp64, rest offset subtracted)."""
        out = np.empty(3 * n, dtype=np.float64)
        nat.check(self._lib.lbm_step_forces(self._h, int(n), nat.ptr(out)))
        self.passos += n
        f = out.reshape(n, 3)
        o = self.offsetForca if self.offsetForca is not None else [0.0, 0.0, 0.0]
        return f - np.asarray(o, dtype=np.float64)

    def passoComForcasAssincrono(self, n, destino=None):
        """passoComForcas enqueued (the reference's medirForcas is async):
        returns a ticket at once; aguardarForcas(ticket) gives the n x 3
        forces (rest offset subtracted) once they have landed.  destino:
        3*n float64 the caller keeps alive (page-locked memory lets the copy
        overlap the next steps)."""
        if destino is None:
            destino = np.empty(3 * n, dtype=np.float64)
        t = C.c_int64()
        nat.check(self._lib.lbm_step_forces_async(self._h, int(n), nat.ptr(destino), C.byref(t)))
        self.passos += n
        if not hasattr(self, "_forcas_async"):
            self._forcas_async = {}
        self._forcas_async[t.value] = destino
        return t.value

    def aguardarForcas(self, ticket, esperar=True):
        """The n x 3 forces of an asynchronous call, or None if not landed
        yet and esperar is False."""
        d = C.c_int()
        nat.check(self._lib.lbm_forces_done(self._h, int(ticket), 1 if esperar else 0, C.byref(d)))
        if not d.value:
            return None
        destino = self._forcas_async.pop(ticket)
        f = destino.reshape(-1, 3)
        o = self.offsetForca if self.offsetForca is not None else [0.0, 0.0, 0.0]
        return f - np.asarray(o, dtype=np.float64)

    # --------------------------------------------------------------- reading
    def lerMacros(self):
        """SolverWebGPU.lerMacros (src/backend/webgpu/solver.js:427-442):
        float32 N*4 (ux, uy, uz, delta)."""
        out = np.empty(4 * self.N, dtype=np.float32)
        nat.check(self._lib.lbm_read_macros(self._h, nat.ptr(out), out.size))
        return out

    def atualizarMacros(self):
        """SolverWebGPU.atualizarMacros (src/backend/webgpu/solver.js:511-520)."""
        nat.check(self._lib.lbm_update_macros(self._h))

    def calibrarRepouso(self):
        """SolverWebGPU.calibrarRepouso (src/backend/webgpu/solver.js:480-484):
        call after definirTipos and before inicializar."""
        self.offsetForca = [0.0, 0.0, 0.0]
        self.offsetForca = self.medirForcas()
        return self.offsetForca

    def medirForcas(self):
        """SolverWebGPU.medirForcas (src/backend/webgpu/solver.js:486-508):
        [fx, fy, fz] in lattice units minus the rest offset."""
        f = np.zeros(3, dtype=np.float64)
        nat.check(self._lib.lbm_forces(self._h, nat.ptr(f)))
        o = self.offsetForca if self.offsetForca is not None else [0.0, 0.0, 0.0]
        return [float(f[0] - o[0]), float(f[1] - o[1]), float(f[2] - o[2])]

    def massa(self) -> float:
        """Sum of delta over the non-solid cells (fp64)."""
        v = C.c_double()
        nat.check(self._lib.lbm_mass(self._h, C.byref(v)))
        return v.value

    def sincronizar(self):
        nat.check(self._lib.lbm_sync(self._h))

    def definirStream(self, cuda_stream_ptr: int):
        nat.check(self._lib.lbm_set_stream(self._h, C.c_void_p(cuda_stream_ptr)))

    def definirBloco(self, block_x: int, min_blocos: int = 0):
        """Launch shape of the step kernel: threads along x per block and the
        variant code of lbm_set_launch (8 or 6 resident blocks per SM; 9
        AoSoA addresses kept; 20 / 21 SoA addressing from one base; 100 + k
        the pipelined SoA step; 0 = default)."""
        nat.check(self._lib.lbm_set_launch(self._h, int(block_x), int(min_blocos)))

    @staticmethod
    def autoajustarLayout(grade, storage="f32", passos=20, estrito=False):
        """Time both layouts of the in-place set on a free stream of this grid
        (lbm_autotune_layout); the faster becomes the default for solvers of
        this grid and storage created afterwards in this process."""
        lib = nat.load()
        dims = nat.Dims(int(grade["nx"]), int(grade["ny"]), int(grade["nz"]))
        lay, a, b = C.c_int(), C.c_float(), C.c_float()
        nat.check(lib.lbm_autotune_layout(C.byref(dims), STORAGE[storage], nat.FLAG_STRICT if estrito else 0,
                                          int(passos), C.byref(lay), C.byref(a), C.byref(b)))
        return {"layout": lay.value, "ms_aosoa": a.value, "ms_soa": b.value}

    def autoajustar(self, passos=20):
        """Measure the step kernel's launch shapes on a copy of the current
        state (lbm_autotune) and keep the fastest: returns the choice and its
        milliseconds per step."""
        bx, by, var, ms = C.c_int(), C.c_int(), C.c_int(), C.c_float()
        nat.check(self._lib.lbm_autotune(self._h, int(passos), C.byref(bx), C.byref(by), C.byref(var), C.byref(ms)))
        return {"block_x": bx.value, "block_y": by.value, "variant": var.value, "ms_per_step": ms.value}

    # --------------------------------------------------------------- state I/O
    def salvarEstado(self) -> bytes:
        """Checkpoint of the population set (include/lbm_state.h)."""
        n = C.c_size_t()
        nat.check(self._lib.lbm_state_bytes(self._h, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        nat.check(self._lib.lbm_save_state(self._h, nat.ptr(buf), n.value))
        return buf.tobytes()

    def carregarEstado(self, blob: bytes):
        """Restore a checkpoint taken by salvarEstado on a solver of the same
        grid, storage form and layout; the step count comes with it."""
        buf = np.frombuffer(blob, np.uint8)
        nat.check(self._lib.lbm_load_state(self._h, nat.ptr(buf), buf.size))
        self.passos = int(np.frombuffer(blob[32:40], np.int64)[0])

    def lerMacrosAssincrono(self, destino=None):
        """Start a macros read-back into destino (4*N float32, kept alive by the
        caller; page-locked memory lets it overlap) and return it at once;
        macrosProntos() tells when it has landed."""
        if destino is None:
            destino = np.empty(4 * self.N, np.float32)
        self._macros_async = destino
        nat.check(self._lib.lbm_read_macros_async(self._h, nat.ptr(destino), destino.size))
        return destino

    def macrosProntos(self) -> bool:
        r = C.c_int()
        nat.check(self._lib.lbm_macros_ready(self._h, C.byref(r)))
        return bool(r.value)

    def definirFecho(self, pesos):
        """Network of the learned closure (cfd__gb300.fecho weights dict);
        configurar(closure=1) then selects it."""
        from .fecho import para_struct
        w = para_struct(pesos)
        nat.check(self._lib.lbm_set_closure(self._h, C.byref(w)))
        self.fontes["passo"] = "cfd__gb300/csrc/lbm_kernels.cuh:k_step_closure"

    def motorFecho(self, motor: int):
        """Tensor-core engine of the closure step: 0 warp mma.sync (default),
        1 CTA tcgen05."""
        nat.check(self._lib.lbm_closure_engine(self._h, int(motor)))

    def estatisticasFecho(self):
        """(fallback cells, fluid cells) over the closure steps since the last call."""
        a, b = C.c_int64(), C.c_int64()
        nat.check(self._lib.lbm_closure_stats(self._h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def info(self):
        i = nat.Info()
        nat.check(self._lib.lbm_get_info(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in nat.Info._fields_}

    # ---------------------------------------------------------------- teardown
    def destruir(self):
        """SolverWebGPU.destruir (src/backend/webgpu/solver.js:523-527)."""
        if getattr(self, "_h", None):
            nat.check(self._lib.lbm_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.destruir()
        except Exception:
            pass
