"""CPU oracle loader — TEST INFRASTRUCTURE ONLY.

Loads oracle/_build/liborc.so (built from the C restatement in this folder by
the Makefile) through ctypes.  Only tests/, ``__graft_entry__.smoke`` and the
``cpu_baseline`` leg of ``bench.py`` import this module, and only to check
results or to time a CPU baseline; the product (``cfd__gb300``) never does.

Parity status: the restatement follows the reference's generated shader
(src/core/emit/ir.js, src/core/emit/wgsl.js) and voxelizer
(src/geom/voxel.js) operation by operation.  The reference's own step cannot
run here (it exists only as WGSL/GLSL text produced by a JavaScript emitter and
this machine has neither a JS engine nor a graphics API), so the oracle is
pinned by the reference's own known-answer tests restated in
tests/test_oracle_kat.py (lattice invariants, uniform flow, shear-wave
viscosity, mass conservation, Couette wall position) and by golden tables
produced from the reference's Python lattice module (tests/golden/).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liborc.so")
_lock = threading.Lock()
_lib = None

F32, F16S, BF16S, F16SR, BF16SR = 0, 1, 2, 4, 5


class OrcParams(C.Structure):
    """Same layout as ``lbm_params`` in include/lbm.h."""

    _fields_ = [
        ("omega_plus", C.c_float), ("magic", C.c_float), ("les_cs", C.c_float),
        ("belt_u", C.c_float * 3), ("inlet_u", C.c_float * 3),
        ("sponge_start", C.c_float), ("sponge_len", C.c_float),
        ("bl_thickness", C.c_float), ("closure", C.c_int32),
    ]


class OrcVoxStats(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int64), ("n_casca", C.c_int64), ("n_dentro", C.c_int64),
        ("n_solido", C.c_int64), ("triangulo_fora", C.c_int64),
        ("oco_suspeito", C.c_int32), ("_pad", C.c_int32), ("n_deferred", C.c_int64),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    srcs = [os.path.join(_HERE, f) for f in ("lbm_oracle.c", "lbm_oracle_impl.h", "vox_oracle.c")]
    if not force and os.path.exists(_LIB_PATH):
        t = os.path.getmtime(_LIB_PATH)
        if all(os.path.getmtime(s) <= t for s in srcs):
            return _LIB_PATH
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            P = C.POINTER
            vp = C.c_void_p
            for sfx in ("f32", "f64"):
                getattr(L, f"orc_step_{sfx}").argtypes = [P(OrcParams), C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int,
                                                          C.c_int64]
                getattr(L, f"orc_init_{sfx}").argtypes = [P(OrcParams), C.c_int, C.c_int, C.c_int, vp, vp, C.c_int]
                getattr(L, f"orc_macros_{sfx}").argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_int]
                getattr(L, f"orc_forces_acc64_{sfx}").argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp]
                getattr(L, f"orc_forces_faithful_{sfx}").argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp]
                getattr(L, f"orc_mass_{sfx}").argtypes = [C.c_int, C.c_int, C.c_int, vp, vp]
                getattr(L, f"orc_mass_{sfx}").restype = C.c_double
                getattr(L, f"orc_run_{sfx}").argtypes = [P(OrcParams), C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int,
                                                         C.c_int64]
                getattr(L, f"orc_run_{sfx}").restype = C.c_int
            L.orc_tables_out.argtypes = [vp] * 6
            L.orc_quantize_f32.argtypes = [vp, C.c_int64, C.c_int]
            L.orc_f16_bits.argtypes = [C.c_float]
            L.orc_f16_bits.restype = C.c_uint16
            L.orc_f16_value.argtypes = [C.c_uint16]
            L.orc_f16_value.restype = C.c_float
            L.orc_bf16_bits.argtypes = [C.c_float]
            L.orc_bf16_bits.restype = C.c_uint16
            L.orc_sr_store_f32.argtypes = [C.c_float, C.c_int, C.c_uint32, C.c_int]
            L.orc_sr_store_f32.restype = C.c_float
            L.orc_sr_cell_hash.argtypes = [C.c_uint32, C.c_int64]
            L.orc_sr_cell_hash.restype = C.c_uint32
            L.orc_voxelize.argtypes = [vp, C.c_int64, vp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, vp, vp, P(OrcVoxStats)]
            L.orc_rasterize.argtypes = [vp, vp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_double, vp, vp]
            L.orc_rasterize.restype = C.c_int64
            L.orc_tri_box.argtypes = [vp, vp, vp, vp]
            L.orc_dist2_point_tri.argtypes = [vp, vp, vp, vp]
            L.orc_dist2_point_tri.restype = C.c_double
            L.orc_montar_tipos.argtypes = [C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_double, vp, P(C.c_double), P(C.c_double)]
            L.orc_area_frontal_corpo.argtypes = [vp, C.c_int, C.c_int, C.c_int]
            L.orc_area_frontal_corpo.restype = C.c_int64
            L.orc_corpo_analitico.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, vp]
            _lib = L
    return _lib


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def params(omega_plus, magic=3.0 / 16.0, les_cs=0.1, inlet_u=(0, 0, 0), belt_u=(0, 0, 0),
           sponge_start=0.0, sponge_len=1.0, bl_thickness=0.0) -> OrcParams:
    p = OrcParams()
    p.omega_plus, p.magic, p.les_cs = omega_plus, magic, les_cs
    for k in range(3):
        p.inlet_u[k] = inlet_u[k]
        p.belt_u[k] = belt_u[k]
    p.sponge_start, p.sponge_len, p.bl_thickness = sponge_start, sponge_len, bl_thickness
    p.closure = 0
    return p


def tables():
    L = lib()
    c = np.zeros(57, np.int32); opp = np.zeros(19, np.int32); mir = np.zeros(57, np.int32)
    w = np.zeros(19, np.float32); sixw = np.zeros(19, np.float32); wd = np.zeros(19, np.float64)
    L.orc_tables_out(_ptr(c), _ptr(opp), _ptr(mir), _ptr(w), _ptr(sixw), _ptr(wd))
    return {"C": c.reshape(19, 3), "OPP": opp, "MIRROR": mir.reshape(3, 19), "W": w, "SIXW": sixw, "Wd": wd}


class Lattice:
    """A/B ping-pong state on the CPU, natural SoA layout, like the reference."""

    def __init__(self, dims, dtype=np.float32, storage=F32, nthreads=1, fast=False):
        self.nx, self.ny, self.nz = dims
        self.N = self.nx * self.ny * self.nz
        self.dtype = np.dtype(dtype)
        self.sfx = "f32" if self.dtype == np.float32 else "f64"
        self.storage = storage
        self.nthreads = nthreads
        self.fast = 1 if fast else 0
        self.a = np.zeros(19 * self.N, self.dtype)
        self.b = np.zeros(19 * self.N, self.dtype)
        self.tipo = np.zeros(self.N, np.uint32)
        self.macros = np.zeros(4 * self.N, np.float32)
        self.p = params(1.0)
        self.steps = 0          # step count (the SR storage forms' rounding seeds); 0 after init / set

    def set_types(self, tipo):
        self.tipo = np.ascontiguousarray(tipo, dtype=np.uint32).reshape(-1)
        assert self.tipo.size == self.N

    def configure(self, **kw):
        self.p = params(**kw)

    def init(self):
        getattr(lib(), f"orc_init_{self.sfx}")(C.byref(self.p), self.nx, self.ny, self.nz,
                                               _ptr(self.tipo), _ptr(self.a), self.storage)
        self.steps = 0

    def set_populations(self, g):
        g = np.asarray(g, np.float64).reshape(-1)
        self.a[:] = g.astype(self.dtype)
        if self.dtype == np.float32 and self.storage != F32:
            lib().orc_quantize_f32(_ptr(self.a), self.a.size, self.storage)
        self.steps = 0

    def step(self, n=1, macros=False):
        L = lib()
        for k in range(n):
            m = _ptr(self.macros) if (macros and k == n - 1) else None
            getattr(L, f"orc_step_{self.sfx}")(C.byref(self.p), self.nx, self.ny, self.nz, _ptr(self.tipo),
                                               _ptr(self.a), _ptr(self.b), m, self.storage, self.nthreads, self.fast,
                                               self.steps)
            self.a, self.b = self.b, self.a
            self.steps += 1

    def run(self, n):
        """n steps in C without returning to Python between steps."""
        which = getattr(lib(), f"orc_run_{self.sfx}")(C.byref(self.p), self.nx, self.ny, self.nz, _ptr(self.tipo),
                                                     _ptr(self.a), _ptr(self.b), n, self.storage, self.nthreads, self.fast,
                                                     self.steps)
        if which == 1:
            self.a, self.b = self.b, self.a
        self.steps += n

    def populations(self):
        return self.a.astype(np.float64)

    def update_macros(self, zero_solids=True):
        getattr(lib(), f"orc_macros_{self.sfx}")(self.nx, self.ny, self.nz, _ptr(self.tipo), _ptr(self.a),
                                                 _ptr(self.macros), 1 if zero_solids else 0)
        return self.macros.copy()

    def forces(self):
        out = np.zeros(3, np.float64)
        getattr(lib(), f"orc_forces_acc64_{self.sfx}")(self.nx, self.ny, self.nz, _ptr(self.tipo), _ptr(self.a), _ptr(out))
        return out

    def forces_faithful(self):
        out = np.zeros(3, self.dtype)
        getattr(lib(), f"orc_forces_faithful_{self.sfx}")(self.nx, self.ny, self.nz, _ptr(self.tipo), _ptr(self.a), _ptr(out))
        return out

    def mass(self):
        return getattr(lib(), f"orc_mass_{self.sfx}")(self.nx, self.ny, self.nz, _ptr(self.tipo), _ptr(self.a))


def voxelize(pos, idx, dims, banda=1.5, selar=True, with_sdf=True):
    nx, ny, nz = dims
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
    idx = np.ascontiguousarray(idx, np.uint32).reshape(-1)
    N = nx * ny * nz
    tipo = np.zeros(N, np.uint8)
    sdf = np.zeros(N, np.float32) if with_sdf else None
    st = OrcVoxStats()
    lib().orc_voxelize(_ptr(pos), pos.size // 3, _ptr(idx), idx.size // 3, nx, ny, nz, banda, 1 if selar else 0,
                       _ptr(tipo), _ptr(sdf), C.byref(st))
    stats = {k: getattr(st, k) for k, _ in OrcVoxStats._fields_ if not k.startswith("_")}
    return tipo, sdf, stats


def rasterize(pos, idx, dims, banda=1.5):
    nx, ny, nz = dims
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
    idx = np.ascontiguousarray(idx, np.uint32).reshape(-1)
    N = nx * ny * nz
    flags = np.zeros(N, np.uint8)
    d2 = np.zeros(N, np.float32)
    fora = lib().orc_rasterize(_ptr(pos), _ptr(idx), idx.size // 3, nx, ny, nz, banda, _ptr(flags), _ptr(d2))
    return flags, d2, fora


def montar_tipos(dims, corpo=None, esteira=True, fracao=0.18):
    nx, ny, nz = dims
    tipo = np.zeros(nx * ny * nz, np.uint32)
    s0, s1 = C.c_double(), C.c_double()
    c = None if corpo is None else np.ascontiguousarray(corpo, np.uint8).reshape(-1)
    lib().orc_montar_tipos(nx, ny, nz, _ptr(c), 1 if esteira else 0, fracao, _ptr(tipo), C.byref(s0), C.byref(s1))
    return tipo, {"inicio": s0.value, "comprimento": s1.value}


def area_frontal_corpo(corpo, dims):
    nx, ny, nz = dims
    c = np.ascontiguousarray(corpo, np.uint8).reshape(-1)
    return int(lib().orc_area_frontal_corpo(_ptr(c), nx, ny, nz))


def corpo_analitico(dims, tipo, cx, cy, cz, raio):
    nx, ny, nz = dims
    out = np.zeros(nx * ny * nz, np.uint8)
    lib().orc_corpo_analitico(nx, ny, nz, 0 if tipo == "esfera" else 1, cx, cy, cz, raio, _ptr(out))
    return out
