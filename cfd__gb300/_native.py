"""ctypes binding of include/lbm.h (and the voxelizer ABI in include/vox.h).

The library is built in-tree by ``cfd__gb300.build.build()``.  There is no CPU
fallback: if the library is missing or cannot be loaded, every solver call
raises ``NativeUnavailable``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

F32, F16S, BF16S, F64, F16SR, BF16SR = 0, 1, 2, 3, 4, 5
FLAG_WRITE_MACROS, FLAG_PINGPONG, FLAG_STRICT, FLAG_SOA, FLAG_AOS = 1, 2, 4, 8, 16

OK, EINVAL, ENOMEM, ECUDA, ETIMEDOUT, ESTATE, ENOTSUP = 0, -1, -2, -3, -4, -5, -6
_NAMES = {EINVAL: "EINVAL", ENOMEM: "ENOMEM", ECUDA: "ECUDA", ETIMEDOUT: "ETIMEDOUT",
          ESTATE: "ESTATE", ENOTSUP: "ENOTSUP"}


class NativeUnavailable(RuntimeError):
    """The sm_103a library is not built or not loadable."""


class LbmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_NAMES.get(code, code)}: {msg}")
        self.code = code


class Dims(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32)]


class Params(C.Structure):
    _fields_ = [
        ("omega_plus", C.c_float), ("magic", C.c_float), ("les_cs", C.c_float),
        ("belt_u", C.c_float * 3), ("inlet_u", C.c_float * 3),
        ("sponge_start", C.c_float), ("sponge_len", C.c_float),
        ("bl_thickness", C.c_float), ("closure", C.c_int32),
    ]


class Info(C.Structure):
    _fields_ = [("n_cells", C.c_int64), ("device_bytes", C.c_int64), ("storage", C.c_int32),
                ("flags", C.c_int32), ("steps", C.c_int64), ("parity", C.c_int32), ("block_x", C.c_int32),
                ("layout", C.c_int32)]


class VoxStats(C.Structure):
    _fields_ = [("n_cells", C.c_int64), ("n_casca", C.c_int64), ("n_dentro", C.c_int64), ("n_solido", C.c_int64),
                ("triangulo_fora", C.c_int64), ("oco_suspeito", C.c_int32), ("flood_iterations", C.c_int32),
                ("n_pairs", C.c_int64), ("n_deferred", C.c_int64), ("ms_raster", C.c_float),
                ("ms_flood", C.c_float), ("ms_total", C.c_float), ("_pad", C.c_float)]


CLOSURE_IN, CLOSURE_H = 6, 32
CLOSURE_NPARAM = CLOSURE_H * CLOSURE_IN + CLOSURE_H + CLOSURE_H * CLOSURE_H + CLOSURE_H + CLOSURE_H + 1


class ClosureWeights(C.Structure):
    _fields_ = [("w1", C.c_float * (CLOSURE_H * CLOSURE_IN)), ("b1", C.c_float * CLOSURE_H),
                ("w2", C.c_float * (CLOSURE_H * CLOSURE_H)), ("b2", C.c_float * CLOSURE_H),
                ("w3", C.c_float * CLOSURE_H), ("b3", C.c_float),
                ("mean", C.c_float * CLOSURE_IN), ("std", C.c_float * CLOSURE_IN),
                ("nu_scale", C.c_float), ("nu_max", C.c_float),
                ("lo", C.c_float * CLOSURE_IN), ("hi", C.c_float * CLOSURE_IN), ("coef", C.c_int32)]


class ClosureCfg(C.Structure):
    _fields_ = [("steps", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float), ("seed", C.c_uint64), ("init", C.c_int32),
                ("_pad", C.c_int32)]


_lib = None
_lock = threading.Lock()

# name -> (restype, argtypes); every entry point declared in include/*.h
SIGNATURES = {
    "lbm_create": (C.c_int, [C.POINTER(Dims), C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "lbm_destroy": (C.c_int, [C.c_void_p]),
    "lbm_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_configure": (C.c_int, [C.c_void_p, C.POINTER(Params)]),
    "lbm_set_types": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_init_equilibrium": (C.c_int, [C.c_void_p]),
    "lbm_set_populations": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_get_populations": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_step": (C.c_int, [C.c_void_p, C.c_int]),
    "lbm_step_forces": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "lbm_step_forces_async": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_int64)]),
    "lbm_forces_done": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, C.POINTER(C.c_int)]),
    "lbm_update_macros": (C.c_int, [C.c_void_p]),
    "lbm_read_macros": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_forces": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_mass": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "lbm_sync": (C.c_int, [C.c_void_p]),
    "lbm_get_info": (C.c_int, [C.c_void_p, C.POINTER(Info)]),
    "lbm_last_error": (C.c_char_p, []),
    "lbm_set_block": (C.c_int, [C.c_void_p, C.c_int]),
    "lbm_set_launch": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "lbm_autotune_layout": (C.c_int, [C.POINTER(Dims), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                      C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "lbm_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                               C.POINTER(C.c_float)]),
    "lbm_forces_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Dims), C.c_void_p, C.c_void_p]),
    "lbm_batch_create": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "lbm_batch_destroy": (C.c_int, [C.c_void_p]),
    "lbm_batch_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_batch_configure": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Params)]),
    "lbm_batch_set_types": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "lbm_batch_init_equilibrium": (C.c_int, [C.c_void_p]),
    "lbm_batch_step": (C.c_int, [C.c_void_p, C.c_int]),
    "lbm_batch_get_populations": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "lbm_batch_forces": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_batch_set_tile": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "lbm_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "lbm_batch_set_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "lbm_batch_get_tile": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "lbm_batch_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_float)]),
    "closure_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(ClosureCfg),
                                C.POINTER(ClosureWeights), C.c_void_p]),
    "closure_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(ClosureWeights),
                               C.POINTER(C.c_float), C.c_void_p]),
    "closure_eval": (C.c_int, [C.POINTER(ClosureWeights), C.c_void_p, C.c_size_t, C.c_int, C.c_void_p]),
    "lbm_closure_engine": (C.c_int, [C.c_void_p, C.c_int]),
    "closure_samples": (C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                  C.c_size_t]),
    "lbm_set_closure": (C.c_int, [C.c_void_p, C.POINTER(ClosureWeights)]),
    "lbm_closure_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "lbm_state_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "lbm_save_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_load_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_read_macros_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lbm_macros_ready": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "vis_fumaca_create": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "vis_fumaca_destroy": (C.c_int, [C.c_void_p]),
    "vis_fumaca_limpar": (C.c_int, [C.c_void_p]),
    "vis_fumaca_passo": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "vis_fumaca_ler": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "vis_fumaca_definir": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "vis_esteiras_create": (C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(C.c_void_p)]),
    "vis_esteiras_destroy": (C.c_int, [C.c_void_p]),
    "vis_esteiras_definir": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "vis_esteiras_ler": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "vis_esteiras_passo": (C.c_int, [C.c_void_p, C.c_float, C.c_int, C.c_uint32]),
    "vis_rasantes_passo": (C.c_int, [C.c_void_p, C.c_float, C.c_int, C.c_uint32, C.c_float]),
    "vis_fumaca_render": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]),
    "vis_cp_triangulos": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_float, C.c_void_p]),
    "vox_voxelize": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.POINTER(Dims), C.c_float, C.c_int,
                               C.c_void_p, C.c_void_p, C.POINTER(VoxStats)]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the library (optionally building it first).  Raises NativeUnavailable."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise NativeUnavailable(
                    f"{path} is missing: build it with cfd__gb300.build.build() (nvcc, sm_103a)")
            _build.build()
        try:
            L = C.CDLL(path)
        except OSError as e:  # pragma: no cover - depends on the machine
            raise NativeUnavailable(f"cannot load {path}: {e}") from e
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def check(rc: int) -> None:
    if rc != OK:
        msg = _lib.lbm_last_error().decode("utf-8", "replace") if _lib is not None else ""
        raise LbmError(rc, msg)


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
