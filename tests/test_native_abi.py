"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute calls: this runs without a GPU)."""
import os
import re

import pytest

from cfd__gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*([a-z_0-9]+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    assert os.path.exists(path)
    lib = _native.load()
    declared = declared_functions()
    assert {"lbm_create", "lbm_step", "lbm_forces"} <= declared
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    assert declared <= set(_native.SIGNATURES), sorted(declared - set(_native.SIGNATURES))


def test_host_validation_without_gpu():
    """Argument checks that fail before any CUDA call."""
    import ctypes as C
    lib = _native.load()
    h = C.c_void_p()
    bad = _native.Dims(0, 4, 4)
    assert lib.lbm_create(C.byref(bad), 0, 0, C.byref(h)) == _native.EINVAL
    assert b"dimensions" in lib.lbm_last_error()
    ok = _native.Dims(4, 4, 4)
    assert lib.lbm_create(C.byref(ok), 9, 0, C.byref(h)) == _native.EINVAL
    assert lib.lbm_create(C.byref(ok), 0, 64, C.byref(h)) == _native.EINVAL
    assert lib.lbm_step(None, 1) == _native.EINVAL


def test_host_validation_of_the_other_entry_points():
    """Null handles and empty inputs of the closure, state, visualisation and
    batch entry points are refused on the host, before any CUDA call."""
    import ctypes as C
    lib = _native.load()
    E = _native.EINVAL
    assert lib.closure_eval(None, None, 0, 0, None) == E
    assert lib.closure_train(None, None, 0, None, None, None) == E
    assert lib.closure_grad(None, None, 0, None, None, None) == E
    assert lib.lbm_set_closure(None, None) == E
    assert lib.lbm_closure_engine(None, 0) == E
    assert lib.lbm_state_bytes(None, None) == E
    assert lib.lbm_save_state(None, None, 0) == E
    assert lib.lbm_load_state(None, None, 0) == E
    assert lib.lbm_read_macros_async(None, None, 0) == E
    assert lib.lbm_macros_ready(None, None) == E
    assert lib.lbm_step_forces_async(None, 1, None, None) == E
    assert lib.lbm_forces_done(None, 1, 0, None) == E
    assert lib.vis_fumaca_create(None, None) == E
    assert lib.vis_fumaca_passo(None, None, None) == E
    assert lib.vis_esteiras_create(None, 0, None) == E
    assert lib.vis_cp_triangulos(None, None, 0, None, 0, C.c_float(0.05), None) == E
    assert lib.lbm_batch_step(None, 1) == E
    assert lib.vox_voxelize(None, 0, None, 0, None, C.c_float(1.5), 1, None, None, None) == E
