"""lbm_forces_noalloc: the force entry point for callers that cannot allocate
device memory (real-time loops, hosts that own every buffer).

Collected last on purpose (test_zz_*): if it fails, a run that stops at the
first failure has already run every other test.  It passes alone in a fresh
process and after the rest of the suite.  The test itself owns the device
buffers (torch), as such a caller would; the entry point allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, nat, pop, tipo, dims, out, stream):
    return lib.lbm_forces_noalloc(C.c_void_p(pop.data_ptr()), C.c_void_p(tipo.data_ptr()), C.byref(dims),
                                  C.c_void_p(out.data_ptr()), C.c_void_p(stream))


def test_noalloc_force_matches_lbm_forces_on_two_calls(native):
    import torch

    from cfd__gb300 import SolverCUDA
    from cfd__gb300 import _native as nat
    from tests.cases import random_state, sphere_tunnel

    lib = nat.load()
    grade, corpo, tipo, esp = sphere_tunnel(64, 32, 32, r=6, cx=20)
    dims = nat.Dims(64, 32, 32)
    s = SolverCUDA(grade)
    s.definirTipos(tipo)
    s.configurar(omegaPlus=1.8, lesCs=0.1, inletU=[0.05, 0, 0], esponja=esp)
    s.definirPopulacoes(random_state(s.N, seed=21))
    d_tipo = torch.tensor(tipo.astype(np.uint8), device="cuda")
    out = torch.empty(3, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):                      # two calls in a row, on two different states
        if call == 1:
            s.passo(7)
        ref = np.array(s.medirForcas())        # the existing entry point (lbm_forces)
        pop = torch.tensor(s.lerPopulacoes().astype(np.float32).reshape(-1), device="cuda")
        out.fill_(float("nan"))
        assert _call(lib, nat, pop, d_tipo, dims, out, stream) == nat.OK, lib.lbm_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-15)
    s.destruir()


def test_noalloc_rejects_grids_beyond_its_scratch(native):
    import torch

    from cfd__gb300 import _native as nat

    lib = nat.load()
    tiny = torch.zeros(8, dtype=torch.float32, device="cuda")
    tipo = torch.zeros(8, dtype=torch.uint8, device="cuda")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    big = nat.Dims(4, 320, 256)                # ny*nz = 81920 > 65536 rows
    assert _call(lib, nat, tiny, tipo, big, out, 0) == nat.EINVAL
    assert b"65536" in lib.lbm_last_error()
