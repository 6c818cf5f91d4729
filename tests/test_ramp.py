"""The inlet ramp of the solver class (SolverWebGPU.rampa / fatorRampa / passo,
src/backend/webgpu/solver.js:323-335, :395-415), on the CPU: the smoothstep
factor, and that passo() advances the ramp and calls the callback (which
re-configures the inlet) before it dispatches the steps.

The solver's library is replaced by a recorder, so no GPU is needed; the
GPU test in test_gpu_ramp.py runs the same ramp against the oracle.
"""
import ctypes as C

import pytest

from cfd__gb300 import _native as nat


class _Recorder:
    """Stands in for the CUDA library: records configure and step calls."""

    def __init__(self, log):
        self.log = log

    def lbm_configure(self, h, p):
        self.log.append(("configure", round(float(p._obj.inlet_u[0]), 9)))
        return nat.OK

    def lbm_step(self, h, n):
        self.log.append(("step", int(n)))
        return nat.OK

    def lbm_init_equilibrium(self, h):
        self.log.append(("init",))
        return nat.OK


def _solver(log, nx=40):
    from cfd__gb300.solver import SolverCUDA
    s = SolverCUDA.__new__(SolverCUDA)
    s._lib = _Recorder(log)
    s._h = C.c_void_p(1)
    s.nx, s.ny, s.nz = nx, 8, 8
    s.N = nx * 64
    s.passos = 0
    s._frente = "A"
    s.cfg = None
    s.offsetForca = None
    s._rampa = None
    return s


def smoothstep(t):
    return t * t * (3 - 2 * t)


def test_factor_is_one_without_ramp():
    s = _solver([])
    assert s.fatorRampa == 1.0


@pytest.mark.parametrize("atual,passos", [(0, 100), (1, 100), (25, 100), (50, 100), (99, 100), (7, 13)])
def test_factor_is_smoothstep(atual, passos):
    s = _solver([])
    s.rampa(passos, None)
    s._rampa["atual"] = atual
    t = atual / passos
    assert s.fatorRampa == smoothstep(t)
    # symmetric about the midpoint, monotone, 0 at the start
    assert smoothstep(0.0) == 0.0 and smoothstep(1.0) == 1.0
    assert abs(smoothstep(t) + smoothstep(1 - t) - 1.0) < 1e-15


def test_factor_ends_at_one():
    s = _solver([])
    s.rampa(10, None)
    s._rampa["atual"] = 10
    assert s.fatorRampa == 1.0
    s._rampa["atual"] = 12
    assert s.fatorRampa == 1.0


def test_passo_applies_before_dispatch():
    """passo(n): the ramp advances by n, the callback gets the new factor and
    re-configures, and only then are the n steps enqueued; once the ramp is
    over the callback is no longer called."""
    log = []
    s = _solver(log)
    u = 0.06

    def aplicar(f):
        log.append(("aplicar", f))
        s.configurar(omegaPlus=1.9, lesCs=0.1, inletU=[u * f, 0.0, 0.0])

    s.rampa(4, aplicar)
    for n in (1, 2, 1, 1, 3):
        s.passo(n)
    f1, f3 = smoothstep(1 / 4), smoothstep(3 / 4)
    assert log == [
        ("aplicar", f1), ("configure", round(float(C.c_float(u * f1).value), 9)), ("step", 1),
        ("aplicar", f3), ("configure", round(float(C.c_float(u * f3).value), 9)), ("step", 2),
        ("aplicar", 1.0), ("configure", round(float(C.c_float(u).value), 9)), ("step", 1),
        ("step", 1),
        ("step", 3),
    ]
    assert s.passos == 8


def test_inicializar_restarts_the_ramp():
    log = []
    s = _solver(log)
    seen = []
    s.rampa(10, seen.append)
    s.passo(4)
    s.inicializar()
    assert s._rampa["atual"] == 0 and s.passos == 0
    s.passo(1)
    assert seen == [smoothstep(0.4), smoothstep(0.1)]


def test_frente_alternates_per_step():
    """The reference swaps its A/B sets once per dispatched step
    (src/backend/webgpu/solver.js:405-410); inicializar leaves the state in B."""
    s = _solver([])
    s.inicializar()
    assert s.frente == "B"
    s.passo(1)
    assert s.frente == "A"
    s.passo(2)
    assert s.frente == "A"
    s.passo(3)
    assert s.frente == "B"
