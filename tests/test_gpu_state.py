"""State I/O (include/lbm_state.h): a checkpoint restored into a fresh
context continues bit for bit; mismatched checkpoints are refused; the
asynchronous macros read-back lands the same field as the synchronous one.
Solid cells carry no state (nothing reads them; in the ping-pong layout their
slots hold whatever the back set held), so comparisons cover the other cells."""
import time

import numpy as np
import pytest

from tests.cases import all_types_tunnel, random_state

pytestmark = pytest.mark.gpu

CFG = dict(omegaPlus=1.9, lesCs=0.12, inletU=[0.05, 0.0, 0.01], beltU=[0.05, 0.0, 0.0])


def _solver(grade, tipo, esp, storage="f32", pingpong=False, **kw):
    from cfd__gb300 import SolverCUDA
    s = SolverCUDA(grade, storage=storage, pingpong=pingpong, escrever_macros=False)
    s.definirTipos(tipo)
    s.configurar(**CFG, esponja=esp, **kw)
    return s


@pytest.mark.parametrize("storage", ["f32", "f16s", "bf16s", "f64"])
@pytest.mark.parametrize("pingpong", [False, True])
def test_checkpoint_continues_bit_exact(native, storage, pingpong):
    grade, tipo, esp = all_types_tunnel()
    g0 = random_state(int(np.prod(list(grade.values()))), seed=31)
    a = _solver(grade, tipo, esp, storage, pingpong)
    a.definirPopulacoes(g0)
    a.passo(7)                      # odd parity
    blob = a.salvarEstado()
    a.passo(9)
    ref = a.lerPopulacoes()
    b = _solver(grade, tipo, esp, storage, pingpong)
    b.carregarEstado(blob)
    assert b.passos == 7 and b.info()["steps"] == 7
    b.passo(9)
    live = ~np.isin(np.asarray(tipo).reshape(-1), [1, 4, 7])
    assert np.array_equal(b.lerPopulacoes()[:, live], ref[:, live])
    a.destruir()
    b.destruir()


def test_checkpoint_refuses_mismatch(native):
    from cfd__gb300._native import LbmError
    grade, tipo, esp = all_types_tunnel()
    a = _solver(grade, tipo, esp)
    a.inicializar()
    blob = a.salvarEstado()
    # the set as it sits in device memory: AoSoA rows padded to the block width
    lay = a.info()["layout"]
    bw = {2: 32, 3: 64}.get(lay, 1)
    nxp = -(-grade["nx"] // bw) * bw
    assert len(blob) == 48 + 19 * nxp * grade["ny"] * grade["nz"] * 4
    for kw in (dict(storage="f16s"), dict(pingpong=True)):
        b = _solver(grade, tipo, esp, **kw)
        with pytest.raises(LbmError, match="EINVAL"):
            b.carregarEstado(blob)
        b.destruir()
    from cfd__gb300 import SolverCUDA
    other = SolverCUDA({"nx": grade["nx"] + 2, "ny": grade["ny"], "nz": grade["nz"]})
    with pytest.raises(LbmError, match="EINVAL"):
        other.carregarEstado(blob)
    other.destruir()
    b = _solver(grade, tipo, esp)
    with pytest.raises(LbmError, match="EINVAL"):
        b.carregarEstado(blob[:-4])
    bad = bytearray(blob)
    bad[0] ^= 0xFF
    with pytest.raises(LbmError, match="EINVAL"):
        b.carregarEstado(bytes(bad))
    b.destruir()
    a.destruir()


def test_checkpoint_with_held_closure_at_an_evaluation_step(native):
    """Closure evaluated every 4th step: a checkpoint taken after 8 steps
    (the next step evaluates the network in both runs) continues bit for bit."""
    from cfd__gb300 import fecho
    grade, tipo, esp = all_types_tunnel()
    g0 = random_state(int(np.prod(list(grade.values()))), seed=32)
    p = fecho.pesos_vazios()
    rng = np.random.default_rng(4)
    p["w1"] = rng.uniform(-1, 1, (32, 6)).astype(np.float32)
    p["w3"] = rng.uniform(-0.3, 0.3, 32).astype(np.float32)
    p["b1"] = np.full(32, 0.1, np.float32)
    p["nu_scale"] = 1e-3
    a = _solver(grade, tipo, esp, closure=4)
    a.definirFecho(p)
    a.definirPopulacoes(g0)
    a.passo(8)
    blob = a.salvarEstado()
    a.passo(10)
    ref = a.lerPopulacoes()
    b = _solver(grade, tipo, esp, closure=4)
    b.definirFecho(p)
    b.carregarEstado(blob)
    b.passo(10)
    live = ~np.isin(np.asarray(tipo).reshape(-1), [1, 4, 7])
    assert np.array_equal(b.lerPopulacoes()[:, live], ref[:, live])
    a.destruir()
    b.destruir()


def test_async_macros_match_sync(native):
    grade, tipo, esp = all_types_tunnel()
    g0 = random_state(int(np.prod(list(grade.values()))), seed=33)
    s = _solver(grade, tipo, esp)
    s.definirPopulacoes(g0)
    s.passo(5)
    dst = s.lerMacrosAssincrono()
    t0 = time.time()
    while not s.macrosProntos():
        assert time.time() - t0 < 30
        time.sleep(0.001)
    s.atualizarMacros()
    assert np.array_equal(dst, s.lerMacros().reshape(-1))
    s.destruir()


def test_async_forces_match_sync(native):
    """lbm_step_forces_async gives the forces lbm_step_forces gives, with
    several calls in flight and tickets awaited out of order."""
    from cfd__gb300._native import LbmError
    grade, tipo, esp = all_types_tunnel()
    g0 = random_state(int(np.prod(list(grade.values()))), seed=34)
    a = _solver(grade, tipo, esp)
    a.definirPopulacoes(g0)
    ref = np.concatenate([a.passoComForcas(3), a.passoComForcas(1), a.passoComForcas(5)])
    b = _solver(grade, tipo, esp)
    b.definirPopulacoes(g0)
    t1 = b.passoComForcasAssincrono(3)
    t2 = b.passoComForcasAssincrono(1)
    t3 = b.passoComForcasAssincrono(5)
    f3 = b.aguardarForcas(t3)
    f1 = b.aguardarForcas(t1, esperar=False)     # older than t3: landed
    f2 = b.aguardarForcas(t2)
    got = np.concatenate([f1, f2, f3])
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max() + 1e-15)
    assert np.array_equal(a.lerPopulacoes(), b.lerPopulacoes())
    with pytest.raises(LbmError, match="EINVAL"):
        b.aguardarForcas(99)
    a.destruir()
    b.destruir()
