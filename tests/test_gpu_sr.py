"""The stochastically rounded 16-bit storage forms (LBM_F16SR, LBM_BF16SR)
against the oracle, which restates the rounding hash and the truncation:
bit-exact in every cell class, in both layouts, in the FAST and STRICT
arithmetic, with the fused force; a checkpoint continues the same rounding
sequence; the forms refuse the ping-pong set."""
import numpy as np
import pytest

from tests.cases import all_types_tunnel, random_state

pytestmark = pytest.mark.gpu

ORC = {"f16sr": 4, "bf16sr": 5}


def _cfg(esp, bl=2):
    return dict(omegaPlus=1.85, lesCs=0.12, inletU=[0.05, 0.0, 0.01], beltU=[0.05, 0.0, 0.0], esponja=esp,
                espessuraCL=bl)


def _pair(storage, soa, strict, bl):
    from cfd__gb300 import SolverCUDA
    from oracle import oracle as O
    grade, tipo, esp = all_types_tunnel(nx=64, ny=24, nz=20)
    cfg = _cfg(esp, bl)
    g0 = random_state(int(np.prod(list(grade.values()))), seed=17)
    s = SolverCUDA(grade, storage=storage, soa=soa, estrito=strict)
    s.definirTipos(tipo)
    s.configurar(**cfg)
    s.definirPopulacoes(g0)
    o = O.Lattice((grade["nx"], grade["ny"], grade["nz"]), dtype=np.float32, storage=ORC[storage], nthreads=8,
                  fast=not strict)
    o.set_types(tipo)
    o.configure(omega_plus=cfg["omegaPlus"], les_cs=cfg["lesCs"], inlet_u=cfg["inletU"], belt_u=cfg["beltU"],
                sponge_start=esp["inicio"], sponge_len=esp["comprimento"], bl_thickness=bl)
    o.set_populations(g0)
    return grade, tipo, g0, s, o


@pytest.mark.parametrize("storage", ["f16sr", "bf16sr"])
@pytest.mark.parametrize("soa", [True, False])
@pytest.mark.parametrize("strict", [False, True])
def test_sr_step_bit_exact(native, storage, soa, strict):
    if strict and not soa:
        pytest.skip("the AoSoA layout is the FAST step's")
    grade, tipo, g0, s, o = _pair(storage, soa, strict, 2)
    assert s.info()["layout"] == (0 if soa else 3)   # AoSoA in blocks of 64 cells
    fl = ~np.isin(tipo, [1, 4, 7])
    for n in (1, 1, 7, 30):
        s.passo(n)
        o.step(n, macros=True)
        gs, go = s.lerPopulacoes()[:, fl], o.populations().reshape(19, -1)[:, fl]
        assert np.array_equal(gs, go), (storage, soa, strict, s.passos, np.abs(gs - go).max())
    assert np.array_equal(s.lerMacros(), o.macros)
    # the fused force: same rounding, force of the state being streamed
    f = s.passoComForcas(3)
    fo = []
    for _ in range(3):
        fo.append(o.forces())
        o.step(1)
    np.testing.assert_allclose(np.asarray(f), np.asarray(fo), rtol=1e-12,
                               atol=1e-12 * np.abs(np.asarray(fo)).max() + 1e-15)
    assert np.array_equal(s.lerPopulacoes()[:, fl], o.populations().reshape(19, -1)[:, fl])
    s.destruir()


def test_sr_differs_from_round_to_nearest(native):
    """The SR form is not the RN form: same start, different states, both
    near each other."""
    from cfd__gb300 import SolverCUDA
    grade, tipo, esp = all_types_tunnel(nx=64, ny=24, nz=20)
    g0 = random_state(int(np.prod(list(grade.values()))), seed=17)
    out = []
    for st in ("f16s", "f16sr"):
        s = SolverCUDA(grade, storage=st)
        s.definirTipos(tipo)
        s.configurar(**_cfg(esp))
        s.definirPopulacoes(g0)
        s.passo(20)
        out.append(s.lerPopulacoes())
        s.destruir()
    fl = ~np.isin(tipo, [1, 4, 7])
    d = np.abs(out[0][:, fl] - out[1][:, fl])
    assert d.max() > 0 and d.max() < 1e-3


def test_sr_checkpoint_continues_the_rounding(native):
    from cfd__gb300 import SolverCUDA
    grade, tipo, esp = all_types_tunnel(nx=64, ny=24, nz=20)
    g0 = random_state(int(np.prod(list(grade.values()))), seed=5)
    a = SolverCUDA(grade, storage="f16sr")
    a.definirTipos(tipo)
    a.configurar(**_cfg(esp))
    a.definirPopulacoes(g0)
    a.passo(5)
    blob = a.salvarEstado()
    a.passo(6)
    b = SolverCUDA(grade, storage="f16sr")
    b.definirTipos(tipo)
    b.configurar(**_cfg(esp))
    b.carregarEstado(blob)
    b.passo(6)
    fl = ~np.isin(tipo, [1, 4, 7])
    assert np.array_equal(a.lerPopulacoes()[:, fl], b.lerPopulacoes()[:, fl])
    for s in (a, b):
        s.destruir()


def test_sr_refusals(native):
    from cfd__gb300 import SolverCUDA
    from cfd__gb300._native import LbmError
    g = {"nx": 32, "ny": 16, "nz": 16}
    with pytest.raises(LbmError, match="ENOTSUP"):
        SolverCUDA(g, storage="f16sr", pingpong=True)


