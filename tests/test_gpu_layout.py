"""The in-place set's AoSoA layout (blocks of 32 cells along x for fp32, 64
for the 16-bit forms, the 19 slots of a block one after the other, rows
padded to a multiple of the block), used whenever the step is the FAST
in-place one with fp32 arithmetic.  The layout is
internal: it must give exactly the states the SoA layout and the oracle
give, in every cell class, for the plain step, the fused force, both
closure engines and checkpoints."""
import numpy as np
import pytest

from tests.cases import all_types_tunnel, random_state

pytestmark = pytest.mark.gpu

CFG = dict(omegaPlus=1.85, lesCs=0.12, inletU=[0.05, 0.0, 0.01], beltU=[0.05, 0.0, 0.0], espessuraCL=2)


def _pair(storage, soa_too=True, nx=64):
    from cfd__gb300 import SolverCUDA
    grade, tipo, esp = all_types_tunnel(nx=nx, ny=24, nz=20)
    g0 = random_state(int(np.prod(list(grade.values()))), seed=21)
    out = []
    for soa in ((False, True) if soa_too else (False,)):
        s = SolverCUDA(grade, storage=storage, soa=soa)
        # AoSoA blocks: 64 cells for the 16-bit forms (layout 3), 32 for fp32 (2)
        assert s.info()["layout"] == (0 if soa else (3 if storage != "f32" else 2))
        s.definirTipos(tipo)
        s.configurar(**CFG, esponja=esp)
        s.definirPopulacoes(g0)
        out.append(s)
    return grade, tipo, esp, g0, out


@pytest.mark.parametrize("storage,nx", [("f32", 64), ("f16s", 64), ("bf16s", 64), ("f16s", 96), ("f32", 40),
                                        ("f16sr", 40)])
def test_aos_step_bit_exact_against_oracle(native, storage, nx):
    """nx = 64: whole blocks; nx = 96 (16-bit, blocks of 64) and 40: rows
    padded to a multiple of the block, the last block partly empty."""
    from oracle import oracle as O
    grade, tipo, esp, g0, (s,) = _pair(storage, soa_too=False, nx=nx)
    dt, q = {"f32": (np.float32, 0), "f16s": (np.float32, 1), "bf16s": (np.float32, 2),
             "f16sr": (np.float32, 4)}[storage]
    o = O.Lattice((grade["nx"], grade["ny"], grade["nz"]), dtype=dt, storage=q, nthreads=8, fast=True)
    o.set_types(tipo)
    o.configure(omega_plus=CFG["omegaPlus"], les_cs=CFG["lesCs"], inlet_u=CFG["inletU"], belt_u=CFG["beltU"],
                sponge_start=esp["inicio"], sponge_len=esp["comprimento"], bl_thickness=CFG["espessuraCL"])
    o.set_populations(g0)
    fl = ~np.isin(tipo, [1, 4, 7])
    for n in (1, 1, 9, 30):
        s.passo(n)
        o.step(n, macros=True)
        assert np.array_equal(s.lerPopulacoes()[:, fl], o.populations().reshape(19, -1)[:, fl]), (storage, s.passos)
    assert np.array_equal(s.lerMacros(), o.macros)
    fo = o.forces()
    np.testing.assert_allclose(s.medirForcas(), fo, rtol=1e-12, atol=1e-12 * np.abs(fo).max() + 1e-15)
    s.atualizarMacros()
    assert np.array_equal(s.lerMacros(), o.update_macros(zero_solids=True))
    np.testing.assert_allclose(s.massa(), o.mass(), rtol=1e-12, atol=1e-13)
    s.destruir()


@pytest.mark.parametrize("storage", ["f32", "f16s"])
def test_aos_equals_soa_with_fused_force(native, storage):
    grade, tipo, esp, g0, (a, b) = _pair(storage)
    fl = ~np.isin(tipo, [1, 4, 7])
    fa = a.passoComForcas(25)
    fb = b.passoComForcas(25)
    assert np.array_equal(a.lerPopulacoes()[:, fl], b.lerPopulacoes()[:, fl])
    np.testing.assert_allclose(fa, fb, rtol=1e-12, atol=1e-12 * np.abs(fb).max() + 1e-15)
    a.passo(7)
    b.passo(7)
    assert np.array_equal(a.lerPopulacoes()[:, fl], b.lerPopulacoes()[:, fl])
    for s in (a, b):
        s.destruir()


@pytest.mark.parametrize("storage,motor,every", [("f32", 0, 1), ("f32", 1, 1), ("f32", 0, 4), ("f16s", 0, 1),
                                                 ("f16s", 1, 1), ("f16sr", 1, 4)])
def test_aos_closure_equals_soa(native, storage, motor, every):
    """The closure steps address either layout (blocks of 32 cells for fp32,
    64 for the 16-bit forms): same states bit for bit."""
    import os

    from cfd__gb300.fecho import carregar
    p = carregar(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cfd__gb300", "pesos",
                              "fecho_coef.npz"))
    grade, tipo, esp, g0, (a, b) = _pair(storage)
    fl = ~np.isin(tipo, [1, 4, 7])
    for s in (a, b):
        s.configurar(**CFG, esponja=esp, closure=every)
        s.definirFecho(p)
        s.motorFecho(motor)
        s.definirPopulacoes(g0)
        s.passo(9)
    assert np.array_equal(a.lerPopulacoes()[:, fl], b.lerPopulacoes()[:, fl])
    assert a.estatisticasFecho() == b.estatisticasFecho()
    for s in (a, b):
        s.destruir()


def test_aos_checkpoint_round_trip(native):
    grade, tipo, esp, g0, (a, b) = _pair("f16s")
    fl = ~np.isin(tipo, [1, 4, 7])
    a.passo(5)
    blob = a.salvarEstado()
    a.passo(6)
    ref = a.lerPopulacoes()[:, fl]
    b2 = _pair("f16s", soa_too=False)[4][0]
    b2.carregarEstado(blob)
    b2.passo(6)
    assert np.array_equal(b2.lerPopulacoes()[:, fl], ref)
    from cfd__gb300._native import LbmError
    with pytest.raises(LbmError, match="layout"):
        b.carregarEstado(blob)          # an SoA context refuses an AoSoA checkpoint
    for s in (a, b, b2):
        s.destruir()


@pytest.mark.parametrize("storage", ["f32", "f16s", "bf16s"])
def test_soa_addressing_variants_equal(native, storage):
    """The SoA step's addressing variants (lbm_set_launch 8: slot pointers,
    20: 32-bit slot offsets, 21: base + slot x N) give the same states bit
    for bit, with the fused force as well (which runs the default)."""
    from cfd__gb300 import SolverCUDA
    grade, tipo, esp = all_types_tunnel(nx=70, ny=24, nz=20)
    g0 = random_state(int(np.prod(list(grade.values()))), seed=33)
    fl = ~np.isin(tipo, [1, 4, 7])
    out = []
    for code in (8, 20, 21):
        s = SolverCUDA(grade, storage=storage, soa=True)
        s.definirTipos(tipo)
        s.configurar(**CFG, esponja=esp)
        s.definirBloco(64, code)
        s.definirPopulacoes(g0)
        s.passo(11)
        s.passoComForcas(3)
        s.passo(4)
        out.append(s.lerPopulacoes()[:, fl])
        s.destruir()
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])
