"""The autotuners (lbm_autotune, lbm_batch_autotune): they time candidate
launch shapes on copies of the state, so after tuning the state and the step
count are exactly what they were, and stepping with the chosen shape gives
the same states bit for bit as the default shape."""
import numpy as np
import pytest

from tests.cases import all_types_tunnel, random_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nx,storage", [(64, "f32"), (64, "f16s"), (70, "f32")])
def test_autotune_keeps_state_and_results(native, nx, storage):
    from cfd__gb300 import SolverCUDA
    grade, tipo, esp = all_types_tunnel(nx=nx, ny=24, nz=20)
    g0 = random_state(int(np.prod(list(grade.values()))), seed=4)
    cfg = dict(omegaPlus=1.85, lesCs=0.12, inletU=[0.05, 0.0, 0.01], beltU=[0.05, 0.0, 0.0], esponja=esp)
    a, b = SolverCUDA(grade, storage=storage), SolverCUDA(grade, storage=storage)
    for s in (a, b):
        s.definirTipos(tipo)
        s.configurar(**cfg)
        s.definirPopulacoes(g0)
        s.passo(3)
    before = a.lerPopulacoes()
    info0 = a.info()
    choice = a.autoajustar(4)
    assert choice["ms_per_step"] > 0 and choice["block_x"] in (32, 64, 128) and choice["block_y"] in (1, 2, 4)
    assert choice["block_x"] * choice["block_y"] <= 128
    assert np.array_equal(a.lerPopulacoes(), before)
    assert a.info()["steps"] == info0["steps"] and a.info()["parity"] == info0["parity"]
    a.passo(9)
    b.passo(9)
    fl = ~np.isin(tipo, [1, 4, 7])
    assert np.array_equal(a.lerPopulacoes()[:, fl], b.lerPopulacoes()[:, fl])
    # a context of the same grid created later starts with the measured shape
    c = SolverCUDA(grade, storage=storage)
    assert c.info()["block_x"] == choice["block_x"]
    for s in (a, b, c):
        s.destruir()


def test_batch_autotune_keeps_states(native):
    from cfd__gb300 import SolverCUDA
    from cfd__gb300.lote import LoteCUDA, sorteio_lote
    tun = sorteio_lote(n=5, seed=11, nx_min=32, nx_max=80)
    lote = LoteCUDA([t[0] for t in tun], storage="f32")
    solos = []
    for k, (g, tipo, cfg, info) in enumerate(tun):
        lote.definirTipos(k, tipo)
        lote.configurar(k, **cfg)
        s = SolverCUDA(g)
        s.definirTipos(tipo)
        s.configurar(**cfg)
        s.inicializar()
        solos.append(s)
    lote.inicializar()
    lote.passo(5)
    for s in solos:
        s.passo(5)
    esc = lote.autoajustar(32)
    assert esc["mode"] in (0, 1) and esc["resident_ctas_per_sm"] in (6, 8) and esc["ms_per_step"] > 0
    assert all(t in (32, 64, 128) for t in esc["tiles"])
    assert lote.passos == 5
    lote.passo(37)
    for s in solos:
        s.passo(37)
    for k, (g, tipo, cfg, info) in enumerate(tun):
        fl = ~np.isin(tipo, [1, 4, 7])
        assert np.array_equal(lote.lerPopulacoes(k)[:, fl], solos[k].lerPopulacoes()[:, fl]), k
    lote.destruir()
    for s in solos:
        s.destruir()


def test_layout_tuner_sets_the_default(native):
    """lbm_autotune_layout times both layouts and makes the faster one the
    default for solvers of that grid and storage; an explicit flag still
    wins, and the two flags together are refused."""
    from cfd__gb300 import SolverCUDA
    from cfd__gb300._native import LbmError
    g = {"nx": 64, "ny": 32, "nz": 24}
    r = SolverCUDA.autoajustarLayout(g, "f16s", passos=4)
    assert r["layout"] in (0, 3) and r["ms_soa"] > 0 and r["ms_aosoa"] > 0
    s = SolverCUDA(g, storage="f16s")
    assert s.info()["layout"] == r["layout"]
    assert SolverCUDA(g, storage="f16s", soa=True).info()["layout"] == 0
    assert SolverCUDA(g, storage="f16s", soa=False).info()["layout"] == 3   # blocks of 64 cells
    # any nx: the rows are padded to a multiple of the block
    assert SolverCUDA({"nx": 70, "ny": 32, "nz": 24}, storage="f32", soa=False).info()["layout"] == 2
    assert SolverCUDA({"nx": 70, "ny": 32, "nz": 24}, storage="f16s", soa=False).info()["layout"] == 3
    from cfd__gb300 import _native as nat
    import ctypes as C
    h = C.c_void_p()
    dims = nat.Dims(64, 32, 24)
    rc = nat.load().lbm_create(C.byref(dims), nat.F32, nat.FLAG_SOA | nat.FLAG_AOS, C.byref(h))
    with pytest.raises(LbmError, match="EINVAL"):
        nat.check(rc)
