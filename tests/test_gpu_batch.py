"""Batched tunnels: every tunnel of a batch equals a separate solver, bit for
bit, through the graph-replayed persistent launch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tunnels():
    from cfd__gb300.lote import sorteio_lote
    # five uneven tunnels (small grids from the same generator as the 64-tunnel workload)
    return sorteio_lote(n=5, seed=11, nx_min=32, nx_max=80)


@pytest.mark.parametrize("storage", ["f32", "f16s", "f16sr"])
@pytest.mark.parametrize("tile", [0, 32])
@pytest.mark.parametrize("mode", [0, 1])
def test_batch_equals_separate_solvers(native, storage, tile, mode):
    """f16sr: the stochastic rounding's seeds follow each tunnel's step count
    through the graph replays and the direct launches."""
    from cfd__gb300 import SolverCUDA
    from cfd__gb300.lote import LoteCUDA
    tun = _tunnels()
    lote = LoteCUDA([t[0] for t in tun], storage=storage)
    lote.definirModo(mode)
    solos = []
    for k, (g, tipo, cfg, info) in enumerate(tun):
        lote.definirTipos(k, tipo)
        lote.configurar(k, **cfg)
        if tile:
            lote.definirLadrilho(k, tile)
        s = SolverCUDA(g, storage=storage)
        s.definirTipos(tipo)
        s.configurar(**cfg)
        s.inicializar()
        solos.append(s)
    lote.inicializar()
    for n in (3, 40):          # direct launches, then a 32-step graph replay + 8 direct
        lote.passo(n)
        for s in solos:
            s.passo(n)
    f = lote.medirForcas()
    for k, (g, tipo, cfg, info) in enumerate(tun):
        fl = ~np.isin(tipo, [1, 4, 7])
        a = lote.lerPopulacoes(k)[:, fl]
        b = solos[k].lerPopulacoes()[:, fl]
        assert np.array_equal(a, b), (k, storage, tile)
        fk = np.asarray(solos[k].medirForcas())
        np.testing.assert_allclose(f[k], fk, rtol=1e-12, atol=1e-12 * np.abs(fk).max() + 1e-15)


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_more_tunnels_than_one_launch_holds(native, mode):
    """70 tunnels of one layout class (nx = 32, AoSoA) and 3 of the other: the
    persistent mode needs two launches for the first class (64 descriptors a
    launch) plus one for the second; every tunnel still equals its separate
    solver."""
    from cfd__gb300 import SolverCUDA
    from cfd__gb300.lote import LoteCUDA, sorteio_lote
    tun = sorteio_lote(n=70, seed=5, nx_min=32, nx_max=32) + sorteio_lote(n=3, seed=6, nx_min=48, nx_max=48)
    lote = LoteCUDA([t[0] for t in tun], storage="f32")
    lote.definirModo(mode)
    for k, (g, tipo, cfg, info) in enumerate(tun):
        lote.definirTipos(k, tipo)
        lote.configurar(k, **cfg)
    lote.inicializar()
    lote.passo(35)
    f = lote.medirForcas()
    for k in (0, 63, 64, 69, 70, 72):
        g, tipo, cfg, info = tun[k]
        s = SolverCUDA(g, storage="f32")
        s.definirTipos(tipo)
        s.configurar(**cfg)
        s.inicializar()
        s.passo(35)
        fl = ~np.isin(tipo, [1, 4, 7])
        assert np.array_equal(lote.lerPopulacoes(k)[:, fl], s.lerPopulacoes()[:, fl]), k
        fk = np.asarray(s.medirForcas())
        np.testing.assert_allclose(f[k], fk, rtol=1e-12, atol=1e-12 * np.abs(fk).max() + 1e-15)
        s.destruir()
    lote.destruir()
