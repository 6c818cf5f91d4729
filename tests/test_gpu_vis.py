"""Visualisation compute (include/lbm_vis.h) on the GPU against
oracle/vis_oracle.py, on the macros of a real solver state.

Smoke: bit-exact where the rake is off; with the rake on, exp() of the CUDA
library and of numpy may differ in the last place, so the emitted voxels are
allowed one fp16 unit.  Particles: bit-exact (integer hash, IEEE fp32)."""
import numpy as np
import pytest

from oracle import vis_oracle as V
from tests.cases import all_types_tunnel, random_state

pytestmark = pytest.mark.gpu


def _state(seed=41):
    from cfd__gb300 import SolverCUDA
    grade, tipo, esp = all_types_tunnel()
    s = SolverCUDA(grade)
    s.definirTipos(tipo)
    s.configurar(omegaPlus=1.9, lesCs=0.12, inletU=[0.05, 0, 0.01], beltU=[0.05, 0, 0], esponja=esp)
    s.definirPopulacoes(random_state(int(np.prod(list(grade.values()))), seed=seed))
    s.passo(3)
    s.atualizarMacros()
    mac = s.lerMacros().reshape(grade["nz"], grade["ny"], grade["nx"], 4)
    return s, grade, np.asarray(tipo).reshape(grade["nz"], grade["ny"], grade["nx"]), mac


R_OFF = {"x": -100.0, "passo_y": 4.0, "passo_z": 4.0, "raio": 1.0, "y0": 1.0, "y1": 10.0, "z0": 1.0, "z1": 10.0}


def test_smoke_step_bit_exact_without_rake(native):
    from cfd__gb300.visual import Fumaca
    s, grade, tipo, mac = _state()
    f = Fumaca(s)
    rng = np.random.default_rng(1)
    cur = rng.uniform(0, 3, f.shape).astype(np.float16)
    f.definir(cur)
    F = {"dt": 30.0, "dissipacao": 0.999, "taxa": 2.4, "avanco": 1.5}
    for _ in range(3):
        ref = V.fumaca_passo(cur, mac, tipo, R_OFF, F)
        f.passo(R_OFF, **F)
        got = f.ler()
        assert np.array_equal(got, ref), np.abs(got.astype(np.float32) - ref.astype(np.float32)).max()
        cur = got
    f.destruir()
    s.destruir()


def test_smoke_step_with_rake(native):
    from cfd__gb300.visual import Fumaca, posicionar_rake
    s, grade, tipo, mac = _state(42)
    f = Fumaca(s)
    ext = {"min": [14.0, 8.0, 6.0], "tamanho": [9.0, 9.0, 9.0], "centro": [18.0, 12.0, 10.0]}
    R = posicionar_rake(grade["ny"], grade["nz"], ext, colunas=5, linhas=4)
    F = {"dt": 20.0, "dissipacao": 0.999, "taxa": 2.4, "avanco": 1.0}
    cur = np.zeros(f.shape, np.float16)
    painted = 0
    for _ in range(4):
        ref = V.fumaca_passo(cur, mac, tipo, R, F)
        f.passo(R, **F)
        got = f.ler()
        g32, r32 = got.astype(np.float32), ref.astype(np.float32)
        tol = np.abs(r32) * 2.0 ** -10 + 2.0 ** -24
        assert (np.abs(g32 - r32) <= tol).all()
        assert np.mean(got == ref) > 0.999
        painted = int((got > 0).sum())
        cur = got
    assert painted > 100
    f.destruir()
    s.destruir()


def test_particles_bit_exact(native):
    from cfd__gb300.visual import Esteiras
    s, grade, tipo, mac = _state(43)
    n = 5000
    rng = np.random.default_rng(2)
    parts = np.zeros((n, 8), np.float32)
    parts[:, 0] = rng.uniform(-1, grade["nx"] + 1, n)
    parts[:, 1] = rng.uniform(-1, grade["ny"] + 1, n)
    parts[:, 2] = rng.uniform(-1, grade["nz"] + 1, n)
    parts[:, 3] = rng.uniform(-5, 300, n)
    e = Esteiras(s, n)
    e.definir(parts)
    for quadro in range(5):
        parts = V.esteiras_passo(parts, mac, 12.5, 6, quadro)
        e.passo(12.5, 6, quadro)
        got = e.ler()
        assert np.array_equal(got, parts)
    assert (parts[:, 7] == 0).any() and (parts[:, 7] == 1).any()
    e.destruir()
    s.destruir()


def test_vis_argument_checks(native):
    from cfd__gb300._native import LbmError
    from cfd__gb300.visual import Esteiras, Fumaca
    s, grade, tipo, mac = _state(44)
    f = Fumaca(s)
    with pytest.raises(LbmError, match="EINVAL"):
        f.definir(np.zeros(10, np.float16))
    e = Esteiras(s, 10)
    with pytest.raises(LbmError, match="EINVAL"):
        e.passo(1.0, 0)
    f.destruir()
    e.destruir()
    s.destruir()


def test_ground_streaks_bit_exact(native):
    from cfd__gb300.visual import Esteiras
    s, grade, tipo, mac = _state(45)
    n = 3000
    rng = np.random.default_rng(3)
    parts = np.zeros((n, 8), np.float32)
    parts[:, 0] = rng.uniform(0, grade["nx"], n)
    parts[:, 1] = rng.uniform(0, grade["ny"], n)
    parts[:, 2] = rng.uniform(0, 4, n)
    parts[:, 3] = rng.uniform(-5, 300, n)
    e = Esteiras(s, n)
    e.definir(parts)
    for quadro in range(4):
        parts = V.esteiras_passo(parts, mac, 9.0, 3, quadro, rasantes=True, altura=5.5)
        e.passo_rasantes(9.0, 3, quadro, altura=5.5)
        assert np.array_equal(e.ler(), parts)
    e.destruir()
    s.destruir()


def test_smoke_render_matches_oracle(native):
    from cfd__gb300.visual import Fumaca, camera_orbita
    s, grade, tipo, mac = _state(46)
    f = Fumaca(s)
    rng = np.random.default_rng(5)
    vol = np.zeros(f.shape, np.float16)
    vol[2:12, 5:18, 8:30] = rng.uniform(0, 1.5, (10, 13, 22)).astype(np.float16)
    f.definir(vol)
    inv, eye = camera_orbita(grade["nx"], grade["ny"], grade["nz"], aspecto=64 / 36)
    kw = dict(largura=64, altura=36, densidade=70.0, g=0.45, passos=48, passos_luz=5, luz=(-0.35, 0.55, 0.76),
              intensidade=1.0, quadro=3)
    got = f.render(inv, eye, **kw)
    ref = V.render(vol, inv, eye, kw["largura"], kw["altura"], kw["densidade"], kw["g"], kw["passos"],
                   kw["passos_luz"], kw["luz"], kw["intensidade"], kw["quadro"])
    assert (ref[..., 3] > 0.05).sum() > 50
    close = np.abs(got - ref) <= 1e-4 + 1e-3 * np.abs(ref)
    assert close.mean() > 0.99, close.mean()
    assert np.abs(got - ref).max() < 2e-2
    f.destruir()
    s.destruir()


def test_surface_cp_bit_exact(native):
    from cfd__gb300.geometry import superelipsoide
    from cfd__gb300.visual import cp_superficie
    s, grade, tipo, mac = _state(47)
    pos, idx = superelipsoide(6.0, 4.0, 3.0, 2.5, 3.0, 600, 0.0, 5)
    pos = (pos + np.array([grade["nx"] * 0.35, grade["ny"] * 0.5, grade["nz"] * 0.5], np.float32)).astype(np.float32)
    got = cp_superficie(s, pos, idx, 0.05)
    ref = V.cp_triangulos(pos, idx, mac, tipo, 0.05)
    assert got.shape == (idx.shape[0],) and np.isfinite(got).all()
    assert np.array_equal(got, ref)
    s.destruir()
