"""CUDA step vs the CPU oracle on identical inputs.

fp32: bit-exact (the kernels are built with -fmad=false and IEEE div/sqrt and
follow the shader's operation order).  The same holds for the fp64 reference form and
for the 16-bit storage forms, whose rounding the oracle reproduces.  The
parity bar for this path (fp32 populations within 1e-5 relative after 1000 steps) is
therefore met with margin; tests assert equality.
Solid cells carry no state in the reference (nothing reads them), so
population comparisons cover the non-solid cells.
"""
import numpy as np
import pytest

from tests.cases import all_types_tunnel, random_state, sphere_tunnel

pytestmark = pytest.mark.gpu

STORAGES = {"f32": (np.float32, 0), "f64": (np.float64, 0), "f16s": (np.float32, 1), "bf16s": (np.float32, 2)}


def _solver(grade, storage="f32", pingpong=False, strict=False):
    from cfd__gb300 import SolverCUDA
    return SolverCUDA(grade, storage=storage, pingpong=pingpong, estrito=strict)


def _oracle(grade, storage, strict=False):
    from oracle import oracle as O
    dt, q = STORAGES[storage]
    return O.Lattice((grade["nx"], grade["ny"], grade["nz"]), dtype=dt, storage=q, nthreads=8, fast=not strict)


def _cfg(esp, **kw):
    base = dict(omegaPlus=1.85, lesCs=0.12, inletU=[0.05, 0.0, 0.01], beltU=[0.05, 0.0, 0.0], esponja=esp,
                espessuraCL=0)
    base.update(kw)
    return base


def _ocfg(c):
    return dict(omega_plus=c["omegaPlus"], les_cs=c["lesCs"], inlet_u=c["inletU"], belt_u=c["beltU"],
                sponge_start=c["esponja"]["inicio"], sponge_len=c["esponja"]["comprimento"],
                bl_thickness=c["espessuraCL"])


def _fluid(tipo):
    t = np.asarray(tipo).reshape(-1)
    return ~np.isin(t, [1, 4, 7])


@pytest.mark.parametrize("storage", ["f32", "f64", "f16s", "bf16s"])
@pytest.mark.parametrize("pingpong", [False, True])
@pytest.mark.parametrize("cs", [0.12, 0.0])
@pytest.mark.parametrize("strict", [False, True])
@pytest.mark.parametrize("bl", [0, 2, 7])
def test_step_bit_exact_all_cell_classes(native, storage, pingpong, cs, strict, bl):
    """bl: the inlet boundary-layer thickness (espessuraCL).  The app sets
    round(0.12 nz) for every tunnel without a belt (index.html:719), here
    round(0.12 * 20) = 2; 7 covers a thicker layer."""
    grade, tipo, esp = all_types_tunnel()
    cfg = _cfg(esp, lesCs=cs, espessuraCL=bl)
    g0 = random_state(int(np.prod(list(grade.values()))), seed=11)
    s = _solver(grade, storage, pingpong, strict)
    s.definirTipos(tipo)
    s.configurar(**cfg)
    s.definirPopulacoes(g0)
    o = _oracle(grade, storage, strict)
    o.set_types(tipo)
    o.configure(**_ocfg(cfg))
    o.set_populations(g0)
    fl = _fluid(tipo)
    for n in (1, 1, 7, 40):
        s.passo(n)
        o.step(n, macros=True)
        gs = s.lerPopulacoes()[:, fl]
        go = o.populations().reshape(19, -1)[:, fl]
        assert np.array_equal(gs, go), f"{storage} pingpong={pingpong} strict={strict} after {s.passos}: max diff {np.abs(gs - go).max()}"
    m = s.lerMacros()
    assert np.array_equal(m, o.macros), "pulled macros differ"
    fs = np.array(s.medirForcas())
    fo = o.forces()
    # fp64 sums in different orders: within 1e-12 of the force's magnitude
    # (a small component can lose relative digits to cancellation)
    np.testing.assert_allclose(fs, fo, rtol=1e-12, atol=1e-12 * np.abs(fo).max() + 1e-15)
    s.atualizarMacros()
    assert np.array_equal(s.lerMacros(), o.update_macros(zero_solids=True))
    np.testing.assert_allclose(s.massa(), o.mass(), rtol=1e-12, atol=1e-13)
    s.destruir()


def test_init_matches_oracle(native):
    grade, tipo, esp = all_types_tunnel()
    cfg = _cfg(esp)
    s = _solver(grade)
    s.definirTipos(tipo)
    s.configurar(**cfg)
    s.inicializar()
    o = _oracle(grade, "f32")
    o.set_types(tipo)
    o.configure(**_ocfg(cfg))
    o.init()
    # init writes every cell, solids included (src/core/emit/wgsl.js:285-299)
    assert np.array_equal(s.lerPopulacoes(), o.populations().reshape(19, -1))


def test_config1_sphere_1000_steps(native):
    """128x64x64, sphere D=16 at (40,32,32), Re 100 (omega 1.908397), Cs 0.1,
    1000 steps from uniform equilibrium.  Both arithmetic modes equal their
    oracle restatement bit for bit; the FAST mode stays within the stated
    1e-5 relative bar of the literal (STRICT) restatement."""
    grade, corpo, tipo, esp = sphere_tunnel(128, 64, 64, r=8, cx=40)
    nu = 0.05 * 16 / 100
    cfg = dict(omegaPlus=1 / (3 * nu + 0.5), lesCs=0.1, inletU=[0.05, 0, 0], beltU=[0, 0, 0], esponja=esp,
               espessuraCL=0)
    fl = _fluid(tipo)
    out = {}
    for strict in (True, False):
        s = _solver(grade, strict=strict)
        s.definirTipos(tipo)
        s.configurar(**cfg)
        s.inicializar()
        o = _oracle(grade, "f32", strict)
        o.set_types(tipo)
        o.configure(**_ocfg(cfg))
        o.init()
        s.passo(1000)
        o.run(1000)
        gs = s.lerPopulacoes()[:, fl]
        go = o.populations().reshape(19, -1)[:, fl]
        assert np.abs(gs - go).max() / np.abs(go).max() <= 1e-5   # the stated bar
        assert np.array_equal(gs, go)                              # and in fact bit-exact
        out[strict] = gs
        s.destruir()
    rel = np.abs(out[False] - out[True]).max() / np.abs(out[True]).max()
    assert rel <= 1e-5, rel


def test_config1_sphere_boundary_layer_1000_steps(native):
    """The config-1 sphere with the inlet boundary layer the app gives a
    tunnel without a belt, espessuraCL = round(0.12 nz) = 8
    (index.html:719): 1000 steps bit-exact against the oracle, and the inlet
    plane carries the 1/7-power profile below z = 8."""
    grade, corpo, tipo, esp = sphere_tunnel(128, 64, 64, r=8, cx=40)
    nu = 0.05 * 16 / 100
    cfg = dict(omegaPlus=1 / (3 * nu + 0.5), lesCs=0.1, inletU=[0.05, 0, 0], beltU=[0, 0, 0], esponja=esp,
               espessuraCL=round(0.12 * 64))
    fl = _fluid(tipo)
    s = _solver(grade)
    s.definirTipos(tipo)
    s.configurar(**cfg)
    s.inicializar()
    o = _oracle(grade, "f32")
    o.set_types(tipo)
    o.configure(**_ocfg(cfg))
    o.init()
    s.passo(1000)
    o.run(1000)
    gs = s.lerPopulacoes()[:, fl]
    go = o.populations().reshape(19, -1)[:, fl]
    assert np.array_equal(gs, go)
    # inlet cells (x = 0) hold the equilibrium of u_in * blf(z)
    g = s.lerPopulacoes().reshape(19, 64, 64, 128)
    inlet = g[:, :, 32, 0]                                 # (19, z)
    ux = (inlet[[1, 7, 9, 11, 13]].sum(0) - inlet[[2, 8, 10, 12, 14]].sum(0)) / (1 + inlet.sum(0))
    zc = np.arange(64) + 0.5
    prof = np.where(zc < 8, (zc / 8.0) ** (1 / 7), 1.0) * 0.05
    np.testing.assert_allclose(ux[1:], prof[1:], rtol=2e-6, atol=1e-9)
    s.destruir()


def test_inplace_equals_pingpong_full_size(native):
    """Size-independent property at the full config-1 size: the in-place
    layout and the reference's A/B scheme give the same state bitwise."""
    grade, corpo, tipo, esp = sphere_tunnel(128, 64, 64, r=8, cx=40, esteira=True, floor_mirror=False)
    cfg = _cfg(esp, omegaPlus=1.9083969, lesCs=0.1)
    a = _solver(grade)
    b = _solver(grade, pingpong=True)
    for s in (a, b):
        s.definirTipos(tipo)
        s.configurar(**cfg)
        s.inicializar()
    fa = a.passoComForcas(1000)
    fb = b.passoComForcas(1000)
    fl = _fluid(tipo)
    assert np.array_equal(a.lerPopulacoes()[:, fl], b.lerPopulacoes()[:, fl])
    np.testing.assert_allclose(fa, fb, rtol=1e-11, atol=1e-13)


def test_fused_force_equals_measured_force(native):
    grade, corpo, tipo, esp = sphere_tunnel(64, 32, 32, r=6, cx=20)
    s = _solver(grade)
    s.definirTipos(tipo)
    s.configurar(**_cfg(esp, beltU=[0, 0, 0]))
    s.inicializar()
    for _ in range(5):
        f_before = np.array(s.medirForcas())
        fused = s.passoComForcas(1)[0]
        np.testing.assert_allclose(fused, f_before, rtol=1e-12, atol=1e-12 * np.abs(f_before).max() + 1e-14)


def test_rest_offset_on_zero_state(native):
    """calibrarRepouso on the all-zero state equals sum over links of 2 w_i c_i
    (src/backend/webgpu/solver.js:457-479); zero for a body away from walls."""
    grade, corpo, tipo, esp = sphere_tunnel(48, 32, 32, r=6, cx=20)
    s = _solver(grade)
    s.definirTipos(tipo)
    s.configurar(**_cfg(esp))
    off = s.calibrarRepouso()
    np.testing.assert_allclose(off, [0, 0, 0], atol=1e-12)
    # a body resting on the floor has a net downward offset
    t = tipo.reshape(32, 32, 48).copy()
    t[1:4, 10:20, 10:20] = 1
    s.definirTipos(t.reshape(-1))
    off2 = s.calibrarRepouso()
    assert off2[2] != 0.0


@pytest.mark.parametrize("storage", ["f32", "f16s", "bf16s"])
@pytest.mark.parametrize("strict", [False, True])
@pytest.mark.parametrize("kz", [4, 8, 16])
def test_pipelined_step_equals_plain_step(native, storage, strict, kz):
    """The software-pipelined step (cp.async prefetch along z) is the same
    arithmetic as the plain step: states must be identical."""
    grade, tipo, esp = all_types_tunnel(nx=70, ny=20, nz=37)
    cfg = _cfg(esp)
    g0 = random_state(int(np.prod(list(grade.values()))), seed=3)
    a = _solver(grade, storage, strict=strict)
    b = _solver(grade, storage, strict=strict)
    b.definirBloco(64, 100 + kz)
    for s in (a, b):
        s.definirTipos(tipo)
        s.configurar(**cfg)
        s.definirPopulacoes(g0)
    for n in (1, 2, 9):
        a.passo(n)
        b.passo(n)
        fl = _fluid(tipo)
        assert np.array_equal(a.lerPopulacoes()[:, fl], b.lerPopulacoes()[:, fl]), (storage, strict, kz, a.passos)


@pytest.mark.parametrize("dims", [(640, 320, 256), (512, 512, 440)])
def test_largest_grids_keep_uniform_flow(native, dims):
    """Size-independent check at the reference's largest preset (640x320x256,
    src/backend/caps.js:75) and past the 2^31 population-index limit
    (512x512x440: 19 N > 2^31, the 64-bit offset path): a uniform flow in a
    periodic all-fluid box stays bit-identical in every cell (the property
    tests/nucleo.html:107-130 checks), with the fp64 mass equal to N times
    the common delta."""
    from cfd__gb300 import SolverCUDA
    nx, ny, nz = dims
    N = nx * ny * nz
    s = SolverCUDA({"nx": nx, "ny": ny, "nz": nz}, escrever_macros=False)
    s.definirTipos(np.zeros(N, np.uint32))
    s.configurar(omegaPlus=1.9, lesCs=0.1, inletU=[0.05, 0.01, -0.02], esponja={"inicio": nx + 10, "comprimento": 4})
    s.inicializar()
    s.passo(6)
    s.atualizarMacros()
    m = s.lerMacros().reshape(-1, 4)
    for k in range(4):
        assert m[:, k].min() == m[:, k].max(), k
    np.testing.assert_allclose(m[0, :3], [0.05, 0.01, -0.02], rtol=1e-6)
    assert abs(float(m[0, 3])) < 1e-6
    mass = s.massa()                      # N identical deltas, summed in fp64
    assert abs(mass - N * float(m[0, 3])) <= 1e-9 * max(1.0, abs(mass))
    s.destruir()
