"""Pins the CPU oracle against the reference's own known-answer tests and its
published results (README.md:100-101, :120).  CPU only."""
import numpy as np

from tests import kat


def make(grade):
    return kat.OracleSolver(grade)


def test_uniform_flow_preserved():
    eu, ed = kat.uniform_flow(make)
    assert eu < 1e-6 and ed < 1e-6           # tests/nucleo.html:128
    assert eu < 5e-8                          # published drift 1.9e-8 (README.md:120)


def test_shear_wave_viscosity():
    rows = kat.shear_wave(make)
    errs = [abs(r[3]) for r in rows]
    assert max(errs) < 2.0                    # tests/nucleo.html:187
    # published range 0.04 - 1.07 % for omega 0.6 - 1.8 (README.md:120)
    assert 0.03 < min(errs) < 0.05 and 1.0 < max(errs) < 1.1


def test_block_mass_conservation():
    r = kat.block_mass(make)
    assert r["nan"] == 0
    assert abs(r["mass1"] - r["mass0"]) < 1e-3 * r["N"] * 1e-4 + 1e-4   # tests/nucleo.html:233
    assert 0.05 < r["umax"] < 0.15                                       # :235


def test_couette_wall_position():
    # 4x4 instead of 8x8 in x, y: the flow is homogeneous there, so every
    # column is bitwise the same and the profile is identical.
    rows = kat.couette(make, nx=4, ny=4)
    worst = max(abs(r["a"] - r["a_teorico"]) / r["a_teorico"] for r in rows)
    spread = max(r["z0"] for r in rows) - min(r["z0"] for r in rows)
    assert worst < 0.05 and spread < 0.06     # tests/validacao.html:181-184
    # published: slope error 0.00 %, walls at 0.500 and 32.501 (README.md:100-101)
    for r in rows:
        assert abs(r["z0"] - 0.5) < 2e-3 and abs(r["z1"] - 32.5) < 2e-3
    assert worst < 1e-3


def test_faithful_and_fp64_force_orders_agree(orc):
    from tests.cases import random_state, sphere_tunnel
    grade, corpo, tipo, esp = sphere_tunnel(48, 24, 24, r=5)
    lat = orc.Lattice((48, 24, 24))
    lat.set_types(tipo)
    lat.set_populations(random_state(lat.N, 1))
    f64 = lat.forces()
    f32 = lat.forces_faithful()
    assert np.all(np.isfinite(f64))
    np.testing.assert_allclose(f32, f64, rtol=1e-5, atol=1e-7)
