"""The reference's known-answer tests and published validation results, run
on the GPU through the solver class API (tests/nucleo.html,
tests/validacao.html; published numbers README.md:100-105, :120)."""
import numpy as np
import pytest

from tests import kat

pytestmark = pytest.mark.gpu


def make(grade):
    from cfd__gb300 import SolverCUDA
    return SolverCUDA(grade)


def test_uniform_flow(native):
    eu, ed = kat.uniform_flow(make)
    assert eu < 1e-6 and ed < 1e-6
    assert eu < 5e-8


def test_shear_wave(native):
    rows = kat.shear_wave(make)
    errs = [abs(r[3]) for r in rows]
    assert max(errs) < 2.0
    assert 0.03 < min(errs) < 0.05 and 1.0 < max(errs) < 1.1


def test_block_mass(native):
    r = kat.block_mass(make)
    assert r["nan"] == 0
    assert abs(r["mass1"] - r["mass0"]) < 1e-3 * r["N"] * 1e-4 + 1e-4
    assert 0.05 < r["umax"] < 0.15


def test_couette_reference_size(native):
    rows = kat.couette(make)                 # 8x8x34 as tests/validacao.html:123
    worst = max(abs(r["a"] - r["a_teorico"]) / r["a_teorico"] for r in rows)
    spread = max(r["z0"] for r in rows) - min(r["z0"] for r in rows)
    assert worst < 1e-3 and spread < 1e-3
    for r in rows:
        assert abs(r["z0"] - 0.5) < 2e-3 and abs(r["z1"] - 32.5) < 2e-3


@pytest.mark.parametrize("cid", ["esfera-re50", "esfera-re100", "cilindro-re100"])
def test_published_validation_cases(native, cid):
    """Cd (and St) of the reference's validation cases against the values its
    WebGPU run published: within 0.5 %, and within the page's own 15 % of the
    correlation."""
    from cfd__gb300.validacao import CASOS, PUBLICADOS, classificar
    caso = next(c for c in CASOS if c["id"] == cid)
    r = kat.validation_case(make, caso)
    assert r["divergiu"] is None
    pub = PUBLICADOS[cid]
    assert abs(r["cd"] - pub["cd"]) / pub["cd"] < 5e-3, (r["cd"], pub["cd"])
    assert classificar(r["cd"], r["ref"])["ok"]
    if "st" in pub:
        st = r["st"]["st"]
        assert abs(st - pub["st"]) / pub["st"] < 5e-3, (st, pub["st"])
