"""D3Q19 tables and identities against the reference's own lattice (golden
fixture generated from legacy/cfd/lattice.py) and the JS self-check."""
import json
import os

import numpy as np

from cfd__gb300 import lattice as L

GOLD = os.path.join(os.path.dirname(__file__), "golden", "lattice_legacy.json")


def _gold():
    with open(GOLD) as f:
        return json.load(f)


def test_self_check():
    assert L.self_check()


def test_tables_match_reference_python_lattice():
    g = _gold()
    assert g["Q"] == L.Q
    assert np.array_equal(np.array(g["C"]), L.C)
    assert np.array_equal(np.array(g["W"]), L.W)
    assert np.array_equal(np.array(g["OPP"]), L.OPP)
    for k, v in g["MAGIC"].items():
        assert L.MAGIC[k] == v


def test_equilibrium_and_moments_match_reference():
    g = _gold()
    s = g["samples"]
    eq = L.equilibrium(np.array(s["delta"]), np.array(s["u"]))
    np.testing.assert_allclose(eq, np.array(s["eq"]), rtol=0, atol=1e-17)
    d, u = L.moments(eq)
    np.testing.assert_allclose(d, np.array(s["moments_delta"]), rtol=0, atol=1e-16)
    np.testing.assert_allclose(u, np.array(s["moments_u"]), rtol=0, atol=1e-16)


def test_viscosity_relations_match_reference():
    g = _gold()
    for w, nu, wm in zip(g["omega"], g["nu_from_omega"], g["omega_minus_wall"]):
        assert abs(L.nu_from_omega(w) - nu) <= 1e-16
        assert abs(L.omega_minus_from_lambda(w, L.MAGIC["WALL"]) - wm) <= 1e-15
        # Lambda round trip
        assert abs(L.lambda_from_omegas(w, wm) - 3 / 16) < 1e-14


def test_oracle_tables_match(orc):
    t = orc.tables()
    assert np.array_equal(t["C"], L.C)
    assert np.array_equal(t["OPP"], L.OPP)
    for ax in range(3):
        assert [L.espelhar_idx(i, ax) for i in range(19)] == list(t["MIRROR"][ax])
    # weights as the 9-significant-digit literals the emitter prints
    assert np.array_equal(t["W"], np.array([f"{w:.9g}" for w in L.W], dtype=np.float32))
    assert np.array_equal(t["SIXW"][1:], np.array([f"{6 * w:.9g}" for w in L.W[1:]], dtype=np.float32))
    assert np.array_equal(t["Wd"], L.W)


def test_half_and_bf16_rounding(orc):
    """The oracle's fp16/bf16 conversions against numpy's IEEE rounding."""
    lib = orc.lib()
    rng = np.random.default_rng(3)
    vals = np.concatenate([rng.normal(0, 1, 2000), rng.normal(0, 1e-5, 2000), [0.0, -0.0, 65504.0, 7e-8, 3e-8, 1e6]])
    for v in vals.astype(np.float32):
        with np.errstate(over="ignore"):      # 1e6 overflows to inf on purpose
            want = np.array([v], np.float32).astype(np.float16).view(np.uint16)[0]
        assert lib.orc_f16_bits(float(v)) == want, v
        back = np.array([want], np.uint16).view(np.float16).astype(np.float32)[0]
        assert np.float32(lib.orc_f16_value(int(want))) == back or (np.isnan(back))
