"""What the trained closure gains over the method without it: coarse runs of
the learned-closure workload (320x160x128, the 20k-triangle superellipsoid
on a no-slip floor, u_in 0.06, held-out Re 10 000 on the 96-cell length) with
the committed network (cfd__gb300/pesos/fecho_coef.npz, evaluated every
step) and with Smagorinsky Cs 0.12, scored against the filtered fine run's
drag (2x resolution, tests/golden/closure_fine_re10000.json, made by
tests/golden/make_closure_fixture.py): the closure's Cd error must not exceed
Smagorinsky's.  Both engines of the network are run; 12 000 coarse steps
each (the same physical time as the fine run's 24 000), Cd from the force
averaged over blocks of 250 steps, mean of the second half.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "closure_fine_re10000.json")
PESOS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cfd__gb300", "pesos",
                     "fecho_coef.npz")


@pytest.fixture(scope="module")
def coarse():
    from cfd__gb300.estudos import tuneis_fecho
    (gc, tc, ec, ac), _ = tuneis_fecho(2026)
    return gc, tc, ec, ac


def test_closure_beats_smagorinsky_against_fine_run(native, coarse):
    from cfd__gb300.estudos import rodar_fecho
    from cfd__gb300.fecho import carregar
    fine = json.load(open(GOLD))
    assert not fine["diverged"] and np.isfinite(fine["cd"])
    gc, tc, ec, ac = coarse
    smag, _ = rodar_fecho(gc, tc, ec, ac, 10000, 12000, 250, u=0.06, comprimento=96.0, cs=0.12)
    assert not smag["diverged"]
    e_smag = abs(smag["cd"] - fine["cd"]) / abs(fine["cd"])
    p = carregar(PESOS)
    for motor in (0, 1):
        clo, _ = rodar_fecho(gc, tc, ec, ac, 10000, 12000, 250, u=0.06, comprimento=96.0, cs=0.12, closure=p,
                             cada_k=1, motor=motor)
        assert not clo["diverged"], motor
        e_clo = abs(clo["cd"] - fine["cd"]) / abs(fine["cd"])
        assert clo["fallback_rate"] < 0.05, (motor, clo["fallback_rate"])
        assert e_clo <= e_smag, (motor, clo["cd"], smag["cd"], fine["cd"])
