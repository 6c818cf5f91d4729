"""The inlet ramp through the GPU solver against the oracle: the app's
start-up (index.html:757-772 ramps the inlet over one domain crossing) on a
tunnel with the app's boundary layer.  Every passo(n) re-configures the inlet
with the new smoothstep factor before it dispatches, as
src/backend/webgpu/solver.js:398-402 does; the oracle is configured with the
same factor before the same n steps.  States must be identical after every
call."""
import numpy as np
import pytest

from tests.cases import sphere_tunnel

pytestmark = pytest.mark.gpu


def test_ramp_bit_exact_against_oracle(native):
    from cfd__gb300 import SolverCUDA
    from oracle import oracle as O

    grade, corpo, tipo, esp = sphere_tunnel(48, 24, 24, r=4, cx=14, floor_mirror=False)
    u, bl = 0.06, round(0.12 * 24)
    base = dict(omegaPlus=1.92, lesCs=0.1, beltU=[0.0, 0.0, 0.0], esponja=esp, espessuraCL=bl)
    s = SolverCUDA(grade)
    s.definirTipos(tipo)
    s.configurar(**base, inletU=[0.0, 0.0, 0.0])
    seen = []

    def aplicar(f):
        seen.append(f)
        s.configurar(**base, inletU=[u * f, 0.0, 0.0])

    s.rampa(48, aplicar)
    s.inicializar()
    o = O.Lattice((grade["nx"], grade["ny"], grade["nz"]), nthreads=8, fast=True)
    o.set_types(tipo)
    o.configure(omega_plus=1.92, les_cs=0.1, inlet_u=[0.0, 0.0, 0.0], sponge_start=esp["inicio"],
                sponge_len=esp["comprimento"], bl_thickness=bl)
    o.init()
    fl = ~np.isin(tipo, [1, 4, 7])
    atual = 0
    for n in (1, 3, 8, 20, 16, 10):
        s.passo(n)
        if atual < 48:
            atual += n
            t = atual / 48
            f = 1.0 if atual >= 48 else t * t * (3 - 2 * t)
            o.configure(omega_plus=1.92, les_cs=0.1, inlet_u=[u * f, 0.0, 0.0], sponge_start=esp["inicio"],
                        sponge_len=esp["comprimento"], bl_thickness=bl)
        o.run(n)
        assert np.array_equal(s.lerPopulacoes()[:, fl], o.populations().reshape(19, -1)[:, fl]), s.passos
    # one call per passo() while the ramp runs (steps 1, 4, 12, 32, 48); the
    # call that reaches step 48 applies the full speed, the next one none
    assert len(seen) == 5 and seen[-1] == 1.0 and abs(seen[0] - (1 / 48) ** 2 * (3 - 2 / 48)) < 1e-15
    assert s.fatorRampa == 1.0
    s.destruir()
