"""The visualisation restatement (oracle/vis_oracle.py) on fields with known
answers: zero flow keeps the smoke, a one-cell shift moves it by one cell,
the rake paints filaments where the reference's formula puts them, and the
particle hash and respawn follow src/render/renderer.js.  CPU only."""
import numpy as np

from oracle import vis_oracle as V

R_OFF = {"x": -100.0, "passo_y": 4.0, "passo_z": 4.0, "raio": 1.0, "y0": 1.0, "y1": 10.0, "z0": 1.0, "z1": 10.0}


def _field(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0, 2, shape).astype(np.float16)


def test_zero_flow_keeps_density():
    cur = _field((6, 7, 8), 1)
    mac = np.zeros((6, 7, 8, 4), np.float32)
    tipo = np.zeros((6, 7, 8), np.uint8)
    out = V.fumaca_passo(cur, mac, tipo, R_OFF, {"dt": 10.0, "dissipacao": 1.0, "taxa": 0.0, "avanco": 0.5})
    assert np.array_equal(out, np.minimum(cur, np.float16(4.0)))


def test_one_cell_shift_moves_by_one_cell():
    cur = _field((5, 6, 12), 2)
    mac = np.zeros((5, 6, 12, 4), np.float32)
    mac[..., 0] = 0.05
    tipo = np.zeros((5, 6, 12), np.uint8)
    out = V.fumaca_passo(cur, mac, tipo, R_OFF, {"dt": 20.0, "dissipacao": 1.0, "taxa": 0.0, "avanco": 1.0})
    # (the last column's forward check reads past the edge: clamp-to-edge)
    assert np.array_equal(out[:, :, 1:-1], cur[:, :, :-2])
    assert (out[:, :, 0] == 0).all()          # traced from outside the domain


def test_solids_are_empty_and_rake_paints_filaments():
    shape = (12, 12, 10)
    cur = np.zeros(shape, np.float16)
    mac = np.zeros(shape + (4,), np.float32)
    tipo = np.zeros(shape, np.uint8)
    tipo[3, 3, 3] = 1
    R = {"x": 4.5, "passo_y": 4.0, "passo_z": 4.0, "raio": 1.0, "y0": 1.0, "y1": 11.0, "z0": 1.0, "z1": 11.0}
    F = {"dt": 10.0, "dissipacao": 1.0, "taxa": 2.4, "avanco": 0.5}
    out = V.fumaca_passo(cur, mac, tipo, R, F).astype(np.float32)
    assert out[3, 3, 3] == 0
    # filament centres at y, z = y0 + (j + 1/2) passo = 3, 7; voxel centres 2.5 / 3.5 are
    # half a cell off: r = sqrt(0.5^2 + 0.5^2), density 2.4 exp(-5.5 r^2)
    expect = 2.4 * np.exp(-5.5 * 0.5)
    np.testing.assert_allclose(out[2, 2, 4], expect, rtol=2e-3)
    assert out[2, 2, 8] == 0                   # outside the emission slice (|dx| > 1.5)
    assert out[0, 0, 4] == 0                   # outside the rake's extent


def test_particle_hash_and_respawn():
    h = V._hash01(np.array([0, 1, 2, 12345], np.uint32))
    assert ((h >= 0) & (h < 1)).all() and len(set(h.tolist())) == 4
    mac = np.zeros((8, 16, 32, 4), np.float32)
    mac[..., 0] = 0.05
    parts = np.zeros((4, 8), np.float32)
    parts[0, :4] = [10.0, 8.0, 4.0, 100.0]      # moves
    parts[1, :4] = [30.9, 8.0, 4.0, 100.0]      # leaves at the outlet -> respawn
    parts[2, :4] = [10.0, 8.0, 4.0, 1.0]        # life runs out -> respawn
    parts[3, :4] = [20.0, 5.0, 2.0, 100.0]
    mac[2, 5, 20, :3] = 0.0                     # particle 3 sits in a still cell -> respawn
    out = V.esteiras_passo(parts, mac, 20.0, 4, 7)
    np.testing.assert_allclose(out[0, :4], [10.0 + 1.0, 8.0, 4.0, 99.0], rtol=1e-6)
    assert out[0, 7] == 1.0 and np.array_equal(out[0, 4:7], parts[0, :3])
    for i in (1, 2, 3):
        assert out[i, 7] == 0.0 and 2.0 <= out[i, 0] < 5.0 and 220.0 <= out[i, 3] < 480.0
        assert np.array_equal(out[i, 4:7], out[i, :3])
