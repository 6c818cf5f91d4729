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


def _slab_chord(o, d, lo, hi):
    """Length of the ray o + t d (t >= 0) inside the box [lo, hi], float64."""
    with np.errstate(divide="ignore", invalid="ignore"):
        ta = (lo[:, None, None] - o[:, None, None]) / d
        tb = (hi[:, None, None] - o[:, None, None]) / d
    t0 = np.maximum(np.nanmax(np.minimum(ta, tb), axis=0), 0.0)
    t1 = np.nanmin(np.maximum(ta, tb), axis=0)
    return np.where(t1 > t0, t1 - t0, 0.0)


def test_render_known_answers():
    """Empty volume: a black, transparent image.  Uniform density d in the
    box: opacity 1 - exp(-sigma d L) with L the chord of each pixel's ray
    through the domain box (Beer-Lambert; the march samples the chord at
    `passos` jittered points, hence the tolerance), rays that miss the box
    stay empty, and the colour channels keep the 0.96 : 0.97 : 1 tint of
    src/render/fumaca.js:330-336."""
    nz, ny, nx = 8, 8, 16
    W, H = 48, 32
    ivp = np.zeros(16, np.float32)
    ivp[0] = ivp[5] = ivp[10] = ivp[15] = 1.0          # clip -> world: (ndx, ndy, 1)
    eye = (0.0, 0.0, -3.0)
    kw = dict(largura=W, altura=H, g=0.3, passos=96, passos_luz=6, luz=(0.3, 0.5, 0.8), intensidade=1.0, quadro=3)
    img0 = V.render(np.zeros((nz, ny, nx), np.float16), ivp, eye, densidade=0.8, **kw)
    assert not img0.any()

    d0, sigma = 0.5, 0.8
    img = V.render(np.full((nz, ny, nx), d0, np.float16), ivp, eye, densidade=sigma, **kw)
    iy, ix = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    ndx = (ix + 0.5) / W * 2 - 1
    ndy = 1 - (iy + 0.5) / H * 2
    d = np.stack([ndx - eye[0], ndy - eye[1], np.ones_like(ndx) - eye[2]])
    d /= np.linalg.norm(d, axis=0)
    k = 2.0 / nx
    lo = np.array([-nx * 0.5 * k, -ny * 0.5 * k, 0.0])
    hi = np.array([nx * 0.5 * k, ny * 0.5 * k, nz * k])
    L = _slab_chord(np.array(eye), d, lo, hi)
    hit = L > 1e-3
    assert hit.any() and (~hit).any()
    want = 1.0 - np.exp(-sigma * d0 * L)
    ds = L[hit] / kw["passos"]
    # at most one of the jittered samples can fall on the far face
    assert np.all(np.abs(img[..., 3][hit] - want[hit]) <= sigma * d0 * ds + 1e-4)
    assert not img[~(L > 0)].any()
    r, g, b = img[..., 0][hit], img[..., 1][hit], img[..., 2][hit]
    assert (b > 0).all()
    np.testing.assert_allclose(r / b, 0.96, rtol=1e-5)
    np.testing.assert_allclose(g / b, 0.97, rtol=1e-5)


def test_cp_samples_along_the_normal_and_flips_into_fluid():
    """One triangle in the plane z = 5 facing +z: Cp reads the macros delta
    1.8 cells along the normal (cell z = 6); with that cell solid it reads
    1.8 cells the other way (z = 3), as the body shader does
    (src/render/renderer.js:168-180); Cp = delta / (1.5 u_ref^2)."""
    nz, ny, nx = 10, 8, 8
    mac = np.zeros((nz, ny, nx, 4), np.float32)
    mac[..., 3] = (np.arange(nz, dtype=np.float32) * np.float32(1e-3))[:, None, None]
    tipo = np.zeros((nz, ny, nx), np.uint8)
    pos = np.array([[2.2, 2.2, 5.0], [5.2, 2.2, 5.0], [2.2, 5.2, 5.0]], np.float32)
    idx = np.array([[0, 1, 2]], np.uint32)
    u = np.float32(0.05)
    den = np.float32(1.5) * u * u
    cp = V.cp_triangulos(pos, idx, mac, tipo, u)
    assert cp[0] == np.float32(6e-3) / den
    tipo[6, 3, 3] = 1                      # the cell above the centroid (3.2, 3.2, 6.8) is solid
    cp = V.cp_triangulos(pos, idx, mac, tipo, u)
    assert cp[0] == np.float32(3e-3) / den
    # the opposite winding faces -z: the same two samples, swapped
    tipo[:] = 0
    cp = V.cp_triangulos(pos, idx[:, ::-1].copy(), mac, tipo, u)
    assert cp[0] == np.float32(3e-3) / den
