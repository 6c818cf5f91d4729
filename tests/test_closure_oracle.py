"""The closure's CPU restatement (oracle/closure_oracle.py) checked on its
own: the hand-derived fp64 gradient against central differences, the bf16
rounding, feature identities and the sample builder on fields with known
answers.  CPU only."""
import ctypes as C

import numpy as np

from oracle import closure_oracle as CO


def _weights(rng, scale=0.5):
    return rng.normal(0.0, scale, 1313)


def test_gradient_matches_central_differences():
    rng = np.random.default_rng(3)
    v = _weights(rng)
    feats = rng.normal(0.0, 1.0, (40, 6)).astype(np.float32)
    target = np.abs(rng.normal(0.0, 1e-3, 40)).astype(np.float32)
    mean, std, s = np.zeros(6), np.ones(6), 1e-3
    loss, g = CO.loss_grad64(v, feats, target, mean, std, s)
    h = 1e-6
    idx = rng.choice(1313, 60, replace=False)
    idx = np.concatenate([idx, [0, 191, 192, 224, 1247, 1279, 1280, 1312]])
    for i in idx:
        vp, vm = v.copy(), v.copy()
        vp[i] += h
        vm[i] -= h
        fd = (CO.loss_grad64(vp, feats, target, mean, std, s)[0] - CO.loss_grad64(vm, feats, target, mean, std, s)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-7, (i, fd, g[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5, 0.0, np.inf], np.float32)
    r = CO.bf16(x)
    exp = np.array([1.0, 1.0, 1.0 + 2.0 ** -6, 1.0, -2.5, 0.0, np.inf], np.float32)
    assert np.array_equal(r, exp)
    assert np.isnan(CO.bf16(np.array([np.nan], np.float32)))[0]


def test_feature_identities():
    a = np.float32(2e-3)
    f = CO.features(a, a, a, 0, 0, 0, 1.0, 0.0, 0.6)
    assert f[3] == 0.0
    np.testing.assert_allclose(f[1], np.sqrt(1.5), rtol=1e-6)
    np.testing.assert_allclose(f[0], np.log(np.sqrt(6.0) * 2e-3 + 1e-9), rtol=1e-6)
    np.testing.assert_allclose(f[4], 1 / 0.6, rtol=1e-7)
    # pure shear: Pi_xy only -> trace 0, det 0, off-diagonal share 1
    f = CO.features(0, 0, 0, 1e-3, 0, 0, 1.0, 0.01, 0.6)
    assert f[1] == 0.0 and f[2] == 0.0
    np.testing.assert_allclose(f[3], 1.0, rtol=1e-6)
    np.testing.assert_allclose(f[5], 1.0, rtol=1e-6)


def test_samples_linear_shear_has_no_residual_stress():
    """u_x = g z on the fine grid: the filtered velocity is the same line and
    the residual stress has no xz part, so nu_t = 0 everywhere.  On the
    coarse grid du_x/dz = 2 g, so S_xz = g and Pi_xz = -(2/3) tau0 g."""
    nx, ny, nz = 16, 12, 20
    gam = 1e-3
    z = np.arange(nz, dtype=np.float32)[:, None, None]
    mac = np.zeros((nz, ny, nx, 4), np.float32)
    mac[..., 0] = gam * (z + 0.0)
    tipo = np.zeros((nz, ny, nx), np.uint8)
    f, t = CO.samples(mac, tipo, 0.55, 0, nx // 2)
    cz, cy, cx = nz // 2, ny // 2, nx // 2
    t3 = t.reshape(cz, cy, cx)
    inner = t3[1:-1, 1:-1, 1:-1]
    assert np.isfinite(inner).all() and (inner == 0).all()
    assert np.isnan(t3[0]).all() and np.isnan(t3[:, :, 0]).all()
    # Pi = -(2/3) tau0 S, S_xz = 2 gam / 2 -> qs = sqrt(2 * 2 Pxz^2) = 2 |Pxz|
    pxz = (2.0 / 3.0) * 0.55 * gam
    np.testing.assert_allclose(f.reshape(cz, cy, cx, 6)[1:-1, 1:-1, 1:-1, 0], np.log(2 * pxz + 1e-9), rtol=1e-5)


def test_samples_solid_masks_neighbours():
    nx, ny, nz = 16, 16, 16
    rng = np.random.default_rng(0)
    mac = rng.normal(0, 1e-2, (nz, ny, nx, 4)).astype(np.float32)
    tipo = np.zeros((nz, ny, nx), np.uint8)
    tipo[8, 8, 8] = 1                 # one solid fine cell -> coarse (4, 4, 4)
    f, t = CO.samples(mac, tipo, 0.55, 0, nx // 2)
    t3 = t.reshape(8, 8, 8)
    for c in [(4, 4, 4), (3, 4, 4), (5, 4, 4), (4, 3, 4), (4, 5, 4), (4, 4, 3), (4, 4, 5)]:
        assert np.isnan(t3[c])
    assert np.isfinite(t3[2, 2, 2]) and np.isfinite(t3[4, 5, 5])


def test_abi_struct_sizes():
    from cfd__gb300 import _native as nat
    assert C.sizeof(nat.ClosureWeights) == 4 * (1313 + 27)
    assert C.sizeof(nat.ClosureCfg) == 40
    assert nat.ClosureCfg.seed.offset == 24


def test_weights_round_trip_and_scaling(tmp_path):
    from cfd__gb300 import fecho
    rng = np.random.default_rng(9)
    p = fecho.pesos_vazios()
    p["w2"] = rng.normal(0, 1, (32, 32)).astype(np.float32)
    p["b3"] = np.float32(-0.5)
    f = rng.normal(0, 1, (5000, 6)).astype(np.float32)
    t = np.where(rng.random(5000) < 0.3, 0.0, rng.lognormal(-8, 1, 5000)).astype(np.float32)
    n = fecho.normalizacao(f, t)
    p.update(n)
    p["coef"] = 1
    assert (n["lo"] < n["hi"]).all() and n["nu_scale"] > 0 and n["nu_max"] > n["nu_scale"]
    # the struct the C ABI sees holds the same numbers
    q = fecho.de_struct(fecho.para_struct(p))
    assert np.array_equal(fecho.vetor(q), fecho.vetor(p)) and q["coef"] == 1
    path = tmp_path / "w.npz"
    fecho.salvar(p, path)
    r = fecho.carregar(path)
    assert np.array_equal(fecho.vetor(r), fecho.vetor(p))
    for k in ("mean", "std", "lo", "hi"):
        assert np.array_equal(r[k], p[k])
    assert r["coef"] == 1 and r["nu_scale"] == p["nu_scale"]


def test_committed_weights_load():
    import os

    from cfd__gb300 import fecho
    p = fecho.carregar(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cfd__gb300",
                                    "pesos", "fecho_coef.npz"))
    assert p["coef"] == 1 and np.isfinite(fecho.vetor(p)).all() and p["std"][0] > 1e20
