"""CPU restatement of the learned closure (include/lbm_closure.h) — TEST
INFRASTRUCTURE ONLY: tests/ use it as the checker for the CUDA kernels in
cfd__gb300/csrc/closure.cu and closure_mlp.cuh.  Nothing in the product
imports it.

The closure has no counterpart in the reference (its sub-grid model is the
closed-form Smagorinsky relaxation time, src/core/emit/ir.js:262-301), so
this file is the definition the kernels are checked against:

  * features()        the six raw features of a non-equilibrium stress in
                      IEEE fp32 (the kernels use approximate sqrt, log and
                      division for them: tests compare with a tolerance);
  * forward64(),
    loss_grad64()     the 6-32-32-1 MLP, its normalised MSE loss and the
                      hand-derived gradient, all in fp64 (the training
                      kernels' gradient is checked against this);
  * eval_bf16()       the inference path of the fused step: normalised
                      features and weights rounded to bf16 (round to nearest
                      even; the CTA engine also rounds the biases, which ride
                      in the K dimension as products with a constant 1),
                      products summed exactly
                      (fp64 here, fp32 in the tensor cores), hidden
                      activations ReLU'd and rounded to bf16, output
                      nu = nu_scale * softplus(y), NaN when not finite or
                      above nu_max;
  * samples()         the 2x2x2 box filter of a fine run's macros, the
                      filtered strain rate by central differences, the
                      residual stress, the target nu_t and the features of
                      -(2/3) rho (tau0c + 3 nu_t) S, in fp64 up to the
                      features (the kernels: fp32, centred moments).
"""
from __future__ import annotations

import numpy as np

NI, NH = 6, 32
SHAPES = (("w1", (NH, NI)), ("b1", (NH,)), ("w2", (NH, NH)), ("b2", (NH,)), ("w3", (NH,)), ("b3", ()))


def unpack(v):
    """Flat 1313-vector (w1, b1, w2, b2, w3, b3) -> dict of fp64 arrays."""
    v = np.asarray(v, np.float64)
    out, o = {}, 0
    for k, s in SHAPES:
        n = int(np.prod(s)) if s else 1
        out[k] = v[o:o + n].reshape(s) if s else float(v[o])
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[k], np.float64).reshape(-1) for k, _ in SHAPES])


def features(pxx, pyy, pzz, pxy, pxz, pyz, rinv, delta, tau0):
    """Raw features, IEEE fp32, the formulas of closure_features (closure_mlp.cuh)."""
    f32 = np.float32
    xx, yy, zz, xy, xz, yz = (np.asarray(a, f32) for a in (pxx, pyy, pzz, pxy, pxz, pyz))
    rinv = np.asarray(rinv, f32)
    delta = np.asarray(delta, f32)
    off = xy * xy + xz * xz + yz * yz
    pp = xx * xx + yy * yy + zz * zz + f32(2.0) * off
    qs = np.sqrt(f32(2.0) * pp)
    out = np.empty(xx.shape + (6,), f32)
    out[..., 0] = np.log(qs * rinv + f32(1e-9))
    out[..., 1] = (xx + yy + zz) / (qs + f32(1e-12))
    det = xx * (yy * zz - yz * yz) - xy * (xy * zz - yz * xz) + xz * (xy * yz - yy * xz)
    out[..., 2] = det / (qs * qs * qs + f32(1e-30))
    out[..., 3] = off / (f32(0.5) * pp + f32(1e-30))
    out[..., 4] = f32(1.0) / f32(tau0)
    out[..., 5] = f32(100.0) * delta
    return out


def normalise(feats, mean, std):
    mean = np.asarray(mean, np.float32)
    inv = np.where(np.asarray(std, np.float32) != 0, np.float32(1.0) / np.asarray(std, np.float32), np.float32(0.0))
    return (np.asarray(feats, np.float32) - mean) * inv


def softplus(y):
    return np.where(y > 20.0, y, np.log1p(np.exp(np.minimum(y, 20.0))))


def forward64(P, x):
    """x: normalised features (m, 6) -> (y, h1, h2), fp64."""
    x = np.asarray(x, np.float64)
    h1 = np.maximum(x @ P["w1"].T + P["b1"], 0.0)
    h2 = np.maximum(h1 @ P["w2"].T + P["b2"], 0.0)
    y = h2 @ P["w3"] + P["b3"]
    return y, h1, h2


def loss_grad64(v, feats, target, mean, std, nu_scale):
    """Loss mean(((s softplus(y) - t) / s)^2) and its gradient (flat, fp64)."""
    P = unpack(v)
    x = normalise(feats, mean, std).astype(np.float64)
    t = np.asarray(target, np.float64)
    m = x.shape[0]
    y, h1, h2 = forward64(P, x)
    s = float(nu_scale)
    r = (s * softplus(y) - t) / s
    loss = float(np.mean(r * r))
    dy = 2.0 * r / (1.0 + np.exp(-y)) / m
    g = {"w3": h2.T @ dy, "b3": float(dy.sum())}
    dh2 = np.outer(dy, P["w3"]) * (h2 > 0)
    g["w2"] = dh2.T @ h1
    g["b2"] = dh2.sum(axis=0)
    dh1 = (dh2 @ P["w2"]) * (h1 > 0)
    g["w1"] = dh1.T @ x
    g["b1"] = dh1.sum(axis=0)
    return loss, pack(g)


def bf16(a):
    """Round fp32 values to bf16 (nearest even), returned as fp32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    nan = (u & 0x7F800000) == 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    r = np.where(nan, u, r).astype(np.uint32)
    return r.view(np.float32)


def eval_bf16(v, feats, mean, std, nu_scale, nu_max, bias_bf16=False, lo=None, hi=None):
    """nu per row as a tensor-core engine computes it (see module text);
    bias_bf16: the biases rounded to bf16 (the CTA engine carries them in the
    K dimension), else fp32 (the warp engine starts its accumulators at them)."""
    P = unpack(np.asarray(v, np.float32).astype(np.float64))
    x = bf16(normalise(feats, mean, std)).astype(np.float64)
    w1 = bf16(P["w1"].astype(np.float32)).astype(np.float64)
    w2 = bf16(P["w2"].astype(np.float32)).astype(np.float64)
    w3 = bf16(P["w3"].astype(np.float32)).astype(np.float64)
    rb = bf16 if bias_bf16 else (lambda a: np.asarray(a, np.float32))
    b1 = rb(np.float32(P["b1"])).astype(np.float64)
    b2 = rb(np.float32(P["b2"])).astype(np.float64)
    b3 = float(rb(np.array([P["b3"]], np.float32))[0])
    a1 = (x @ w1.T + b1).astype(np.float32)
    h1 = bf16(np.maximum(a1, 0)).astype(np.float64)
    a2 = (h1 @ w2.T + b2).astype(np.float32)
    h2 = bf16(np.maximum(a2, 0)).astype(np.float64)
    y = (h2 @ w3 + b3).astype(np.float32).astype(np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        nu = float(np.float32(nu_scale)) * softplus(y)
    ok = np.isfinite(nu) & (nu >= 0) & (nu <= float(np.float32(nu_max)))
    f = np.asarray(feats, np.float32)
    if lo is not None:
        ok &= (f >= np.asarray(lo, np.float32)).all(axis=1)
    if hi is not None:
        ok &= (f <= np.asarray(hi, np.float32)).all(axis=1)
    return np.where(ok, nu, np.nan), y


def samples(mac, tipo, tau0c, x0, x1, s_min=0.0):
    """mac: fine macros (nz, ny, nx, 4) = (ux, uy, uz, delta); tipo (nz, ny, nx).
    Returns (feats (rows, 6), target (rows,)) in the row order of
    closure_samples (X fastest over [x0, x1), then Y, then Z)."""
    f32, f64 = np.float32, np.float64
    mac = np.asarray(mac, f64)
    nz, ny, nx = tipo.shape
    cz, cy, cx = nz // 2, ny // 2, nx // 2
    m = mac[:2 * cz, :2 * cy, :2 * cx].reshape(cz, 2, cy, 2, cx, 2, 4)
    t = np.asarray(tipo)[:2 * cz, :2 * cy, :2 * cx].reshape(cz, 2, cy, 2, cx, 2)
    ok = (t == 0).all(axis=(1, 3, 5))
    u = m.mean(axis=(1, 3, 5))
    dev = m - u[:, None, :, None, :, None, :]
    tau = {}
    for name, a, b in (("xx", 0, 0), ("yy", 1, 1), ("zz", 2, 2), ("xy", 0, 1), ("xz", 0, 2), ("yz", 1, 2)):
        tau[name] = (dev[..., a] * dev[..., b]).mean(axis=(1, 3, 5))
    valid = np.zeros((cz, cy, cx), bool)
    core = ok[1:-1, 1:-1, 1:-1] & ok[1:-1, 1:-1, :-2] & ok[1:-1, 1:-1, 2:] & ok[1:-1, :-2, 1:-1] & \
        ok[1:-1, 2:, 1:-1] & ok[:-2, 1:-1, 1:-1] & ok[2:, 1:-1, 1:-1]
    valid[1:-1, 1:-1, 1:-1] = core
    G = np.zeros((cz, cy, cx, 3, 3), f64)    # G[..., a, b] = d u_b / d x_a
    G[:, :, 1:-1, 0, :] = 0.5 * (u[:, :, 2:, :3] - u[:, :, :-2, :3])
    G[:, 1:-1, :, 1, :] = 0.5 * (u[:, 2:, :, :3] - u[:, :-2, :, :3])
    G[1:-1, :, :, 2, :] = 0.5 * (u[2:, :, :, :3] - u[:-2, :, :, :3])
    sxx, syy, szz = G[..., 0, 0], G[..., 1, 1], G[..., 2, 2]
    sxy = 0.5 * (G[..., 0, 1] + G[..., 1, 0])
    sxz = 0.5 * (G[..., 0, 2] + G[..., 2, 0])
    syz = 0.5 * (G[..., 1, 2] + G[..., 2, 1])
    txx, tyy, tzz, txy, txz, tyz = (tau[k] for k in ("xx", "yy", "zz", "xy", "xz", "yz"))
    tr3 = (txx + tyy + tzz) / 3.0
    ss = sxx * sxx + syy * syy + szz * szz + 2.0 * (sxy * sxy + sxz * sxz + syz * syz)
    ts = (txx - tr3) * sxx + (tyy - tr3) * syy + (tzz - tr3) * szz + 2.0 * (txy * sxy + txz * sxz + tyz * syz)
    with np.errstate(divide="ignore", invalid="ignore"):
        nut = np.where((2.0 * ss > s_min * s_min) & (ss > 1e-30), np.maximum(0.0, -ts / (2.0 * ss)), 0.0)
    delta = u[..., 3]
    rho = 1.0 + delta
    k = -(2.0 / 3.0) * rho * (tau0c + 3.0 * nut)
    feats = features(k * sxx, k * syy, k * szz, k * sxy, k * sxz, k * syz, (1.0 / rho).astype(f32),
                     delta.astype(f32), tau0c)
    nut = nut.astype(f32)
    sl = (slice(None), slice(None), slice(x0, x1))
    tgt = np.where(valid, nut, np.nan).astype(f32)[sl].reshape(-1)
    fe = np.where(valid[..., None], feats, f32(0.0))[sl].reshape(-1, 6)
    return fe, tgt
