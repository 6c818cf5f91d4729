"""CPU restatement of the visualisation compute (include/lbm_vis.h) — TEST
INFRASTRUCTURE ONLY: tests/ use it as the checker for cfd__gb300/csrc/vis.cu.
Nothing in the product imports it.

numpy float32, each operation rounded as written (the kernels are built with
-fmad=false), density volumes in float16 as the reference's rgba16float
volume:
  * fumaca_passo   one smoke step: back-trace (src/render/fumaca.js:147-160),
                   MacCormack correction with the eight-corner limiter,
                   dissipation, domain cut-off and rake (:96-132, :186-218);
                   trilinear samples with clamp-to-edge at t = p - 0.5,
                   interpolated along x, y, z as a + f (b - a);
  * esteiras_passo one frame of the streak particles
                   (src/render/renderer.js:51-116) or of the ground streaks
                   (src/render/rasante.js:95-149), with the integer hash;
  * render         the ray-march of the smoke volume into an image
                   (src/render/fumaca.js:257-349).
exp() of the rake and of the ray-march may differ from the GPU's expf in the
last place; tests allow for that where it is used.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def _sample(vol, ax, ay, az):
    nz, ny, nx = vol.shape
    v = vol.astype(np.float32)
    tx, ty, tz = ax - f32(0.5), ay - f32(0.5), az - f32(0.5)
    bx, by, bz = np.floor(tx), np.floor(ty), np.floor(tz)
    fx, fy, fz = tx - bx, ty - by, tz - bz
    x0 = np.clip(bx.astype(np.int64), 0, nx - 1); x1 = np.clip(bx.astype(np.int64) + 1, 0, nx - 1)
    y0 = np.clip(by.astype(np.int64), 0, ny - 1); y1 = np.clip(by.astype(np.int64) + 1, 0, ny - 1)
    z0 = np.clip(bz.astype(np.int64), 0, nz - 1); z1 = np.clip(bz.astype(np.int64) + 1, 0, nz - 1)

    def lerp(a, b, f):
        return a + f * (b - a)
    c00 = lerp(v[z0, y0, x0], v[z0, y0, x1], fx)
    c10 = lerp(v[z0, y1, x0], v[z0, y1, x1], fx)
    c01 = lerp(v[z1, y0, x0], v[z1, y0, x1], fx)
    c11 = lerp(v[z1, y1, x0], v[z1, y1, x1], fx)
    return lerp(lerp(c00, c10, fy), lerp(c01, c11, fy), fz)


def _inside(shape, ax, ay, az):
    nz, ny, nx = shape
    return ((ax >= f32(0.5)) & (ay >= f32(0.5)) & (az >= f32(0.5)) & (ax <= f32(nx) - f32(0.5)) &
            (ay <= f32(ny) - f32(0.5)) & (az <= f32(nz) - f32(0.5)))


def rake(R, F, px, py, pz):
    meia = np.maximum(f32(1.5), f32(F["avanco"]) * f32(0.6))
    dx = np.abs(px - f32(R["x"]))
    ay = (py - f32(R["y0"])) / f32(R["passo_y"])
    az = (pz - f32(R["z0"])) / f32(R["passo_z"])
    fy = np.abs((ay - np.floor(ay)) - f32(0.5)) * f32(R["passo_y"])
    fz = np.abs((az - np.floor(az)) - f32(0.5)) * f32(R["passo_z"])
    r = np.sqrt(fy * fy + fz * fz) / np.maximum(f32(R["raio"]), f32(1e-3))
    with np.errstate(over="ignore"):
        val = f32(F["taxa"]) * np.exp(-r * r * f32(5.5)) * (f32(1.0) - f32(0.35) * dx / meia)
    off = (dx > meia) | (py < f32(R["y0"])) | (py > f32(R["y1"])) | (pz < f32(R["z0"])) | (pz > f32(R["z1"]))
    return np.where(off, f32(0.0), val).astype(np.float32)


def fumaca_passo(cur, mac, tipo, R, F):
    """cur: float16 (nz, ny, nx); mac: float32 (nz, ny, nx, 4); tipo: (nz, ny, nx)."""
    nz, ny, nx = cur.shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    px, py, pz = x.astype(f32) + f32(0.5), y.astype(f32) + f32(0.5), z.astype(f32) + f32(0.5)
    ux, uy, uz = (mac[..., k].astype(np.float32) for k in range(3))
    solid = np.isin(np.asarray(tipo), [1, 4, 7])
    dt = f32(F["dt"])
    ax, ay, az = px - ux * dt, py - uy * dt, pz - uz * dt
    d = _sample(cur, ax, ay, az)
    d = np.where(_inside(cur.shape, ax, ay, az), d, f32(0.0))
    mid = np.where(solid, f32(0.0), d).astype(np.float16)
    chapeu = mid.astype(np.float32)
    voltando = _sample(mid, px + ux * dt, py + uy * dt, pz + uz * dt)
    original = cur.astype(np.float32)
    d = chapeu + f32(0.5) * (original - voltando)
    bx, by, bz = np.floor(ax - f32(0.5)), np.floor(ay - f32(0.5)), np.floor(az - f32(0.5))
    lo = np.full(cur.shape, f32(1e30))
    hi = np.full(cur.shape, f32(-1e30))
    c = cur.astype(np.float32)
    for k in range(8):
        qx = np.clip((bx + f32(k & 1)).astype(np.int64), 0, nx - 1)
        qy = np.clip((by + f32((k >> 1) & 1)).astype(np.int64), 0, ny - 1)
        qz = np.clip((bz + f32((k >> 2) & 1)).astype(np.int64), 0, nz - 1)
        v = c[qz, qy, qx]
        lo = np.minimum(lo, v)
        hi = np.maximum(hi, v)
    d = np.minimum(np.maximum(d, lo), hi) * f32(F["dissipacao"])
    d = np.where(_inside(cur.shape, ax, ay, az), d, f32(0.0))
    d = np.maximum(d, rake(R, F, px, py, pz))
    d = np.minimum(np.maximum(d, f32(0.0)), f32(4.0))
    return np.where(solid, f32(0.0), d).astype(np.float16)


def _hash01(n):
    n = np.asarray(n, np.uint32)
    with np.errstate(over="ignore"):
        x = n * np.uint32(747796405) + np.uint32(2891336453)
        x = ((x >> ((x >> np.uint32(28)) + np.uint32(4))) ^ x) * np.uint32(277803737)
    return ((x >> np.uint32(22)) ^ x).astype(np.float32) / f32(4294967296.0)


def esteiras_passo(parts, mac, dt_quadro, nsub, quadro, rasantes=False, altura=0.0):
    """parts: float32 (n, 8) = pos xyzw, ant xyzw; mac: float32 (nz, ny, nx, 4).
    rasantes: the ground streaks (src/render/rasante.js:95-149)."""
    nz, ny, nx = mac.shape[:3]
    P = np.array(parts, np.float32, copy=True)

    def nearest(px, py, pz):
        ix = np.clip(px.astype(np.int64), 0, nx - 1)
        iy = np.clip(py.astype(np.int64), 0, ny - 1)
        iz = np.clip(pz.astype(np.int64), 0, nz - 1)
        return mac[iz, iy, ix].astype(np.float32)
    m = nearest(P[:, 0], P[:, 1], P[:, 2])
    ns = max(int(nsub), 1)
    dt = f32(dt_quadro) / f32(ns)
    x, y, z = P[:, 0].copy(), P[:, 1].copy(), P[:, 2].copy()
    for _ in range(ns):
        u = nearest(x, y, z)
        x = x + u[:, 0] * dt
        y = y + u[:, 1] * dt
        z = z + u[:, 2] * dt
    w = P[:, 3] - f32(1.0)
    fx, fy, fz = f32(nx), f32(ny), f32(nz)
    zmin = f32(0.4) if rasantes else f32(0.5)
    fora = (x >= fx - f32(1.0)) | (x < f32(1.0)) | (y < f32(1.0)) | (y >= fy - f32(1.0)) | (z < zmin) | \
        (z >= fz - f32(1.0))
    presa = np.sqrt(m[:, 0] * m[:, 0] + m[:, 1] * m[:, 1] + m[:, 2] * m[:, 2]) < f32(1e-5)
    renasce = fora | presa | (w <= f32(0.0))
    with np.errstate(over="ignore"):
        s = np.arange(P.shape[0], dtype=np.uint32) * np.uint32(3) + np.uint32(quadro) * np.uint32(7919)
    if rasantes:
        h = _hash01(s + np.uint32(2))
        rx = f32(1.5) + _hash01(s) * f32(4.0)
        ry = f32(1.0) + _hash01(s + np.uint32(1)) * (fy - f32(2.0))
        rz = f32(0.6) + h * h * h * f32(altura)
        rw = f32(150.0) + _hash01(s + np.uint32(5)) * f32(320.0)
    else:
        rx = f32(2.0) + _hash01(s) * f32(3.0)
        ry = f32(2.0) + _hash01(s + np.uint32(1)) * (fy - f32(4.0))
        rz = f32(0.5) + _hash01(s + np.uint32(2)) * (fz - f32(2.0))
        rw = f32(220.0) + _hash01(s + np.uint32(5)) * f32(260.0)
    out = np.empty_like(P)
    out[:, 0] = np.where(renasce, rx, x)
    out[:, 1] = np.where(renasce, ry, y)
    out[:, 2] = np.where(renasce, rz, z)
    out[:, 3] = np.where(renasce, rw, w)
    out[:, 4] = np.where(renasce, rx, P[:, 0])
    out[:, 5] = np.where(renasce, ry, P[:, 1])
    out[:, 6] = np.where(renasce, rz, P[:, 2])
    out[:, 7] = np.where(renasce, f32(0.0), f32(1.0))
    return out


def _fract(x):
    return x - np.floor(x)


def render(vol, inv_view_proj, olho, largura, altura, densidade, g, passos, passos_luz, luz, intensidade, quadro):
    """Ray-march of a float16 volume (src/render/fumaca.js:257-349) into an
    (altura, largura, 4) float32 image; no opaque depth; rays that miss give 0."""
    nz, ny, nx = vol.shape
    m = np.asarray(inv_view_proj, np.float32)
    iy, ix = np.meshgrid(np.arange(altura), np.arange(largura), indexing="ij")
    fx, fy = ix.astype(f32) + f32(0.5), iy.astype(f32) + f32(0.5)
    ndx = fx / f32(largura) * f32(2.0) - f32(1.0)
    ndy = f32(1.0) - fy / f32(altura) * f32(2.0)
    h = [((m[i] * ndx + m[4 + i] * ndy) + m[8 + i] * f32(1.0)) + m[12 + i] for i in range(4)]
    alvo = [h[0] / h[3], h[1] / h[3], h[2] / h[3]]
    o = [f32(v) for v in olho]
    d = [alvo[0] - o[0], alvo[1] - o[1], alvo[2] - o[2]]
    ln = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    d = [d[0] / ln, d[1] / ln, d[2] / ln]
    k = (f32(1.0) / f32(nx)) * f32(2.0)
    lo = [-f32(nx) * f32(0.5) * k, -f32(ny) * f32(0.5) * k, f32(0.0)]
    hi = [f32(nx) * f32(0.5) * k, f32(ny) * f32(0.5) * k, f32(nz) * k]
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        inv = [f32(1.0) / d[a] for a in range(3)]
        ta = [(lo[a] - o[a]) * inv[a] for a in range(3)]
        tb = [(hi[a] - o[a]) * inv[a] for a in range(3)]
    tmin = np.maximum(np.maximum(np.minimum(ta[0], tb[0]), np.minimum(ta[1], tb[1])), np.minimum(ta[2], tb[2]))
    tmax = np.minimum(np.minimum(np.maximum(ta[0], tb[0]), np.maximum(ta[1], tb[1])), np.maximum(ta[2], tb[2]))
    t0 = np.maximum(tmin, f32(0.0))
    t1 = tmax
    hit = t1 > t0
    ds = (t1 - t0) / f32(passos)
    ll = np.sqrt(f32(luz[0]) ** 2 + f32(luz[1]) ** 2 + f32(luz[2]) ** 2)
    L = [f32(luz[0]) / ll, f32(luz[1]) / ll, f32(luz[2]) / ll]
    gg = f32(g)
    g2 = gg * gg
    cos = d[0] * L[0] + d[1] * L[1] + d[2] * L[2]
    dd = f32(1.0) + g2 - f32(2.0) * gg * cos
    fase = (f32(1.0) - g2) / (f32(12.566370614) * np.maximum(dd * np.sqrt(dd), f32(1e-4)))
    qx = fx + f32(quadro) * f32(0.618)
    qy = fy + f32(quadro) * f32(0.618)
    p3x, p3y, p3z = _fract(qx * f32(0.1031)), _fract(qy * f32(0.1031)), _fract(qx * f32(0.1031))
    dt_ = p3x * (p3y + f32(33.33)) + p3y * (p3z + f32(33.33)) + p3z * (p3x + f32(33.33))
    p3x, p3y, p3z = p3x + dt_, p3y + dt_, p3z + dt_
    jitter = _fract((p3x + p3y) * p3z) * ds

    def dens(wx, wy, wz):
        px = wx / k + f32(nx) * f32(0.5)
        py = wy / k + f32(ny) * f32(0.5)
        pz = wz / k
        ux, uy, uz = px / f32(nx), py / f32(ny), pz / f32(nz)
        out = (ux < 0) | (uy < 0) | (uz < 0) | (ux > 1) | (uy > 1) | (uz > 1)
        v = _sample(vol, np.where(out, f32(1.0), px), np.where(out, f32(1.0), py), np.where(out, f32(1.0), pz))
        return np.where(out, f32(0.0), v).astype(np.float32)
    T = np.ones(fx.shape, np.float32)
    Lr, Lg, Lb = (np.zeros(fx.shape, np.float32) for _ in range(3))
    s = t0 + jitter
    sigma = f32(densidade)
    dl = (hi[2] - lo[2]) / f32(passos_luz) * f32(0.9)
    alive = hit.copy()
    for _ in range(passos):
        alive &= ~(T < f32(0.01))
        wx, wy, wz = o[0] + d[0] * s, o[1] + d[1] * s, o[2] + d[2] * s
        dv = dens(wx, wy, wz)
        s = s + ds
        act = alive & ~(dv <= f32(0.001))
        st = dv * sigma
        with np.errstate(over="ignore", invalid="ignore"):
            atenua = f32(1.0) - np.exp(-st * ds)
            tau = np.zeros(fx.shape, np.float32)
            for j in range(1, passos_luz + 1):
                off = f32(j) * dl
                tau = tau + dens(wx + L[0] * off, wy + L[1] * off, wz + L[2] * off) * sigma * dl
            lz = np.exp(-tau)
            amb = f32(0.16) + f32(0.10) * np.exp(-tau * f32(0.35))
            c = T * atenua * (lz * fase * f32(3.6) + amb) * f32(intensidade)
            Lr = np.where(act, Lr + c * f32(0.96), Lr)
            Lg = np.where(act, Lg + c * f32(0.97), Lg)
            Lb = np.where(act, Lb + c * f32(1.0), Lb)
            T = np.where(act, T * np.exp(-st * ds), T)
    img = np.zeros((altura, largura, 4), np.float32)
    img[..., 0] = np.where(hit, Lr, 0)
    img[..., 1] = np.where(hit, Lg, 0)
    img[..., 2] = np.where(hit, Lb, 0)
    img[..., 3] = np.where(hit, f32(1.0) - T, 0)
    return img


def cp_triangulos(pos, idx, mac, tipo, u_ref):
    """Surface Cp per triangle at its centroid (src/render/renderer.js:168-180)."""
    nz, ny, nx = np.asarray(tipo).shape
    p = np.asarray(pos, np.float32).reshape(-1, 3)
    t = np.asarray(idx, np.int64).reshape(-1, 3)
    v0, v1, v2 = p[t[:, 0]], p[t[:, 1]], p[t[:, 2]]
    e1, e2 = v1 - v0, v2 - v0
    n = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1], e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                  e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], axis=1)
    ln = np.sqrt(n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1] + n[:, 2] * n[:, 2])
    n = n / ln[:, None]
    cen = ((v0 + v1) + v2) / f32(3.0)
    fora = cen + n * f32(1.8)

    def cell(q):
        ix = np.clip(q[:, 0].astype(np.int64), 0, nx - 1)
        iy = np.clip(q[:, 1].astype(np.int64), 0, ny - 1)
        iz = np.clip(q[:, 2].astype(np.int64), 0, nz - 1)
        return iz, iy, ix
    solid = np.isin(np.asarray(tipo)[cell(fora)], [1, 4, 7])
    fora = np.where(solid[:, None], cen - n * f32(1.8), fora)
    delta = np.asarray(mac, np.float32)[cell(fora) + (3,)]
    return delta / np.maximum(f32(1.5) * f32(u_ref) * f32(u_ref), f32(1e-12))
