"""Learned eddy-viscosity closure (include/lbm_closure.h) from Python.

The reference's only sub-grid model is the closed-form Smagorinsky relaxation
time (src/core/emit/ir.js:262-301).  This module holds the network that
replaces it when ``configurar(closure=1)``: weights as a dict of numpy arrays,
training (hand-written CUDA forward / backward / Adam), evaluation through the
tensor-core path the fused step uses, and the training samples cut from a
fine run.

Network: 6 -> 32 -> 32 -> 1, ReLU hidden layers, output nu_scale *
softplus(y): the eddy viscosity nu_t, or (coef = 1) a per-cell Smagorinsky
coefficient Cs^2 that the step uses with its own |S| estimate.  Features
(raw, then normalised (x - mean) / std):
    x0 = ln(qs/rho + 1e-9), qs = sqrt(2 Pi:Pi)
    x1 = tr(Pi) / (qs + 1e-12)
    x2 = det(Pi) / (qs^3 + 1e-30)
    x3 = (Pxy^2 + Pxz^2 + Pyz^2) / (Pi:Pi / 2 + 1e-30)
    x4 = 1 / tau0
    x5 = 100 delta
of the non-equilibrium stress Pi of the pulled populations.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat

NI, NH = nat.CLOSURE_IN, nat.CLOSURE_H
NP = nat.CLOSURE_NPARAM
CAMPOS = ("w1", "b1", "w2", "b2", "w3", "b3")
FORMAS = {"w1": (NH, NI), "b1": (NH,), "w2": (NH, NH), "b2": (NH,), "w3": (NH,), "b3": ()}


def pesos_vazios():
    """Zero weights, identity normalisation, nu_scale 1, nu_max 1."""
    d = {k: np.zeros(s, np.float32) for k, s in FORMAS.items()}
    d["mean"] = np.zeros(NI, np.float32)
    d["std"] = np.ones(NI, np.float32)
    d["nu_scale"] = 1.0
    d["nu_max"] = 1.0
    d["lo"] = np.full(NI, -np.inf, np.float32)
    d["hi"] = np.full(NI, np.inf, np.float32)
    d["coef"] = 0
    return d


def vetor(p) -> np.ndarray:
    """The 1313 trainable parameters in ABI order (w1, b1, w2, b2, w3, b3)."""
    return np.concatenate([np.asarray(p[k], np.float32).reshape(-1) for k in CAMPOS])


def de_vetor(v, base=None):
    p = dict(pesos_vazios() if base is None else base)
    o = 0
    for k in CAMPOS:
        n = int(np.prod(FORMAS[k])) if FORMAS[k] else 1
        p[k] = np.asarray(v[o:o + n], np.float32).reshape(FORMAS[k]) if FORMAS[k] else np.float32(v[o])
        o += n
    return p


def para_struct(p) -> nat.ClosureWeights:
    w = nat.ClosureWeights()
    v = vetor(p)
    C.memmove(C.addressof(w), v.ctypes.data, 4 * NP)
    for a in range(NI):
        w.mean[a] = float(p["mean"][a])
        w.std[a] = float(p["std"][a])
    w.nu_scale = float(p["nu_scale"])
    w.nu_max = float(p["nu_max"])
    lo = p.get("lo", np.full(NI, -np.inf))
    hi = p.get("hi", np.full(NI, np.inf))
    for a in range(NI):
        w.lo[a] = float(lo[a])
        w.hi[a] = float(hi[a])
    w.coef = int(p.get("coef", 0))
    return w


def de_struct(w: nat.ClosureWeights, base=None):
    v = np.frombuffer((C.c_float * NP).from_address(C.addressof(w)), np.float32).copy()
    p = de_vetor(v, base)
    p["mean"] = np.array(w.mean[:], np.float32)
    p["std"] = np.array(w.std[:], np.float32)
    p["nu_scale"] = float(w.nu_scale)
    p["nu_max"] = float(w.nu_max)
    p["lo"] = np.array(w.lo[:], np.float32)
    p["hi"] = np.array(w.hi[:], np.float32)
    p["coef"] = int(w.coef)
    return p


def _rows(feats, target=None):
    f = np.ascontiguousarray(feats, np.float32).reshape(-1, NI)
    if target is None:
        return f, None
    t = np.ascontiguousarray(target, np.float32).reshape(-1)
    if t.size != f.shape[0]:
        raise ValueError("features and targets differ in length")
    return f, t


def gradiente(feats, target, p):
    """(loss, grad[1313]) of the normalised MSE on all rows, fp32 kernels."""
    L = nat.load()
    f, t = _rows(feats, target)
    w = para_struct(p)
    loss = C.c_float()
    g = np.zeros(NP, np.float32)
    nat.check(L.closure_grad(nat.ptr(f), nat.ptr(t), f.shape[0], C.byref(w), C.byref(loss), nat.ptr(g)))
    return float(loss.value), g


def treinar(feats, target, p, passos, lote=65536, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, semente=2026,
            iniciar=True):
    """Adam on minibatches drawn with replacement; returns (weights, loss per step)."""
    L = nat.load()
    f, t = _rows(feats, target)
    w = para_struct(p)
    cfg = nat.ClosureCfg(int(passos), int(lote), float(lr), float(beta1), float(beta2), float(eps),
                         int(semente), 1 if iniciar else 0, 0)
    hist = np.zeros(max(1, int(passos)), np.float32)
    nat.check(L.closure_train(nat.ptr(f), nat.ptr(t), f.shape[0], C.byref(cfg), C.byref(w), nat.ptr(hist)))
    return de_struct(w, p), hist[:int(passos)]


def avaliar(p, feats, motor=0):
    """nu_t per row through a tensor-core engine of the step (0 warp mma.sync,
    1 CTA tcgen05); NaN = Smagorinsky fallback."""
    L = nat.load()
    f, _ = _rows(feats)
    out = np.empty(f.shape[0], np.float32)
    w = para_struct(p)
    nat.check(L.closure_eval(C.byref(w), nat.ptr(f), f.shape[0], int(motor), nat.ptr(out)))
    return out


def amostras(solver, tau0_grosso, x0=None, x1=None, s_min=0.0):
    """Rows of closure_samples for a fine SolverCUDA: (feats[m, 6], target[m]),
    one row per coarse cell with x0 <= X < x1, target NaN where not usable,
    0 where the filtered strain rate |S| is below s_min."""
    L = nat.load()
    cx, cy, cz = solver.nx // 2, solver.ny // 2, solver.nz // 2
    x0 = 0 if x0 is None else int(x0)
    x1 = cx if x1 is None else int(x1)
    m = (x1 - x0) * cy * cz
    f = np.empty((m, NI), np.float32)
    t = np.empty(m, np.float32)
    nat.check(L.closure_samples(solver._h, float(tau0_grosso), float(s_min), x0, x1, nat.ptr(f), nat.ptr(t), m))
    return f, t


def normalizacao(feats, target, q_escala=0.9, q_max=0.999, fator_max=20.0, q_faixa=1e-4):
    """mean / std of the features; nu_scale = the q_escala quantile of the
    positive targets; nu_max = fator_max times their q_max quantile; the
    trained range [lo, hi] of each raw feature = its q_faixa and 1 - q_faixa
    quantiles (a constant feature gets its value +- 1 %)."""
    f, t = _rows(feats, target)
    mean = f.mean(axis=0).astype(np.float32)
    std = f.std(axis=0).astype(np.float32)
    std[std < 1e-6] = 1.0
    pos = t[t > 0]
    escala = float(np.quantile(pos, q_escala)) if pos.size else 1e-4
    alto = float(np.quantile(pos, q_max)) if pos.size else escala
    lo = np.quantile(f, q_faixa, axis=0)
    hi = np.quantile(f, 1.0 - q_faixa, axis=0)
    larg = np.maximum(hi - lo, 0.01 * np.abs(hi))
    lo = np.where(hi - lo < 1e-9, lo - larg, lo)
    hi = np.where(hi - lo < 1e-9, hi + larg, hi)
    return {"mean": mean, "std": std, "nu_scale": max(escala, 1e-8), "nu_max": float(fator_max * max(alto, escala)),
            "lo": lo.astype(np.float32), "hi": hi.astype(np.float32)}


def salvar(p, caminho):
    """Weights to an .npz file."""
    np.savez(caminho, **{k: np.asarray(v) for k, v in p.items()})


def carregar(caminho):
    d = np.load(caminho)
    p = pesos_vazios()
    for k in d.files:
        v = d[k]
        if k == "coef":
            p[k] = int(v)
        else:
            p[k] = float(v) if k in ("nu_scale", "nu_max") else (np.float32(v) if v.shape == () else v.astype(np.float32))
    return p
