"""Studies of the storage forms and the batched form on one GB300.

    python -m cfd__gb300.estudos precisao [--steps 10000] [--grid 512,256,192]
    python -m cfd__gb300.estudos lote [--steps 256]
    python -m cfd__gb300.estudos fecho [--steps 24000] [--pesos w.npz]
    python -m cfd__gb300.estudos casos

precisao: the 512x256x192 precision workload (25.2 M cells): the seeded
superellipsoid (semi-axes 80x32x22 cells, 20k triangles, 0.3-cell jitter)
voxelized on the GPU and centred vertically, free-slip walls on every side
(the sphere case's tunnel, tests/validacao.html:224-231), u_in 0.05,
nu 0.008 (omega+ 1.9084), Smagorinsky Cs 0.1.  The same run in four storage
forms: fp32, fp16 of g*2^10, bf16 — all with fp32 arithmetic — and the fp64
fp64 reference form (fp64 storage and arithmetic).  Reported per form: MLUPS and fraction of
the HBM roofline (bytes per cell 152 / 76 / 76 / 304), the drag coefficient
averaged over the last quarter of the run (Maskell-corrected, theta 2.5) and
its error against the fp64 run, and the relative L2 error of the velocity
field against the fp64 run.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np

BYTES = {"f32": 152, "f16s": 76, "bf16s": 76, "f64": 304, "f16sr": 76, "bf16sr": 76}


def _peak():
    import os
    p = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def malha_precisao(grade):
    """Mesh of the precision workload: the seeded superellipsoid (semi-axes
    80x32x22 cells, 20k triangles, 0.3-cell jitter), nose at 0.28 nx, centred
    in y and z."""
    from .geometry import colocar, superelipsoide
    pos, idx = superelipsoide(80.0, 32.0, 22.0, 2.5, 3.0, 20000, 0.3, 2027)
    pos = colocar(pos, grade, nariz=0.28, folga_piso=0.0)
    dz = 0.5 * grade["nz"] - 0.5 * (pos[:, 2].min() + pos[:, 2].max())
    pos[:, 2] += np.float32(dz)
    return pos, idx


def caso_precisao(grade, voxelizador=None):
    """Cell types, parameters and frontal area of the precision workload.
    voxelizador(pos, idx, grade) -> VOXEL codes; default: the GPU voxelizer."""
    from .tunel import areaFrontalCorpo, montarTipos
    pos, idx = malha_precisao(grade)
    if voxelizador is None:
        from .voxel import voxelizar
        corpo = voxelizar(pos, idx, grade, sdf=False)["tipo"]
    else:
        corpo = voxelizador(pos, idx, grade)
    mt = montarTipos(grade, corpo=corpo, esteira=False)
    t = mt["tipo"].reshape(grade["nz"], grade["ny"], grade["nx"])
    t[0, :, 1:grade["nx"] - 1] = 6          # free-slip floor as well
    area = areaFrontalCorpo(corpo, grade)
    nu = 0.008
    cfg = dict(omegaPlus=1.0 / (3.0 * nu + 0.5), lesCs=0.1, inletU=[0.05, 0.0, 0.0], esponja=mt["esponja"])
    return mt["tipo"], cfg, area


def _subnormal_share(s, fluid):
    """Where the fp16 store's rounding sits: of the fluid cells' stored values
    g·2^10 at the end of the run, the share that is zero, the share in the
    subnormal range (0 < |v| < 2^-14, where fp16 keeps fewer than 11 bits),
    and per direction the median |g|.  A per-direction power-of-two scale
    changes the rounding of the subnormal share only: a normal fp16 value
    keeps 11 significant bits at any exponent."""
    g = s.lerPopulacoes()
    out = {"per_direction_median_abs_g": [], "per_direction_subnormal_share": []}
    n_sub = n_zero = n_all = 0
    for i in range(19):
        v = np.abs(g[i, fluid]) * 1024.0
        z = int(np.count_nonzero(v == 0.0))
        sb = int(np.count_nonzero((v > 0.0) & (v < 2.0 ** -14)))
        n_zero += z
        n_sub += sb
        n_all += v.size
        out["per_direction_median_abs_g"].append(float(np.median(v)) / 1024.0)
        out["per_direction_subnormal_share"].append(sb / v.size)
    out["zero_share"] = n_zero / n_all
    out["subnormal_share"] = n_sub / n_all
    return out


def precisao(steps=10000, grade=None, forms=("f64", "f32", "f16s", "bf16s", "f16sr", "bf16sr"), sample=50):
    import torch

    from .forces import coeficientes
    from .solver import SolverCUDA
    from .units import LatticeUnits
    grade = grade or {"nx": 512, "ny": 256, "nz": 192}
    tipo, cfg, area = caso_precisao(grade)
    N = int(tipo.size)
    units = LatticeUnits(0.05)
    fluid = ~np.isin(tipo, [1, 4, 7])
    out = {"grid": grade, "cells": N, "steps": steps, "frontal_area": area, "forms": {}}
    ref_u = None
    stream = torch.cuda.Stream()
    for form in forms:
        s = SolverCUDA(grade, storage=form, escrever_macros=False)
        s.definirStream(stream.cuda_stream)
        s.definirTipos(tipo)
        s.configurar(**cfg)
        s.calibrarRepouso()
        s.inicializar()
        cds = []
        ms_total = 0.0
        done = 0
        while done < steps:
            n = min(sample, steps - done)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.passo(n)
            e1.record(stream)
            e1.synchronize()
            ms_total += e0.elapsed_time(e1)
            done += n
            f = s.medirForcas()
            cds.append(coeficientes(f, units, area, grade)["cd"])
        s.atualizarMacros()
        m = s.lerMacros().reshape(-1, 4)[:, :3].astype(np.float64)[fluid]
        sub = _subnormal_share(s, fluid) if form in ("f16s", "f16sr") else None
        s.destruir()
        tail = cds[len(cds) * 3 // 4:]
        cd = float(np.mean(tail))
        mlups = N * steps / (ms_total / 1e3) / 1e6
        rec = {"MLUPS": mlups, "roofline_frac": BYTES[form] * mlups * 1e6 / 1e9 / _peak(),
               "cd": cd, "cd_finite": bool(np.isfinite(cds).all())}
        if sub is not None:
            rec["stored_values"] = sub
        if ref_u is None:
            ref_u, ref_cd = m, cd
        else:
            rec["cd_err_vs_f64"] = (cd - ref_cd) / ref_cd
            rec["u_l2_rel_err_vs_f64"] = float(np.linalg.norm(m - ref_u) / np.linalg.norm(ref_u))
        out["forms"][form] = rec
    return out


def lote(n_tunnels=64, steps=256, storages=("f32", "f16s", "f16sr"), seed=2026):
    """Batched workload: n tunnels drawn by sorteio_lote (96x48x48 to
    256x128x128).  Aggregate MLUPS = sum N_k * steps / time, for the batch in
    mode 0 (a captured graph of per-tunnel chains), in mode 1 (one persistent
    launch per step over all tunnels' tiles) with the cost model's tiles, in
    the configuration lbm_batch_autotune measures best (its choices are
    recorded), and for the same tunnels run one after another with the
    single-tunnel solver.  Every form is timed over `steps` steps between CUDA
    events after 64 warm-up steps."""
    import torch

    from .lote import LoteCUDA, sorteio_lote
    from .solver import SolverCUDA
    tun = sorteio_lote(n_tunnels, seed)
    cells = sum(t[0]["nx"] * t[0]["ny"] * t[0]["nz"] for t in tun)
    out = {"tunnels": n_tunnels, "cells": cells, "steps": steps,
           "omega_flagged": int(sum(t[3]["flag_omega"] for t in tun)), "forms": {}}
    stream = torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def novo(st, modo):
        L = LoteCUDA([t[0] for t in tun], storage=st)
        L.definirStream(stream.cuda_stream)
        L.definirModo(modo)
        for k, (g, tipo, cfg, info) in enumerate(tun):
            L.definirTipos(k, tipo)
            L.configurar(k, **cfg)
        L.inicializar()
        return L

    def cronometrar(L):
        L.passo(64)
        torch.cuda.synchronize()
        e0.record(stream)
        L.passo(steps)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    for st in storages:
        ms_modes = {}
        for modo in (0, 1):
            L = novo(st, modo)
            ms_modes[modo] = cronometrar(L)
            L.destruir()
        L = novo(st, 0)
        L.passo(64)
        escolha = L.autoajustar(64)
        ms_tuned = cronometrar(L)
        classes = {}
        for k, (g, tipo, cfg, info) in enumerate(tun):
            classes.setdefault(g["nx"], escolha["tiles"][k])
        L.destruir()
        ms_seq = 0.0
        for g, tipo, cfg, info in tun:
            s = SolverCUDA(g, storage=st, escrever_macros=False)
            s.definirStream(stream.cuda_stream)
            s.definirTipos(tipo)
            s.configurar(**cfg)
            s.inicializar()
            s.passo(8)
            torch.cuda.synchronize()
            e0.record(stream)
            s.passo(steps)
            e1.record(stream)
            e1.synchronize()
            ms_seq += e0.elapsed_time(e1)
            s.destruir()
        mlups = lambda ms: cells * steps / (ms / 1e3) / 1e6
        out["forms"][st] = {"mode0_graph_of_chains_MLUPS": mlups(ms_modes[0]),
                            "mode1_persistent_launch_MLUPS": mlups(ms_modes[1]),
                            "tuned_MLUPS": mlups(ms_tuned),
                            "tuner_choice": {"mode": escolha["mode"],
                                             "resident_ctas_per_sm": escolha["resident_ctas_per_sm"],
                                             "tile_x_per_nx": {str(k): v for k, v in sorted(classes.items())},
                                             "measured_ms_per_step": escolha["ms_per_step"]},
                            "sequential_MLUPS": mlups(ms_seq),
                            "mode1_vs_sequential": ms_seq / ms_modes[1],
                            "tuned_vs_sequential": ms_seq / ms_tuned}
    return out


def tuneis_fecho(seed=2026):
    """The coarse 320x160x128 mesh-body tunnel and its 2x fine twin
    640x320x256: the same 20k-triangle superellipsoid (48x20x14 cells on the
    coarse grid) with every vertex scaled by 2, the floor two fine rows thick
    so the no-slip wall sits where the coarse one does.  Returns
    ((grid, types, sponge, frontal area), ...) for coarse and fine."""
    from .geometry import corpo_config2
    from .tunel import areaFrontalCorpo, montarTipos
    from .voxel import voxelizar
    gc = {"nx": 320, "ny": 160, "nz": 128}
    gf = {"nx": 640, "ny": 320, "nz": 256}
    pos, idx = corpo_config2(gc, seed)
    out = []
    for g, k in ((gc, 1.0), (gf, 2.0)):
        vox = voxelizar((pos * np.float32(k)).astype(np.float32), idx, g, sdf=False)
        mt = montarTipos(g, corpo=vox["tipo"], esteira=False)
        if k == 2.0:
            t = mt["tipo"].reshape(g["nz"], g["ny"], g["nx"])
            row = t[1, 1:g["ny"] - 1, 1:g["nx"] - 1]
            row[row == 0] = 7
        out.append((g, mt["tipo"], mt["esponja"], areaFrontalCorpo(vox["tipo"], g)))
    return out[0], out[1]


def rodar_fecho(g, tipo, esp, area, re, passos, bloco, u=0.06, comprimento=96.0, cs=0.12, closure=None, cada_k=1,
                colher=None, snapshots=4, intervalo=1000, cronometrar=False, stream=None, motor=0):
    """One run of the learned-closure workload's tunnel: Re on `comprimento`
    cells, u_in u, Smagorinsky Cs cs, or the network `closure` (weights
    dict) evaluated every `cada_k` steps on engine `motor`.  Cd (Maskell,
    src/core/forces.js:55-95) of the force averaged over each block of
    `bloco` steps; reported: the mean and std of the second half of the
    blocks.  colher(s): called at the last `snapshots` states `intervalo`
    steps apart (training samples)."""
    import torch

    from .forces import coeficientes
    from .solver import SolverCUDA
    from .units import LatticeUnits
    units = LatticeUnits(u)
    nu = u * comprimento / re
    s = SolverCUDA(g, escrever_macros=False)
    if stream is not None:
        s.definirStream(stream.cuda_stream)
    s.definirTipos(tipo)
    s.configurar(omegaPlus=1.0 / (3.0 * nu + 0.5), lesCs=cs, inletU=[u, 0.0, 0.0], esponja=esp,
                 closure=cada_k if closure is not None else 0)
    if closure is not None:
        s.definirFecho(closure)
        s.motorFecho(motor)
        s.estatisticasFecho()
    s.inicializar()
    cds, feito, amos = [], 0, []
    t0 = time.time()
    while feito < passos:
        n = min(bloco, passos - feito)
        f = s.passoComForcas(n)
        feito += n
        c = coeficientes(f.mean(axis=0), units, area, g)["cd"]
        cds.append(c)
        if not np.isfinite(c) or abs(c) > 100:
            break
        if colher is not None and feito > passos - snapshots * intervalo and (passos - feito) % intervalo == 0:
            amos.append(colher(s))
    rec = {"Re": re, "omega_plus": 1.0 / (3.0 * nu + 0.5), "steps": feito, "diverged": bool(feito < passos),
           "wall_s": time.time() - t0}
    tail = cds[len(cds) // 2:]
    rec["cd"] = float(np.mean(tail)) if tail and not rec["diverged"] else float("nan")
    rec["cd_std"] = float(np.std(tail)) if tail and not rec["diverged"] else float("nan")
    if closure is not None:
        fb, fl = s.estatisticasFecho()
        rec["fallback_cells"], rec["network_cell_evaluations"] = fb, fl
        rec["fallback_rate"] = fb / max(fl, 1)
    if cronometrar and not rec["diverged"]:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        st = stream if stream is not None else torch.cuda.current_stream()
        e0.record(st)
        s.passo(400)
        e1.record(st)
        e1.synchronize()
        rec["ms_per_step"] = e0.elapsed_time(e1) / 400
        rec["MLUPS"] = s.N / rec["ms_per_step"] / 1e3
    s.destruir()
    return rec, amos


def fecho(re_treino=(2000, 5000, 20000), re_teste=10000, passos_finos=24000, snapshots=4, intervalo=1000,
          por_snapshot=300000, passos_treino=3000, cs=0.12, u=0.06, comprimento=96.0, semente=2026,
          s_min=2e-4, escalas=(2.0, 1.0, 0.5, 0.25, 0.125), cada=8, forma="coef", pesos_saida=None):
    """Learned-closure workload.

    Fine runs (2x resolution, FP32, Smagorinsky Cs) at the training and the
    held-out Reynolds numbers; at their last `snapshots` states `intervalo`
    fine steps apart, a-priori samples (closure_samples: 2x2x2 box filter,
    least-squares eddy viscosity of the resolved residual stress, coarse-grid
    features; target 0 where the filtered strain rate is below s_min);
    `por_snapshot` valid rows drawn from x in [0.25, 0.85) of the coarse
    length.  forma "nu": the network's output is nu_t and the target the
    a-priori eddy viscosity; forma "coef" (default): the output is a
    per-cell Smagorinsky Cs^2 used with the step's own |S| estimate, the
    target nu_t / |S| of the filtered field, feature x0 (the magnitude,
    whose in-situ distribution is dominated by grid-scale non-equilibrium
    at omega near 2) switched off and the bounded invariants x1..x3 checked
    against their mathematical range only.  Training on the training
    Reynolds numbers (targets clipped at the 99.9th percentile of their
    positive values; batch 65 536, Adam).
    A-posteriori calibration: coarse runs at the training Reynolds numbers
    with nu_t scaled by each factor in `escalas`; the factor with the
    smallest mean |Cd error| against the fine runs is kept.  Evaluation at
    the held-out Reynolds number: a-priori (held-out samples, network and
    Smagorinsky against the target) and a-posteriori (coarse runs: learned
    closure every step and every `cada`-th step, Smagorinsky, no model; Cd
    over the second half of passos_finos / 2 coarse steps, from the force
    averaged over each block of steps, against the fine run's Cd over the
    same physical time).  Step time of each coarse form from 400 steps
    timed alone, and the fallback rate of the network."""
    import torch

    from .fecho import amostras, avaliar, normalizacao, pesos_vazios, salvar, treinar
    (gc, tc, ec, ac), (gf, tf, ef, af) = tuneis_fecho(semente)
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(semente)
    cx = gc["nx"]
    x0, x1 = int(0.25 * cx), int(0.85 * cx)
    out = {"coarse": gc, "fine": gf, "frontal_area": {"coarse": ac, "fine": af}, "u_in": u, "cs": cs,
           "length_coarse": comprimento, "s_min": s_min, "fine_runs": {}, "calibration": {}, "coarse_runs": {}}

    def rodar(g, tipo, esp, area, re, passos, bloco, closure=None, cada_k=1, colher=None, cs_run=cs,
              cronometrar=False):
        return rodar_fecho(g, tipo, esp, area, re, passos, bloco, u=u, comprimento=comprimento * g["nx"] / cx,
                           cs=cs_run, closure=closure, cada_k=cada_k, colher=colher, snapshots=snapshots,
                           intervalo=intervalo, cronometrar=cronometrar, stream=stream)

    def colhedor(re):
        tau0c = 3.0 * u * comprimento / re + 0.5

        def colher(s):
            f, t = amostras(s, tau0c, x0, x1, s_min=s_min)
            ok = np.flatnonzero(np.isfinite(t))
            pick = rng.choice(ok, size=min(por_snapshot, ok.size), replace=False)
            pick.sort()
            return f[pick], t[pick]
        return colher

    dados = {}
    for re in tuple(re_treino) + (re_teste,):
        rec, amos = rodar(gf, tf, ef, af, re, passos_finos, intervalo // 2, colher=colhedor(re))
        out["fine_runs"][str(re)] = rec
        if amos:
            dados[re] = (np.concatenate([a[0] for a in amos]), np.concatenate([a[1] for a in amos]))
            rec["samples"] = int(dados[re][1].size)
            rec["target_mean"] = float(dados[re][1].mean())
            rec["target_zero_fraction"] = float((dados[re][1] == 0).mean())
    treino = [re for re in re_treino if re in dados]
    F = np.concatenate([dados[re][0] for re in treino])
    T = np.concatenate([dados[re][1] for re in treino])
    def alvo(Fx, Tx, re):
        if forma != "coef":
            return Tx
        tau0c = 3.0 * u * comprimento / re + 0.5
        s_abs = 1.5 * np.exp(Fx[:, 0].astype(np.float64)) / (tau0c + 3.0 * Tx)   # |S| of the filtered field
        return np.where(Tx > 0, Tx / np.maximum(s_abs, 1e-30), 0.0).astype(np.float32)
    T = np.concatenate([alvo(dados[re][0], dados[re][1], re) for re in treino])
    pos = T[T > 0]
    t_clip = float(np.quantile(pos, 0.999)) if pos.size else 1.0
    T = np.minimum(T, np.float32(t_clip))
    p = pesos_vazios()
    p.update(normalizacao(F, T))
    if forma == "coef":
        p["coef"] = 1
        p["mean"][0], p["std"][0] = 0.0, 1e30
        bound = np.array([np.inf, 1.2248, 0.069, 1.0], np.float32)
        p["lo"][:4] = -bound
        p["hi"][:4] = bound
    t0 = time.time()
    p, hist = treinar(F, T, p, passos=int(passos_treino * 2 // 3), lote=65536, lr=2e-3, semente=semente)
    p, hist2 = treinar(F, T, p, passos=int(passos_treino // 3), lote=65536, lr=5e-4, semente=semente + 1,
                       iniciar=False)
    out["training"] = {"samples": int(T.size), "Re": list(treino), "steps": int(passos_treino), "batch": 65536,
                       "seconds": time.time() - t0, "loss_first": float(hist[:10].mean()),
                       "loss_last": float(hist2[-50:].mean()), "nu_scale": p["nu_scale"], "nu_max": p["nu_max"],
                       "target_clip": t_clip, "form": forma}
    # a-priori on the held-out Reynolds number
    if re_teste in dados:
        Fv, Tv = dados[re_teste]
        tau0c = 3.0 * u * comprimento / re_teste + 0.5
        s_mag = 1.5 * np.exp(Fv[:, 0].astype(np.float64)) / (tau0c + 3.0 * Tv)   # |S| from x0
        out_net = avaliar(p, Fv)
        nu_net = out_net * s_mag if forma == "coef" else out_net
        Tv = np.minimum(Tv, np.float32(t_clip * (np.max(s_mag) if forma == "coef" else 1.0)))
        nu_smag = cs * cs * s_mag
        ok = np.isfinite(nu_net)

        def metr(a, b):
            return {"rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                    "corr": float(np.corrcoef(a, b)[0, 1]), "mean_ratio": float(a.mean() / b.mean())}
        out["a_priori"] = {"Re": re_teste, "rows": int(Tv.size), "closure": metr(nu_net[ok], Tv[ok]),
                           "smagorinsky": metr(nu_smag, Tv), "fallback_rows": int((~ok).sum())}
    passos_grossos = passos_finos // 2
    bloco_g = intervalo // 4

    def escalado(c):
        q = dict(p)
        q["nu_scale"] = p["nu_scale"] * c
        return q
    # a-posteriori calibration on the training Reynolds numbers
    melhor, melhor_err = 1.0, float("inf")
    for c in escalas:
        errs = []
        for re in treino:
            rec, _ = rodar(gc, tc, ec, ac, re, passos_grossos, bloco_g, closure=escalado(c), cada_k=cada)
            fine_cd = out["fine_runs"][str(re)]["cd"]
            errs.append(abs(rec["cd"] - fine_cd) / abs(fine_cd))
        e = float(np.mean(errs)) if np.all(np.isfinite(errs)) else float("inf")
        out["calibration"][str(c)] = {"cd_abs_err_per_Re": errs, "mean": e}
        if e < melhor_err:
            melhor, melhor_err = c, e
    smag_train = []
    for re in treino:
        rec, _ = rodar(gc, tc, ec, ac, re, passos_grossos, bloco_g)
        smag_train.append(abs(rec["cd"] - out["fine_runs"][str(re)]["cd"]) / abs(out["fine_runs"][str(re)]["cd"]))
    out["calibration"]["chosen"] = melhor
    out["calibration"]["smagorinsky_cd_abs_err_per_Re"] = smag_train
    pf = escalado(melhor)
    if pesos_saida:
        salvar(pf, pesos_saida)
    for nome, clo, k, c_s in (("smagorinsky", None, 1, cs), ("closure_every_step", pf, 1, cs),
                              (f"closure_every_{cada}", pf, cada, cs), ("no_model", None, 1, 0.0)):
        rec, _ = rodar(gc, tc, ec, ac, re_teste, passos_grossos, bloco_g, closure=clo, cada_k=k, cs_run=c_s,
                       cronometrar=True)
        out["coarse_runs"][nome] = rec
    fine_cd = out["fine_runs"][str(re_teste)]["cd"]
    for nome, rec in out["coarse_runs"].items():
        rec["cd_err_vs_fine"] = (rec["cd"] - fine_cd) / fine_cd
    sm = out["coarse_runs"]["smagorinsky"]
    out["closure_overhead"] = {nome: rec["ms_per_step"] / sm["ms_per_step"] - 1.0
                               for nome, rec in out["coarse_runs"].items()
                               if nome.startswith("closure") and "ms_per_step" in rec}
    return out


def estavel(s, u_ref, fator=6.0, passo_amostra=11):
    """The stability check of tests/estabilidade.html:49-72: recompute the
    macros, read them back and sample every 11th cell; the run has diverged
    if a sampled |u| is not finite or exceeds 6 times the free stream.
    Returns (stable, max sampled |u|)."""
    s.atualizarMacros()
    m = s.lerMacros().reshape(-1, 4)[::passo_amostra, :3].astype(np.float64)
    u = np.sqrt((m * m).sum(1))
    if not np.isfinite(u).all():
        return False, float("nan")
    mu = float(u.max())
    return mu <= fator * u_ref, mu


def rodar_caso(grade, tipo, cfg, area, passos, u, janela, storage="f32", bloco=1000, checar=True):
    """Run `passos` steps with the fused force of every step; Cd / Cl per step
    (Maskell, theta 2.5, src/core/forces.js:55-95); the stability check every
    `bloco` steps.  Returns the per-step coefficients and the window means."""
    from .forces import coeficientes
    from .solver import SolverCUDA
    from .units import LatticeUnits
    s = SolverCUDA(grade, storage=storage, escrever_macros=False)
    s.definirTipos(tipo)
    s.configurar(**cfg)
    s.calibrarRepouso()
    s.inicializar()
    units = LatticeUnits(u)
    cd, cl, feito, maxu, divergiu = [], [], 0, [], None
    t0 = time.time()
    while feito < passos:
        n = min(bloco, passos - feito)
        f = s.passoComForcas(n)
        for k in range(n):
            c = coeficientes(list(f[k]), units, area, grade)
            cd.append(c["cd"])
            cl.append(c["cl"])
        feito += n
        if checar:
            ok, mu = estavel(s, u)
            maxu.append(mu)
            if not ok:
                divergiu = feito
                break
    wall = time.time() - t0
    s.destruir()
    cd, cl = np.asarray(cd), np.asarray(cl)
    a, b = janela
    rec = {"storage": storage, "steps_run": feito, "diverged_at": divergiu, "max_u_per_check": maxu, "wall_s": wall}
    if divergiu is None and len(cd) >= b:
        w = slice(a, b)
        rec.update(cd_mean=float(cd[w].mean()), cd_std=float(cd[w].std(ddof=1)), cl_mean=float(cl[w].mean()),
                   cl_std=float(cl[w].std(ddof=1)), window=[a, b])
    return rec, cd, cl


def casos(storage_judge="f64"):
    """The stated outputs of the plain-method workloads.

    Mesh body, 320x160x128 (no-slip floor, u_in 0.06, Cs 0.12): Re 2000 on
    the body's 96-cell length gives nu = 0.00288 and omega+ = 1.96603 (on its
    48-cell semi-axis, nu = 0.00144 and omega+ = 1.98287); both are above the
    reference's stability ceiling omega_max = 1.90 (src/core/units.js:60-92).
    10 000 steps of each with the stability check of tests/estabilidade.html
    every 1000; Cd / Cl averaged over steps 5000-10000 if it survives; then
    the run at the clamped viscosity (omega+ = 1.90, as Units does,
    src/core/units.js:157-164), with its fp64 run as the accuracy judge.

    Sphere, 128x64x64 (D = 16 at (40, 32, 32), Re 100, Cs 0.1): the Cd series
    over 4000 steps in fp32 and fp64, and the fp32 error against fp64."""
    from .cargas import GRIDS, carga
    from .lattice import nu_from_omega, omega_from_nu
    from .tunel import areaFrontalCorpo, corpoAnalitico, montarTipos
    from .voxel import voxelizar
    out = {"mesh_body": {}, "sphere": {}}
    g2 = GRIDS["320x160x128"]
    tipo, cfg, desc = carga("320x160x128")
    from .geometry import corpo_config2
    pos, idx = corpo_config2(g2)
    corpo = voxelizar(pos, idx, g2, sdf=False)["tipo"]
    area = areaFrontalCorpo(corpo, g2)
    out["mesh_body"]["workload"] = desc
    out["mesh_body"]["frontal_area"] = area
    omega48 = omega_from_nu(0.06 * 48 / 2000)
    for nome, omega in (("re2000", cfg["omegaPlus"]), ("re2000_on_semi_axis_48", omega48),
                        ("clamped_omega_1.90", 1.90)):
        c = dict(cfg, omegaPlus=omega)
        rec, cd, _ = rodar_caso(g2, tipo, c, area, 10000, 0.06, (5000, 10000))
        rec["omega_plus"] = omega
        rec["nu"] = nu_from_omega(omega)
        rec["Re_length_96"] = 0.06 * 96 / rec["nu"]
        rec["cd_series_every_100"] = [float(v) for v in cd[::100]]
        out["mesh_body"][nome] = rec
    judge = dict(cfg, omegaPlus=1.90)
    rj, cdj, _ = rodar_caso(g2, tipo, judge, area, 10000, 0.06, (5000, 10000), storage=storage_judge)
    out["mesh_body"]["clamped_omega_1.90_" + storage_judge] = {k: v for k, v in rj.items() if k != "max_u_per_check"}
    c32 = out["mesh_body"]["clamped_omega_1.90"]
    if "cd_mean" in c32 and "cd_mean" in rj:
        c32["cd_err_vs_" + storage_judge] = (c32["cd_mean"] - rj["cd_mean"]) / rj["cd_mean"]
        c32["cl_abs_err_vs_" + storage_judge] = c32["cl_mean"] - rj["cl_mean"]

    g1 = {"nx": 128, "ny": 64, "nz": 64}
    corpo1 = corpoAnalitico(g1, {"tipo": "esfera", "cx": 40, "cy": 32, "cz": 32, "raio": 8})
    mt = montarTipos(g1, corpo=corpo1, esteira=False)
    t1 = mt["tipo"].reshape(64, 64, 128)
    t1[0, :, 1:127] = 6
    nu = 0.05 * 16 / 100
    cfg1 = dict(omegaPlus=omega_from_nu(nu), lesCs=0.1, inletU=[0.05, 0.0, 0.0], beltU=[0.0, 0.0, 0.0],
                esponja=mt["esponja"])
    area1 = areaFrontalCorpo(corpo1, g1)
    series = {}
    for st in ("f32", storage_judge):
        rec, cd, cl = rodar_caso(g1, mt["tipo"], cfg1, area1, 4000, 0.05, (3000, 4000), storage=st, checar=False)
        series[st] = cd
        out["sphere"][st] = {k: v for k, v in rec.items() if k != "max_u_per_check"}
        out["sphere"][st]["cd_series_every_10"] = [float(v) for v in cd[::10]]
    d = series["f32"] - series[storage_judge]
    out["sphere"]["frontal_area"] = area1
    out["sphere"]["cd_final_err_vs_" + storage_judge] = float(d[-1] / series[storage_judge][-1])
    out["sphere"]["cd_series_max_abs_err_vs_" + storage_judge] = float(np.abs(d).max())
    out["sphere"]["cd_series_max_rel_err_after_500_vs_" + storage_judge] = float(
        np.abs(d[500:] / series[storage_judge][500:]).max())
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["precisao", "lote", "fecho", "casos"])
    ap.add_argument("--pesos", default=None, help="fecho: write the trained weights (.npz) here")
    ap.add_argument("--cada", type=int, default=8, help="fecho: the held form's evaluation period (calibration)")
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--grid", default="512,256,192")
    ap.add_argument("--out", default=None, help="also write the result (JSON) to this file")
    a = ap.parse_args(argv)
    nx, ny, nz = (int(v) for v in a.grid.split(","))
    t0 = time.time()
    if a.study == "lote":
        r = lote(steps=a.steps)
    elif a.study == "fecho":
        r = fecho(passos_finos=a.steps, pesos_saida=a.pesos, cada=a.cada)
    elif a.study == "casos":
        r = casos()
    else:
        r = precisao(a.steps, {"nx": nx, "ny": ny, "nz": nz})
    r["wall_s"] = time.time() - t0
    r["command"] = "python -m cfd__gb300.estudos " + " ".join(argv if argv is not None else sys.argv[1:])
    print(json.dumps(r))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(r, f, indent=1)
            f.write("\n")


if __name__ == "__main__":
    main()
