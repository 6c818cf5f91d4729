"""Studies of the storage forms and the batched form on one GB300.

    python -m cfd__gb300.estudos precisao [--steps 10000] [--grid 512,256,192]

precisao: the 512x256x192 precision workload (25.2 M cells): the seeded
superellipsoid (semi-axes 80x32x22 cells, 20k triangles, 0.3-cell jitter)
voxelized on the GPU and centred vertically, free-slip walls on every side
(the sphere case's tunnel, tests/validacao.html:224-231), u_in 0.05,
nu 0.008 (omega+ 1.9084), Smagorinsky Cs 0.1.  The same run in four storage
forms: fp32, fp16 of g*2^10, bf16 — all with fp32 arithmetic — and the fp64
judge (fp64 storage and arithmetic).  Reported per form: MLUPS and fraction of
the HBM roofline (bytes per cell 152 / 76 / 76 / 304), the drag coefficient
averaged over the last quarter of the run (Maskell-corrected, theta 2.5) and
its error against the fp64 run, and the relative L2 error of the velocity
field against the fp64 run.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

BYTES = {"f32": 152, "f16s": 76, "bf16s": 76, "f64": 304}


def _peak():
    import os
    p = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def caso_precisao(grade):
    from .geometry import colocar, superelipsoide
    from .tunel import areaFrontalCorpo, montarTipos
    from .voxel import voxelizar
    pos, idx = superelipsoide(80.0, 32.0, 22.0, 2.5, 3.0, 20000, 0.3, 2027)
    pos = colocar(pos, grade, nariz=0.28, folga_piso=0.0)
    dz = 0.5 * grade["nz"] - 0.5 * (pos[:, 2].min() + pos[:, 2].max())
    pos[:, 2] += np.float32(dz)
    vox = voxelizar(pos, idx, grade, sdf=False)
    mt = montarTipos(grade, corpo=vox["tipo"], esteira=False)
    t = mt["tipo"].reshape(grade["nz"], grade["ny"], grade["nx"])
    t[0, :, 1:grade["nx"] - 1] = 6          # free-slip floor as well
    area = areaFrontalCorpo(vox["tipo"], grade)
    nu = 0.008
    cfg = dict(omegaPlus=1.0 / (3.0 * nu + 0.5), lesCs=0.1, inletU=[0.05, 0.0, 0.0], esponja=mt["esponja"])
    return mt["tipo"], cfg, area


def precisao(steps=10000, grade=None, forms=("f64", "f32", "f16s", "bf16s"), sample=50):
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
        s.destruir()
        tail = cds[len(cds) * 3 // 4:]
        cd = float(np.mean(tail))
        mlups = N * steps / (ms_total / 1e3) / 1e6
        rec = {"MLUPS": mlups, "roofline_frac": BYTES[form] * mlups * 1e6 / 1e9 / _peak(),
               "cd": cd, "cd_finite": bool(np.isfinite(cds).all())}
        if ref_u is None:
            ref_u, ref_cd = m, cd
        else:
            rec["cd_err_vs_f64"] = (cd - ref_cd) / ref_cd
            rec["u_l2_rel_err_vs_f64"] = float(np.linalg.norm(m - ref_u) / np.linalg.norm(ref_u))
        out["forms"][form] = rec
    return out


def lote(n_tunnels=64, steps=256, storages=("f32", "f16s"), seed=2026):
    """Batched workload: n tunnels drawn by sorteio_lote (96x48x48 to
    256x128x128).  Aggregate MLUPS = sum N_k * steps / time, for the batch
    (one persistent launch per step, CUDA-graph replay) and for the same
    tunnels run one after another with the single-tunnel solver."""
    import torch

    from .lote import LoteCUDA, sorteio_lote
    from .solver import SolverCUDA
    tun = sorteio_lote(n_tunnels, seed)
    cells = sum(t[0]["nx"] * t[0]["ny"] * t[0]["nz"] for t in tun)
    out = {"tunnels": n_tunnels, "cells": cells, "steps": steps,
           "omega_flagged": int(sum(t[3]["flag_omega"] for t in tun)), "forms": {}}
    stream = torch.cuda.Stream()
    for st in storages:
        ms_modes = {}
        for modo in (0, 1):
            L = LoteCUDA([t[0] for t in tun], storage=st)
            L.definirStream(stream.cuda_stream)
            L.definirModo(modo)
            for k, (g, tipo, cfg, info) in enumerate(tun):
                L.definirTipos(k, tipo)
                L.configurar(k, **cfg)
            L.inicializar()
            L.passo(64)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            L.passo(steps)
            e1.record(stream)
            e1.synchronize()
            ms_modes[modo] = e0.elapsed_time(e1)
            L.destruir()
        ms_batch = ms_modes[0]
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
        out["forms"][st] = {"batched_MLUPS": cells * steps / (ms_batch / 1e3) / 1e6,
                            "persistent_launch_MLUPS": cells * steps / (ms_modes[1] / 1e3) / 1e6,
                            "sequential_MLUPS": cells * steps / (ms_seq / 1e3) / 1e6,
                            "speedup": ms_seq / ms_batch}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["precisao", "lote"])
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--grid", default="512,256,192")
    a = ap.parse_args(argv)
    nx, ny, nz = (int(v) for v in a.grid.split(","))
    t0 = time.time()
    if a.study == "lote":
        r = lote(steps=a.steps)
    else:
        r = precisao(a.steps, {"nx": nx, "ny": ny, "nz": nz})
    r["wall_s"] = time.time() - t0
    print(json.dumps(r))


if __name__ == "__main__":
    main()
