"""Run a few steps of a benchmark workload on cuda:0 — the program the
committed ncu summaries under profiles/ capture.

    python -m cfd__gb300.perfil [--grid 512x256x192|320x160x128]
                                [--storage f32|f16s|bf16s|f64] [--steps K] [--warmup W]
                                [--closure K] [--engine 0|1] [--block BX] [--variant MINB]
                                [--forces] [--soa | --aos]

W warm-up steps, then K steps, then a synchronize; prints the wall time.
The step kernel runs once per step (k_step_inplace, or k_step_closure with
--closure), so `ncu -k regex:k_step -s W -c C` captures steps W .. W+C-1.
"""
from __future__ import annotations

import argparse
import os
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", default="512x256x192",
                    help="a bench workload (512x256x192, 320x160x128) or any NXxNYxNZ: a free-stream tunnel")
    ap.add_argument("--storage", default="f32", choices=["f32", "f16s", "bf16s", "f64", "f16sr", "bf16sr"])
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--closure", type=int, default=0, help="learned closure evaluated every K steps (0: off)")
    ap.add_argument("--engine", type=int, default=0)
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--variant", type=int, default=0, help="lbm_set_launch min_blocks code")
    ap.add_argument("--forces", action="store_true", help="steps with the fused force (passoComForcas)")
    ap.add_argument("--soa", action="store_true", help="keep the in-place set in the SoA layout")
    ap.add_argument("--aos", action="store_true", help="keep the in-place set in the AoSoA layout")
    ap.add_argument("--lote", type=int, default=0,
                    help="instead: the batched workload of this many seeded tunnels (--mode 0/1)")
    ap.add_argument("--mode", type=int, default=1)
    a = ap.parse_args(argv)
    if a.lote:
        return lote(a)
    from . import build as B
    B.build()
    from .cargas import GRIDS, carga
    from .solver import SolverCUDA
    if a.grid in GRIDS:
        grade = GRIDS[a.grid]
        tipo, cfg, desc = carga(a.grid)
    else:
        from .tunel import montarTipos
        nx, ny, nz = (int(v) for v in a.grid.split("x"))
        grade = {"nx": nx, "ny": ny, "nz": nz}
        mt = montarTipos(grade, esteira=False)
        tipo = mt["tipo"]
        cfg = dict(omegaPlus=1.85, lesCs=0.1, inletU=[0.05, 0.0, 0.0], beltU=[0.0, 0.0, 0.0], esponja=mt["esponja"])
        desc = f"{a.grid} free-stream tunnel, u_in 0.05, omega+ 1.85, Cs 0.1"
    s = SolverCUDA(grade, storage=a.storage, escrever_macros=False, soa=True if a.soa else (False if a.aos else None))
    s.definirTipos(tipo)
    s.configurar(**cfg, closure=a.closure)
    if a.closure:
        from .fecho import carregar
        s.definirFecho(carregar(os.path.join(os.path.dirname(os.path.abspath(__file__)), "pesos", "fecho_coef.npz")))
        s.motorFecho(a.engine)
    if a.block or a.variant:
        s.definirBloco(a.block or 64, a.variant)
    s.inicializar()
    run = s.passoComForcas if a.forces else s.passo
    run(a.warmup)
    s.sincronizar()
    t0 = time.perf_counter()
    run(a.steps)
    s.sincronizar()
    dt = time.perf_counter() - t0
    N = int(tipo.size)
    print(f"{desc}: {a.storage}, layout {s.info()['layout']}, {a.steps} steps in {dt * 1e3:.2f} ms ({N * a.steps / dt / 1e6:.0f} MLUPS wall)")
    s.destruir()


def lote(a):
    from . import build as B
    B.build()
    from .lote import LoteCUDA, sorteio_lote
    tun = sorteio_lote(a.lote, 2026)
    L = LoteCUDA([t[0] for t in tun], storage=a.storage)
    L.definirModo(a.mode)
    for k, (g, tipo, cfg, info) in enumerate(tun):
        L.definirTipos(k, tipo)
        L.configurar(k, **cfg)
    L.inicializar()
    L.passo(a.warmup)
    t0 = time.perf_counter()
    L.passo(a.steps)
    L.medirForcas()
    dt = time.perf_counter() - t0
    print(f"{a.lote} tunnels, {L.celulas} cells, mode {a.mode}: {a.steps} steps in {dt * 1e3:.2f} ms "
          f"({L.celulas * a.steps / dt / 1e6:.0f} MLUPS wall)")
    L.destruir()


if __name__ == "__main__":
    main()
