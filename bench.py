"""Throughput of the D3Q19 wind-tunnel step on GB300 (MLUPS, % of HBM roofline).

Default workload (--grid 512x256x192): the precision workload, 25.2 M cells,
a seeded superellipsoid mesh (semi-axes 80x32x22 cells, 20k triangles,
0.3-cell jitter) voxelized on the GPU, free-slip walls, equilibrium inlet,
outlet + sponge, u_in 0.05, nu 0.008 (omega+ 1.9084), Smagorinsky Cs 0.1.
`value` is the fp32 step; the fp16 (g * 2^10) and bf16 storage forms are
timed beside it, with the Cd and velocity errors against the fp64 run that
the precision study recorded (results/precisao_512x256x192.json).
--grid 320x160x128 selects the mesh-body tunnel (no-slip floor, u_in 0.06,
Re 2000, Cs 0.12), where the learned closure and the visualisation compute
are also timed.  One "step" = one D3Q19 step over every cell (MLUPS counts
all nx*ny*nz cells, as the reference's tests/desempenho.html:67-70).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--grid 512x256x192|320x160x128] [--storage f32|f16s|bf16s|f16sr|bf16sr|f64]

Timing: W + 2W untimed warm-up steps, then K steps between CUDA events on
the solver's stream, repeated R >= 5 times so the repeats span at least a
second; the median is reported.

--impl reference times the reference's step on the host cores instead: the
reference has no runnable CPU step of its own (its step exists only as
generated WGSL/GLSL), so that arm runs the CPU restatement in oracle/ with all
host threads on the same workload.

Multi-GPU: the tunnel does not shard here (replicas only): every rank runs its
own copy and `value` sums the ranks' cells (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# The metric string both arms print (so the two lines' values can be divided).
METRIC = "MLUPS & % HBM roofline on 1 GB300, FP16-store vs FP32 plain, Cd err \u22641% vs FP64"
from cfd__gb300.cargas import GRIDS  # noqa: E402

GRID = GRIDS["320x160x128"]
BYTES_PER_CELL = {"f32": 152, "f16s": 76, "bf16s": 76, "f64": 304, "f16sr": 76, "bf16sr": 76}


def oracle_voxelizer(pos, idx, grade):
    from oracle import oracle as O
    return O.voxelize(pos, idx, (grade["nx"], grade["ny"], grade["nz"]), with_sdf=False)[0]


def workload(grid="512x256x192", cpu_voxelizer=False):
    """(cell types, solver parameters, description) of a bench workload
    (cfd__gb300/cargas.py).  The reference arm voxelizes with the CPU
    restatement, ours on the GPU (the two give identical masks)."""
    from cfd__gb300.cargas import carga
    return carga(grid, oracle_voxelizer if cpu_voxelizer else None)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, copy burst)"
    return 6800.0, "fallback 6.8 TB/s"


def ncu_traffic(storage="f32", grid="512x256x192"):
    """Per-launch DRAM bytes (read + write) of the step kernel, from the
    committed ncu summary of the same storage form and grid."""
    p = os.path.join(ROOT, "profiles", f"lbm_step_{storage}_{grid}.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def precision_study(grid):
    """The recorded result of the precision study (Cd and velocity error of
    each storage form against the fp64 run), if one is committed."""
    p = os.path.join(ROOT, "results", f"precisao_{grid}.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    out = {"recorded": True, "source": d.get("command"), "steps": d.get("steps"), "forms": {}}
    for k, v in d.get("forms", {}).items():
        out["forms"][k] = {kk: v[kk] for kk in ("cd", "cd_err_vs_f64", "u_l2_rel_err_vs_f64") if kk in v}
        if "stored_values" in v:
            out["forms"][k]["subnormal_share_of_stored_values"] = v["stored_values"]["subnormal_share"]
    return out


class Clocks:
    """nvidia-smi sampling; summary() keeps the samples taken inside the
    window marked by start()/stop()."""

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        self.t0 = time.perf_counter()

    def stop(self):
        self.t1 = time.perf_counter()

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            if self.t0 is not None and not (self.t0 <= t <= (self.t1 or t) + 0.05):
                continue
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def voxelizer_timing(repeats=3):
    """GPU voxelization of the 20k-triangle body onto 320x160x128 (ms)."""
    from cfd__gb300.geometry import corpo_config2
    from cfd__gb300.voxel import voxelizar
    pos, idx = corpo_config2(GRID)
    best = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        r = voxelizar(pos, idx, GRID)
        wall = (time.perf_counter() - t0) * 1e3
        st = r["stats"]
        if best is None or wall < best["wall_ms"]:
            best = {"wall_ms": wall, "gpu_ms": st["msTotal"], "raster_ms": st["msRasterizacao"],
                    "flood_ms": st["msInundacao"], "triangles": int(idx.shape[0]), "pairs": st["pares"],
                    "pairs_fp64": st["paresFp64"], "flood_passes": st["passesInundacao"],
                    "solid_cells": st["nSolido"]}
    return best


def cpu_voxelizer_ms():
    from cfd__gb300.geometry import corpo_config2
    from oracle import oracle as O
    pos, idx = corpo_config2(GRID)
    t0 = time.perf_counter()
    O.voxelize(pos, idx, (GRID["nx"], GRID["ny"], GRID["nz"]))
    return (time.perf_counter() - t0) * 1e3


def cpu_model():
    """CPU model of the host, from /proc/cpuinfo (x86 'model name', Arm 'CPU part')."""
    try:
        txt = open("/proc/cpuinfo").read()
    except OSError:
        return "unknown"
    for key in ("model name", "Model"):
        for line in txt.splitlines():
            if line.lower().startswith(key.lower()) and ":" in line:
                return line.split(":", 1)[1].strip()
    parts = sorted({line.split(":", 1)[1].strip() for line in txt.splitlines() if line.startswith("CPU part")})
    impl = sorted({line.split(":", 1)[1].strip() for line in txt.splitlines() if line.startswith("CPU implementer")})
    return f"Arm CPU implementer {','.join(impl)} part {','.join(parts)}" if parts else "unknown"


def _oracle_lattice(grade, tipo, cfg, threads):
    from oracle import oracle as O
    lat = O.Lattice((grade["nx"], grade["ny"], grade["nz"]), nthreads=threads)
    lat.set_types(tipo)
    lat.configure(omega_plus=cfg["omegaPlus"], les_cs=cfg["lesCs"], inlet_u=cfg["inletU"], belt_u=cfg["beltU"],
                  sponge_start=cfg["esponja"]["inicio"], sponge_len=cfg["esponja"]["comprimento"],
                  bl_thickness=cfg.get("espessuraCL", 0.0))
    lat.init()
    return lat


def cpu_measure(grid, tipo, cfg, target_s=10.0, threads=None):
    """The oracle step on the host cores, bounded to ~target_s seconds."""
    threads = threads or (os.cpu_count() or 1)
    grade = GRIDS[grid]
    lat = _oracle_lattice(grade, tipo, cfg, threads)
    lat.run(1)  # warm-up
    t0 = time.perf_counter()
    lat.run(1)
    one = time.perf_counter() - t0
    n = max(1, min(200, int(target_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    lat.run(n)
    dt = time.perf_counter() - t0
    N = int(tipo.size)
    return {"value": N * n / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{n} full steps of the {grid} tunnel (fp32 oracle restatement, {threads} threads)",
            "seconds": dt}


def run_reference(args):
    """The reference's step on the host cores.  The reference has no CPU step
    of its own (its step exists only as generated WGSL/GLSL for a browser
    GPU), so this arm times the CPU restatement in oracle/ on all host
    threads: W untimed warm-up steps, then up to K timed steps of the same
    workload (fewer when K steps would take over a minute; the line says how
    many)."""
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    tipo, cfg, desc = workload(args.grid, cpu_voxelizer=True)
    grade = GRIDS[args.grid]
    N = int(tipo.size)
    lat = _oracle_lattice(grade, tipo, cfg, threads)
    t0 = time.perf_counter()
    lat.run(args.warmup)
    per = (time.perf_counter() - t0) / max(1, args.warmup)
    k = max(1, min(args.steps, int(60.0 / max(per, 1e-6))))
    t0 = time.perf_counter()
    lat.run(k)
    dt = time.perf_counter() - t0
    v = N * k / dt / 1e6
    sample = f"{k} of the requested {args.steps} steps of the {args.grid} tunnel after {args.warmup} warm-up steps"
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "MLUPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / k * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc, "cells": N, "storage": "f32"},
        "cpu_baseline": {"kind": "port", "cores": threads, "sample": sample, "value": v, "unit": "MLUPS",
                         "cpu_model": cpu_model()},
        "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's step exists only as generated WGSL/GLSL for a browser GPU; this arm times its "
                "CPU restatement (oracle/, fp32, A/B ping-pong) on all host threads",
    }
    print(json.dumps(line))
    return 0


def time_steps(s, stream, K):
    """K steps bracketed by CUDA events on the solver's stream (ms)."""
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    s.passo(K)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def timed(s, stream, K, barrier=None, min_total_ms=1000.0, min_repeats=5):
    """K steps timed R >= min_repeats times, R large enough that the timed
    repeats span at least min_total_ms: (median ms of K steps, R)."""
    first = time_steps(s, stream, K)
    R = max(min_repeats, int(math.ceil(min_total_ms / max(first, 1e-3))))
    R = min(R, 5000)
    times = []
    for _ in range(R):
        if barrier:
            barrier()
        times.append(time_steps(s, stream, K))
    return statistics.median(times), R


def reduce_max(value, world, device="cpu"):
    """Max of a per-rank value over the ranks (the slowest rank's time)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def closure_forms(make, stream, steps, N, ms_plain):
    """Step time of the learned closure (coefficient form, weights trained by
    `python -m cfd__gb300.estudos fecho`) evaluated every step, every 8th and
    every 16th step (warp engine) and every step on the CTA tcgen05 engine,
    against the Smagorinsky step of the same tunnel."""
    from cfd__gb300.fecho import carregar
    p = carregar(os.path.join(ROOT, "cfd__gb300", "pesos", "fecho_coef.npz"))
    out = {}
    for every, motor in ((1, 0), (8, 0), (16, 0), (1, 1)):
        s = make("f32", closure=every, pesos=p)
        s.motorFecho(motor)
        s.passo(16)
        ms, R = timed(s, stream, steps, min_total_ms=500.0)
        fb, fl = s.estatisticasFecho()
        name = f"closure_every_{every}" + ("_tcgen05" if motor else "")
        out[name] = {"MLUPS": N * steps / (ms / 1e3) / 1e6, "overhead_vs_smagorinsky": (ms / steps) / ms_plain - 1.0,
                     "fallback_rate": fb / max(fl, 1), "repeats": R,
                     "engine": "CTA tcgen05.mma, TMEM accumulators" if motor else "warp mma.sync"}
        s.destruir()
    return out


def vis_timing(make, stream, N, peak):
    """Visualisation compute on the 320x160x128 tunnel (include/lbm_vis.h): one
    smoke step (back-trace + MacCormack, fp16 volume; algorithmic bytes per
    voxel: 2 x 16 B macros + 2 x 1 B types + 2 B current x 3 reads + 2 B
    intermediate write + read + 2 B next write = 44 B), a 640x360 ray-march
    of the volume, and one frame of 65 536 streak particles in 8 sub-steps."""
    import torch

    from cfd__gb300.visual import Esteiras, Fumaca, camera_orbita, posicionar_rake
    s = make("f32")
    s.passo(20)
    s.atualizarMacros()
    f = Fumaca(s)
    ext = {"min": [0.28 * GRID["nx"], GRID["ny"] * 0.5 - 20, 3], "tamanho": [96, 40, 28],
           "centro": [0.28 * GRID["nx"] + 48, GRID["ny"] * 0.5, 17]}
    rake = posicionar_rake(GRID["ny"], GRID["nz"], ext)
    for _ in range(5):
        f.passo(rake, dt=44.0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(20):
        f.passo(rake, dt=44.0)
    e1.record(stream)
    e1.synchronize()
    ms_smoke = e0.elapsed_time(e1) / 20
    inv, eye = camera_orbita(GRID["nx"], GRID["ny"], GRID["nz"])
    f.render(inv, eye, largura=640, altura=360)
    t0 = time.perf_counter()
    img = f.render(inv, eye, largura=640, altura=360)
    ms_render = (time.perf_counter() - t0) * 1e3
    rng = np.random.default_rng(0)
    n = 65536
    parts = np.zeros((n, 8), np.float32)
    parts[:, 0] = rng.uniform(2, 5, n)
    parts[:, 1] = rng.uniform(2, GRID["ny"] - 2, n)
    parts[:, 2] = rng.uniform(1, GRID["nz"] - 2, n)
    parts[:, 3] = rng.uniform(200, 400, n)
    e = Esteiras(s, n)
    e.definir(parts)
    e.passo(24.0, 8, 0)
    torch.cuda.synchronize()
    e0.record(stream)
    for q in range(20):
        e.passo(24.0, 8, q)
    e1.record(stream)
    e1.synchronize()
    ms_parts = e0.elapsed_time(e1) / 20
    out = {"smoke_step_ms": ms_smoke, "smoke_Mvoxels_per_s": N / ms_smoke / 1e3,
           "smoke_roofline_frac": 44 * N / (ms_smoke / 1e3) / 1e9 / peak,
           "render_640x360_ms_e2e": ms_render, "render_mean_alpha": float(img[..., 3].mean()),
           "particles_65536x8_ms": ms_parts}
    e.destruir()
    f.destruir()
    s.destruir()
    return out


def run_ours(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from cfd__gb300 import SolverCUDA
    from cfd__gb300 import build as B

    B.build()
    grade = GRIDS[args.grid]
    tipo, cfg, desc = workload(args.grid)
    N = int(tipo.size)
    stream = torch.cuda.Stream()
    vox = voxelizer_timing() if not args.no_forms else None

    def maker(tp, cf, gr):
        def make(storage, closure=0, pesos=None, soa=None):
            s = SolverCUDA(gr, storage=storage, escrever_macros=False, soa=soa)
            s.definirStream(stream.cuda_stream)
            s.definirTipos(tp)
            s.configurar(**cf, closure=closure)
            if pesos is not None:
                s.definirFecho(pesos)
            s.inicializar()
            return s
        return make

    make = maker(tipo, cfg, grade)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    peak, peak_src = peaks()
    s = make(args.storage)
    s.passo(args.warmup)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        s.passo(2 * args.warmup)        # keeps the GPU busy while the sampler starts
        time.sleep(0.3)
        barrier()
        clk.start()
        t0 = time.perf_counter()
        ms, R = timed(s, stream, args.steps, barrier=barrier)
        wall = time.perf_counter() - t0
        clk.stop()
    barrier()
    ms = reduce_max(ms, world, device="cuda")
    ms_step = ms / args.steps
    mlups = N * args.steps / (ms / 1e3) / 1e6 * world

    # roofline of the step kernel (one launch per step)
    bpc = BYTES_PER_CELL[args.storage]
    achieved = bpc * N / (ms_step / 1e3) / 1e9
    traffic = ncu_traffic(args.storage, args.grid)

    # end to end through the public API: every step configures (parameters by
    # value in the launch) and its force (24 B) comes back to the host.  The
    # reference's medirForcas is asynchronous; the pipelined form reads step
    # k's force while step k+1 runs (page-locked double buffer), the
    # synchronous form waits for every step.
    E = max(200, min(2000, int(2000.0 / max(ms_step, 1e-3))))
    import torch as _t
    bufs = [_t.empty(3, dtype=_t.float64, pin_memory=True).numpy() for _ in range(2)]
    s.passoComForcas(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prev = None
    for k in range(E):
        s.configurar(**cfg)
        tk = s.passoComForcasAssincrono(1, bufs[k % 2])
        if prev is not None:
            s.aguardarForcas(prev)
        prev = tk
    s.aguardarForcas(prev)
    e2e_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(E):
        s.configurar(**cfg)
        s.passoComForcas(1)
    e2e_sync_s = time.perf_counter() - t0
    e2e = {"value": N * E / e2e_s / 1e6 * world, "unit": "MLUPS", "h2d_bytes_per_step": 52,
           "d2h_bytes_per_step": 24, "steps": E,
           "path": "per step SolverCUDA.configurar + passoComForcasAssincrono(1), the previous step's force "
                   "awaited (C ABI lbm_configure, lbm_step_forces_async, lbm_forces_done)",
           "synchronous_value": N * E / e2e_sync_s / 1e6 * world,
           "synchronous_path": "per step SolverCUDA.configurar + passoComForcas(1) (lbm_step_forces, waits)"}
    s.destruir()

    forms = {}
    if not args.no_forms:
        # the fused-force variant of the step on the device (what e2e runs),
        # without the host: K steps of passoComForcas between CUDA events
        s2 = make(args.storage)
        s2.passoComForcas(args.warmup)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s2.passoComForcas(args.steps)
        e1.record(stream)
        e1.synchronize()
        msf = e0.elapsed_time(e1)
        forms["fused_force_step_device"] = {"MLUPS": N * args.steps / (msf / 1e3) / 1e6,
                                            "note": "passoComForcas(K): step with the fused force, its per-step "
                                                    "slot clear and one read-back of the K forces"}
        s2.destruir()
        for st in ("f16s", "bf16s", "f16sr", "bf16sr"):
            s2 = make(st)
            s2.passo(args.warmup)
            ms2, R2 = timed(s2, stream, args.steps)
            m2 = N * args.steps / (ms2 / 1e3) / 1e6
            a2 = BYTES_PER_CELL[st] * N / (ms2 / args.steps / 1e3) / 1e9
            forms[st] = {"MLUPS": m2, "vs_f32": m2 / (mlups / world), "repeats": R2,
                         "roofline": {"bound": "hbm", "achieved": a2, "peak": peak, "unit": "GB/s", "frac": a2 / peak,
                                      "traffic": ncu_traffic(st, args.grid), "algorithmic_bytes_per_cell": 76}}
            s2.destruir()
        forms["precision_study"] = precision_study(args.grid)
        # the metric's comparison in one place: each 16-bit store form's speed
        # against the fp32 step (this run) and its recorded Cd error vs fp64
        ps = (forms["precision_study"] or {}).get("forms", {})
        cmp16 = {}
        for st in ("f16s", "bf16s", "f16sr", "bf16sr"):
            e = ps.get(st, {}).get("cd_err_vs_f64")
            cmp16[st] = {"MLUPS": forms[st]["MLUPS"], "vs_f32": forms[st]["vs_f32"], "cd_err_vs_f64": e,
                         "meets_1pct_cd": None if e is None else abs(e) <= 0.01}
        forms["fp16_store_vs_fp32"] = cmp16
        # the step kernel's addressing variants side by side (lbm_set_launch
        # codes): in the AoSoA layout (the default; blocks of 64 cells for
        # the 16-bit forms) and, for the 16-bit forms, in SoA
        variants = {}
        for st in ("f32", "f16s", "bf16s"):
            row = {}
            codes = [("aosoa_recompute_addresses", 8, False), ("aosoa_keep_addresses", 9, False)]
            if st != "f32":
                codes += [("soa_slot_pointers", 8, True), ("soa_slot_offsets_32bit", 20, True),
                          ("soa_base_plus_slot_times_n", 21, True), ("soa_80_registers", 6, True)]
            for name, code, soa in codes:
                s2 = make(st, soa=soa)
                s2.definirBloco(64, code)
                s2.passo(args.warmup)
                ms2, _ = timed(s2, stream, args.steps, min_total_ms=300.0)
                row[name] = {"MLUPS": N * args.steps / (ms2 / 1e3) / 1e6,
                             "roofline_frac": BYTES_PER_CELL[st] * N / (ms2 / args.steps / 1e3) / 1e9 / peak}
                s2.destruir()
            variants[st] = row
        forms["step_variants"] = variants
        # the in-place set's two layouts side by side (AoSoA is the default:
        # blocks of 32 cells for fp32, 64 for the 16-bit forms, rows padded
        # to a multiple of the block; the layout code says which)
        lay = {}
        for st in ("f32", "f16s", "bf16s", "f16sr"):
            row = {}
            for name, soa in (("aosoa", False), ("soa", True)):
                s2 = SolverCUDA(grade, storage=st, escrever_macros=False, soa=soa)
                s2.definirStream(stream.cuda_stream)
                s2.definirTipos(tipo)
                s2.configurar(**cfg)
                s2.inicializar()
                s2.passo(args.warmup)
                ms2, _ = timed(s2, stream, args.steps, min_total_ms=300.0)
                row[name] = {"MLUPS": N * args.steps / (ms2 / 1e3) / 1e6, "layout": s2.info()["layout"],
                             "roofline_frac": BYTES_PER_CELL[st] * N / (ms2 / args.steps / 1e3) / 1e9 / peak}
                s2.destruir()
            lay[st] = row
        forms["layouts"] = lay
        # the mesh-body tunnel: its plain step, the learned closure (trained
        # on that tunnel's body) and the visualisation compute
        g2 = GRIDS["320x160x128"]
        tipo2, cfg2, desc2 = workload("320x160x128")
        N2 = int(tipo2.size)
        make2 = maker(tipo2, cfg2, g2)
        s2 = make2("f32")
        s2.passo(args.warmup)
        ms2, R2 = timed(s2, stream, args.steps)
        s2.destruir()
        forms["f32_320x160x128"] = {"MLUPS": N2 * args.steps / (ms2 / 1e3) / 1e6, "workload": desc2, "repeats": R2,
                                    "roofline_frac": 152 * N2 / (ms2 / args.steps / 1e3) / 1e9 / peak}
        forms.update(closure_forms(make2, stream, args.steps, N2, ms2 / args.steps))
        forms["visual"] = vis_timing(make2, stream, N2, peak)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_measure(args.grid, tipo, cfg, target_s=args.cpu_seconds)
        cpu.pop("seconds", None)
        one = cpu_measure(args.grid, tipo, cfg, target_s=max(2.0, args.cpu_seconds / 4), threads=1)
        cpu["single_thread_MLUPS"] = one["value"]
        cpu["cpu_model"] = cpu_model()
        if vox is not None:
            cpu["voxelizer_320x160x128_ms_1_thread"] = cpu_voxelizer_ms()
    if rank == 0:
        line = {
            "metric": METRIC,
            "value": mlups, "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "repeats": R, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"f32": "f32", "f16s": "f16 storage / f32 math", "bf16s": "bf16 storage / f32 math",
                      "f16sr": "f16 storage, stochastic rounding / f32 math",
                      "bf16sr": "bf16 storage, stochastic rounding / f32 math", "f64": "f64"}[args.storage],
            "data": "synthetic",
            "config": {"workload": desc, "cells": N, "storage": args.storage, "layout": "in-place (esoteric pull)",
                       "parallelism": "replicas" if world > 1 else "single",
                       "timing": f"median of {R} timed repeats of {args.steps} steps (CUDA events on the solver's "
                                 f"stream), {args.warmup} + {2 * args.warmup} warm-up steps",
                       "l2": f"state {N * 19 * (bpc // 38) / 1e6:.0f} MB > 126 MB L2 (inputs larger than L2)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                         "kernel": "k_step_inplace", "algorithmic_bytes_per_cell": bpc},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": args.steps * R,
            "gpu_launches_note": f"{args.steps} step kernels per timed repeat, {R} repeats",
            "clocks": clk.summary(),
            "forms": forms,
            "voxelizer": vox,
            "wall_s_timed": wall,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=40)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--storage", default="f32", choices=["f32", "f16s", "bf16s", "f64", "f16sr", "bf16sr"])
    ap.add_argument("--grid", default="512x256x192", choices=sorted(GRIDS))
    ap.add_argument("--no-forms", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
