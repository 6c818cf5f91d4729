"""The benchmark workloads (cell types and solver parameters), shared by
bench.py and the profiling driver (python -m cfd__gb300.perfil).

* 512x256x192 — the precision workload: 25.2 M cells, the seeded
  superellipsoid mesh (semi-axes 80x32x22 cells, 20k triangles, 0.3-cell
  jitter) centred in y and z, free-slip walls on every side, u_in 0.05,
  nu 0.008 (omega+ 1.9084), Smagorinsky Cs 0.1.
* 320x160x128 — the mesh-body workload: 6.55 M cells, the superellipsoid
  48x20x14 cells two cells above a no-slip floor (PAREDE), u_in 0.06, Re 2000
  on the 96-cell length (nu 0.00288, omega+ 1.98295), Cs 0.12.

The reference measures on vehicle meshes missing from its checkout; these
seeded bodies stand in for them.
"""
from __future__ import annotations

GRIDS = {
    "512x256x192": {"nx": 512, "ny": 256, "nz": 192},
    "320x160x128": {"nx": 320, "ny": 160, "nz": 128},
}
U_IN, RE, LEN, CS = 0.06, 2000.0, 96.0, 0.12


def carga(grid="512x256x192", voxelizador=None):
    """(cell types uint32[N], configurar() keywords, description).
    voxelizador(pos, idx, grade) -> VOXEL codes; default: the GPU voxelizer."""
    from .tunel import montarTipos
    grade = GRIDS[grid]
    if voxelizador is None:
        from .voxel import voxelizar

        def voxelizador(pos, idx, g):
            return voxelizar(pos, idx, g, sdf=False)["tipo"]
    if grid == "512x256x192":
        from .estudos import caso_precisao
        tipo, cfg, _ = caso_precisao(grade, voxelizador)
        cfg = dict(cfg, beltU=[0.0, 0.0, 0.0])
        return tipo, cfg, ("512x256x192 tunnel, voxelized superellipsoid mesh 80x32x22 cells, 20k triangles, "
                           "0.3-cell jitter, free-slip walls, u_in 0.05, nu 0.008, Cs 0.1")
    from .geometry import corpo_config2
    nu = U_IN * LEN / RE
    pos, idx = corpo_config2(grade)
    corpo = voxelizador(pos, idx, grade)
    mt = montarTipos(grade, corpo=corpo, esteira=False)
    cfg = dict(omegaPlus=1.0 / (3.0 * nu + 0.5), lesCs=CS, inletU=[U_IN, 0.0, 0.0], beltU=[0.0, 0.0, 0.0],
               esponja=mt["esponja"])
    return mt["tipo"], cfg, ("320x160x128 tunnel, voxelized superellipsoid mesh 48x20x14 cells, 20k triangles, "
                             "0.3-cell jitter, no-slip floor, u_in 0.06, Re 2000, Cs 0.12")
