"""The CPU voxelizer restatement against the reference's own sanity checks
(tests/geometria.html:160-163 on examples/cube_example.stl) and geometric
known answers.  CPU only."""
import numpy as np

from tests import vox_cases as V


def test_cube_example_geometry_sanity(orc):
    pos, idx, g = V.cube_example()
    tipo, sdf, st = orc.voxelize(pos, idx, (g["nx"], g["ny"], g["nz"]))
    from cfd__gb300.voxel import areaFrontal
    af = areaFrontal(tipo, g)
    frac = st["n_solido"] / st["n_cells"]
    assert st["n_solido"] > 200 and frac < 0.35 and af > 50     # tests/geometria.html:160-163
    # a 24-cell cube: the shell marks every voxel the surface touches, so the
    # solid spans 24 to 26 cells per axis
    assert 24 ** 3 <= st["n_solido"] <= 26 ** 3
    assert 24 * 24 <= af <= 26 * 26
    assert not st["oco_suspeito"]


def test_sphere_volume_and_sdf_sign(orc):
    g = {"nx": 48, "ny": 48, "nz": 48}
    pos, idx, _ = V.sphere_mesh(g, r=12.0)
    tipo, sdf, st = orc.voxelize(pos, idx, (48, 48, 48))
    # conservative shell: between the r = 12 and r = 13.5 ball volumes
    assert 4 / 3 * np.pi * 12 ** 3 < st["n_solido"] < 4 / 3 * np.pi * 13.5 ** 3
    assert (sdf[tipo == 0] > 0).all() and (sdf[tipo != 0] <= 0).all()


def test_sealing_closes_small_gaps(orc):
    g = {"nx": 48, "ny": 48, "nz": 48}
    pos, idx, _ = V.sphere_mesh(g, r=12.0, n_tri=3000, hole=(12, 1, 10, 2))   # a 1 x 2 quad hole
    t_seal, _, s_seal = orc.voxelize(pos, idx, (48, 48, 48), selar=True)
    t_open, _, s_open = orc.voxelize(pos, idx, (48, 48, 48), selar=False)
    assert s_open["n_dentro"] == 0 and s_open["oco_suspeito"]        # the flood leaks in
    assert s_seal["n_dentro"] > 5000 and not s_seal["oco_suspeito"]  # sealed
