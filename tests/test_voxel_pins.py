"""Hand-derived voxel masks, asserted on the CPU voxelizer restatement itself
(no GPU, no comparison with the CUDA voxelizer).

The expected masks follow from the comparisons of the reference's voxelizer
(src/geom/voxel.js):

* a triangle in the plane x = X touches the voxel box [x, x + 1] iff
  |X - (x + 1/2)| <= 1/2 (the box-axis test `min > h || max < -h`, :85-88,
  is inclusive), so a face on a voxel face (X integer) marks both voxels
  x = X - 1 and x = X, a face strictly inside a voxel marks only that voxel;
* the same inclusive test on the other two axes gives the face's extent:
  voxels x with X0 - 1 <= x <= X1 for a face spanning [X0, X1];
* the distance prefilter d2 <= 0.75 (:212) admits every voxel whose box
  touches the triangle (0.75 is the squared half-diagonal), including a
  corner-only contact, where d2 = 0.75 exactly;
* the flood fills from the six domain faces through 6-neighbours
  (:278-327); with sealing, the shell dilated by one cell is the barrier and
  one non-cascading growth gives the skin back (:333-355); classification:
  shell -> CASCA (1), not reached -> DENTRO (2), else FLUIDO (0) (:401-407).

All coordinates below are dyadic or exact float32 values, so every
comparison of the restatement (fp64 with JavaScript semantics) is exact and
the masks are determined.
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "cube_example.json")


def _cube(lo, size):
    d = json.load(open(GOLD))
    p = np.array(d["positions"], np.float64) * np.asarray(size, np.float64) + np.asarray(lo, np.float64)
    return p.astype(np.float32), np.array(d["indices"], np.uint32)


def _box_shell(dims, faces_x, faces_y, faces_z, span):
    """Expected mask of a closed axis-aligned box: faces_a = the voxel
    indices each face plane marks along axis a (a set per face pair), span =
    the inclusive voxel range of the box's shell along each axis."""
    nx, ny, nz = dims
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    (x0, x1), (y0, y1), (z0, z1) = span
    inbox = (x >= x0) & (x <= x1) & (y >= y0) & (y <= y1) & (z >= z0) & (z <= z1)
    onface = np.isin(x, list(faces_x)) | np.isin(y, list(faces_y)) | np.isin(z, list(faces_z))
    shell = inbox & onface
    inside = inbox & ~onface
    t = np.zeros((nz, ny, nx), np.uint8)
    t[shell] = 1
    t[inside] = 2
    return t.reshape(-1)


@pytest.mark.parametrize("selar", [True, False])
def test_face_aligned_cube(orc, selar):
    """Cube [10, 26] x [8, 24] x [6, 22], every face on a voxel face: each
    face marks the two voxel layers either side of it; the shell spans
    [lo - 1, lo + size] on every axis and the interior [lo + 1, lo + size - 2]
    is DENTRO."""
    dims = (40, 32, 28)
    lo, size = np.array([10, 8, 6]), 16
    pos, idx = _cube(lo, size)
    t, sdf, st = orc.voxelize(pos, idx, dims, selar=selar)
    exp = _box_shell(dims, {9, 10, 25, 26}, {7, 8, 23, 24}, {5, 6, 21, 22}, ((9, 26), (7, 24), (5, 22)))
    assert np.array_equal(t, exp)
    assert st["n_casca"] == 18 ** 3 - 14 ** 3 and st["n_dentro"] == 14 ** 3
    assert not st["oco_suspeito"]
    # signed distance: non-positive in shell and interior voxels, positive in
    # fluid voxels, band + 1 = 2.5 where no triangle's band reaches
    assert (sdf[t != 0] <= 0).all() and (sdf[t == 0] > 0).all()
    assert sdf.reshape(28, 32, 40)[0, 0, 0] == np.float32(2.5)


def test_reference_cube_at_the_geometry_page_scale(orc):
    """examples/cube_example.stl (the unit cube) placed as the geometry page
    places it on the 'baixa' preset (tests/geometria.html:89-124): 240x120x96,
    body length nx / 10 = 24 cells (src/backend/caps.js:78), nose at 0.28 nx,
    centred in y, resting one cell above z = 0 (src/geom/prepare.js defaults).
    The faces sit at x = 67.2 and 91.2 (inside voxels 67 and 91), y = 48 and
    72, z = 1 and 25 (on voxel faces)."""
    from cfd__gb300.prepara import colocar
    d = json.load(open(GOLD))
    grade = {"nx": 240, "ny": 120, "nz": 96}
    r = colocar(np.array(d["positions"], np.float32), (0, 1, 2), grade, 24)
    pos = r["positions"].reshape(-1, 3)
    assert sorted(set(pos[:, 1].tolist())) == [48.0, 72.0] and sorted(set(pos[:, 2].tolist())) == [1.0, 25.0]
    assert sorted(set(pos[:, 0].tolist())) == [float(np.float32(67.2)), float(np.float32(91.2))]
    t, _, st = orc.voxelize(pos, np.array(d["indices"], np.uint32), (240, 120, 96))
    exp = _box_shell((240, 120, 96), {67, 91}, {47, 48, 71, 72}, {0, 1, 24, 25}, ((67, 91), (47, 72), (0, 25)))
    assert np.array_equal(t, exp)
    assert st["n_dentro"] == 23 * 22 * 22 and st["n_casca"] == 25 * 26 * 26 - 23 * 22 * 22
    # the page's own sanity bounds (tests/geometria.html:160-163)
    from cfd__gb300.voxel import areaFrontal
    af = areaFrontal(t, grade)
    assert st["n_solido"] > 200 and st["n_solido"] / st["n_cells"] < 0.35 and af > 50
    assert af == 26 * 26   # voxel.js areaFrontal: the whole YZ shadow, y 47..72 and z 0..25


def _plate(z, x0, x1, y0, y1):
    p = np.array([[x0, y0, z], [x1, y0, z], [x1, y1, z], [x0, y1, z]], np.float32)
    return p, np.array([[0, 1, 2], [0, 2, 3]], np.uint32)


@pytest.mark.parametrize("z,layers", [(10.25, [10]), (10.5, [10]), (10.0, [9, 10])])
def test_open_plate(orc, z, layers):
    """A zero-thickness horizontal plate [8.25, 30.75] x [4.5, 20.0]: one
    voxel layer when the plane lies inside a voxel, two when it lies on a
    voxel face; x from ceil(8.25 - 1) = 8 to floor(30.75) = 30, y from
    ceil(4.5 - 1) = 4 to 20 (the edge at 20.0 touches voxel 20's face).  The
    flood passes around an open plate: no DENTRO, and with more than 500
    shell cells the mask is flagged as possibly hollow."""
    dims = (40, 28, 24)
    pos, idx = _plate(z, 8.25, 30.75, 4.5, 20.0)
    for selar in (True, False):
        t, _, st = orc.voxelize(pos, idx, dims, selar=selar)
        exp = np.zeros((24, 28, 40), np.uint8)
        for zz in layers:
            exp[zz, 4:21, 8:31] = 1
        assert np.array_equal(t, exp.reshape(-1)), (z, selar)
        assert st["n_dentro"] == 0
        assert st["oco_suspeito"] == (st["n_casca"] > 500)


def test_corner_contact_is_shell(orc):
    """A triangle whose only contact with a voxel is the voxel's corner
    point: the inclusive tests mark it, and d2 = 0.75 passes the prefilter.
    The triangle (12, 12, 12), (15, 12, 12), (12, 15, 12) lies in the voxel
    face plane z = 12 and touches voxel (11, 11, 11) at its corner (12, 12, 12)."""
    pos = np.array([[12, 12, 12], [15, 12, 12], [12, 15, 12]], np.float32)
    t, _, _ = orc.voxelize(pos, np.array([[0, 1, 2]], np.uint32), (24, 24, 24), selar=False)
    t = t.reshape(24, 24, 24)
    assert t[11, 11, 11] == 1                     # z, y, x
    assert t[11, 11, 10] == 0 and t[11, 10, 11] == 0 and t[10, 11, 11] == 0
