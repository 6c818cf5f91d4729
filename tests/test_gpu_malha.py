"""A mesh file through the whole chain: parsed (cfd__gb300/malha.py), placed
(cfd__gb300/prepara.py) and voxelized on the GPU, bit-identical to the CPU
voxelizer restatement on the same placed positions; then the surface Cp of
the placed mesh after a few steps of the tunnel."""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_stl_file_to_voxels_and_cp(native):
    from cfd__gb300 import SolverCUDA, malha, prepara
    from cfd__gb300.geometry import superelipsoide
    from cfd__gb300.tunel import montarTipos
    from cfd__gb300.visual import cp_superficie
    from cfd__gb300.voxel import voxelizar
    from oracle import oracle as O
    pos, idx = superelipsoide(2.2, 0.9, 0.6, 2.5, 3.0, 3000, 0.0, 13)
    tris = pos[idx].reshape(-1, 9)
    data = b"\0" * 80 + struct.pack("<I", len(tris)) + b"".join(
        struct.pack("<3f", 0, 0, 0) + struct.pack("<9f", *t) + b"\0\0" for t in tris)
    m = malha.ler(data, "carro.stl")
    g = {"nx": 96, "ny": 48, "nz": 40}
    r = prepara.preparar(m, g, celulasPorComprimento=30)
    vox = voxelizar(r["positions"], r["indices"], g, sdf=False)
    ref = O.voxelize(r["positions"], r["indices"], (g["nx"], g["ny"], g["nz"]), with_sdf=False)[0]
    assert np.array_equal(vox["tipo"], ref)
    assert (vox["tipo"] != 0).sum() > 500
    mt = montarTipos(g, corpo=vox["tipo"], esteira=False)
    s = SolverCUDA(g)
    s.definirTipos(mt["tipo"])
    s.configurar(omegaPlus=1.8, lesCs=0.1, inletU=[0.05, 0, 0], esponja=mt["esponja"])
    s.inicializar()
    s.passo(200)
    s.atualizarMacros()
    cp = cp_superficie(s, r["positions"], r["indices"], 0.05)
    assert np.isfinite(cp).all() and cp.max() > 0.2       # stagnation at the nose
    s.destruir()
