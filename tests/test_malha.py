"""Mesh ingestion (cfd__gb300/malha.py, src/geom/parse.js) and placement
(cfd__gb300/prepara.py, src/geom/prepare.js) on synthetic files built here,
including the quirks the reference tolerates.  CPU only."""
import base64
import json
import struct

import numpy as np
import pytest

from cfd__gb300 import malha, prepara

TRI = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0], [0, 0, 0, 0, 1, 0, 0, 0, 1], [1.5, -2, 3, 4, 5.25, -6, 7, 8, 9]],
               np.float32)


def stl_bin(tris, header=b"", base=80, cut=0, count=None):
    h = header.ljust(base, b"\0")[:base]
    n = len(tris) if count is None else count
    body = b"".join(struct.pack("<3f", 0, 0, 1) + struct.pack("<9f", *t) + b"\0\0" for t in tris)
    data = h + struct.pack("<I", n) + body
    return data[:len(data) - cut] if cut else data


def test_stl_binary_and_its_quirks():
    r = malha.ler(stl_bin(TRI))
    assert r["formato"] == "stl-binario" and r["nTriangulos"] == 3
    assert np.array_equal(r["positions"], TRI.reshape(-1)) and np.array_equal(r["indices"], np.arange(9))
    # 79-byte header: the count is found where the arithmetic closes
    r = malha.ler(stl_bin(TRI, base=79))
    assert r["nTriangulos"] == 3 and np.array_equal(r["positions"], TRI.reshape(-1))
    assert any("stl-header-size: 79-byte" in a for a in r["avisos"])
    # a binary file whose header starts with "solid"
    r = malha.ler(stl_bin(TRI, header=b"solid exported by a CAD tool"))
    assert r["formato"] == "stl-binario" and any("stl-solid-binary" in a for a in r["avisos"])
    assert r["nome"] == "solid exported by a CAD tool"
    # one byte short: the incomplete last record is dropped, with a warning
    r = malha.ler(stl_bin(TRI, cut=1))
    assert r["nTriangulos"] == 2 and any("stl-truncated" in a for a in r["avisos"])


def test_stl_ascii():
    txt = "solid caixa\n"
    for t in TRI:
        txt += " facet normal 0 0 1\n  outer loop\n"
        for k in range(3):
            txt += "   vertex {} {} {}\n".format(*t[3 * k:3 * k + 3])
        txt += "  endloop\n endfacet\n"
    txt += "   vertex 1 2 3\nendsolid\n"
    r = malha.ler(txt.encode())
    assert r["formato"] == "stl-ascii" and r["nome"] == "caixa" and r["nTriangulos"] == 3
    assert np.array_equal(r["positions"], TRI.reshape(-1))
    assert any("stl-trailing-vertices" in a for a in r["avisos"])
    with pytest.raises(ValueError):
        malha.ler(b"not a mesh at all, just text of some length that is not stl" * 3)


def test_obj_polygons_negative_indices_and_range_quirk():
    txt = "# comment\no corpo\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nf 1/1/1 2//1 3 4\nv 2 2 2\nf -1 -2 -3\n"
    r = malha.ler(txt.encode(), "x.obj")
    assert r["formato"] == "obj" and r["nome"] == "corpo" and r["nVertices"] == 5
    assert r["indices"].tolist() == [0, 1, 2, 0, 2, 3, 4, 3, 2]
    # an out-of-range index is dropped on its own (the reference's filter)
    r = malha.ler(b"v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\nf 1 2 9\n", "y.obj")
    assert r["indices"].tolist() == [0, 1, 2, 0, 1] and any("obj-index-range" in a for a in r["avisos"])


def test_ply_ascii_and_binary():
    txt = ("ply\nformat ascii 1.0\nelement vertex 4\nproperty float nx\nproperty float x\nproperty float y\n"
           "property float z\nelement face 1\nproperty list uchar int vertex_indices\nend_header\n"
           "9 0 0 0\n9 1 0 0\n9 1 1 0\n9 0 1 0\n4 0 1 2 3\n")
    r = malha.ler(txt.encode())
    assert r["formato"] == "ply" and r["indices"].tolist() == [0, 1, 2, 0, 2, 3]
    assert np.array_equal(r["positions"].reshape(-1, 3)[2], [1, 1, 0])
    head = ("ply\nformat binary_little_endian 1.0\nelement vertex 3\nproperty float x\nproperty float y\n"
            "property float z\nproperty uchar red\nelement face 1\nproperty uchar flags\n"
            "property list uchar uint vertex_indices\nend_header\n").encode()
    body = b"".join(struct.pack("<3fB", *v, 7) for v in ([0, 0, 0], [2, 0, 0], [0, 3, 0]))
    body += struct.pack("<BB3I", 1, 3, 0, 1, 2)
    r = malha.ler(head + body)
    assert r["indices"].tolist() == [0, 1, 2] and np.array_equal(r["positions"], [0, 0, 0, 2, 0, 0, 0, 3, 0])


def _gltf_json(buffer_entry):
    return {"asset": {"version": "2.0", "generator": "teste"}, "scene": 0,
            "scenes": [{"name": "cena", "nodes": [0]}],
            "nodes": [{"translation": [10, 0, 0], "scale": [2, 2, 2], "children": [1]},
                      {"rotation": [0, 0, np.sin(np.pi / 4), np.cos(np.pi / 4)], "mesh": 0}],
            "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "indices": 1}]}],
            "buffers": [buffer_entry],
            "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 36},
                            {"buffer": 0, "byteOffset": 36, "byteLength": 6}],
            "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"},
                          {"bufferView": 1, "componentType": 5123, "count": 3, "type": "SCALAR"}]}


def _expected_gltf():
    # rotate 90 degrees about z, then scale 2, then translate x by 10
    v = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float64)
    rot = np.stack([-v[:, 1], v[:, 0], v[:, 2]], axis=1)
    return (rot * 2 + np.array([10, 0, 0])).astype(np.float32).reshape(-1)


def test_glb_and_gltf_with_node_transforms():
    bin_ = struct.pack("<9f", 1, 0, 0, 0, 1, 0, 0, 0, 1) + struct.pack("<3H", 0, 1, 2)
    js = json.dumps(_gltf_json({"byteLength": len(bin_)})).encode()
    js += b" " * ((4 - len(js) % 4) % 4)
    binp = bin_ + b"\0" * ((4 - len(bin_) % 4) % 4)
    glb = struct.pack("<III", 0x46546C67, 2, 12 + 8 + len(js) + 8 + len(binp))
    glb += struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(binp), 0x004E4942) + binp
    r = malha.ler(glb)
    assert r["formato"] == "glb" and r["nome"] == "cena" and r["indices"].tolist() == [0, 1, 2]
    np.testing.assert_allclose(r["positions"], _expected_gltf(), atol=1e-6)
    uri = "data:application/octet-stream;base64," + base64.b64encode(bin_).decode()
    r = malha.ler(json.dumps(_gltf_json({"byteLength": len(bin_), "uri": uri})).encode(), "m.gltf")
    assert r["formato"] == "gltf"
    np.testing.assert_allclose(r["positions"], _expected_gltf(), atol=1e-6)


def test_extentos_counts_non_finite():
    e = malha.extentos(np.array([0, 0, 0, 1, 2, 3, np.nan, 0, 0], np.float32))
    assert e["min"] == [0, 0, 0] and e["max"] == [1, 2, 3] and e["naoFinitos"] == 1
    assert e["centro"] == [0.5, 1.0, 1.5]


def _car(flow_axis=1, up_axis=2, nose_low=True):
    """A car-like block: long along flow_axis, symmetric across the lateral
    axis, a cabin at the rear half only (taller tail)."""
    from cfd__gb300.geometry import superelipsoide
    body, idx = superelipsoide(2.2, 0.9, 0.4, 2.5, 3.0, 800, 0.0, 9)
    cab, idx2 = superelipsoide(0.8, 0.7, 0.35, 2.5, 3.0, 400, 0.0, 9)
    cab = cab + np.array([0.9 if nose_low else -0.9, 0.0, 0.45], np.float32)
    pos = np.concatenate([body, cab])
    idx = np.concatenate([idx, idx2 + body.shape[0]])
    lat = 3 - flow_axis - up_axis
    out = np.empty_like(pos)
    out[:, flow_axis], out[:, lat], out[:, up_axis] = pos[:, 0], pos[:, 1], pos[:, 2]
    return {"positions": out.reshape(-1), "indices": idx.reshape(-1), "avisos": []}


def test_prepare_guesses_axes_sense_unit_and_places():
    g = {"nx": 320, "ny": 160, "nz": 128}
    m = _car(flow_axis=1, up_axis=0, nose_low=True)
    r = prepara.preparar(m, g)
    assert r["eixos"]["ordem"] == [1, 2, 0]
    assert r["unidade"]["nome"] == "metros" and abs(r["comprimentoM"] - 4.4) < 0.05
    ext = r["extentos"]
    assert abs(ext["min"][0] - 0.28 * 320) < 1e-3 and abs(ext["tamanho"][0] - round(0.34 * 320)) < 1e-2
    assert abs(ext["min"][2] - 1.0) < 1e-3 and abs(ext["centro"][1] - 80.0) < 1e-2
    # the placed nose is the lower end
    p = r["positions"].reshape(-1, 3)
    front = p[p[:, 0] < ext["min"][0] + 0.2 * ext["tamanho"][0], 2].max()
    back = p[p[:, 0] > ext["max"][0] - 0.2 * ext["tamanho"][0], 2].max()
    assert front < back
    # a model loaded tail-first is turned round (half turn, not a reflection)
    r2 = prepara.preparar(_car(flow_axis=1, up_axis=0, nose_low=False), g)
    assert r2["sentido"]["inverter"] and r2["sentido"]["aplicado"]
    # millimetres and a manual override
    mm = dict(m, positions=m["positions"] * np.float32(1000))
    assert prepara.preparar(mm, g)["unidade"]["nome"] == "milímetros"
    assert prepara.preparar(m, g, ordem=[1, 0, 2])["eixos"]["manual"]


def test_units_guess():
    assert prepara.palpitar_unidade(4.5)["nome"] == "metros"
    assert prepara.palpitar_unidade(450)["nome"] == "centímetros"
    assert prepara.palpitar_unidade(1.0)["nome"] == "metros"
    assert prepara.palpitar_unidade(0.3)["nome"] == "normalizado"
    assert prepara.palpitar_unidade(1e6)["nome"] == "desconhecida"
