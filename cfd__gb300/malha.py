"""Mesh ingestion: STL, OBJ, PLY, glTF and GLB into one triangle soup for the
voxelizer (src/geom/parse.js).

Output of `ler`, for every format:

    {"positions": float32[3*nv], "indices": uint32[3*nt], "nome", "formato",
     "avisos": [str], "nTriangulos", "nVertices"}

Triangles are not welded.  Format detection trusts content over names, as
the reference does: a binary STL is recognised by the arithmetic
84 + 50 n = file size (also with a header of 76..84 bytes, or a file a few
bytes short), not by its first word.  Numbers parsed from text are taken as
doubles and stored as float32, as JS numbers stored into a Float32Array are.
The OBJ index filter keeps the reference's behaviour of dropping each
out-of-range index on its own (src/geom/parse.js:221-224).
"""
from __future__ import annotations

import base64
import json
import re
import struct

import numpy as np

TAM_TRI_BIN = 50
TAM_CABECALHO = 84


def contagem_stl_binario(buf: bytes):
    """src/geom/parse.js:59-98: {n, base, truncado, deslocado} or None."""
    if len(buf) < TAM_CABECALHO:
        return None

    def tentar(base):
        if base + 4 > len(buf):
            return None
        n = struct.unpack_from("<I", buf, base)[0]
        if n == 0 or n > 200e6:
            return None
        return n, base + 4 + n * TAM_TRI_BIN

    padrao = tentar(80)
    if padrao and padrao[1] == len(buf):
        return {"n": padrao[0], "base": 84, "truncado": 0, "deslocado": 0}
    for base in range(76, 85):
        if base == 80:
            continue
        t = tentar(base)
        if t and t[1] == len(buf):
            return {"n": t[0], "base": base + 4, "truncado": 0, "deslocado": base - 80}
    if padrao:
        folga = len(buf) - padrao[1]
        disponivel = (len(buf) - TAM_CABECALHO) // TAM_TRI_BIN
        if -TAM_TRI_BIN <= folga <= 4 and disponivel > 0:
            n = min(padrao[0], disponivel)
            return {"n": n, "base": 84, "truncado": padrao[0] - n, "deslocado": 0}
    return None


def _stl_binario(buf, info, avisos):
    n, base = info["n"], info["base"]
    if info["deslocado"]:
        avisos.append(f"stl-header-size: {base - 4}-byte header (80 expected); triangle count read at byte "
                      f"{base - 4}, the offset where 4 + 50 n bytes follow exactly")
    rec = np.frombuffer(buf, dtype=np.dtype([("nrm", "<f4", 3), ("v", "<f4", 9), ("attr", "<u2")]), count=n,
                        offset=base)
    positions = np.ascontiguousarray(rec["v"].reshape(-1)).astype(np.float32)
    if info["truncado"] > 0:
        avisos.append(f"stl-truncated: {info['truncado']} declared triangle(s) missing from the end of the "
                      "file; read the complete ones")
    return positions, np.arange(n * 3, dtype=np.uint32)


_VERTEX = re.compile(r"vertex\s+(-?[\d.eE+-]+)\s+(-?[\d.eE+-]+)\s+(-?[\d.eE+-]+)")


def _num(s):
    try:
        return float(s)
    except ValueError:
        return float("nan")


def _stl_ascii(texto, avisos):
    verts = []
    for m in _VERTEX.finditer(texto):
        verts.extend((_num(m.group(1)), _num(m.group(2)), _num(m.group(3))))
    if not verts:
        raise ValueError("stl-ascii-empty: no vertex lines")
    if len(verts) % 9:
        sobra = (len(verts) % 9) // 3
        avisos.append(f"stl-trailing-vertices: {sobra} vertex line(s) after the last full triangle, dropped")
        verts = verts[:len(verts) - len(verts) % 9]
    positions = np.array(verts, np.float64).astype(np.float32)
    return positions, np.arange(positions.size // 3, dtype=np.uint32)


def parse_stl(buf: bytes, avisos=None):
    """src/geom/parse.js:151-172."""
    avisos = [] if avisos is None else avisos
    b = contagem_stl_binario(buf)
    if b:
        cab = buf[:min(80, b["base"] - 4)].decode("latin1")
        cab = re.sub(r"\0.*$", "", cab, flags=re.S).strip()
        if re.match(r"^solid", cab, re.I):
            avisos.append("stl-solid-binary: the header text begins with 'solid' but the size fits the binary "
                          "layout (84 + 50 n bytes); read as binary")
        pos, idx = _stl_binario(buf, b, avisos)
        return {"positions": pos, "indices": idx, "formato": "stl-binario", "nome": cab}
    texto = buf.decode("utf-8", errors="replace")
    if not re.match(r"^\s*solid", texto, re.I):
        raise ValueError("stl-unknown: the size does not fit the binary layout and the text does not begin "
                         "with 'solid'")
    m = re.search(r"^\s*solid[ \t]*(.*)$", texto, re.M)
    pos, idx = _stl_ascii(texto, avisos)
    return {"positions": pos, "indices": idx, "formato": "stl-ascii", "nome": (m.group(1) if m else "").strip()}


def _parse_int(s):
    m = re.match(r"^\s*([+-]?\d+)", s)
    return int(m.group(1)) if m else None


def parse_obj(texto: str, avisos=None):
    """src/geom/parse.js:176-223."""
    avisos = [] if avisos is None else avisos
    vx, tris, nome = [], [], ""
    for linha in texto.split("\n"):
        if linha[:1] == "#":
            continue
        t = linha.strip()
        if not t:
            continue
        if t.startswith("v "):
            p = re.split(r"\s+", t)
            vx.extend(_num(p[i]) if i < len(p) else float("nan") for i in (1, 2, 3))
        elif t.startswith("f "):
            idx = []
            for s in re.split(r"\s+", t)[1:]:
                i = _parse_int(s.split("/")[0])
                if i is None:
                    continue
                r = i - 1 if i > 0 else len(vx) // 3 + i
                if r >= 0:
                    idx.append(r)
            for k in range(1, len(idx) - 1):
                tris.extend((idx[0], idx[k], idx[k + 1]))
        elif t.startswith("o ") or t.startswith("g "):
            if not nome:
                nome = t[2:].strip()
    if not tris:
        raise ValueError("obj-no-faces: no face with three or more vertices")
    nv = len(vx) // 3
    fora = sum(1 for i in tris if i < 0 or i >= nv)
    if fora:
        avisos.append(f"obj-index-range: {fora} face index/indices outside the vertex list, dropped")
    return {"positions": np.array(vx, np.float64).astype(np.float32),
            "indices": np.array([i for i in tris if 0 <= i < nv], np.uint32), "formato": "obj", "nome": nome}


_PLY_TIPOS = {"char": "b", "int8": "b", "uchar": "B", "uint8": "B", "short": "h", "int16": "h", "ushort": "H",
              "uint16": "H", "int": "i", "int32": "i", "uint": "I", "uint32": "I", "float": "f", "float32": "f",
              "double": "d", "float64": "d"}


def parse_ply(buf: bytes, avisos=None):
    """src/geom/parse.js:227-336."""
    avisos = [] if avisos is None else avisos
    cab = buf[:65536].decode("latin1")
    fim = cab.find("end_header")
    if fim < 0:
        raise ValueError("ply-header: end_header not found in the first 64 KiB")
    inicio = cab.find("\n", fim) + 1
    formato, atual, elementos = None, None, []
    for l in re.split(r"\r?\n", cab[:fim]):
        p = re.split(r"\s+", l.strip())
        if p[0] == "format":
            formato = p[1]
        elif p[0] == "element":
            atual = {"nome": p[1], "contagem": int(float(p[2])), "props": []}
            elementos.append(atual)
        elif p[0] == "property" and atual is not None:
            if p[1] == "list":
                atual["props"].append({"lista": True, "tipoTam": p[2], "tipoItem": p[3], "nome": p[4]})
            else:
                atual["props"].append({"lista": False, "tipo": p[1], "nome": p[2]})
    ev = next((e for e in elementos if e["nome"] == "vertex"), None)
    ef = next((e for e in elementos if e["nome"] == "face"), None)
    if ev is None:
        raise ValueError("ply-vertex: no vertex element declared")
    positions = np.zeros(ev["contagem"] * 3, np.float32)
    tris = []
    ix = next((k for k, q in enumerate(ev["props"]) if q["nome"] == "x"), -1)
    if formato == "ascii":
        texto = buf.decode("latin1")
        corpo = texto[texto.find("\n", texto.find("end_header")) + 1:]
        tok = [s for s in re.split(r"\s+", corpo) if s]
        p = 0
        for i in range(ev["contagem"]):
            for k in range(len(ev["props"])):
                v = _num(tok[p]) if p < len(tok) else float("nan")
                p += 1
                if ix <= k < ix + 3:
                    positions[i * 3 + (k - ix)] = v
        if ef is not None:
            for i in range(ef["contagem"]):
                n = int(_num(tok[p])); p += 1
                face = [int(_num(tok[p + k])) for k in range(n)]
                p += n
                for k in range(1, n - 1):
                    tris.extend((face[0], face[k], face[k + 1]))
    else:
        e = "<" if formato == "binary_little_endian" else ">"
        p = [inicio]

        def ler(tipo):
            c = _PLY_TIPOS.get(tipo)
            if c is None:
                raise ValueError(f"ply-type: property type {tipo} not recognised")
            v = struct.unpack_from(e + c, buf, p[0])[0]
            p[0] += struct.calcsize(c)
            return v
        for i in range(ev["contagem"]):
            for k, q in enumerate(ev["props"]):
                v = ler(q["tipo"])
                if ix <= k < ix + 3:
                    positions[i * 3 + (k - ix)] = v
        if ef is not None:
            pl = next((q for q in ef["props"] if q["lista"]), None)
            for i in range(ef["contagem"]):
                for q in ef["props"]:
                    if q is not pl:
                        ler(q["tipo"])
                        continue
                    n = ler(q["tipoTam"])
                    face = [ler(q["tipoItem"]) for _ in range(n)]
                    for k in range(1, n - 1):
                        tris.extend((face[0], face[k], face[k + 1]))
    if not tris:
        raise ValueError("ply-faces: no face element or no faces")
    return {"positions": positions, "indices": np.array(tris, np.uint32), "formato": "ply", "nome": ""}


_COMP = {5120: ("<i1", 1), 5121: ("<u1", 1), 5122: ("<i2", 2), 5123: ("<u2", 2), 5125: ("<u4", 4),
         5126: ("<f4", 4)}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}


def _mat_mul(a, b):
    """Column-major 4x4 product (src/geom/parse.js:348-357)."""
    o = [0.0] * 16
    for c in range(4):
        for r in range(4):
            o[c * 4 + r] = (a[r] * b[c * 4] + a[4 + r] * b[c * 4 + 1] + a[8 + r] * b[c * 4 + 2] +
                            a[12 + r] * b[c * 4 + 3])
    return o


def _trs(t, r, s):
    """src/geom/parse.js:359-371."""
    x, y, z, w = r
    x2, y2, z2 = x + x, y + y, z + z
    xx, xy, xz = x * x2, x * y2, x * z2
    yy, yz, zz = y * y2, y * z2, z * z2
    wx, wy, wz = w * x2, w * y2, w * z2
    return [(1 - (yy + zz)) * s[0], (xy + wz) * s[0], (xz - wy) * s[0], 0,
            (xy - wz) * s[1], (1 - (xx + zz)) * s[1], (yz + wx) * s[1], 0,
            (xz + wy) * s[2], (yz - wx) * s[2], (1 - (xx + yy)) * s[2], 0,
            t[0], t[1], t[2], 1]


def _montar_gltf(js, buffers, avisos):
    """Scene walk with node transforms, all TRIANGLES primitives concatenated
    (src/geom/parse.js:388-498)."""
    pos_acc, idx_acc, total = [], [], 0

    def dados(i_acc):
        acc = js["accessors"][i_acc]
        comp = _COMP.get(acc.get("componentType"))
        n = _NCOMP.get(acc.get("type"))
        if not comp or not n:
            raise ValueError(f"gltf-accessor: accessor {i_acc} has a component type this reader does not take")
        if acc.get("bufferView") is None:
            return np.zeros(acc["count"] * n, comp[0])
        bv = js["bufferViews"][acc["bufferView"]]
        buf = buffers[bv.get("buffer", 0)] if bv.get("buffer", 0) < len(buffers) else None
        if buf is None:
            raise ValueError("gltf-buffer-view: refers to a buffer that was not loaded")
        base = bv.get("byteOffset", 0) + acc.get("byteOffset", 0)
        passo = bv.get("byteStride", 0)
        if not passo or passo == comp[1] * n:
            return np.frombuffer(buf, comp[0], acc["count"] * n, base).copy()
        out = np.zeros(acc["count"] * n, comp[0])
        for i in range(acc["count"]):
            out[i * n:(i + 1) * n] = np.frombuffer(buf, comp[0], n, base + i * passo)
        return out

    def visitar(i_node, pai):
        nonlocal total
        nodes = js.get("nodes", [])
        if i_node >= len(nodes):
            return
        node = nodes[i_node]
        local = node["matrix"] if "matrix" in node else _trs(node.get("translation", [0, 0, 0]),
                                                           node.get("rotation", [0, 0, 0, 1]),
                                                           node.get("scale", [1, 1, 1]))
        M = _mat_mul(pai, local)
        if node.get("mesh") is not None:
            for prim in js["meshes"][node["mesh"]].get("primitives", []):
                if prim.get("mode") is not None and prim["mode"] != 4:
                    avisos.append(f"gltf-mode: primitive of mode {prim['mode']} is not a triangle list, skipped")
                    continue
                if (prim.get("extensions") or {}).get("KHR_draco_mesh_compression"):
                    avisos.append("gltf-draco: Draco-compressed primitive skipped (no decoder here); export it "
                                  "uncompressed")
                    continue
                i_pos = (prim.get("attributes") or {}).get("POSITION")
                if i_pos is None:
                    continue
                p = dados(i_pos).astype(np.float64).reshape(-1, 3)
                x, y, z = p[:, 0], p[:, 1], p[:, 2]
                tr = np.empty_like(p)
                tr[:, 0] = M[0] * x + M[4] * y + M[8] * z + M[12]
                tr[:, 1] = M[1] * x + M[5] * y + M[9] * z + M[13]
                tr[:, 2] = M[2] * x + M[6] * y + M[10] * z + M[14]
                pos_acc.append(tr.reshape(-1).astype(np.float32))
                nv = p.shape[0]
                if prim.get("indices") is not None:
                    ind = (dados(prim["indices"]).astype(np.int64) + total).astype(np.uint32)
                else:
                    ind = np.arange(total, total + nv, dtype=np.uint32)
                idx_acc.append(ind)
                total += nv
        for f in node.get("children", []):
            visitar(f, M)

    cenas = js.get("scenes")
    cena = cenas[js.get("scene", 0)] if cenas else None
    raizes = cena.get("nodes", []) if cena else list(range(len(js.get("nodes", []))))
    ident = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1]
    for r in raizes:
        visitar(r, ident)
    if not pos_acc:
        raise ValueError("gltf-empty: no triangle geometry in the scene")
    return np.concatenate(pos_acc), np.concatenate(idx_acc)


def _b64(uri):
    return base64.b64decode(uri.split(",", 1)[1])


def parse_glb(buf: bytes, avisos=None):
    """src/geom/parse.js:500-532."""
    avisos = [] if avisos is None else avisos
    if struct.unpack_from("<I", buf, 0)[0] != 0x46546C67:
        raise ValueError("glb-magic: the file does not start with the glTF magic bytes")
    versao = struct.unpack_from("<I", buf, 4)[0]
    if versao != 2:
        avisos.append(f"glb-version: container version {versao}, read as glTF 2.0")
    js, bins, p = None, [], 12
    while p + 8 <= len(buf):
        tam, tipo = struct.unpack_from("<II", buf, p)
        dados = buf[p + 8:p + 8 + tam]
        if tipo == 0x4E4F534A:
            js = json.loads(dados.decode("utf-8"))
        elif tipo == 0x004E4942:
            bins.append(dados)
        p += 8 + tam + ((4 - tam % 4) % 4)
    if js is None:
        raise ValueError("glb-json: no JSON chunk")
    buffers = []
    for i, b in enumerate(js.get("buffers", [])):
        if b.get("uri") is None:
            buffers.append(bins[0] if bins else (bins[i] if i < len(bins) else None))
        elif b["uri"].startswith("data:"):
            buffers.append(_b64(b["uri"]))
        else:
            avisos.append(f"gltf-external-buffer: {b['uri']} is a separate file and was not loaded")
            buffers.append(None)
    if not buffers:
        buffers.append(bins[0] if bins else None)
    cenas = js.get("scenes")
    nome = (cenas[js.get("scene", 0)].get("name") if cenas else None) or (js.get("asset") or {}).get("generator", "")
    pos, idx = _montar_gltf(js, buffers, avisos)
    return {"positions": pos, "indices": idx, "formato": "glb", "nome": nome}


def parse_gltf(texto: str, avisos=None):
    """src/geom/parse.js:534-545."""
    avisos = [] if avisos is None else avisos
    js = json.loads(texto)
    buffers = []
    for b in js.get("buffers", []):
        if (b.get("uri") or "").startswith("data:"):
            buffers.append(_b64(b["uri"]))
        else:
            avisos.append(f"gltf-external-buffer: {b.get('uri')} is a separate file and was not loaded (a .glb "
                          "carries its buffers inside)")
            buffers.append(None)
    cenas = js.get("scenes")
    nome = (cenas[js.get("scene", 0)].get("name") if cenas else None) or ""
    pos, idx = _montar_gltf(js, buffers, avisos)
    return {"positions": pos, "indices": idx, "formato": "gltf", "nome": nome}


def ler(buf: bytes, nome_arquivo: str = ""):
    """Any supported format, decided by content, the name only as a tie-break
    (src/geom/parse.js:555-585)."""
    avisos = []
    m = re.search(r"\.([a-z0-9]+)$", nome_arquivo, re.I)
    ext = m.group(1).lower() if m else ""
    magia = struct.unpack_from("<I", buf, 0)[0] if len(buf) >= 4 else 0
    inicio = buf[:1024].decode("latin1")
    if magia == 0x46546C67:
        r = parse_glb(buf, avisos)
    elif re.match(r"^ply\s", inicio):
        r = parse_ply(buf, avisos)
    elif ext == "gltf" or re.match(r'^\s*\{[\s\S]*"asset"', inicio):
        r = parse_gltf(buf.decode("utf-8"), avisos)
    elif ext == "obj" or re.search(r"^\s*(v\s|vn\s|vt\s|#|mtllib|o\s|g\s)", inicio, re.M):
        r = parse_stl(buf, avisos) if contagem_stl_binario(buf) else parse_obj(buf.decode("utf-8", "replace"), avisos)
    else:
        r = parse_stl(buf, avisos)
    nt = r["indices"].size // 3
    if not nt:
        raise ValueError(f"{r['formato']}: the file holds no triangles")
    return dict(r, avisos=avisos, nTriangulos=nt, nVertices=r["positions"].size // 3)


def extentos(positions):
    """Bounding box and count of non-finite vertices (src/geom/parse.js:588-605)."""
    p = np.asarray(positions, np.float64).reshape(-1, 3)
    ok = np.isfinite(p.sum(axis=1))
    q = p[ok]
    mn = q.min(axis=0) if q.size else np.full(3, np.inf)
    mx = q.max(axis=0) if q.size else np.full(3, -np.inf)
    return {"min": mn.tolist(), "max": mx.tolist(), "tamanho": (mx - mn).tolist(), "centro": ((mn + mx) / 2).tolist(),
            "naoFinitos": int((~ok).sum())}
