"""From the mesh as exported to the mesh placed in the tunnel
(src/geom/prepare.js): guesses of the flow axis, the lateral and vertical
axes (mirror symmetry on a coarse occupancy grid), the nose direction (the
silhouette is lower at the nose), the file unit, and the placement in
lattice coordinates.  Every guess is returned with its confidence and can be
overridden, as in the reference.

Arithmetic follows the reference: doubles, with the Float32Array stores of
the placed positions rounding to float32 after each stage.
"""
from __future__ import annotations

import math

import numpy as np

from .malha import extentos


def ocupacao(pos, ext, K=24):
    """Occupancy of a K^3 grid over the bounding box (src/geom/prepare.js:37-48)."""
    p = np.asarray(pos, np.float64).reshape(-1, 3)
    ok = np.isfinite(p.sum(axis=1))
    p = p[ok]
    inv = [K / t if t > 0 else 0.0 for t in ext["tamanho"]]
    ijk = []
    for a in range(3):
        v = (p[:, a] - ext["min"][a]) * inv[a]
        ijk.append(np.clip(np.trunc(v).astype(np.int64), 0, K - 1))
    oc = np.zeros((K, K, K), np.uint8)          # [c][b][a]
    oc[ijk[2], ijk[1], ijk[0]] = 1
    return oc


def simetria(oc, eixo):
    """Fraction of occupied cells whose mirror along `eixo` is occupied
    (src/geom/prepare.js:51-67)."""
    ocupados = int(oc.sum())
    if not ocupados:
        return 0.0
    axis = {0: 2, 1: 1, 2: 0}[eixo]               # oc is indexed [z][y][x]
    return float((oc & np.flip(oc, axis=axis)).sum()) / ocupados


def palpitar_eixos(pos, ext):
    """src/geom/prepare.js:74-104: flow = longest extent; of the other two the
    more mirror-symmetric is lateral, the other vertical."""
    ordem_tam = sorted([0, 1, 2], key=lambda a: -ext["tamanho"][a])
    fluxo = ordem_tam[0]
    r0, r1 = [a for a in (0, 1, 2) if a != fluxo]
    oc = ocupacao(pos, ext)
    sim = [simetria(oc, a) for a in range(3)]
    lateral = r0 if sim[r0] >= sim[r1] else r1
    vertical = r1 if lateral == r0 else r0
    return {"ordem": [fluxo, lateral, vertical], "simetrias": sim, "confianca": abs(sim[r0] - sim[r1]),
            "talvezInvertido": None}


def palpitar_sentido(pos, ordem, ext, N=12):
    """src/geom/prepare.js:133-163: tallest silhouette in the first and last
    20 % along the flow axis; the nose is the lower end."""
    ex, ez = ordem[0], ordem[2]
    x0 = ext["min"][ex]
    comprimento = max(ext["tamanho"][ex], 1e-12)
    zb = ext["min"][ez]
    p = np.asarray(pos, np.float64).reshape(-1, 3)
    x, z = p[:, ex], p[:, ez]
    ok = np.isfinite(x + z)
    x, z = x[ok], z[ok]
    k = np.clip(np.floor((x - x0) / comprimento * N), 0, N - 1).astype(np.int64)
    h = z - zb
    alturas = np.zeros(N)
    np.maximum.at(alturas, k, h)
    alturas = np.maximum(alturas, 0.0)
    m = int(round(N * 0.2))
    frente = float(alturas[:m].sum() / m)
    tras = float(alturas[N - m:].sum() / m)
    escala = max(frente, tras, 1e-12)
    return {"inverter": frente > tras, "alturaFrente": frente, "alturaTras": tras,
            "confianca": abs(tras - frente) / escala}


def palpitar_unidade(comprimento):
    """src/geom/prepare.js:177-204: the factor that takes the file to metres."""
    for fator, nome, lo, hi in ((1, "metros", 0.5, 30), (0.01, "centímetros", 50, 3000),
                                (0.001, "milímetros", 500, 30000), (0.0254, "polegadas", 20, 1200)):
        if lo <= comprimento <= hi:
            return {"fator": fator, "nome": nome, "tipico": [lo, hi], "normalizado": False, "confianca": "plausível"}
    if 0.2 < comprimento < 2.5:
        return {"fator": 1, "nome": "normalizado", "normalizado": True, "confianca": "nenhuma",
                "aviso": f"unit-normalised: longest side {comprimento:.3f} looks like a unit-scaled model; give "
                         "the body's real length (comprimentoM), since Re and Cd use it"}
    return {"fator": 1, "nome": "desconhecida", "normalizado": True, "confianca": "nenhuma",
            "aviso": f"unit-unknown: longest side {comprimento:.4g} fits no unit's usual range; give the body's "
                     "real length (comprimentoM)"}


def colocar(positions, ordem, grade, celulas_por_comprimento, espelhar=(False, False, False), fracao_entrada=0.28,
            assentar_no_piso=True, folga_piso=1, guinada_graus=0):
    """src/geom/prepare.js:226-300: permute / mirror, yaw about the vertical,
    scale so the length spans celulas_por_comprimento cells, nose at
    fracao_entrada * nx, centred in y, on the floor (or centred in z)."""
    p = np.asarray(positions, np.float32).reshape(-1, 3)
    s0 = np.empty_like(p)
    for a in range(3):
        v = p[:, ordem[a]]
        s0[:, a] = -v if espelhar[a] else v
    if guinada_graus:
        t = guinada_graus * math.pi / 180
        cs, sn = math.cos(t), math.sin(t)
        e0 = extentos(s0)
        cx, cy = e0["centro"][0], e0["centro"][1]
        x = s0[:, 0].astype(np.float64) - cx
        y = s0[:, 1].astype(np.float64) - cy
        s0[:, 0] = (cx + x * cs - y * sn).astype(np.float32)
        s0[:, 1] = (cy + x * sn + y * cs).astype(np.float32)
    ext = extentos(s0)
    comprimento = max(ext["tamanho"][0], 1e-12)
    s = celulas_por_comprimento / comprimento
    ax = grade["nx"] * fracao_entrada - ext["min"][0] * s
    ay = grade["ny"] * 0.5 - ext["centro"][1] * s
    az = (folga_piso - ext["min"][2] * s) if assentar_no_piso else (grade["nz"] * 0.5 - ext["centro"][2] * s)
    out = np.empty_like(s0)
    out[:, 0] = (s0[:, 0].astype(np.float64) * s + ax).astype(np.float32)
    out[:, 1] = (s0[:, 1].astype(np.float64) * s + ay).astype(np.float32)
    out[:, 2] = (s0[:, 2].astype(np.float64) * s + az).astype(np.float32)
    ef = extentos(out)
    bloqueio = (ef["tamanho"][1] * ef["tamanho"][2]) / (grade["ny"] * grade["nz"])
    avisos = []
    for a, nome in ((0, "x"), (1, "y"), (2, "z")):
        lim = (grade["nx"], grade["ny"], grade["nz"])[a]
        if ef["min"][a] < 0 or ef["max"][a] > lim:
            avisos.append(f"body-outside: along {nome} the body spans {ef['min'][a]:.1f} to {ef['max'][a]:.1f}, "
                          f"the grid 0 to {lim}")
    if bloqueio > 0.10:
        avisos.append(f"blockage: the body's box covers {bloqueio * 100:.1f} % of the cross-section; past 10 % the "
                      "Maskell blockage correction is not reliable, so widen the grid")
    return {"positions": out.reshape(-1), "escala": s, "extentos": ef, "bloqueioCaixa": bloqueio, "avisos": avisos}


def preparar(malha, grade, **opcoes):
    """src/geom/prepare.js:306-354: the whole pipeline with every guess exposed
    and overridable (ordem, unidade, comprimentoM, inverterSentido, espelhar,
    celulasPorComprimento, fracaoEntrada, assentarNoPiso, folgaPiso,
    guinadaGraus)."""
    pos = malha["positions"]
    ext = extentos(pos)
    if opcoes.get("ordem") is not None:
        eixos = {"ordem": list(opcoes["ordem"]), "confianca": 1, "simetrias": None, "manual": True}
    else:
        eixos = palpitar_eixos(pos, ext)
    comp_arq = ext["tamanho"][eixos["ordem"][0]]
    unidade = opcoes.get("unidade") or palpitar_unidade(comp_arq)
    comprimento_m = opcoes.get("comprimentoM", comp_arq * unidade["fator"])
    sentido = palpitar_sentido(pos, eixos["ordem"], ext)
    inverter = opcoes.get("inverterSentido")
    inverter = sentido["inverter"] if inverter is None else inverter
    # a half turn about the vertical (x -> -x, y -> -y), not a reflection
    espelhar = opcoes.get("espelhar") or ((True, True, False) if inverter else (False, False, False))
    kw = {k2: opcoes[k1] for k1, k2 in (("fracaoEntrada", "fracao_entrada"), ("assentarNoPiso", "assentar_no_piso"),
                                         ("folgaPiso", "folga_piso"), ("guinadaGraus", "guinada_graus"))
          if opcoes.get(k1) is not None}
    col = colocar(pos, eixos["ordem"], grade,
                  opcoes.get("celulasPorComprimento", int(math.floor(grade["nx"] * 0.34 + 0.5))), espelhar, **kw)
    avisos = list(malha.get("avisos", [])) + col["avisos"]
    if unidade.get("aviso"):
        avisos.append(unidade["aviso"])
    if sentido["confianca"] < 0.12:
        avisos.append(f"direction-guess: front and rear heights are close ({sentido['alturaFrente']:.2f}, "
                      f"{sentido['alturaTras']:.2f}), so the flow direction is a guess; check that the flow meets "
                      "the nose and set inverterSentido otherwise")
    return dict(col, indices=malha["indices"], eixos=eixos,
                sentido=dict(sentido, aplicado=inverter, manual=opcoes.get("inverterSentido") is not None),
                unidade=unidade, comprimentoM=comprimento_m, extentosOriginais=ext, avisos=avisos)
