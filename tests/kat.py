"""The reference's known-answer tests, restated once and run against any
solver object with the reference's class API (the GPU SolverCUDA) or against
the CPU oracle through OracleSolver below.

Sources: tests/nucleo.html:107-237 (uniform flow, shear wave, mass
conservation) and tests/validacao.html:122-184 (Couette wall position).
"""
import math
import os

import numpy as np

from cfd__gb300 import lattice as L


class OracleSolver:
    """The CPU oracle behind the reference's method names (tests only)."""

    def __init__(self, grade, nthreads=None):
        from oracle import oracle as O
        self.O = O
        self.nx, self.ny, self.nz = grade["nx"], grade["ny"], grade["nz"]
        self.N = self.nx * self.ny * self.nz
        self.lat = O.Lattice((self.nx, self.ny, self.nz), nthreads=nthreads or min(8, os.cpu_count() or 1))
        self.passos = 0
        self.frente = "A"

    def definirTipos(self, t):
        self.lat.set_types(t)

    def configurar(self, omegaPlus, lesCs=0.1, inletU=(0, 0, 0), beltU=(0, 0, 0), esponja=None, magic=3 / 16,
                   espessuraCL=0):
        esp = esponja or {"inicio": math.floor(self.nx * 0.82 + 0.5),
                          "comprimento": max(4, math.floor(self.nx * 0.18 + 0.5))}
        self.lat.configure(omega_plus=omegaPlus, magic=magic, les_cs=lesCs, inlet_u=inletU, belt_u=beltU,
                           sponge_start=esp["inicio"], sponge_len=esp["comprimento"], bl_thickness=espessuraCL)

    def inicializar(self):
        self.lat.init()
        self.passos = 0

    def definirCampo(self, fn, equilibrium=L.equilibrium):
        z, y, x = np.meshgrid(np.arange(self.nz), np.arange(self.ny), np.arange(self.nx), indexing="ij")
        r = fn(x, y, z)
        delta = np.broadcast_to(np.asarray(r.get("delta", 0.0), np.float64), x.shape)
        u = np.stack([np.broadcast_to(np.asarray(c, np.float64), x.shape) for c in r["u"]], -1)
        g = equilibrium(delta, u)
        self.lat.set_populations(np.ascontiguousarray(np.moveaxis(g, -1, 0).reshape(19, -1)))

    def passo(self, n=1):
        self.lat.run(n)
        self.passos += n

    def atualizarMacros(self):
        self._m = self.lat.update_macros()

    def lerMacros(self):
        return self._m

    def medirForcas(self):
        return list(self.lat.forces())


def uniform_flow(make):
    """tests/nucleo.html:107-130: all fluid 64x32x32, omega 1, Cs 0, u (0.05,0,0), 200 steps."""
    s = make({"nx": 64, "ny": 32, "nz": 32})
    s.definirTipos(np.zeros(s.N, np.uint32))
    s.configurar(omegaPlus=1.0, lesCs=0.0, inletU=[0.05, 0, 0])
    s.inicializar()
    s.passo(200)
    s.atualizarMacros()
    m = s.lerMacros()
    err_u = max(np.abs(m[0::4] - 0.05).max(), np.abs(m[1::4]).max(), np.abs(m[2::4]).max())
    err_d = np.abs(m[3::4]).max()
    return float(err_u), float(err_d)


def shear_wave(make, omegas=(0.6, 1.0, 1.5, 1.8)):
    """tests/nucleo.html:140-188: u_x = A0 sin(2 pi y / 64) decays as exp(-nu k^2 t)."""
    NY, A0, T = 64, 0.02, 400
    k = 2 * math.pi / NY
    rows = []
    for om in omegas:
        s = make({"nx": 8, "ny": NY, "nz": 8})
        s.definirTipos(np.zeros(s.N, np.uint32))
        s.configurar(omegaPlus=om, lesCs=0.0, inletU=[0, 0, 0])
        s.frente = "A"
        s.definirCampo(lambda x, y, z: {"delta": 0, "u": [A0 * np.sin(k * y), 0 * y, 0 * y]}, L.equilibrium)
        s.passo(T)
        s.atualizarMacros()
        mm = s.lerMacros()
        ux = mm[0::4].astype(np.float64).reshape(8, NY, 8)
        sn = np.sin(k * np.arange(NY))[None, :, None] * np.ones((8, NY, 8))
        amp = (ux * sn).sum() / (sn * sn).sum()
        nu_t = L.nu_from_omega(om)
        nu_m = -math.log(abs(amp) / A0) / (k * k * T)
        rows.append((om, nu_t, nu_m, 100 * (nu_m - nu_t) / nu_t))
    return rows


def block_mass(make, steps=500):
    """tests/nucleo.html:193-237: 12^3 SOLIDO block in a periodic 96x48x48 box."""
    s = make({"nx": 96, "ny": 48, "nz": 48})
    t = np.zeros((48, 48, 96), np.uint32)
    t[18:30, 18:30, 30:42] = 1
    s.definirTipos(t.reshape(-1))
    s.configurar(omegaPlus=1.2, lesCs=0.0, inletU=[0.05, 0, 0], esponja={"inicio": 1e9, "comprimento": 1})
    s.inicializar()
    s.atualizarMacros()
    m0 = s.lerMacros()
    mass0 = float(m0[3::4].astype(np.float64).sum())
    s.passo(steps)
    s.atualizarMacros()
    m3 = s.lerMacros()
    mass1 = float(m3[3::4].astype(np.float64).sum())
    ux, uy, uz, dd = (m3[i::4].astype(np.float64) for i in range(4))
    nan = int((~np.isfinite(ux + uy + uz + dd)).sum())
    umax = float(np.sqrt(ux * ux + uy * uy + uz * uz).max())
    return {"N": s.N, "mass0": mass0, "mass1": mass1, "nan": nan, "umax": umax}


def couette(make, omegas=(0.7, 1.0, 1.6), nx=8, ny=8):
    """tests/validacao.html:122-184: floor SOLIDO, top SOLIDO_MOVEL at U=0.04."""
    nz, U = 34, 0.04
    rows = []
    for om in omegas:
        s = make({"nx": nx, "ny": ny, "nz": nz})
        t = np.zeros((nz, ny, nx), np.uint32)
        t[0] = 1
        t[nz - 1] = 4
        s.definirTipos(t.reshape(-1))
        s.configurar(omegaPlus=om, lesCs=0, inletU=[0, 0, 0], beltU=[U, 0, 0], esponja={"inicio": 1e9, "comprimento": 1})
        s.inicializar()
        H = nz - 2
        passos = math.ceil(4 * H * H / L.nu_from_omega(om))
        s.passo(passos)
        s.atualizarMacros()
        m = s.lerMacros()
        ux = m[0::4].astype(np.float64).reshape(nz, ny, nx)
        perfil = ux[1:nz - 1].mean(axis=(1, 2))
        z = np.arange(1, nz - 1, dtype=np.float64)
        n = perfil.size
        sx, sy, sxx, sxy = z.sum(), perfil.sum(), (z * z).sum(), (z * perfil).sum()
        a = (n * sxy - sx * sy) / (n * sxx - sx * sx)
        b = (sy - a * sx) / n
        rows.append({"omega": om, "a": a, "a_teorico": U / H, "z0": -b / a, "z1": (U - b) / a})
    return rows


def validation_case(make, caso):
    """One case of tests/validacao.html:198-300 (sphere / cylinder vs
    correlation), driven through the solver class API."""
    from cfd__gb300.forces import JanelaCd, coeficientes, strouhal
    from cfd__gb300.tunel import areaFrontalCorpo, corpoAnalitico, montarTipos
    from cfd__gb300.units import LatticeUnits
    from cfd__gb300.validacao import uLbParaOmega

    grade = caso["grade"]
    D = caso["diametroCelulas"]
    uLb = uLbParaOmega(caso["re"], D, 1.90)
    nuLb = uLb * D / caso["re"]
    omega = 1 / (nuLb / (1 / 3) + 0.5)
    units = LatticeUnits(uLb)
    s = make(grade)
    corpo = corpoAnalitico(grade, {"tipo": caso["forma"], "cx": grade["nx"] * 0.30, "cy": grade["ny"] * 0.5,
                                   "cz": grade["nz"] * 0.5, "raio": D / 2})
    mt = montarTipos(grade, corpo=corpo, esteira=False)
    tipo, esponja = mt["tipo"], mt["esponja"]
    t = tipo.reshape(grade["nz"], grade["ny"], grade["nx"])
    t[0, :, 1:grade["nx"] - 1] = 6
    s.definirTipos(tipo)
    s.configurar(omegaPlus=omega, lesCs=0, inletU=[uLb, 0, 0], esponja=esponja)
    s.inicializar()
    af = areaFrontalCorpo(corpo, grade)
    travessia = math.ceil(grade["nx"] / uLb)
    transiente = math.floor(caso["travessiasTransiente"] * travessia + 0.5)
    medida = math.floor(caso["travessiasMedida"] * travessia + 0.5)
    if caso.get("perturbacao"):
        a = caso["perturbacao"]["grausGuinada"] * math.pi / 180
        s.configurar(omegaPlus=omega, lesCs=0, esponja=esponja, inletU=[uLb * math.cos(a), 0, uLb * math.sin(a)])
        s.passo(caso["perturbacao"]["passos"])
        s.configurar(omegaPlus=omega, lesCs=0, inletU=[uLb, 0, 0], esponja=esponja)
    k = 0
    while k < transiente:
        s.passo(min(2000, transiente - k))
        k += 2000
    jan = JanelaCd(4000)
    serie_cl = []
    divergiu = None
    for k in range(0, medida, 100):
        s.passo(100)
        f = s.medirForcas()
        co = coeficientes(f, units, af, grade, corrigirBloqueio=True,
                          theta=1.0 if caso["forma"] == "cilindro" else 2.5)
        if not math.isfinite(co["cd"]):
            divergiu = s.passos
            break
        jan.adicionar(co["cd"])
        serie_cl.append(co["cl"])
    st = strouhal(serie_cl, 100, D, uLb) if caso.get("referenciaSt") else None
    return {"cd": jan.media, "desvio": jan.desvio, "ref": caso["referencia"](), "st": st, "omega": omega,
            "uLb": uLb, "af": af, "divergiu": divergiu, "passos": s.passos}
