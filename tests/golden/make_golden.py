"""Generates tests/golden/lattice_legacy.json from the reference's own Python
lattice module (legacy/cfd/lattice.py of ceschmiedel/CFD_, a numpy restatement
of src/core/lattice.js kept by the reference as a cross-check).

Run in a checkout that has the reference next to it:
    python tests/golden/make_golden.py /path/to/reference
The output is committed; tests never read the reference at run time.
"""
import importlib.util
import json
import os
import sys

import numpy as np


def main(ref_root):
    spec = importlib.util.spec_from_file_location("ref_lattice", os.path.join(ref_root, "legacy", "cfd", "lattice.py"))
    L = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(L)
    rng = np.random.default_rng(20261203)
    delta = rng.normal(0.0, 1e-3, size=64)
    u = rng.uniform(-0.1, 0.1, size=(64, 3))
    eq = L.equilibrium(delta, u)
    d2, u2 = L.moments(eq)
    omegas = [0.6, 1.0, 1.5, 1.8, 1.9, 1.98]
    out = {
        "source": "legacy/cfd/lattice.py",
        "Q": int(L.Q), "CS2": float(L.CS2),
        "C": L.C.astype(int).tolist(), "W": L.W.tolist(), "OPP": L.OPP.astype(int).tolist(),
        "MAGIC": {k: float(v) for k, v in L.MAGIC.items()},
        "samples": {"delta": delta.tolist(), "u": u.tolist(), "eq": eq.tolist(),
                    "moments_delta": d2.tolist(), "moments_u": u2.tolist()},
        "omega": omegas,
        "nu_from_omega": [float(L.nu_from_omega(w)) for w in omegas],
        "omega_minus_wall": [float(L.omega_minus_from_lambda(w, L.MAGIC["WALL"])) for w in omegas],
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lattice_legacy.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} REFERENCE_CHECKOUT")
    main(sys.argv[1])
