"""Make tests/golden/closure_fine_re10000.json: the drag of the fine
(640x320x256, 2x resolution) run of the learned-closure workload at the
held-out Reynolds number 10 000, the reference the closure gain test scores
the coarse runs against.

    python tests/golden/make_closure_fixture.py [--steps 24000]

Runs on cuda:0 (about a minute on one GB300): the 20k-triangle
superellipsoid of the mesh-body workload scaled by two, u_in 0.06, Re 10 000
on the 192-cell fine length, Smagorinsky Cs 0.12, fp32; Cd from the force
averaged over blocks of 500 steps, mean of the second half
(cfd__gb300.estudos.rodar_fecho, the closure study's own measurement).
"""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=24000)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                  "closure_fine_re10000.json"))
    a = ap.parse_args()
    from cfd__gb300 import build
    build.build()
    from cfd__gb300.estudos import rodar_fecho, tuneis_fecho
    _, (gf, tf, ef, af) = tuneis_fecho(2026)
    rec, _ = rodar_fecho(gf, tf, ef, af, 10000, a.steps, 500, u=0.06, comprimento=192.0, cs=0.12)
    out = {"grid": gf, "Re": 10000, "u_in": 0.06, "cs": 0.12, "length_cells": 192, "steps": rec["steps"],
           "block": 500, "cd": rec["cd"], "cd_std": rec["cd_std"], "diverged": rec["diverged"],
           "frontal_area": af, "command": "python tests/golden/make_closure_fixture.py --steps %d" % a.steps}
    with open(a.out, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
