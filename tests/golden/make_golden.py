"""Regenerates the golden fixtures in this directory from the CPU oracle.

The reference (pbosler/lpmKokkos) cannot be built here, and it records no BVE trajectories,
so the oracle's own outputs -- pinned to the reference's recorded Poisson table and
known answers by tests/test_oracle_golden.py -- are frozen as fixtures:

  bve_<seed>_L2.npz : icosahedral / cubed-sphere level 2, RH54 + 2 Gaussian vortices
                      (seed 20261203); velocity and stream function at vertices and faces;
                      the state after 2 RK4 steps (dt 0.01, Omega 2 pi, face quirk on).

Run:  python tests/golden/make_golden.py
"""
import hashlib
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

SEED, NG, DT, OMEGA, NSTEPS = 20261203, 2, 0.01, 2 * math.pi, 2


def make(seed_kind):
    m = O.mesh(seed_kind, 2)
    zv = O.rh54_gaussians(m["vx"], SEED, NG)
    zf = O.rh54_gaussians(m["fx"], SEED, NG)
    uv, uf, pv, pf = O.velocity(m["vx"], m["fx"], zf, m["farea"], m["fmask"], psi=True)
    out = O.rk4(m["vx"], zv, uv, m["fx"], zf, uf, m["farea"], m["fmask"], DT, OMEGA, NSTEPS)
    arrays = dict(vx=m["vx"], fx=m["fx"], farea=m["farea"], fmask=m["fmask"], vzeta=zv, fzeta=zf,
                  vu=uv, fu=uf, vpsi=pv, fpsi=pf,
                  rk_vx=out[0], rk_vzeta=out[1], rk_vvel=out[2], rk_fx=out[3], rk_fzeta=out[4], rk_fvel=out[5])
    name = f"bve_{'icos' if seed_kind == 0 else 'cube'}_L2.npz"
    np.savez_compressed(os.path.join(HERE, name), **arrays)
    h = hashlib.sha256(b"".join(np.ascontiguousarray(arrays[k]).tobytes() for k in sorted(arrays))).hexdigest()
    return name, h


def main():
    meta = {"seed": SEED, "gaussians": NG, "dt": DT, "omega": OMEGA, "rk4_steps": NSTEPS, "quirk": True,
            "files": {}}
    for k in (0, 1):
        name, h = make(k)
        meta["files"][name] = h
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(json.dumps(meta, indent=1))


if __name__ == "__main__":
    main()
