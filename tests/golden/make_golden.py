"""Generate the golden parity fixtures in this folder from the reference itself.

Each case is a small D3Q19 lattice described cell by cell (kind flags, boundary
values, Guo force field, initial f-bar).  The script writes the case file, runs
``oracle/_ref/plb_case`` -- a driver that builds the case through the
reference's own construction API (MultiBlockLattice3D, defineDynamics, the
regularized / Zou-He boundary instantiators, initializeMomentumExchange) and
calls ``collideAndStream()`` -- and packs the reference's outputs into
``<case>.npz``:

  flags, bcval, force, f_init (after lattice.initialize()), f_final,
  stats (step, avRhoBar, avUSqr, maxUSqr, drag_x, drag_y, drag_z) per
  recorded step, energy / density (computeAverageEnergy/Density at the end),
  and the case parameters.

The large lid-driven cavity (64^3, 1000 steps) is stored as a fingerprint
(sha256 of the f-bar bytes, reductions, sampled populations) because its
arrays are 40 MB.

Run from the repository root on a machine with the reference checkout:

    make -f oracle/Makefile.ref -j8 REF=<palabos checkout>
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)

from lbcases import (  # noqa: E402
    CASES, BIG_CASES, CaseSpec, write_case_file, read_result_file,
)

DRIVER = os.path.join(ROOT, "oracle", "_ref", "plb_case")


def run_reference(spec: CaseSpec, tmp: str):
    cpath = os.path.join(tmp, spec.name + ".case")
    rpath = os.path.join(tmp, spec.name + ".res")
    write_case_file(spec, cpath)
    subprocess.run([DRIVER, cpath, rpath], check=True)
    return read_result_file(rpath, spec)


def main(argv):
    if not os.path.exists(DRIVER):
        raise SystemExit("build oracle/_ref/plb_case first (make -f oracle/Makefile.ref)")
    only = set(argv[1:])
    with tempfile.TemporaryDirectory() as tmp:
        for builder in CASES:
            spec = builder()
            if only and spec.name not in only:
                continue
            res = run_reference(spec, tmp)
            extra = {}
            if spec.rho_bar0 is not None:
                extra = dict(rho_bar0=spec.rho_bar0, j0=spec.j0, rho_bar_final=res["rho_bar_final"],
                             j_final=res["j_final"])
            for what in ("lattice", "density", "velocity"):
                if "binary_" + what in res:
                    extra["binary_" + what] = res["binary_" + what]
            if "state_plb" in res:
                extra.update(state_plb=res["state_plb"], state_dat=res["state_dat"])
            if "dstate_plb" in res:
                extra.update(dstate_plb=res["dstate_plb"], dstate_dat=res["dstate_dat"])
            if spec.sparse is not None:
                extra.update(sparse=spec.sparse, in_lattice=res["in_lattice"], compare=spec.compare)
            np.savez_compressed(
                os.path.join(HERE, spec.name + ".npz"),
                flags=spec.flags, bcval=spec.bcval, force=spec.force,
                f_init=res["f_init"], f_final=res["f_final"], stats=res["stats"],
                energy=res["energy"], density=res["density"],
                meta=json.dumps(spec.meta()), **extra,
            )
            print(f"{spec.name}: {spec.nx}x{spec.ny}x{spec.nz}, {spec.nsteps} steps, "
                  f"E={res['energy']:.12e} rho={res['density']:.12e}")
        for builder in BIG_CASES:
            spec = builder()
            if only and spec.name not in only:
                continue
            res = run_reference(spec, tmp)
            ff = np.ascontiguousarray(res["f_final"])
            rng = np.random.default_rng(7)
            sample_idx = rng.choice(ff.size, size=4096, replace=False)
            fp = dict(
                meta=spec.meta(),
                sha256_f_final=hashlib.sha256(ff.tobytes()).hexdigest(),
                sha256_f_init=hashlib.sha256(np.ascontiguousarray(res["f_init"]).tobytes()).hexdigest(),
                energy=res["energy"], density=res["density"],
                stats=res["stats"].tolist(),
                sample_idx=sample_idx.tolist(),
                sample_val=[float.hex(float(v)) for v in ff.reshape(-1)[sample_idx]],
                f_final_abs_sum=float(np.abs(ff).sum()),
            )
            with open(os.path.join(HERE, spec.name + ".json"), "w") as f:
                json.dump(fp, f, indent=1)
            print(f"{spec.name}: E={res['energy']:.12e} sha={fp['sha256_f_final'][:16]}")


if __name__ == "__main__":
    main(sys.argv)
