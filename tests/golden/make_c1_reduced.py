"""Exact J and K of the reduced ERI + J/K workload, for the GPU parity test.

The workload is quiqbox_gb300.workloads.reduced_shell_molecule() (4 H + 2 heavy atoms,
the bench workload's atom density and basis statistics, 36 functions) with the density
random_density(nfun, seed).  The fixture stores the flattened basis and the density
themselves (so the test needs no generator and no floating-point agreement between
machines), and J and K from the oracle's quad-precision instance (the reference's
recursions in 113-bit arithmetic) over every canonical function quartet, without
screening.  Run from the repository root:

    python tests/golden/make_c1_reduced.py
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def main(seed=3):
    import __graft_entry__ as ge
    import oracle
    qb = ge.load_package()
    from quiqbox_gb300.workloads import random_density, reduced_shell_molecule
    atoms, coords, bs = reduced_shell_molecule(seed=seed)
    fb = qb.flatten(bs)
    D = random_density(fb.nfun, seed)
    J, K = oracle.jk(fb, D, exact=True)
    out = {"source": "oracle quad-precision instance, all canonical quartets, no screening",
           "workload": "reduced_shell_molecule(n_h=4, n_heavy=2, seed=%d)" % seed, "seed": seed,
           "nfun": int(fb.nfun), "atoms": list(atoms),
           "fun_ptr": [int(x) for x in fb.fun_ptr], "ijk": [int(x) for x in np.asarray(fb.ijk).reshape(-1)],
           "center": [float(x) for x in np.asarray(fb.center).reshape(-1)],
           "alpha": [float(x) for x in fb.alpha], "weight": [float(x) for x in fb.weight],
           "D_colmajor": [float(x) for x in D.reshape(-1, order="F")],
           "J_colmajor": [float(x) for x in J.reshape(-1, order="F")],
           "K_colmajor": [float(x) for x in K.reshape(-1, order="F")]}
    dst = Path(__file__).with_name("c1_reduced_jk.json")
    dst.write_text(json.dumps(out))
    print("wrote", dst, "nfun", fb.nfun)


if __name__ == "__main__":
    main()
