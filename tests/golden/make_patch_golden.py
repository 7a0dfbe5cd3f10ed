"""Oracle S11 of the coarse patch-antenna problem (committed fixture).

    python tests/golden/make_patch_golden.py

Runs the CPU oracle (direct solve, complex128) on the probe-fed patch mesh
at h_fine = 5 mm, h_coarse = 15 mm with Debye FR-4, the jk0 absorbing box
and a 50-ohm lumped port whose weights are normalised once at 2.5 GHz (as
the stacked-patch design does, stacked_patch.py:691-694), at 2.2, 2.5 and
2.8 GHz, and writes patch_antenna_S.json.  The GPU test compares the batched sweep with it, so
no direct solve runs at test time.
"""
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import edgefem_oracle as O  # noqa: E402
from edgefem_gb300.mesh import patch_antenna_mesh  # noqa: E402

FREQS = [2.2e9, 2.5e9, 2.8e9]
F_NORM = 2.5e9
DEBYE = (4.488, 4.312, 1.0 / (2 * math.pi * 2.5e9))
MESH = dict(h_fine=5e-3, h_coarse=15e-3)


def main():
    m = patch_antenna_mesh(**MESH)
    prob = O.make_problem(m)
    prob.pec = np.union1d(prob.pec, O.build_edge_pec(prob.topo.tri_edges, m.tri_phys, 10))
    port = O.build_lumped_port(prob, 20, (0.0, 0.0, 1.0), 50.0)
    w_mid = 2 * math.pi * F_NORM
    eps_mid = O.tet_eps(prob, w_mid, eps_models={101: O.debye_eps(*DEBYE)})
    port = O.normalize_port_weights(prob, w_mid, eps_mid, [port], use_abc=True, abc_tags=(50,))[0]
    out = {"mesh": MESH, "debye": DEBYE, "freqs": FREQS, "f_norm": F_NORM, "S11": []}
    for f in FREQS:
        w = 2 * math.pi * f
        eps = O.tet_eps(prob, w, eps_models={101: O.debye_eps(*DEBYE)})
        S = O.calculate_sparams(prob, w, eps, [port], use_abc=True, abc_tags=(50,))
        out["S11"].append([float(S[0, 0].real), float(S[0, 0].imag)])
        print(f, S[0, 0], flush=True)
    with open(os.path.join(HERE, "patch_antenna_S.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
