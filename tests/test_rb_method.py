"""The reduced-basis guesses of the batched engine (BatchOptions.rb_samples),
checked as a method on the CPU with the oracle's systems: on the 8x4x20
slab guide, the Galerkin solutions on the orthonormalised direct solutions
at 16 evenly spaced sample frequencies (of 48 over 8-12 GHz) meet a
relative residual far below the batched tolerance (1e-8) at every
frequency, and four of those samples leave residuals far above it.  No
GPU: the engine's
own form is compared with its from-zero sweep and the oracle in
test_rb_sweep.py."""
import math

import numpy as np
import scipy.sparse.linalg as spla

import edgefem_oracle as O
from edgefem_gb300.mesh import waveguide_mesh

A_WR90 = 0.02286


def _sweep():
    m = waveguide_mesh(8, 4, 20, A_WR90, 10.16e-3, 50e-3, slab=(20e-3, 30e-3))
    prob = O.make_problem(m)
    ports = O.waveguide_ports(prob, A_WR90, 10e9)
    eps = O.tet_eps(prob, 2 * math.pi * 10e9, eps_regions={101: 2.2 * (1 - 0.001j)})
    return O.EigenmodeSweep(prob, ports, eps)


def _worst_residual(sw, freqs, basis):
    worst = 0.0
    for f in freqs:
        s = sw.system(2 * math.pi * f)
        Y = np.linalg.solve(basis.T @ (s.A @ basis), basis.T @ s.B)
        R = s.B - s.A @ (basis @ Y)
        worst = max(worst, max(np.linalg.norm(R[:, k]) / np.linalg.norm(s.B[:, k]) for k in range(s.B.shape[1])))
    return worst


def test_galerkin_guesses_from_sixteen_samples():
    sw = _sweep()
    freqs = np.linspace(8e9, 12e9, 48)
    # the engine's sample rule: round(i (F - 1) / (n - 1)), half away from zero
    samples = sorted(set(int(math.floor(i * 47 / 15 + 0.5)) for i in range(16)))
    assert len(samples) == 16 and samples[0] == 0 and samples[-1] == 47
    V = np.column_stack([spla.splu(sw.system(2 * math.pi * freqs[i]).A.tocsc()).solve(
        sw.system(2 * math.pi * freqs[i]).B) for i in samples])
    Q, _ = np.linalg.qr(V)
    assert _worst_residual(sw, freqs, Q) < 1e-9
    # four samples leave residuals the Krylov phase has to remove
    Q4, _ = np.linalg.qr(V[:, [0, 1, 10, 11, 20, 21, 30, 31]])
    assert _worst_residual(sw, freqs, Q4) > 1e-6
