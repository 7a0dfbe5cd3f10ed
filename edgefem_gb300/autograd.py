"""|S_ji|^2 as a differentiable function of the per-tetrahedron permittivity.

`SParamPower` is a `torch.autograd.Function` whose forward runs the GPU
eigenmode solve (the semantics of calculate_sparams_eigenmode,
src/assemble_maxwell.cpp:637-787) or, with `driven=True`, the driven-port
solve (calculate_sparams, src/assemble_maxwell.cpp:352-394: lumped or wave
ports with real weights, ABC, Debye media), and whose backward returns the
hand-written adjoint sensitivity d|S_ji|^2 / d eps_r(tet) computed in the
same call (efg_sparams_eigenmode_adjoint / efg_sparams_driven_adjoint: the
adjoint vector of a port is its scaled forward solution because A is
complex symmetric, a per-tetrahedron contraction kernel and, for eigenmode
ports, the propagation-constant terms).  The reference has no sensitivity code; this
is the inverse-design entry point layered on its forward model.

The variable is the real part of eps_r per tetrahedron; a fixed imaginary
part (loss) may be given.  PyTorch is only the autograd front end: the
forward and the gradient come from the CUDA library, never from torch ops.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np
import torch

from . import sdk


class SParamPower(torch.autograd.Function):
    """y = |S_ji(eps)|^2 for eps = eps_real (+ 1j * eps_imag) per tetrahedron."""

    @staticmethod
    def forward(ctx, eps_real: torch.Tensor, mesh: "sdk.Mesh", params: "sdk.MaxwellParams", bc: "sdk.BC",
                ports: Sequence["sdk.WavePort"], out_j: int, in_i: int,
                eps_imag: Optional[np.ndarray], opts: Optional["sdk.SolveOptions"], driven: bool = False):
        if eps_real.dim() != 1 or eps_real.numel() != mesh.num_tets:
            raise ValueError(f"eps_real must be a vector of {mesh.num_tets} per-tetrahedron values")
        er = eps_real.detach().to("cpu", torch.float64).numpy()
        eps = er.astype(np.complex128)
        if eps_imag is not None:
            eps = eps + 1j * np.asarray(eps_imag, np.float64)
        saved = params.eps_r_tet
        params.eps_r_tet = eps
        try:
            adjoint = sdk.sparams_driven_adjoint if driven else sdk.sparams_eigenmode_adjoint
            grad, S = adjoint(mesh, params, bc, ports, out_j, in_i, opts)
        finally:
            params.eps_r_tet = saved
        ctx.save_for_backward(torch.from_numpy(grad).to(eps_real.device, eps_real.dtype))
        ctx.S = S
        return eps_real.new_tensor(float(abs(S[out_j, in_i]) ** 2))

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return (grad_out * g,) + (None,) * 9


def sparam_power(eps_real: torch.Tensor, mesh, params, bc, ports, out_j: int = 1, in_i: int = 0,
                 eps_imag=None, opts=None, driven: bool = False) -> torch.Tensor:
    """|S_{out_j, in_i}|^2 with gradient d/d eps_real through the adjoint;
    `driven` selects the driven-port formulation (calculate_sparams)."""
    return SParamPower.apply(eps_real, mesh, params, bc, ports, int(out_j), int(in_i), eps_imag, opts,
                             bool(driven))
