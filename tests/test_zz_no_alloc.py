"""Allocation-free Jacobi-COCG entry point (efg_solve_linear_device_noalloc)
against the allocating efg_solve_linear run with the same (Jacobi)
preconditioner on the same complex-symmetric system.  The file name keeps
it last in collection order, so the GPU test also runs after every other
test has used the device."""
import ctypes as C
import math

import numpy as np
import pytest

import edgefem_gb300 as em
from edgefem_gb300 import _lib

MAX_ROWS = 131072  # EFG_NOALLOC_MAX_ROWS in include/edgefem_gb300.h

_fn = _lib.lib.efg_solve_linear_device_noalloc
_fn.restype = C.c_int
_fn.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int32,
                C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_int32)]


def _call(n, rp, ci, v, b, x, tol, maxit, stream=None):
    it, rs, cv = C.c_int32(-1), C.c_double(-1.0), C.c_int32(-1)
    rc = _fn(n, rp, ci, v, b, x, tol, maxit, stream, C.byref(it), C.byref(rs), C.byref(cv))
    return rc, it.value, rs.value, cv.value


def test_noalloc_rejects_oversize_and_bad_arguments():
    # Checked before any CUDA call: runs without a GPU.
    rc, *_ = _call(MAX_ROWS + 1, None, None, None, None, None, 1e-10, 100)
    assert rc == -1
    msg = _lib.lib.efg_last_error().decode()
    assert "exceeds the fixed scratch capacity" in msg and str(MAX_ROWS) in msg
    assert _call(16, None, None, None, None, None, 1e-10, 100)[0] == -1
    assert "null array pointer" in _lib.lib.efg_last_error().decode()
    assert _call(16, None, None, None, None, None, 0.0, 100)[0] == -1
    assert _call(16, None, None, None, None, None, 1e-10, 0)[0] == -1
    # n = 0 is an empty, converged solve.
    assert _call(0, None, None, None, None, None, 1e-10, 100) == (0, 0, 0.0, 1)


@pytest.mark.gpu
def test_noalloc_matches_solve_linear(gpu, wr90_mesh):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch has no CUDA device")
    M = em.Mesh.from_arrays(wr90_mesh)
    bc = em.build_edge_pec(M, 1)
    p = em.MaxwellParams()
    p.omega = 2 * math.pi * 10e9
    p.eps_r = 1 - 0.05j
    asm = gpu.assemble_maxwell(M, p, bc, [], -1)
    n = asm.A.n
    assert n <= MAX_ROWS
    rp, ci, v = asm.A.csr()
    rng = np.random.default_rng(7)
    b = rng.normal(size=n) + 1j * rng.normal(size=n)
    b[bc.pec_array()] = 0
    tol, maxit = 1e-10, 100000
    # the entry point is the Jacobi form: compare with solve_linear's Jacobi
    # preconditioner (use_ilut=False), not its default auxiliary space
    ref = gpu.solve_linear(asm.A, b, em.SolveOptions(use_bicgstab=False, tolerance=tol, max_iterations=maxit,
                                                     use_ilut=False))
    assert ref.converged and "Jacobi" in ref.method and "Block" not in ref.method

    # The caller owns every device array.
    dev = torch.device("cuda:0")
    d_rp = torch.from_numpy(np.ascontiguousarray(rp, np.int32)).to(dev)
    d_ci = torch.from_numpy(np.ascontiguousarray(ci, np.int32)).to(dev)
    d_v = torch.from_numpy(np.ascontiguousarray(v, np.complex128).view(np.float64)).to(dev)
    d_b = torch.from_numpy(np.ascontiguousarray(b, np.complex128).view(np.float64)).to(dev)
    torch.cuda.synchronize()
    scale = np.linalg.norm(ref.x)
    for call in range(2):  # two calls in a row on the same scratch
        d_x = torch.full((2 * n,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc, iters, res, conv = _call(n, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_b.data_ptr(),
                                     d_x.data_ptr(), tol, maxit)
        assert rc == 0, _lib.lib.efg_last_error().decode()
        assert conv == 1 and 0 < iters <= maxit and res <= tol
        x = d_x.cpu().numpy().view(np.complex128)
        assert np.all(np.isfinite(x))
        assert np.linalg.norm(x - ref.x) <= 1e-8 * scale, f"call {call}"
        # Same algorithm; FP64 atomic reduction order differs run to run, so
        # the iteration counts agree only closely.
        assert abs(iters - ref.iters) <= 0.1 * ref.iters
        if call == 0:
            # after one call, a further call takes no device memory
            torch.cuda.synchronize()
            free0, _ = torch.cuda.mem_get_info()

    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device memory changed by {free0 - free1} bytes across a call"

    # a caller-owned stream, with the inputs written on that same stream
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        d_b2 = d_b * 1.0
        d_x2 = torch.full((2 * n,), float("nan"), dtype=torch.float64, device=dev)
    rc, iters, res, conv = _call(n, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_b2.data_ptr(),
                                 d_x2.data_ptr(), tol, maxit, C.c_void_p(side.cuda_stream))
    assert rc == 0 and conv == 1, _lib.lib.efg_last_error().decode()
    side.synchronize()
    x = d_x2.cpu().numpy().view(np.complex128)
    assert np.linalg.norm(x - ref.x) <= 1e-8 * scale


@pytest.mark.gpu
def test_noalloc_rejects_missing_diagonal(gpu):
    """A CSR row without its diagonal entry is an error, not a silent
    fallback (the allocating solve rejects it too)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch has no CUDA device")
    dev = torch.device("cuda:0")
    n = 4
    rp = np.array([0, 1, 2, 3, 4], np.int32)
    ci = np.array([0, 1, 3, 3], np.int32)  # row 2 stores column 3 only
    v = np.array([2.0, 2.0, 1.0, 2.0], np.complex128)
    d = [torch.from_numpy(a).to(dev) for a in (rp, ci, v.view(np.float64), np.ones(n, np.complex128).view(np.float64))]
    d_x = torch.zeros(2 * n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc, *_ = _call(n, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(), d_x.data_ptr(), 1e-10, 100)
    assert rc == -1
    assert "row 2 has no diagonal entry" in _lib.lib.efg_last_error().decode()
