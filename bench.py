#!/usr/bin/env python3
"""Benchmark: frequency points/s of the batched eigenmode sweep on one GB300
(one JSON line on stdout).

Workload (default): WR-90 box 22.86 x 10.16 x 50 mm with a centred
dielectric slab (z in [20, 30] mm, eps_r = 2.2 (1 - 0.001j)), 40x20x100 hex
cells split into 6 tets (480,000 tets, 580,560 edges), two TE10 wave ports,
64 frequencies uniform over 8-12 GHz, relative FP64 residual tolerance 1e-8.
A step is one full solve of all 64 frequencies x 2 active ports with the
operator resident in HBM, nothing carried over from the previous step.
Synthetic mesh (no gmsh here).

The batched form measured is the double-float engine (Krylov vectors and
the K/M products in double-float on the FP32 pipes, about 48 bits, every
convergence confirmed on an FP64-accurate true residual) in its default
form: 16 sample frequencies solved first, every column started from the
Galerkin solution on their orthonormalised solutions (--rb-samples 0:
every column from zero; the `batched_cold` object times that form too).
The FP32 Krylov + FP64 refinement form (--precision 0) is the same engine
with complex64 vectors; it needs about eight times the iterations on this
system.

Reported beside it: the plain unbatched FP64 GPU path at 8 band-spanning
frequencies, |dS| of both against the complex128 oracle at the band edges
and at one frequency the sample phase did not solve, the SpMM roofline,
the single-vector SpMVs, the measured CPU baseline (the oracle solved to
convergence on the host's threads), and an end-to-end number through the
public API from host arrays.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os

# Single-threaded BLAS for the NumPy set-up work; the oracle's C solver sets
# its OpenMP thread count explicitly (all host threads).
for _v in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ.setdefault(_v, "1")
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# The headline metric as stated for this path; the batched form measured is
# the double-float engine (FP32-pipe arithmetic at ~48 bits with
# true-residual confirmation), the successor of the FP32 + FP64-refinement
# form (precision 0, still selectable).
METRIC = "freq points/s at |\u0394S|\u22641e-6: batched FP32+FP64-refine vs plain; SpMV GB/s"
C0 = 299792458.0


def workload_spec(name: str):
    if name == "slab":
        return dict(workload="wr90_slab_40x20x100_64f", grid=(40, 20, 100), slab=(20e-3, 30e-3),
                    eps_slab=2.2 * (1 - 0.001j), freqs=np.linspace(8e9, 12e9, 64), tol=1e-8)
    if name == "medium":
        return dict(workload="wr90_slab_24x12x60_64f", grid=(24, 12, 60), slab=(20e-3, 30e-3),
                    eps_slab=2.2 * (1 - 0.001j), freqs=np.linspace(8e9, 12e9, 64), tol=1e-8)
    if name == "small":
        return dict(workload="wr90_8x4x20_16f", grid=(8, 4, 20), slab=None, eps_slab=None,
                    freqs=np.linspace(8e9, 12e9, 16), tol=1e-8)
    if name in ("uneven", "uneven_small"):
        # 32 (or 4) WR-90 guides of seeded lengths 30-80 mm and grids between
        # 20x10x40 and 48x24x120 cells, per-tet eps_r ~ U[1, 4] (1 - 0.002j),
        # 16 frequencies over 8-12 GHz, one batch.
        return dict(workload="wr90_uneven_32x16f" if name == "uneven" else "wr90_uneven_4x16f",
                    kind="multi", n_inst=32 if name == "uneven" else 4, seed=2024,
                    freqs=np.linspace(8e9, 12e9, 16), tol=1e-8, eps_slab=None)
    if name in ("patch", "patch_small"):
        # Probe-fed patch on Debye FR-4 (4.4(1 - 0.02j) at 2.5 GHz) in an
        # absorbing air box, 50-ohm lumped port, 101 frequencies over 2-3 GHz.
        mesh_kw = {} if name == "patch" else dict(h_fine=2e-3, h_coarse=8e-3)
        return dict(workload="patch_fr4_debye_abc_101f" if name == "patch" else "patch_fr4_debye_abc_101f_coarse",
                    kind="driven", mesh_kw=mesh_kw, debye=(4.488, 4.312, 1.0 / (2 * math.pi * 2.5e9)),
                    freqs=np.linspace(2e9, 3e9, 101), tol=1e-8, eps_slab=None)
    raise SystemExit(f"unknown workload {name}")


def _mesh_module():
    """edgefem_gb300/mesh.py loaded by path: pure numpy, so the CPU reference
    arm builds its meshes without loading the CUDA library."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_efg_mesh", os.path.join(ROOT, "edgefem_gb300", "mesh.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def build_problem(spec):
    em = _mesh_module()
    if spec.get("kind") == "multi":
        rng = np.random.default_rng(spec["seed"])
        out = []
        for _ in range(spec["n_inst"]):
            t = rng.uniform()
            grid = (int(round(20 + 28 * t)), int(round(10 + 14 * t)), int(round(40 + 80 * t)))
            L = rng.uniform(30e-3, 80e-3)
            m = em.waveguide_mesh(*grid, 22.86e-3, 10.16e-3, L)
            m.eps_tet = rng.uniform(1.0, 4.0, m.num_tets) * (1 - 0.002j)
            out.append(m)
        return out
    if spec.get("kind") == "driven":
        return em.patch_antenna_mesh(**spec["mesh_kw"])
    a, b, L = 22.86e-3, 10.16e-3, 50e-3
    arrays = em.waveguide_mesh(*spec["grid"], a, b, L, slab=spec["slab"])
    return arrays


def setup_instance(arrays, spec):
    import edgefem_gb300 as em
    if spec.get("kind") == "driven":
        mesh = em.Mesh.from_arrays(arrays)
        bc = em.build_edge_pec(mesh, 1)
        bc.dirichlet_edges |= em.build_edge_pec(mesh, 10).dirichlet_edges
        ports = [em.build_lumped_port(mesh, 20, 50.0, (0.0, 0.0, 1.0))]
        p = em.MaxwellParams()
        p.set_debye_region(101, *spec["debye"])
        p.use_abc = True
        p.abc_surface_tags = {50}
        # port weights normalised once at mid-band (stacked_patch.py:691-694)
        p.omega = 2 * math.pi * float(np.median(spec["freqs"]))
        ports = em.normalize_port_weights(mesh, p, bc, ports,
                                          em.SolveOptions(use_bicgstab=False, tolerance=1e-10, max_iterations=400000))
        return em.BatchInstance(mesh, p, bc, ports)
    a = 22.86e-3
    mesh = em.Mesh.from_arrays(arrays)
    bc = em.build_edge_pec(mesh, 1)
    mode = em.solve_te10_mode(em.RectWaveguidePort(a, 10.16e-3), float(spec["freqs"][0]))
    kc_sq = (math.pi / a) ** 2
    ports = [em.build_wave_port_2d(mesh, t, mode, bc.dirichlet_edges, kc_sq) for t in (2, 3)]
    p = em.MaxwellParams()
    if spec["eps_slab"] is not None:
        p.set_eps_r_region(101, spec["eps_slab"])
    if getattr(arrays, "eps_tet", None) is not None:
        p.eps_r_tet = arrays.eps_tet
    return em.BatchInstance(mesh, p, bc, ports)


def setup_instances(problem, spec):
    return [setup_instance(a, spec) for a in (problem if isinstance(problem, list) else [problem])]


def representative(problem):
    """Index of the median-size instance (the plain and CPU baselines' case)."""
    if not isinstance(problem, list):
        return 0
    sizes = [m.num_tets for m in problem]
    return int(np.argsort(sizes)[len(sizes) // 2])


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum, one ncu capture
# of two full-width launches, mean) of the batched SpMM on the named
# workload, precision and column width; None where no capture exists.
MEASURED_SPMM_TRAFFIC = {("wr90_slab_40x20x100_64f", 2, 128): 4.323e9,
                         ("wr90_slab_40x20x100_64f", 2, 32): 1.0054e9}


def spmm_bytes(rows: int, nnz: int, rhs: int, precision: int = 2) -> int:
    """Algorithmic bytes of one batched SpMM launch: per nonzero the column
    index, K and M high words (16 B) and, in double-float, their low words
    (16 B); row pointer and side-row index once per row; the p gather counted
    once per right-hand side and the q write (8 B complex64, 16 B complex
    double-float)."""
    vec = 8 if precision == 0 else 16
    per_nz = 16 if precision == 0 else 32
    return nnz * per_nz + (rows + 1) * 4 + rows * 4 + 2 * rows * rhs * vec


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum, one
# ncu capture, mean over its launches) of the single-right-hand-side SpMVs
# on the named workload; None where no capture exists.  The 40x20x100 entry
# is the 24x12x60 capture (25.84 MB per launch against 26.86 MB algorithmic)
# scaled to the larger operator by the algorithmic bytes.
MEASURED_SPMV_TRAFFIC = {("wr90_slab_40x20x100_64f", "efgk_spmv32"): 1.186e8,
                         ("wr90_slab_24x12x60_64f", "efgk_spmv32"): 2.584e7}


def spmv_measure(em, inst, freq, peak, workload, launches=20):
    """Plain single-right-hand-side CSR SpMVs on the workload's assembled
    A(omega) at one frequency, through the kernel C-ABI on torch-owned
    device arrays: the complex64 product with FP32 accumulation
    (efgk_spmv32, the FP32 Krylov form) and the complex128 product
    (efgk_spmv64, the plain FP64 form).  Each launch is timed alone with
    CUDA events on the launching stream, after a 512 MB write that flushes
    L2 and a 256 MB read that leaves it clean (no write-backs inside the
    timed launch).  Algorithmic bytes per launch: nnz (s_v + 4) + (n + 1) 4 + 2 n s_x
    (values and column indices streamed once, x gathered once, y written),
    s_v = s_x = 8 (complex64) or 16 (complex128)."""
    import ctypes as C

    import scipy.sparse as sp
    import torch
    from edgefem_gb300 import _lib
    p = inst.params
    p.omega = 2 * math.pi * float(freq)
    asm = em.assemble_maxwell(inst.mesh, p, inst.bc, [], -1)
    rp, ci, v = asm.A.csr()
    n, nnz = asm.A.n, int(ci.size)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream()
    d_rp = torch.from_numpy(np.ascontiguousarray(rp, np.int32)).to(dev)
    d_ci = torch.from_numpy(np.ascontiguousarray(ci, np.int32)).to(dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    flush_view = flush[: 256 << 20]
    rng = np.random.default_rng(5)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    y_ref = sp.csr_matrix((v, ci, rp), shape=(n, n)) @ x
    out = {}
    d_status = torch.zeros(1, dtype=torch.int32, device=dev)
    for form, fname, cdt, rdt, sv in (("complex64", "efgk_spmv32", np.complex64, np.float32, 8),
                                      ("complex64_bulk", "efgk_spmv32_bulk", np.complex64, np.float32, 8),
                                      ("complex128", "efgk_spmv64", np.complex128, np.float64, 16)):
        fn = getattr(_lib.lib, fname)
        fn.restype = C.c_int
        bulk = fname.endswith("_bulk")
        fn.argtypes = ([C.c_int32, C.c_int32] + [C.c_void_p] * 7) if bulk else ([C.c_int32] + [C.c_void_p] * 6)
        d_v = torch.from_numpy(np.ascontiguousarray(v.astype(cdt)).view(rdt)).to(dev)
        d_x = torch.from_numpy(np.ascontiguousarray(x.astype(cdt)).view(rdt)).to(dev)
        d_y = torch.empty(2 * n, dtype=d_v.dtype, device=dev)
        ptrs = (d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_x.data_ptr(), d_y.data_ptr())

        def call():
            if bulk:
                rc = fn(n, nnz, *ptrs, d_status.data_ptr(), stream.cuda_stream)
            else:
                rc = fn(n, *ptrs, stream.cuda_stream)
            if rc != 0:
                raise RuntimeError(f"{fname} failed with CUDA error {rc}")

        for _ in range(3):
            call()
        evs = []
        for i in range(launches):
            # Write 512 MB (evicts the operands), then read 256 MB so the
            # dirty lines of that write are written back before the launch.
            flush.fill_(i & 0xFF)
            flush_view.max()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            call()
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
        nbytes = nnz * (sv + 4) + (n + 1) * 4 + 2 * n * sv
        y = d_y.cpu().numpy().view(cdt).astype(np.complex128)
        achieved = nbytes / (ms / 1e3) / 1e9
        if bulk and int(d_status.item()) != 0:
            raise RuntimeError(f"{fname}: a bulk copy never completed")
        out[form] = {"kernel": fname.replace("efgk_", "") + "_kernel", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "bytes_per_launch": nbytes, "avg_launch_ms": ms,
                     "launches": launches, "l2": "flushed before every launch (512 MB write, then a 256 MB read)",
                     "traffic": MEASURED_SPMV_TRAFFIC.get((workload, fname)),
                     "max_abs_err_over_max_y": float(np.abs(y - y_ref).max() / np.abs(y_ref).max())}
    # The complex64 product on its sliced-ELLPACK copy (built once on the
    # device from the same CSR arrays); GB/s on the CSR algorithmic bytes, so
    # that its padding counts against it.
    plan, fill, sell = _lib.lib.efgk_sell32_plan, _lib.lib.efgk_sell32_fill, _lib.lib.efgk_spmv32_sell
    plan.restype = fill.restype = sell.restype = C.c_int
    plan.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64), C.c_void_p]
    fill.argtypes = [C.c_int32] + [C.c_void_p] * 8
    sell.argtypes = [C.c_int32] + [C.c_void_p] * 7
    ns = (n + 31) // 32
    d_perm = torch.empty(n, dtype=torch.int32, device=dev)
    d_sp = torch.empty(ns + 1, dtype=torch.int64, device=dev)
    ent = C.c_int64()
    if plan(n, d_rp.data_ptr(), d_perm.data_ptr(), d_sp.data_ptr(), C.byref(ent), stream.cuda_stream) != 0:
        raise RuntimeError("efgk_sell32_plan failed")
    d_sc = torch.empty(ent.value, dtype=torch.int32, device=dev)
    d_sv = torch.empty(2 * ent.value, dtype=torch.float32, device=dev)
    d_v = torch.from_numpy(np.ascontiguousarray(v.astype(np.complex64)).view(np.float32)).to(dev)
    d_x = torch.from_numpy(np.ascontiguousarray(x.astype(np.complex64)).view(np.float32)).to(dev)
    d_y = torch.empty(2 * n, dtype=torch.float32, device=dev)
    if fill(n, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_perm.data_ptr(), d_sp.data_ptr(),
            d_sc.data_ptr(), d_sv.data_ptr(), stream.cuda_stream) != 0:
        raise RuntimeError("efgk_sell32_fill failed")

    def call_sell():
        if sell(n, d_perm.data_ptr(), d_sp.data_ptr(), d_sc.data_ptr(), d_sv.data_ptr(), d_x.data_ptr(),
                d_y.data_ptr(), stream.cuda_stream) != 0:
            raise RuntimeError("efgk_spmv32_sell failed")

    for _ in range(3):
        call_sell()
    evs = []
    for i in range(launches):
        flush.fill_(i & 0xFF)
        flush_view.max()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call_sell()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    nbytes = nnz * 12 + (n + 1) * 4 + 2 * n * 8
    fmt_bytes = ent.value * 12 + n * 4 + (ns + 1) * 8 + 2 * n * 8
    y = d_y.cpu().numpy().view(np.complex64).astype(np.complex128)
    achieved = nbytes / (ms / 1e3) / 1e9
    out["complex64_sell"] = {"kernel": "spmv_sell_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "bytes_per_launch": nbytes, "format_bytes_per_launch": fmt_bytes,
                             "padded_entries": int(ent.value), "avg_launch_ms": ms, "launches": launches,
                             "l2": "flushed before every launch (512 MB write, then a 256 MB read)",
                             "traffic": MEASURED_SPMV_TRAFFIC.get((workload, "efgk_spmv32_sell")),
                             "max_abs_err_over_max_y": float(np.abs(y - y_ref).max() / np.abs(y_ref).max())}
    out["rows"], out["nnz"], out["frequency_hz"] = n, nnz, float(freq)
    out["note"] = ("complex64: the row-pipelined kernel (8 lanes per row, next row's entries in flight); "
                   "complex64_bulk: the matrix streamed through shared memory by bulk asynchronous copies "
                   "(slower: two stages per CTA at a third of the occupancy); complex64_sell: the same product "
                   "on a sliced-ELLPACK copy (32-row slices, rows sorted by length in windows of 1024), GB/s "
                   "on the CSR algorithmic bytes; the complex128 product does 8 FP64 flops per stored entry, "
                   "which GB300's FP64 pipe cannot feed at HBM rate")
    del flush
    return out


def solve_linear_report(em, inst, freq, tol):
    """solve_linear on the workload's assembled operator (assemble_maxwell at
    `freq` with the first port driven, as the reference's design classes
    call it before solve_linear): FP64 COCG iterations and Krylov device
    time with each preconditioner solve_linear can choose - the auxiliary
    space (the matrix from assemble_maxwell carries its mesh data),
    block-Jacobi (the same values as a raw CSR matrix) and Jacobi
    (use_ilut=False)."""
    p = inst.params
    p.omega = 2 * math.pi * float(freq)
    asm = em.assemble_maxwell(inst.mesh, p, inst.bc, inst.ports, 0)
    rp, ci, v = asm.A.csr()
    raw = em.sdk.SpMatC.from_csr(rp, ci, v, asm.A.n)
    out = {"frequency_hz": float(freq), "rows": int(asm.A.n), "tolerance": tol}
    for name, A_, opts in (("aux", asm.A, em.SolveOptions(use_bicgstab=False, tolerance=tol, max_iterations=400000)),
                           ("block_jacobi", raw, em.SolveOptions(use_bicgstab=False, tolerance=tol,
                                                                 max_iterations=400000)),
                           ("jacobi", raw, em.SolveOptions(use_bicgstab=False, tolerance=tol, max_iterations=400000,
                                                           use_ilut=False))):
        em.sdk.krylov_totals(reset=True)
        res = em.solve_linear(A_, asm.b, opts)
        kt = em.sdk.krylov_totals(reset=True)
        out[name] = {"method": res.method, "iterations": res.iters, "converged": res.converged,
                     "device_s": kt["device_ms"] / 1e3}
    return out


def edge_build_measure(em, arrays, reps=3):
    """Mesh ingest on the GPU for the workload's mesh: the global edge
    numbering (build_edges) beside the host mesh construction that contains
    the host numbering (node map, elements, build_edges, quality check), and
    validate_mesh beside the host's; best of `reps`, and whether the GPU
    results are identical to the host's."""
    host_s, dev_ms, call_s = [], [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        M = em.Mesh.from_arrays(arrays)
        host_s.append(time.perf_counter() - t0)
    host = M.topology()
    for _ in range(reps):
        tm = {}
        t0 = time.perf_counter()
        dev = em.build_edges_gpu(arrays, tm)
        call_s.append(time.perf_counter() - t0)
        dev_ms.append(tm["device_ms"])
    q_host_s, q_dev_ms = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        qh = em.validate_mesh(M)
        q_host_s.append(time.perf_counter() - t0)
        tm = {}
        qd = em.validate_mesh_gpu(M, tm)
        q_dev_ms.append(tm["device_ms"])
    return {"tets": int(len(arrays.tets)), "tris": int(len(arrays.tris)), "edges": int(len(host[0])),
            "gpu_device_ms": min(dev_ms), "gpu_call_ms": 1e3 * min(call_s),
            "host_mesh_from_arrays_ms": 1e3 * min(host_s),
            "identical_to_host": bool(all(np.array_equal(h, d) for h, d in zip(host, dev))),
            "validate_mesh": {"gpu_device_ms": min(q_dev_ms), "host_ms": 1e3 * min(q_host_s),
                              "identical_to_host": bool((qh.num_degenerate_tets, qh.num_inverted_tets, qh.min_volume,
                                                         qh.max_aspect_ratio) ==
                                                        (qd.num_degenerate_tets, qd.num_inverted_tets, qd.min_volume,
                                                         qd.max_aspect_ratio))}}


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import edgefem_oracle as O
    return O


def host_threads() -> int:
    return len(os.sched_getaffinity(0))


class OracleSweep:
    """The workload's systems on the CPU oracle (complex128): one K/M
    assembly, A(f) per frequency (oracle.EigenmodeSweep), solved to
    convergence by the oracle's C COCG with the Jacobi + nodal gradient +
    vector-nodal preconditioner (oracle/krylov_c.c) on `threads` host
    threads.  Eigenmode workloads (wave ports) only."""

    def __init__(self, arrays, spec):
        O = _oracle()
        self.O, self.spec = O, spec
        t0 = time.perf_counter()
        self.prob = O.make_problem(arrays)
        f0 = float(spec["freqs"][0])
        ports = O.waveguide_ports(self.prob, 22.86e-3, f0)
        eps_slab = spec.get("eps_slab")
        eps = O.tet_eps(self.prob, 2 * math.pi * f0, eps_regions={101: eps_slab} if eps_slab is not None else None,
                        eps_tet=getattr(arrays, "eps_tet", None))
        self.sweep = O.EigenmodeSweep(self.prob, ports, eps)
        self.inc = O.aux_incidence(self.prob)
        self.setup_s = time.perf_counter() - t0

    def solve_point(self, f, tol, tol1=0.0, threads=0, maxit=10 ** 6):
        """S at frequency f (all ports active in turn) with the per-port solve
        records: iterations and seconds to tol (and to tol1 if given)."""
        t0 = time.perf_counter()
        sys_ = self.sweep.system(2 * math.pi * float(f))
        form_s = time.perf_counter() - t0
        X, recs = [], []
        for k in range(sys_.B.shape[1]):
            r = self.O.cocg_aux_c(self.prob, sys_.A, sys_.B[:, k], tol=tol, tol1=tol1, threads=threads,
                                  inc=self.inc, maxit=maxit)
            X.append(r.pop("x"))
            recs.append(r)
        S = self.O.sparams_from_solution(sys_, np.column_stack(X))
        return S, recs, form_s


def band_indices(F: int, k: int = 8):
    """k frequency indices spread over the band, both ends included."""
    return sorted(set(int(round(v)) for v in np.linspace(0, F - 1, min(k, F))))


def rb_sample_indices(F: int, rb_samples: int, P: int):
    """Frequency indices the batched engine solves first when its
    reduced-basis phase is on (the engine's own rule: min(rb_samples, 64 / P)
    evenly spaced indices, rounded half away from zero, when that is at
    least 2 and F is at least twice it); empty when the phase is off."""
    n = min(rb_samples, 64 // P)
    if n < 2 or F < 2 * n:
        return []
    return sorted(set(int(math.floor(i * (F - 1) / (n - 1) + 0.5)) for i in range(n)))


def oracle_check(arrays, spec, S_batched, plain_rows, tight=1e-12, extra_idx=(), samples=()):
    """Parity of the GPU results at the band edges (and at extra_idx, a
    frequency the reduced-basis phase did not sample) against the complex128
    oracle solved to |r|/|b| < tight, and the measured CPU baseline: the
    same oracle solves timed to the workload's tolerance on all host threads
    (iterations and seconds to that tolerance are recorded during the tight
    solve, set-up of the preconditioner included)."""
    freqs = spec["freqs"]
    threads = host_threads()
    osw = OracleSweep(arrays, spec)
    idx = [0, len(freqs) - 1] + [int(i) for i in extra_idx]
    plain_by_idx = {r["index"]: r for r in plain_rows}
    checks, sec_pts, it_pts = [], [], []
    for fi in idx:
        S_o, recs, form_s = osw.solve_point(freqs[fi], tight, tol1=spec["tol"], threads=threads)
        row = {"freq_hz": float(freqs[fi]), "rb_sample": fi in samples,
               "dS_batched": float(np.abs(S_batched[fi] - S_o).max()),
               "oracle_iterations_to_tol": [r["iterations_tol1"] for r in recs],
               "oracle_iterations_to_tight": [r["iterations"] for r in recs],
               "oracle_relres": [r["relres"] for r in recs]}
        if fi in plain_by_idx:
            row["dS_plain"] = float(np.abs(plain_by_idx[fi]["S"] - S_o).max())
        row["S_oracle"] = [[S_o[i, j].real, S_o[i, j].imag] for i in range(S_o.shape[0]) for j in range(S_o.shape[1])]
        checks.append(row)
        sec_pts.append(form_s + sum(r["seconds_tol1"] for r in recs))
        it_pts.append(sum(r["iterations_tol1"] for r in recs))
    dS_b = max(c["dS_batched"] for c in checks)
    dS_p = max((c["dS_plain"] for c in checks if "dS_plain" in c), default=None)
    cpu = {"value": len(idx) / float(np.sum(sec_pts)), "unit": "freq points/s", "cores": threads, "kind": "port",
           "sample": f"{len(idx)} frequency points ({', '.join(f'{freqs[i]/1e9:.2f}' for i in idx)} GHz, both ports) "
                     f"of the full {osw.prob.n}-edge system solved to |r|/|b| < {spec['tol']:g} by the oracle's "
                     f"complex128 COCG with the Jacobi + nodal gradient + vector-nodal preconditioner (C, OpenMP, "
                     f"{threads} threads): {it_pts} iterations per point, {[round(s, 2) for s in sec_pts]} s per "
                     f"point (A(f) formed from K and M, preconditioner set-up and solves), measured to convergence",
           "seconds_per_point": sec_pts, "iterations_per_point": it_pts}
    return {"tolerance": tight, "points": checks, "dS_batched_max": dS_b, "dS_plain_max": dS_p,
            "oracle_setup_s": osw.setup_s}, cpu


def reference_arm(args, spec):
    """CPU implementation of the path on the host: the reference's Eigen
    solver does not build here (Eigen headers absent), so the oracle's
    restatement runs instead - per step one frequency point of the workload
    (A(f) formed from the K/M split, both ports) solved to the workload's
    tolerance by complex128 COCG with the Jacobi + nodal gradient +
    vector-nodal preconditioner, OpenMP over all host threads.  Steps cycle
    through 8 band-spanning frequencies; every point is solved to
    convergence (nothing extrapolated)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if spec.get("kind") in ("driven", "multi"):
        print(json.dumps({"impl": "reference", "unavailable": "the CPU reference arm covers the single-mesh "
                                                              "eigenmode workloads (slab, medium, small)"}))
        return
    threads = host_threads()
    problem = build_problem(spec)
    osw = OracleSweep(problem, spec)
    freqs = spec["freqs"]
    idx = band_indices(len(freqs))
    times, iters, conv = [], [], True
    for step in range(args.warmup + args.steps):
        fi = idx[(step - args.warmup) % len(idx)]
        t0 = time.perf_counter()
        if step < args.warmup:
            # warm-up: the same set-up and 100 iterations (pages, caches,
            # thread pool); the timed steps solve to convergence
            osw.solve_point(freqs[fi], spec["tol"], threads=threads, maxit=100)
            continue
        _, recs, _ = osw.solve_point(freqs[fi], spec["tol"], threads=threads)
        dt = time.perf_counter() - t0
        conv &= all(r["converged"] for r in recs)
        times.append(dt)
        iters.append(sum(r["iterations"] for r in recs))
    v = len(times) / float(np.sum(times))
    out = {"metric": METRIC, "value": v, "unit": "freq points/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.mean(times)), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
           "config": {"workload": spec["workload"], "rows": int(osw.prob.n), "freqs": len(freqs),
                      "ports": 2, "step": "one frequency point (both ports) solved to convergence",
                      "tolerance": spec["tol"]},
           "impl": "reference",
           "cpu_baseline": {"value": v, "unit": "freq points/s", "cores": threads, "kind": "port",
                            "sample": f"{args.steps} timed frequency points cycling over "
                                      f"{', '.join(f'{freqs[i]/1e9:.2f}' for i in idx)} GHz, each solved to "
                                      f"|r|/|b| < {spec['tol']:g} (both ports; {min(iters)}-{max(iters)} "
                                      f"iterations per point; all converged: {conv}) by the oracle's complex128 "
                                      f"COCG with the Jacobi + nodal gradient + vector-nodal preconditioner in C "
                                      f"on {threads} OpenMP threads (the reference's Eigen BiCGSTAB+ILUT path "
                                      f"is unavailable: Eigen headers absent)"},
           "e2e": {"value": v, "unit": "freq points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def smooth_eps_field(arrays, a, b, L, seed=2024):
    """Per-tet eps_r of the adjoint workload: 1 plus 8 Gaussian bumps
    (centres uniform in the box, amplitudes U[0, 5], sigma 4 mm) at the tet
    centroids, clipped to [1, 6]."""
    lut = arrays.node_index()
    X = arrays.xyz[lut[arrays.tets]].mean(axis=1)
    rng = np.random.default_rng(seed)
    c = rng.uniform([0.0, 0.0, 0.0], [a, b, L], size=(8, 3))
    amp = rng.uniform(0.0, 5.0, 8)
    eps = 1.0 + sum(amp[i] * np.exp(-np.sum((X - c[i]) ** 2, axis=1) / (2 * 4e-3 ** 2)) for i in range(8))
    return np.clip(eps, 1.0, 6.0)


def adjoint_measure(em, steps: int, warmup: int, no_cpu: bool) -> dict:
    """d|S21|^2 / d eps_r of every tet of a WR-90 box (50 mm, 36x16x60 cells,
    207,360 tets) with a smooth seeded eps_r field, at 10 GHz.  Timed: the
    library's adjoint call (assembly, forward and adjoint FP64 solves on the
    GPU, per-tet contraction) per gradient; checked: central differences
    (h = 1e-4) at 20 seeded tets, and (unless --no-cpu) the oracle's
    complex128 adjoint (iterative, relative residual 1e-12), whose time is
    the CPU baseline."""
    a, b, L, f = 22.86e-3, 10.16e-3, 50e-3, 10e9
    arrays = em.waveguide_mesh(36, 16, 60, a, b, L)
    eps = smooth_eps_field(arrays, a, b, L)
    mesh = em.Mesh.from_arrays(arrays)
    bc = em.build_edge_pec(mesh, 1)
    mode = em.solve_te10_mode(em.RectWaveguidePort(a, b), f)
    ports = [em.build_wave_port_2d(mesh, t, mode, bc.dirichlet_edges, (math.pi / a) ** 2) for t in (2, 3)]
    p = em.MaxwellParams()
    p.omega = 2 * math.pi * f
    p.eps_r_tet = eps.astype(np.complex128)
    opts = em.SolveOptions(use_bicgstab=False, max_iterations=400000)  # COCG, default tolerance 1e-10
    for _ in range(warmup):
        em.sparams_eigenmode_adjoint(mesh, p, bc, ports, 1, 0, opts)
    clocks = ClockSampler()
    clocks.start()
    em.sdk.krylov_totals(reset=True)
    t0 = time.perf_counter()
    for _ in range(steps):
        g, S = em.sparams_eigenmode_adjoint(mesh, p, bc, ports, 1, 0, opts)
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    kt = em.sdk.krylov_totals(reset=True)
    # checks at a tight tolerance
    tight = em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=400000)
    g_t, S_t = em.sparams_eigenmode_adjoint(mesh, p, bc, ports, 1, 0, tight)
    rng = np.random.default_rng(7)
    h, fd_err = 1e-4, 0.0
    gmax = float(np.abs(g_t).max())
    for t in rng.choice(arrays.num_tets, 20, replace=False).tolist():
        vals = []
        for s in (1, -1):
            e2 = eps.astype(np.complex128)
            e2[t] += s * h
            p.eps_r_tet = e2
            Sx = em.calculate_sparams_eigenmode(mesh, p, bc, ports, tight)
            vals.append(abs(Sx[1, 0]) ** 2)
        fd = (vals[0] - vals[1]) / (2 * h)
        fd_err = max(fd_err, abs(g_t[t] - fd) / max(abs(fd), 1e-2 * gmax))
    p.eps_r_tet = eps.astype(np.complex128)
    cpu, cpu_err = None, None
    if not no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import edgefem_oracle as O
        prob = O.make_problem(arrays)
        t1 = time.perf_counter()
        threads = host_threads()
        g_o, S_o = O.sparams_eigenmode_adjoint(prob, p.omega, O.waveguide_ports(prob, a, f),
                                               eps.astype(np.complex128), 1, 0, iterative_tol=1e-12,
                                               threads=threads)
        t_cpu = time.perf_counter() - t1
        cpu_err = float(np.abs(g_t - g_o).max() / np.abs(g_o).max())
        cpu = {"value": 1.0 / t_cpu, "unit": "gradients/s", "cores": threads, "kind": "port",
               "sample": f"one complex128 adjoint of the oracle on the full {prob.n}-edge system: its assembly, "
                         f"two COCG solves (Jacobi + nodal gradient + vector-nodal preconditioner in C, "
                         f"{threads} OpenMP threads, relative residual 1e-12; a SuperLU factorisation ran past "
                         f"6 minutes here) and the per-tet contraction"}
    out = {"metric": "adjoint gradients/s: d|S21|^2/d eps_r of every tet at 10 GHz", "value": steps / dt,
           "unit": "gradients/s", "n_gpus": 1, "steps": steps, "warmup": warmup,
           "ms_per_step": dt / steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded smooth eps_r field)",
           "config": {"workload": "wr90_adjoint_36x16x60_smooth_eps", "tets": arrays.num_tets,
                      "edges": mesh.num_edges, "freq_hz": f, "tolerance": opts.tolerance,
                      "timing": "host wall clock around the library call (assembly + 2 solves + contraction)"},
           "krylov": {"iterations_per_gradient": kt["iters"] / max(steps, 1),
                      "solves_per_gradient": kt["solves"] / max(steps, 1)},
           "checks": {"fd_tets": 20, "fd_h": h, "fd_max_rel_err": fd_err, "S21": [S_t[1, 0].real, S_t[1, 0].imag],
                      "cpu_adjoint_max_rel_err": cpu_err},
           "clocks": clk, "cpu_baseline": cpu}
    return out


def adjoint_workload(args):
    import edgefem_gb300 as em
    if em.device_count() < 1:
        raise SystemExit("bench.py needs a CUDA device")
    print(json.dumps(adjoint_measure(em, args.steps, args.warmup, args.no_cpu)))


def correction_fd(em, mesh, q, bc, ports, eps, tets, h, tol=1e-10):
    """Central differences of |S11|^2 (driven port 0) with respect to the
    permittivity of single tets, by correction solves: with x0 the base
    solution and r0 = b - A x0 its residual, A(eps +- h e_t) is
    A +- h dA_t exactly (A is linear in each tet's permittivity, dA_t =
    -k0^2 times the tet's signed mass matrix), so x+- = x0 + d+- with
    A(eps +- h e_t) d+- = r0 -+ h dA_t x0.  The difference of the two
    S11 values is c^T (d+ - d-) / sqrt(Z0): the base solve's error cancels
    and each correction solve is accurate relative to its own small
    right-hand side, so the quotient carries no amplified solver noise.
    Returns [(tet, fd)]."""
    import scipy.sparse as sp
    q.eps_r_tet = eps.copy()
    tight = em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=400000)
    asm = em.assemble_maxwell(mesh, q, bc, ports, 0)
    x0 = em.solve_linear(asm.A, asm.b, tight).x
    rp, ci, v = asm.A.csr()
    A0 = sp.csr_matrix((v, ci, rp), shape=(asm.A.n, asm.A.n))
    r0 = asm.b - A0 @ x0
    arr = mesh.arrays()
    lut = arr.node_index()
    _, te, to, _, _ = mesh.topology()
    pec = np.zeros(asm.A.n, bool)
    pec[bc.pec_array()] = True
    pt = ports[0]
    keep = ~pec[pt.edges]
    c = np.zeros(asm.A.n, np.complex128)
    np.add.at(c, pt.edges[keep], np.conj(pt.weights[keep]))
    vinc = np.sqrt(complex(pt.mode.Z0))
    S0 = (c @ x0 - vinc) / vinc
    k0 = q.omega / C0
    so = em.SolveOptions(use_bicgstab=False, tolerance=tol, max_iterations=400000)
    out = []
    for t in tets:
        _, Ml = em.element_matrices(arr.xyz[lut[arr.tets[t]]])
        sg = to[t].astype(np.float64)
        ed = te[t].astype(np.int64)
        dAx = np.zeros(asm.A.n, np.complex128)
        np.add.at(dAx, ed, -(k0 * k0) * ((sg[:, None] * Ml * sg[None, :]) @ x0[ed]))
        dAx[pec] = 0.0
        d = []
        for sgn in (1.0, -1.0):
            e2 = eps.copy()
            e2[t] += sgn * h
            q.eps_r_tet = e2
            a2 = em.assemble_maxwell(mesh, q, bc, ports, 0)
            d.append(em.solve_linear(a2.A, r0 - sgn * h * dAx, so).x)
        dS = c @ (d[0] - d[1]) / vinc
        Ssum = 2.0 * S0 + c @ (d[0] + d[1]) / vinc
        out.append((int(t), float(np.real(dS * np.conj(Ssum)) / (2 * h))))
    q.eps_r_tet = eps.copy()
    return out


def patch_adjoint_workload(args):
    """d|S11|^2 / d eps_r of every tet of the probe-fed patch (Debye FR-4
    substrate, ABC air box, 50-ohm lumped port normalised at 2.5 GHz) at
    2.5 GHz, reported over the substrate tets.  Timed: the library's driven
    adjoint call (assembly, one forward FP64 solve, per-tet contraction; the
    adjoint vector of the single port is its scaled forward solution) per
    gradient.  Checked, through the same system with the Debye permittivity
    at 2.5 GHz written per tet: central differences (h = 1e-4, correction
    solves) at 20 seeded substrate tets and the three of largest
    sensitivity, and (unless --no-cpu) the oracle's complex128 adjoint
    (its own assembly, forward and adjoint solves by the C COCG)."""
    import edgefem_gb300 as em
    if em.device_count() < 1:
        raise SystemExit("bench.py needs a CUDA device")
    spec = workload_spec("patch")
    arrays = build_problem(spec)
    inst = setup_instance(arrays, spec)
    mesh, bc, ports, p = inst.mesh, inst.bc, inst.ports, inst.params
    f = 2.5e9
    p.omega = 2 * math.pi * f
    opts = em.SolveOptions(use_bicgstab=False, max_iterations=400000)  # COCG, default tolerance 1e-10
    for _ in range(args.warmup):
        em.sparams_driven_adjoint(mesh, p, bc, ports, 0, 0, opts)
    clocks = ClockSampler()
    clocks.start()
    em.sdk.krylov_totals(reset=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        g, S = em.sparams_driven_adjoint(mesh, p, bc, ports, 0, 0, opts)
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    kt = em.sdk.krylov_totals(reset=True)
    sub = np.flatnonzero(np.asarray(arrays.tet_phys) == 101)
    tight = em.SolveOptions(use_bicgstab=False, tolerance=1e-12, max_iterations=400000)
    g_t, S_t = em.sparams_driven_adjoint(mesh, p, bc, ports, 0, 0, tight)
    # The same system with the permittivity per tet (air 1, substrate the
    # Debye value at 2.5 GHz), so single tets can be perturbed.
    eps_s, eps_inf, tau = spec["debye"]
    eps_d = eps_inf + (eps_s - eps_inf) / complex(1.0, p.omega * tau)
    eps = np.ones(arrays.num_tets, np.complex128)
    eps[sub] = eps_d
    q = em.MaxwellParams()
    q.omega, q.use_abc, q.abc_surface_tags, q.eps_r_tet = p.omega, True, {50}, eps
    g_q, _ = em.sparams_driven_adjoint(mesh, q, bc, ports, 0, 0, tight)
    rng = np.random.default_rng(7)
    seeded = rng.choice(sub, 20, replace=False)
    top = sub[np.argsort(-np.abs(g_t[sub]))[:3]]
    h = 1e-4
    t_fd = time.perf_counter()
    fd = correction_fd(em, mesh, q, bc, ports, eps, np.concatenate([seeded, top]), h)
    t_fd = time.perf_counter() - t_fd
    gmax = float(np.abs(g_t[sub]).max())
    rel = [abs(g_t[t] - d) / max(abs(d), 1e-3 * gmax) for t, d in fd]
    cpu, cpu_err = None, None
    if not args.no_cpu:
        O = _oracle()
        t1 = time.perf_counter()
        prob = O.make_problem(arrays)
        prob.pec = np.union1d(prob.pec, O.build_edge_pec(prob.topo.tri_edges, arrays.tri_phys, 10))
        t_setup = time.perf_counter() - t1
        oport = O.WavePort(20, np.asarray(ports[0].edges, np.int64), np.asarray(ports[0].weights, np.complex128),
                           Z0=ports[0].mode.Z0)
        t2 = time.perf_counter()
        g_o, S_o = O.sparams_driven_adjoint(prob, p.omega, eps, [oport], 0, 0, use_abc=True, abc_tags=(50,),
                                            iterative_tol=1e-12, threads=host_threads())
        t_cpu = time.perf_counter() - t2
        cpu_err = float(np.abs(g_t - g_o).max() / np.abs(g_o).max())
        cpu = {"value": 1.0 / t_cpu, "unit": "gradients/s", "cores": host_threads(), "kind": "port",
               "sample": f"one complex128 driven adjoint of the oracle on the full {prob.n}-edge system (its own "
                         f"assembly; forward and adjoint COCG to 1e-12 with the Jacobi + nodal gradient + "
                         f"vector-nodal preconditioner in C on {host_threads()} OpenMP threads): {t_cpu:.1f} s "
                         f"(mesh topology and element matrices, {t_setup:.0f} s, not counted)"}
    out = {"metric": "adjoint gradients/s: d|S11|^2/d eps_r of every tet at 2.5 GHz (patch)", "value": args.steps / dt,
           "unit": "gradients/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (graded jittered patch mesh)",
           "config": {"workload": "patch_fr4_debye_abc_adjoint_2p5ghz", "tets": arrays.num_tets,
                      "substrate_tets": int(sub.size), "edges": mesh.num_edges, "freq_hz": f,
                      "tolerance": opts.tolerance,
                      "timing": "host wall clock around the library call (assembly + 1 solve + contraction)"},
           "krylov": {"iterations_per_gradient": kt["iters"] / max(args.steps, 1),
                      "solves_per_gradient": kt["solves"] / max(args.steps, 1)},
           "checks": {"fd_h": h, "fd_method": "central differences by correction solves (tolerance 1e-10 "
                                               "relative to the correction's right-hand side)",
                      "fd_tets": [[t, float(g_t[t]), d] for t, d in fd], "fd_max_rel_err": float(max(rel)),
                      "fd_rel_err_floor": "1e-3 of the largest substrate gradient", "fd_seconds": t_fd,
                      "per_tet_eps_vs_debye_region_max_rel": float(np.abs(g_q - g_t).max() / np.abs(g_t).max()),
                      "cpu_adjoint_max_rel_err": cpu_err,
                      "S11": [S_t[0, 0].real, S_t[0, 0].imag],
                      "substrate_grad_abs_max": gmax,
                      "air_grad_abs_max": float(np.abs(np.delete(g_t, sub)).max())},
           "clocks": clk, "cpu_baseline": cpu}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="slab",
                    choices=["slab", "medium", "small", "patch", "patch_small", "uneven", "uneven_small",
                             "adjoint", "patch_adjoint"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="leave the adjoint object out of the default line")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--no-vector-aux", action="store_true",
                    help="gradient auxiliary space only (no vector-nodal term) in the batched preconditioner")
    ap.add_argument("--precision", type=int, default=2, choices=[0, 1, 2],
                    help="batched Krylov arithmetic: 2 double-float K and M, 1 double-float K, 0 complex64")
    ap.add_argument("--rb-samples", type=int, default=16,
                    help="sample frequencies of the batched engine's reduced-basis initial guesses "
                         "(0 = every column from zero)")
    ap.add_argument("--cold-steps", type=int, default=2,
                    help="timed solves of the same sweep with every column from zero (0 = skip)")
    args = ap.parse_args()
    if args.workload in ("adjoint", "patch_adjoint"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the adjoint workload has no reference "
                                                                  "implementation (the reference has no adjoint)"}))
            return
        (adjoint_workload if args.workload == "adjoint" else patch_adjoint_workload)(args)
        return
    spec = workload_spec(args.workload)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, spec)
        return

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")

    import edgefem_gb300 as em
    if em.device_count() < 1:
        raise SystemExit("bench.py needs a CUDA device")
    problem = build_problem(spec)
    insts = setup_instances(problem, spec)
    rep = representative(problem)
    arrays = problem[rep] if isinstance(problem, list) else problem
    inst = insts[rep]
    freqs_all = spec["freqs"]
    if world > 1:
        # One sweep of (64 x N) band points sharded across the N GPUs: each
        # rank solves an interleaved 64 of them (weak scaling: fixed work
        # per GPU), as the SDK's sharded sweep entry points do.
        from edgefem_gb300.replicas import shard_indices
        freqs_all = np.linspace(spec["freqs"][0], spec["freqs"][-1], len(spec["freqs"]) * world)
        my_idx = shard_indices(len(freqs_all), rank, world)
    else:
        my_idx = np.arange(len(freqs_all))
    freqs = freqs_all[my_idx]
    driven = spec.get("kind") == "driven"
    bopts = dict(tolerance=spec["tol"], precision=args.precision, formulation=1 if driven else 0,
                 vector_aux=not args.no_vector_aux)
    # The same sweep with every column from zero: its own points/s, and the
    # SpMM launch time at the full column width for the roofline.
    cold = None
    spmm_ms, spmm_n = 0.0, 0
    # (only where the reduced-basis phase engages: otherwise the default
    # solve below is already the from-zero one)
    rb_on = args.precision > 0 and bool(rb_sample_indices(len(freqs), args.rb_samples, len(inst.ports)))
    if args.cold_steps > 0 and rb_on:
        csolver = em.BatchSolver(insts, freqs, em.BatchOptions(time_spmm=True, rb_samples=0, **bopts))
        csolver.solve()
        ct, cit = [], []
        for _ in range(args.cold_steps):
            _, cst = csolver.solve()
            ct.append(cst["solve_ms"])
            cit.append(cst["max_iters"])
            spmm_ms += cst["spmm_ms"]
            spmm_n += cst["spmm_timed"]
        cold = {"value": len(insts) * len(freqs) * len(ct) / (float(np.sum(ct)) / 1e3), "unit": "freq points/s",
                "ms_per_step": float(np.mean(ct)), "steps": len(ct), "iterations_max": int(max(cit)),
                "timing": "CUDA events around the solve, as the value; one untimed solve first",
                "spmm_rhs": csolver.rhs, "spmm_avg_launch_ms": spmm_ms / max(spmm_n, 1)}
        del csolver
    # (with reduced-basis guesses the full-width SpMMs are those of the
    # sample frequencies' engine: rb_samples x ports columns)
    solver = em.BatchSolver(insts, freqs, em.BatchOptions(time_spmm=True, rb_samples=args.rb_samples, **bopts))

    for _ in range(args.warmup):
        solver.solve()
    if dist is not None:
        dist.barrier()
    clocks = ClockSampler()
    clocks.start()
    times, launches, iters = [], 0, []
    S_last = None
    spmm_ms, spmm_n = 0.0, 0
    for _ in range(args.steps):
        S, st = solver.solve()
        times.append(st["solve_ms"])
        spmm_ms += st["spmm_ms"]
        spmm_n += st["spmm_timed"]
        launches += st["kernel_launches"]
        iters.append(st["max_iters"])
        S_last, st_last = S, st
    clk = clocks.stop()
    _, rhs_iters, _ = solver.rhs_stats()
    it_f = rhs_iters.max(axis=(0, 2))  # per frequency: the slowest instance and port
    iter_summary = {"per_frequency_min": int(it_f.min()), "median": float(np.median(it_f)),
                    "mean": float(it_f.mean()), "max": int(it_f.max()),
                    "by_frequency": [int(v) for v in it_f]}
    total_ms = float(np.sum(times))
    if dist is not None:
        # Replicas: every rank solved the full workload on its own GPU; the
        # job's time is the slowest rank's.
        from edgefem_gb300.replicas import max_over_ranks
        total_ms = max_over_ranks(total_ms)
    points = len(insts) * len(freqs_all) * args.steps
    value = points / (total_ms / 1000.0)

    peak, peak_kind = read_peaks()
    # column width of the timed SpMMs: the sample engine's with the
    # reduced-basis phase on (its rule: samples x ports rounded up to a power
    # of two, at least 4), else the engine's own
    spmm_rhs = solver.rhs
    if st_last["rb_samples"] > 0:
        spmm_rhs = 4
        while spmm_rhs < st_last["rb_samples"] * len(inst.ports):
            spmm_rhs *= 2
    bytes_launch = spmm_bytes(solver.rows, solver.nnz, spmm_rhs, args.precision)
    avg_spmm_ms = spmm_ms / spmm_n if spmm_n else None
    achieved = bytes_launch / (avg_spmm_ms / 1000.0) / 1e9 if spmm_n else None
    if cold is not None:
        cb = spmm_bytes(solver.rows, solver.nnz, cold["spmm_rhs"], args.precision)
        cold["spmm_roofline"] = {
            "kernel": "dd_spmm_kernel", "rhs": cold["spmm_rhs"], "bytes_per_launch": cb,
            "achieved": cb / (cold["spmm_avg_launch_ms"] / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
            "frac": cb / (cold["spmm_avg_launch_ms"] / 1000.0) / 1e9 / peak,
            "traffic": MEASURED_SPMM_TRAFFIC.get((spec["workload"], args.precision, cold["spmm_rhs"]))}

    extra = {}
    P_ = len(inst.ports)
    samples = rb_sample_indices(len(freqs), args.rb_samples, P_) if args.precision > 0 else []
    if st_last["rb_samples"] > 0:
        extra["reduced_basis"] = {
            "rb_samples": args.rb_samples, "sample_frequencies": st_last["rb_samples"],
            "sample_indices": samples, "basis_vectors": st_last["rb_basis"],
            "columns_done_at_guess": st_last["rb_done_at_guess"],
            "columns": len(insts) * len(freqs) * P_,
            "sample_solve_ms": st_last["rb_sample_ms"], "basis_and_guess_ms": st_last["rb_ms"],
            "rest_ms": st_last["solve_ms"] - st_last["rb_sample_ms"] - st_last["rb_ms"],
            "note": "sample frequencies solved to a tenth of the tolerance; every column then starts from the "
                    "Galerkin solution on their orthonormalised solutions and iterates only while its true "
                    "residual is above the tolerance"}
    if cold is not None:
        extra["batched_cold"] = cold
        extra["rb_speedup_over_cold"] = value / world / cold["value"] if world == 1 else None
    plain_rows = []
    if rank == 0 and not args.no_plain:
        # Plain unbatched FP64 GPU path on the same mesh at 8 band-spanning
        # frequencies (both ports each): the library call per frequency
        # (assembly, both port solves, S extraction) on the host clock, and
        # the Krylov solves alone on CUDA events (the batched value's timing).
        p = inst.params

        def plain(fi, prec, tol, maxit):
            p.omega = 2 * math.pi * float(freqs[fi])
            so = em.SolveOptions(use_bicgstab=False, tolerance=tol, max_iterations=maxit, preconditioner=prec)
            em.sdk.krylov_totals(reset=True)
            t0 = time.perf_counter()
            if driven:
                S_ = em.calculate_sparams(inst.mesh, p, inst.bc, inst.ports, so)
            else:
                S_ = em.calculate_sparams_eigenmode(inst.mesh, p, inst.bc, inst.ports, so)
            wall = time.perf_counter() - t0
            kt = em.sdk.krylov_totals(reset=True)
            return {"index": fi, "freq_hz": float(freqs[fi]), "S": S_, "wall_s": wall,
                    "device_s": kt["device_ms"] / 1e3, "iterations": kt["iters"]}

        plain(len(freqs) // 2, "aux", spec["tol"], 400000)  # warm-up
        plain_rows = [plain(fi, "aux", spec["tol"], 400000) for fi in band_indices(len(freqs))]
        dev_s = float(sum(r["device_s"] for r in plain_rows))
        wall_s = float(sum(r["wall_s"] for r in plain_rows))
        extra["plain_fp64"] = {
            "value": len(plain_rows) / dev_s, "unit": "freq points/s", "preconditioner": "aux",
            "timing": "CUDA events around the Krylov solves (as the batched value)",
            "value_wall": len(plain_rows) / wall_s,
            "wall_timing": "host clock around calculate_sparams_eigenmode (assembly + solves + S)",
            "frequencies_hz": [r["freq_hz"] for r in plain_rows],
            "iterations": [r["iterations"] for r in plain_rows],
            "device_s": [r["device_s"] for r in plain_rows]}
        extra["batched_over_plain"] = value / world / extra["plain_fp64"]["value"]
        extra["batched_over_plain_wall"] = value / world / extra["plain_fp64"]["value_wall"]
        if cold is not None:
            extra["batched_cold_over_plain"] = cold["value"] / extra["plain_fp64"]["value"]
        if not driven:
            fi = len(freqs) // 2
            jac = plain(fi, "jacobi", spec["tol"], 400000)
            extra["plain_fp64_jacobi"] = {"value": 1.0 / jac["device_s"], "unit": "freq points/s",
                                          "preconditioner": "jacobi", "frequency_hz": jac["freq_hz"],
                                          "iterations": jac["iterations"], "seconds_per_point": jac["device_s"]}
            extra["batched_over_plain_jacobi"] = value / world * jac["device_s"]

    spmv = edge_build = None
    if rank == 0:
        spmv = spmv_measure(em, inst, float(freqs[len(freqs) // 2]), peak, spec["workload"])
        edge_build = edge_build_measure(em, arrays)
        if not args.no_plain and args.workload == "slab":
            extra["solve_linear"] = solve_linear_report(em, inst, float(freqs[len(freqs) // 2]), spec["tol"])

    # End to end through the public API from host arrays: mesh ingest, ports,
    # pattern, H2D, assembly, solve, S back to the host.
    # With several ranks every rank takes part (the sweep is sharded inside
    # sparams_eigenmode_batched and gathered on every rank).
    e2e = None
    if args.e2e_steps > 0 and (rank == 0 or world > 1):
        if dist is not None:
            dist.barrier()
        h0, d0 = em.sdk.transfer_counters()
        t0 = time.perf_counter()
        setup_s = solve_s = 0.0
        for _ in range(args.e2e_steps):
            insts2 = setup_instances(problem, spec)
            S2, st2 = em.sparams_eigenmode_batched(insts2, freqs_all,
                                                   em.BatchOptions(rb_samples=args.rb_samples, **bopts))
            setup_s += st2["setup_ms"] / 1e3
            solve_s += st2["solve_ms"] / 1e3
        t_e2e = time.perf_counter() - t0
        if dist is not None:
            from edgefem_gb300.replicas import max_over_ranks
            t_e2e = max_over_ranks(t_e2e)
        h1, d1 = em.sdk.transfer_counters()
        e2e = {"value": len(insts) * len(freqs_all) * args.e2e_steps / t_e2e, "unit": "freq points/s",
               "h2d_bytes_per_step": int((h1 - h0) / args.e2e_steps),
               "d2h_bytes_per_step": int((d1 - d0) / args.e2e_steps),
               "seconds_per_step": t_e2e / args.e2e_steps,
               "engine_setup_seconds_per_step": setup_s / args.e2e_steps,
               "solve_device_seconds_per_step": solve_s / args.e2e_steps,
               "dS_vs_resident": float(np.nanmax(np.abs(S2[:, my_idx] - S_last)))}
        if world > 1:
            e2e["note"] = "bytes and set-up/solve times of rank 0's share; value over the whole sharded sweep"

    # Parity at the band edges against the complex128 oracle and the
    # measured CPU baseline (the same oracle solves, timed to the workload's
    # tolerance on the host's threads).
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu and not driven and not isinstance(problem, list):
        F = len(freqs)
        mid = next((i for i in range(F // 2, F) if i not in samples), None) if samples else None
        extra["oracle_check"], cpu = oracle_check(arrays, spec, S_last[rep], plain_rows,
                                                  extra_idx=[mid] if mid is not None else [], samples=samples)

    # Configuration 4 (adjoint of |S21|^2 per tet, 207k tets) as a bounded
    # object of the default line: 2 timed gradients, central differences at
    # 20 seeded tets, the oracle's complex128 adjoint.
    if rank == 0 and args.workload == "slab" and not args.no_adjoint:
        extra["adjoint"] = adjoint_measure(em, steps=2, warmup=1, no_cpu=args.no_cpu)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "freq points/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None,
               "dtype": "c64+f64" if args.precision == 0 else "dd(f32x2)+f64", "data": "synthetic",
               "config": {"workload": spec["workload"], "instances": len(insts), "rows": solver.rows,
                          "nnz": solver.nnz,
                          "freqs": len(freqs_all), "freqs_per_gpu": len(freqs), "ports": len(inst.ports),
                          "rhs_per_row": solver.rhs,
                          "tolerance": spec["tol"],
                          "rows_per_chunk": solver.rows_per_chunk, "parallelism": f"freq-shard{world}" if world > 1 else "single-gpu",
                          "precision": ["complex64", "double-float K", "double-float K and M"][args.precision],
                          "preconditioner": "Jacobi + nodal gradient" + ("" if args.no_vector_aux or
                                                                          args.precision == 0
                                                                          else " + vector-nodal"),
                          "l2": "inputs larger than L2 (each [rows x rhs] vector is "
                                f"{solver.rows * solver.rhs * (8 if args.precision == 0 else 16) / 1e6:.0f} MB)",
                          "rb_samples": args.rb_samples if samples else 0,
                          "form": ("reduced-basis guesses from " + str(len(samples)) + " sample frequencies, then "
                                   if samples else "") + "batched block COCG from the guesses"},
               "iterations_max": int(np.max(iters)), "iterations": iter_summary, "gpu_launches": int(launches),
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak if achieved else None,
                            "traffic": MEASURED_SPMM_TRAFFIC.get((spec["workload"], args.precision, spmm_rhs)),
                            "rhs": spmm_rhs,
                            "kernel": "batch_spmm_kernel" if args.precision == 0 else "dd_spmm_kernel",
                            "bytes_per_launch": bytes_launch, "avg_launch_ms": avg_spmm_ms,
                            "note": "SpMM launches at the full column width of the timed solves (the sample "
                                    "frequencies' engine with reduced-basis guesses; batched_cold.spmm_roofline "
                                    "has the 128-column form); the double-float SpMM is bound by its instruction "
                                    "issue (TwoProd/TwoSum arithmetic, about half of the issue slots) and the "
                                    "latency of its p gathers, not HBM"
                                    if args.precision > 0 else "latency-bound gather",
                            "peak_kind": peak_kind},
               "clocks": clk, "e2e": e2e, "cpu_baseline": cpu, "spmv": spmv,
               "edge_build": edge_build}
        out.update(extra)
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
