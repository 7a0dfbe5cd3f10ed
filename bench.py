#!/usr/bin/env python3
"""Benchmark: frequency points/s of the batched complex64 + FP64-refinement
eigenmode sweep on one GB300 (one JSON line on stdout).

Workload (default): WR-90 box 22.86 x 10.16 x 50 mm with a centred
dielectric slab (z in [20, 30] mm, eps_r = 2.2 (1 - 0.001j)), 40x20x100 hex
cells split into 6 tets (480,000 tets, 580,560 edges), two TE10 wave ports,
64 frequencies uniform over 8-12 GHz, relative FP64 residual tolerance 1e-8.
A step is one full solve of all 64 frequencies x 2 active ports from x = 0
with the operator resident in HBM.  Synthetic mesh (no gmsh here).

Reported beside it: the plain unbatched FP64 GPU path on the same mesh,
|dS| of the batched result against a tight FP64 solve, the SpMM roofline,
the CPU baseline, and an end-to-end number through the public API from
host arrays.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os

# Single-threaded BLAS: the CPU legs time one core per process, and the
# reference arm forks its worker processes after numpy is loaded.
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
# of two full-width launches, mean) of the batched SpMM on the named workload
# and precision; None where no capture exists.
MEASURED_SPMM_TRAFFIC = {("wr90_slab_40x20x100_64f", 2): 5.365e9}


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
    for form, fname, cdt, rdt, sv in (("complex64", "efgk_spmv32", np.complex64, np.float32, 8),
                                      ("complex128", "efgk_spmv64", np.complex128, np.float64, 16)):
        fn = getattr(_lib.lib, fname)
        fn.restype = C.c_int
        fn.argtypes = [C.c_int32] + [C.c_void_p] * 6
        d_v = torch.from_numpy(np.ascontiguousarray(v.astype(cdt)).view(rdt)).to(dev)
        d_x = torch.from_numpy(np.ascontiguousarray(x.astype(cdt)).view(rdt)).to(dev)
        d_y = torch.empty(2 * n, dtype=d_v.dtype, device=dev)
        ptrs = (d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_x.data_ptr(), d_y.data_ptr(), stream.cuda_stream)

        def call():
            rc = fn(n, *ptrs)
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
        out[form] = {"kernel": fname.replace("efgk_", "") + "_kernel", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "bytes_per_launch": nbytes, "avg_launch_ms": ms,
                     "launches": launches, "l2": "flushed before every launch (512 MB write, then a 256 MB read)",
                     "traffic": MEASURED_SPMV_TRAFFIC.get((workload, fname)),
                     "max_abs_err_over_max_y": float(np.abs(y - y_ref).max() / np.abs(y_ref).max())}
    out["rows"], out["nnz"], out["frequency_hz"] = n, nnz, float(freq)
    out["note"] = ("the complex128 product does 8 FP64 flops per stored entry, which GB300's FP64 pipe "
                   "cannot feed at HBM rate; the complex64 product runs on the FP32 pipes")
    del flush
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


def oracle_system(arrays, spec, f):
    """(problem, A, b) of the workload at frequency f from the CPU oracle:
    the eigenmode system (first port active) or the driven-port system."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import edgefem_oracle as O
    prob = O.make_problem(arrays)
    w = 2 * math.pi * f
    if spec.get("kind") == "driven":
        prob.pec = np.union1d(prob.pec, O.build_edge_pec(prob.topo.tri_edges, arrays.tri_phys, 10))
        eps = O.tet_eps(prob, w, eps_models={101: O.debye_eps(*spec["debye"])})
        ports = [O.build_lumped_port(prob, 20, (0.0, 0.0, 1.0), 50.0)]
        A, b = O.assemble_maxwell(prob, w, eps, ports, 0, use_abc=True, abc_tags=(50,))
        return prob, A, b
    ports = O.waveguide_ports(prob, 22.86e-3, f)
    eps_slab = spec["eps_slab"]
    eps = O.tet_eps(prob, w, eps_regions={101: eps_slab} if eps_slab is not None else None,
                    eps_tet=getattr(arrays, "eps_tet", None))
    sys_ = O.eigenmode_system(prob, w, ports, eps)
    return prob, sys_.A, sys_.B[:, 0]


def cpu_baseline(arrays, spec, iters_per_point: int, seconds: float, eps_slab=None):
    """Bounded CPU sample: Jacobi-COCG in complex128 (the oracle's CPU
    restatement) on the same assembled system at one frequency, timed for
    `seconds`; points/s extrapolated with the measured iterations per point."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import edgefem_oracle as O
    f = float(spec["freqs"][len(spec["freqs"]) // 2])
    prob, A, b = oracle_system(arrays, spec, f)
    _, it, _, t_it = O.cocg_jacobi(A, b, tol=1e-300, maxit=10 ** 9, max_seconds=seconds,
                                   prec=O.aux_preconditioner(prob, A, vector=True))
    return {"value": 1.0 / (iters_per_point * t_it), "unit": "freq points/s", "cores": 1, "kind": "port",
            "sample": f"{it} COCG iterations with the Jacobi + nodal gradient + vector-nodal preconditioner "
                      f"(complex128, SciPy CSR, 1 thread) on the full "
                      f"{prob.n}-edge system at {f/1e9:.3f} GHz, {t_it*1e3:.2f} ms/iteration, extrapolated "
                      f"to {iters_per_point} iterations per frequency point (all ports), the FP64 GPU count"}


_REF = {}


def _ref_worker(seconds):
    """One core: COCG with the auxiliary preconditioner on the system the
    parent assembled (inherited through fork), for `seconds`."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import edgefem_oracle as O
    _, _, _, t_it = O.cocg_jacobi(_REF["A"], _REF["b"], tol=1e-300, maxit=10 ** 9, max_seconds=seconds,
                                  prec=_REF["prec"])
    return t_it


def reference_arm(args, spec):
    """CPU implementation of the path on all host cores: the reference Eigen
    path does not build here (Eigen headers absent), so the CPU restatement
    runs instead - complex128 COCG with the Jacobi + nodal auxiliary
    preconditioner (SciPy), one process per core, each timing iterations on
    the workload's system (assembled once, at the middle frequency; the
    per-iteration cost is the same at every frequency).  Points/s = sum over
    cores of 1 / (iterations per point x seconds per iteration)."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import edgefem_oracle as O
    cores = len(os.sched_getaffinity(0))
    problem = build_problem(spec)
    arrays = problem[representative(problem)] if isinstance(problem, list) else problem
    iters_per_point = args.ref_iters_per_point
    f = float(spec["freqs"][len(spec["freqs"]) // 2])
    prob, A, b = oracle_system(arrays, spec, f)
    _REF.update(A=A, b=b, prec=O.aux_preconditioner(prob, A, vector=True))
    # This process never touches the GPU, so forked workers are safe and
    # share the assembled system.
    ctx = mp.get_context("fork")
    per = max(3.0, args.ref_seconds)
    values = []
    with ctx.Pool(cores) as pool:
        for step in range(args.warmup + args.steps):
            t_it = np.array(pool.map(_ref_worker, [per] * cores))
            thr = float(np.sum(1.0 / (iters_per_point * t_it)))
            if step >= args.warmup:
                values.append(thr)
    v = float(np.mean(values))
    out = {"metric": METRIC, "value": v, "unit": "freq points/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1000.0 * len(spec["freqs"]) / v, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
           "config": {"workload": spec["workload"], "rows": int(A.shape[0]), "freqs": len(spec["freqs"]),
                      "ports": 1 if spec.get("kind") == "driven" else 2},
           "impl": "reference",
           "cpu_baseline": {"value": v, "unit": "freq points/s", "cores": cores, "kind": "port",
                            "sample": f"{cores} processes x {per:.0f} s of complex128 COCG with the Jacobi + "
                                      f"nodal gradient + vector-nodal preconditioner (SciPy, 1 thread each) on the full "
                                      f"{A.shape[0]}-edge system at {f/1e9:.3f} GHz; extrapolated to "
                                      f"{iters_per_point} iterations per point (reference Eigen path "
                                      f"unavailable: Eigen headers absent)"},
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


def adjoint_workload(args):
    """d|S21|^2 / d eps_r of every tet of a WR-90 box (50 mm, 36x16x60 cells,
    207,360 tets) with a smooth seeded eps_r field, at 10 GHz.  Timed: the
    library's adjoint call (assembly, forward and adjoint FP64 solves on the
    GPU, per-tet contraction) per gradient; checked: central differences
    (h = 1e-4) at 20 seeded tets, and (unless --no-cpu) the oracle's
    complex128 adjoint (iterative, relative residual 1e-12), whose time is
    the CPU baseline."""
    import edgefem_gb300 as em
    if em.device_count() < 1:
        raise SystemExit("bench.py needs a CUDA device")
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
    for _ in range(args.warmup):
        em.sparams_eigenmode_adjoint(mesh, p, bc, ports, 1, 0, opts)
    clocks = ClockSampler()
    clocks.start()
    em.sdk.krylov_totals(reset=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
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
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import edgefem_oracle as O
        prob = O.make_problem(arrays)
        t1 = time.perf_counter()
        g_o, S_o = O.sparams_eigenmode_adjoint(prob, p.omega, O.waveguide_ports(prob, a, f),
                                               eps.astype(np.complex128), 1, 0, iterative_tol=1e-12)
        t_cpu = time.perf_counter() - t1
        cpu_err = float(np.abs(g_t - g_o).max() / np.abs(g_o).max())
        cpu = {"value": 1.0 / t_cpu, "unit": "gradients/s", "cores": 1, "kind": "port",
               "sample": f"one complex128 adjoint of the oracle on the full {prob.n}-edge system: two COCG "
                         f"solves (Jacobi + nodal gradient + vector-nodal preconditioner, SciPy CSR, 1 thread, "
                         f"relative residual 1e-12; a SuperLU factorisation ran past 6 minutes here) and the "
                         f"per-tet contraction"}
    out = {"metric": "adjoint gradients/s: d|S21|^2/d eps_r of every tet at 10 GHz", "value": args.steps / dt,
           "unit": "gradients/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded smooth eps_r field)",
           "config": {"workload": "wr90_adjoint_36x16x60_smooth_eps", "tets": arrays.num_tets,
                      "edges": mesh.num_edges, "freq_hz": f, "tolerance": opts.tolerance,
                      "timing": "host wall clock around the library call (assembly + 2 solves + contraction)"},
           "krylov": {"iterations_per_gradient": kt["iters"] / max(args.steps, 1),
                      "solves_per_gradient": kt["solves"] / max(args.steps, 1)},
           "checks": {"fd_tets": 20, "fd_h": h, "fd_max_rel_err": fd_err, "S21": [S_t[1, 0].real, S_t[1, 0].imag],
                      "cpu_adjoint_max_rel_err": cpu_err},
           "clocks": clk, "cpu_baseline": cpu}
    print(json.dumps(out))


def patch_adjoint_workload(args):
    """d|S11|^2 / d eps_r of every tet of the probe-fed patch (Debye FR-4
    substrate, ABC air box, 50-ohm lumped port normalised at 2.5 GHz) at
    2.5 GHz, reported over the substrate tets.  Timed: the library's driven
    adjoint call (assembly, one forward FP64 solve, per-tet contraction; the
    adjoint vector of the single port is its scaled forward solution) per
    gradient.  Checked: central differences (h = 1e-3, and 1e-4 beside it)
    at the three substrate tets of largest sensitivity, through the same
    system with the Debye permittivity at 2.5 GHz written per tet."""
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
    # Central differences at two steps.  The 1e-12 solves leave S with an
    # error near 2e-12, which a difference quotient amplifies by |S| / h
    # (about 800 at h = 1e-4, against gradients near 1e-5 per tet); at
    # h = 1e-3 that noise is ten times smaller and the truncation error of
    # the central difference stays far below it.
    picks = sub[np.argsort(-np.abs(g_t[sub]))[:3]]
    fd, fd_err = {}, {}
    for h in (1e-3, 1e-4):
        fd[h], fd_err[h] = [], 0.0
        for t in picks.tolist():
            vals = []
            for sgn in (1, -1):
                e2 = eps.copy()
                e2[t] += sgn * h
                q.eps_r_tet = e2
                vals.append(abs(em.calculate_sparams(mesh, q, bc, ports, tight)[0, 0]) ** 2)
            d = (vals[0] - vals[1]) / (2 * h)
            fd[h].append([int(t), float(g_t[t]), float(d)])
            fd_err[h] = max(fd_err[h], abs(g_t[t] - d) / abs(d))
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
           "checks": {"fd_h": 1e-3, "fd_tets": fd[1e-3], "fd_max_rel_err": fd_err[1e-3],
                      "fd_h_1e-4": {"fd_tets": fd[1e-4], "fd_max_rel_err": fd_err[1e-4]},
                      "per_tet_eps_vs_debye_region_max_rel": float(np.abs(g_q - g_t).max() / np.abs(g_t).max()),
                      "S11": [S_t[0, 0].real, S_t[0, 0].imag],
                      "substrate_grad_abs_max": float(np.abs(g_t[sub]).max()),
                      "air_grad_abs_max": float(np.abs(np.delete(g_t, sub)).max())},
           "clocks": clk, "cpu_baseline": None}
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
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--no-vector-aux", action="store_true",
                    help="gradient auxiliary space only (no vector-nodal term) in the batched preconditioner")
    ap.add_argument("--precision", type=int, default=2, choices=[0, 1, 2],
                    help="batched Krylov arithmetic: 2 double-float K and M, 1 double-float K, 0 complex64")
    ap.add_argument("--ref-seconds", type=float, default=10.0)
    ap.add_argument("--ref-iters-per-point", type=int, default=0,
                    help="iterations per frequency point for the CPU extrapolation (0 = measured FP64 count)")
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
        if args.ref_iters_per_point <= 0:
            # Plain FP64 COCG iterations per point (all ports) with the Jacobi +
            # gradient + vector-nodal preconditioner, as the GPU plain path
            # measured them on these workloads (slab 40x20x100 at 10.03 GHz:
            # 1728); the CPU restatement does the same iterations.
            args.ref_iters_per_point = {"slab": 1728, "medium": 2 * 500, "small": 2 * 150,
                                        "patch": 4000, "patch_small": 1500, "uneven": 2 * 1000,
                                        "uneven_small": 2 * 1000}[args.workload]
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
    freqs = spec["freqs"]
    driven = spec.get("kind") == "driven"
    bopts = dict(tolerance=spec["tol"], precision=args.precision, formulation=1 if driven else 0,
                 vector_aux=not args.no_vector_aux)
    solver = em.BatchSolver(insts, freqs, em.BatchOptions(time_spmm=True, **bopts))

    for _ in range(args.warmup):
        solver.solve()
    if dist is not None:
        dist.barrier()
    clocks = ClockSampler()
    clocks.start()
    times, spmm_ms, spmm_n, launches, iters = [], 0.0, 0, 0, []
    S_last = None
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
    points = len(insts) * len(freqs) * args.steps * world
    value = points / (total_ms / 1000.0)

    peak, peak_kind = read_peaks()
    bytes_launch = spmm_bytes(solver.rows, solver.nnz, solver.rhs, args.precision)
    avg_spmm_ms = spmm_ms / max(spmm_n, 1)
    achieved = bytes_launch / (avg_spmm_ms / 1000.0) / 1e9

    extra = {}
    if rank == 0 and not args.no_plain:
        # Plain unbatched FP64 GPU path on the same mesh at one frequency (both ports).
        fi = len(freqs) // 2
        p = inst.params
        p.omega = 2 * math.pi * float(freqs[fi])
        def plain(prec, tol, maxit):
            so = em.SolveOptions(use_bicgstab=False, tolerance=tol, max_iterations=maxit, preconditioner=prec)
            st_ = {}
            t0 = time.perf_counter()
            if driven:
                em.sdk.krylov_totals(reset=True)
                S_ = em.calculate_sparams(inst.mesh, p, inst.bc, inst.ports, so)
                st_ = em.sdk.krylov_totals(reset=True)
            else:
                S_ = em.calculate_sparams_eigenmode(inst.mesh, p, inst.bc, inst.ports, so, st_)
            return S_, time.perf_counter() - t0, st_

        S_ref, _, pst_ref = plain("aux", 1e-12, 600000)
        S_plain, t_plain, pst = plain("aux", spec["tol"], 400000)
        if driven:  # Jacobi alone needs far more iterations here; time a bounded sample
            S_jac, t_jac, pst_jac = S_plain, float("nan"), {"iters": None}
        else:
            S_jac, t_jac, pst_jac = plain("jacobi", spec["tol"], 400000)
        dS = float(np.abs(S_last[rep, fi] - S_ref).max())
        extra["plain_fp64"] = {"value": 1.0 / t_plain, "unit": "freq points/s", "preconditioner": "aux",
                               "iterations": pst["iters"], "seconds_per_point": t_plain,
                               "dS_vs_tight_fp64": float(np.abs(S_plain - S_ref).max())}
        extra["plain_fp64_jacobi"] = {"value": 1.0 / t_jac, "unit": "freq points/s", "preconditioner": "jacobi",
                                      "iterations": pst_jac["iters"], "seconds_per_point": t_jac,
                                      "dS_vs_tight_fp64": float(np.abs(S_jac - S_ref).max())}
        extra["batched_over_plain"] = value / world / (1.0 / t_plain)
        extra["batched_over_plain_jacobi"] = None if driven else value / world / (1.0 / t_jac)
        if driven:
            extra["plain_fp64_jacobi"] = None
        extra["dS_batched_vs_tight_fp64"] = dS
        extra["tight_fp64_iterations"] = pst_ref["iters"]
        iters_per_point = pst["iters"]
    else:
        iters_per_point = None

    spmv = edge_build = None
    if rank == 0:
        spmv = spmv_measure(em, inst, float(freqs[len(freqs) // 2]), peak, spec["workload"])
        edge_build = edge_build_measure(em, arrays)

    # End to end through the public API from host arrays: mesh ingest, ports,
    # pattern, H2D, assembly, solve, S back to the host.
    e2e = None
    if rank == 0 and args.e2e_steps > 0:
        h0, d0 = em.sdk.transfer_counters()
        t0 = time.perf_counter()
        setup_s = solve_s = 0.0
        for _ in range(args.e2e_steps):
            insts2 = setup_instances(problem, spec)
            S2, st2 = em.sparams_eigenmode_batched(insts2, freqs, em.BatchOptions(**bopts))
            setup_s += st2["setup_ms"] / 1e3
            solve_s += st2["solve_ms"] / 1e3
        t_e2e = time.perf_counter() - t0
        h1, d1 = em.sdk.transfer_counters()
        e2e = {"value": len(insts) * len(freqs) * args.e2e_steps / t_e2e, "unit": "freq points/s",
               "h2d_bytes_per_step": int((h1 - h0) / args.e2e_steps),
               "d2h_bytes_per_step": int((d1 - d0) / args.e2e_steps),
               "seconds_per_step": t_e2e / args.e2e_steps,
               "engine_setup_seconds_per_step": setup_s / args.e2e_steps,
               "solve_device_seconds_per_step": solve_s / args.e2e_steps,
               "dS_vs_resident": float(np.nanmax(np.abs(S2 - S_last)))}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu and iters_per_point:
        cpu = cpu_baseline(arrays, spec, iters_per_point, args.cpu_seconds, spec["eps_slab"])

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "freq points/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None,
               "dtype": "c64+f64" if args.precision == 0 else "dd(f32x2)+f64", "data": "synthetic",
               "config": {"workload": spec["workload"], "instances": len(insts), "rows": solver.rows,
                          "nnz": solver.nnz,
                          "freqs": len(freqs), "ports": len(inst.ports), "rhs_per_row": solver.rhs,
                          "tolerance": spec["tol"],
                          "rows_per_chunk": solver.rows_per_chunk, "parallelism": f"replicas{world}",
                          "precision": ["complex64", "double-float K", "double-float K and M"][args.precision],
                          "preconditioner": "Jacobi + nodal gradient" + ("" if args.no_vector_aux or
                                                                          args.precision == 0
                                                                          else " + vector-nodal"),
                          "l2": "inputs larger than L2 (each [rows x rhs] vector is "
                                f"{solver.rows * solver.rhs * (8 if args.precision == 0 else 16) / 1e6:.0f} MB)"},
               "iterations_max": int(np.max(iters)), "iterations": iter_summary, "gpu_launches": int(launches),
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak,
                            "traffic": MEASURED_SPMM_TRAFFIC.get((spec["workload"], args.precision)),
                            "kernel": "batch_spmm_kernel" if args.precision == 0 else "dd_spmm_kernel",
                            "bytes_per_launch": bytes_launch, "avg_launch_ms": avg_spmm_ms,
                            "note": "the double-float SpMM is bound by FP32 issue (TwoProd/TwoSum "
                                    "arithmetic), not HBM; the vector phases run near HBM peak"
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
