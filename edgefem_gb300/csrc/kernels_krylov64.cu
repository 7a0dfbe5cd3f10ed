// Plain FP64 Krylov kernels: complex CSR SpMV, COCG and BiCGStab with the
// Jacobi or the nodal auxiliary-space preconditioner, port overlaps.
// One right-hand side per solve.
//
// Preconditioners (both complex symmetric, as COCG requires):
//   Jacobi  z = D^-1 r
//   aux     z = D^-1 r + G Dn^-1 G^T r
// with G the discrete gradient (edge-node incidence, rows of PEC edges
// zeroed) and Dn = diag(G^T A G).  The aux term smooths the gradient
// null-space of the curl-curl operator that Jacobi alone leaves slow
// (the additive two-space smoother of Hiptmair, SIAM J. Numer. Anal. 36
// (1998), with Jacobi in both spaces).
//
// COCG runs as four kernels per iteration with device-resident scalars so
// a host loop can capture many iterations in one CUDA graph:
//   K1  q = A p, pq += p^T q                                (SpMV + dot)
//   K2  alpha = rho_k/pq; x += alpha p; r -= alpha q;
//       rho_{k+1} += r^T D^-1 r; rr += |r|^2
//   K2b (aux) s = G^T r; t = Dn^-1 s; rho_{k+1} += s^T t    (node pass)
//   K3  convergence test; beta; p = D^-1 r + G t + beta p
// Accumulators are double-buffered by iteration parity.  Every kernel is a
// grid-stride loop over a fixed grid (a few blocks per SM), so a reduction
// costs a few hundred atomics, not one per 256 rows.
#include <cuda_runtime.h>

#include "edgefem_gb300_kernels.h"
#include "sc_layout.h"

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double2 cconjmul(double2 a, double2 b) {  // conj(a) * b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// Block-wide sum of NV doubles, then one atomicAdd each into dst[k]
// (dst[k] == nullptr skips).  All threads of the block must call it.
template <int NV>
__device__ __forceinline__ void block_reduce_add(double (&v)[NV], double *const (&dst)[NV]) {
  __shared__ double sh[NV][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  }
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][warp] = v[k];
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = lane < nw ? sh[k][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0 && dst[k]) atomicAdd(dst[k], s);
    }
  }
}

constexpr int kL = 4;     // lanes per row in the SpMV
constexpr int kBS = 256;  // threads per block

// Sub-warp CSR row product: L lanes per row; the row sum ends up in all L lanes.
template <int L>
__device__ __forceinline__ double2 row_dot(int row, int lane, const int *__restrict__ rowptr,
                                           const int *__restrict__ colidx, const double2 *__restrict__ vals,
                                           const double2 *__restrict__ x) {
  double2 acc = make_double2(0.0, 0.0);
  const int b = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
  for (int k = b + lane; k < e; k += L) acc = cfma(__ldg(vals + k), __ldg(x + __ldg(colidx + k)), acc);
  // Only the L lanes of this row's group take part: other groups of the
  // warp may already have left their row loop.
  const unsigned mask = ((1u << L) - 1u) << (threadIdx.x & 31 & ~(L - 1));
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) {
    acc.x += __shfl_xor_sync(mask, acc.x, o);
    acc.y += __shfl_xor_sync(mask, acc.y, o);
  }
  return acc;
}

__device__ __forceinline__ bool stopped(const double *sc) { return sc[SC_STATUS] != 0.0; }

// Block-uniform stop test for kernels that reach a __syncthreads: one read
// by thread 0, shared with the block.
__device__ __forceinline__ bool block_stopped(const double *sc) {
  __shared__ int s_stop;
  if (threadIdx.x == 0) s_stop = stopped(sc) ? 1 : 0;
  __syncthreads();
  return s_stop != 0;
}

// Auxiliary-space data: per edge its (tail, head) node index or (-1, -1) for
// a PEC edge; per node its incident non-PEC edges with the incidence sign.
struct Aux {
  const int2 *enodes;
  const int *nptr, *nedge;
  const signed char *nsign;
  const double2 *dninv;
  double2 *t;
  int nn;
  // vector-nodal space (npi = 3): per edge weights (x_head - x_tail)/2, per
  // (node, component) omega / diag(Pi^T A Pi) and the node values t_d
  int npi;
  const double *piw;
  const double2 *dpinv;
  double2 *tp;
  // block-Jacobi (bs > 0): column-major inverses of the diagonal blocks
  // and the preconditioned vector z
  const double2 *bjinv;
  double2 *z;
  int bs;
};

__device__ __forceinline__ double2 aux_term(const Aux &ax, int e) {
  const int2 en = ax.enodes[e];
  if (en.x < 0) return make_double2(0.0, 0.0);
  double2 z = csub(ax.t[en.y], ax.t[en.x]);
  for (int d = 0; d < ax.npi; ++d) {
    const double w = ax.piw[3 * e + d];
    const double2 a = ax.tp[3 * en.x + d], b = ax.tp[3 * en.y + d];
    z.x += w * (a.x + b.x);
    z.y += w * (a.y + b.y);
  }
  return z;
}

// -------------------------------------------------------------------- SpMV
__global__ void __launch_bounds__(kBS) spmv64_kernel(int n, const int *__restrict__ rowptr,
                                                    const int *__restrict__ colidx,
                                                    const double2 *__restrict__ vals,
                                                    const double2 *__restrict__ x, double2 *__restrict__ y) {
  const int lane = threadIdx.x % kL;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) / kL; row < n; row += gridDim.x * blockDim.x / kL) {
    const double2 s = row_dot<kL>(row, lane, rowptr, colidx, vals, x);
    if (lane == 0) y[row] = s;
  }
}

// Complex64 CSR SpMV with FP32 accumulation: the single-right-hand-side
// operator product of an FP32 Krylov iteration.  A group of kL32 = 8 lanes
// takes one row at a time (grid-stride over rows, one wave of resident
// blocks); each lane loads up to kU32 = 3 of the row's entries per pass
// (predicated, so the 13- and 19-entry rows of a Kuhn-split hex grid take
// one pass) and longer rows finish in a tail loop.  Rows are pipelined: the
// column and value loads of the group's next row are issued before this
// row's x gathers are consumed, and row bounds are read two rows ahead, so
// a group waits about one DRAM latency per row instead of three dependent
// ones (bounds, entries, gather).  The x gather (8 bytes per entry) is
// served by L1/L2: a row's columns lie within a few hex-grid layers of the
// row.  An FP64 complex SpMV does 8 FP64 flops per stored entry, which
// GB300's FP64 pipe cannot feed at HBM rate; this form runs on the FP32
// pipes and is bound by HBM (12 bytes per entry).
__device__ __forceinline__ float2 cfma32(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

constexpr int kL32 = 8;  // lanes per row in the complex64 SpMV
constexpr int kU32 = 3;  // entries per lane per pass

// Predicated first-pass loads of one row: entries k0, k0 + kL32, ... below e
// (column -1 and value 0 past the end).
__device__ __forceinline__ void spmv32_pass(int k0, int e, const int *__restrict__ colidx,
                                            const float2 *__restrict__ vals, int (&c)[kU32],
                                            float2 (&a)[kU32]) {
#pragma unroll
  for (int u = 0; u < kU32; ++u) {
    const int k = k0 + u * kL32;
    const bool ok = k < e;
    c[u] = ok ? __ldg(colidx + k) : -1;
    a[u] = ok ? __ldg(vals + k) : make_float2(0.f, 0.f);
  }
}

__global__ void __launch_bounds__(kBS) spmv32_kernel(int n, const int *__restrict__ rowptr,
                                                    const int *__restrict__ colidx,
                                                    const float2 *__restrict__ vals,
                                                    const float2 *__restrict__ x, float2 *__restrict__ y) {
  const int lane = threadIdx.x % kL32;
  // Only this row's lanes take part in the shuffles: other groups of the
  // warp may have left the row loop.
  const unsigned mask = ((1u << kL32) - 1u) << (threadIdx.x & 31 & ~(kL32 - 1));
  const int stride = gridDim.x * blockDim.x / kL32;
  int row = (blockIdx.x * blockDim.x + threadIdx.x) / kL32;
  if (row >= n) return;
  int b = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
  int nrow = row + stride, nb = 0, ne = 0;
  if (nrow < n) nb = __ldg(rowptr + nrow), ne = __ldg(rowptr + nrow + 1);
  int c[kU32];
  float2 a[kU32];
  spmv32_pass(b + lane, e, colidx, vals, c, a);
  while (true) {
    float2 xv[kU32];
#pragma unroll
    for (int u = 0; u < kU32; ++u) xv[u] = c[u] >= 0 ? __ldg(x + c[u]) : make_float2(0.f, 0.f);
    // Next row's entries and the bounds of the row after it.
    int c2[kU32];
    float2 a2[kU32];
    spmv32_pass(nb + lane, nrow < n ? ne : 0, colidx, vals, c2, a2);
    const int nnrow = nrow + stride;
    int nnb = 0, nne = 0;
    if (nnrow < n) nnb = __ldg(rowptr + nnrow), nne = __ldg(rowptr + nnrow + 1);
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kU32; ++u) acc = cfma32(a[u], xv[u], acc);
    for (int k = b + lane + kU32 * kL32; k < e; k += kL32)
      acc = cfma32(__ldg(vals + k), __ldg(x + __ldg(colidx + k)), acc);
#pragma unroll
    for (int o = kL32 / 2; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(mask, acc.x, o);
      acc.y += __shfl_xor_sync(mask, acc.y, o);
    }
    if (lane == 0) y[row] = acc;
    if (nrow >= n) break;
    row = nrow, b = nb, e = ne;
    nrow = nnrow, nb = nnb, ne = nne;
#pragma unroll
    for (int u = 0; u < kU32; ++u) c[u] = c2[u], a[u] = a2[u];
  }
}

// -------------------------------------------------------------------- COCG
__global__ void __launch_bounds__(kBS) cocg_k1(int n, const int *__restrict__ rowptr,
                                              const int *__restrict__ colidx,
                                              const double2 *__restrict__ vals,
                                              const double2 *__restrict__ p, double2 *__restrict__ q,
                                              double *sc, int P) {
  if (block_stopped(sc)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc[SC_RHO + 2 * P] = 0.0;
    sc[SC_RHO + 2 * P + 1] = 0.0;
    sc[SC_RR + P] = 0.0;
  }
  const int lane = threadIdx.x % kL;
  double v[2] = {0.0, 0.0};
  const int stride = gridDim.x * blockDim.x / kL;
  // Uniform trip count per sub-warp: rows beyond n are skipped inside.
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) / kL; row < n; row += stride) {
    const double2 s = row_dot<kL>(row, lane, rowptr, colidx, vals, p);
    if (lane == 0) {
      q[row] = s;
      const double2 d = cmul(p[row], s);
      v[0] += d.x;
      v[1] += d.y;
    }
  }
  double *const dst[2] = {sc + SC_PQ + 2 * P, sc + SC_PQ + 2 * P + 1};
  block_reduce_add<2>(v, dst);
}

__global__ void __launch_bounds__(kBS) cocg_k2(int n, const double2 *__restrict__ dinv, double2 *x, double2 *r,
                                              const double2 *__restrict__ p, const double2 *__restrict__ q,
                                              double *sc, int P, int rho_diag) {
  if (block_stopped(sc)) return;
  const int Q = 1 - P;
  const double2 rho = make_double2(sc[SC_RHO + 2 * Q], sc[SC_RHO + 2 * Q + 1]);
  const double2 pq = make_double2(sc[SC_PQ + 2 * P], sc[SC_PQ + 2 * P + 1]);
  if (pq.x == 0.0 && pq.y == 0.0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[SC_STATUS] = EFGK_BREAKDOWN;
    return;
  }
  const double2 alpha = cdiv(rho, pq);
  const double2 malpha = make_double2(-alpha.x, -alpha.y);
  double v[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = cfma(alpha, p[i], x[i]);
    const double2 ri = cfma(malpha, q[i], r[i]);
    r[i] = ri;
    if (rho_diag) {
      const double2 rz = cmul(ri, cmul(dinv[i], ri));
      v[0] += rz.x;
      v[1] += rz.y;
    }
    v[2] += ri.x * ri.x + ri.y * ri.y;
  }
  double *const dst[3] = {sc + SC_RHO + 2 * P, sc + SC_RHO + 2 * P + 1, sc + SC_RR + P};
  block_reduce_add<3>(v, dst);
}

// Node pass: t = Dn^-1 G^T r, and s^T t into the rho slot.
__global__ void __launch_bounds__(kBS) aux_node_kernel(const Aux ax, const double2 *__restrict__ r, double *sc,
                                                      int P, int check_stop) {
  if (check_stop && block_stopped(sc)) return;
  double v[2] = {0.0, 0.0};
  for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < ax.nn; nd += gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int k = ax.nptr[nd]; k < ax.nptr[nd + 1]; ++k) {
      const double2 re = r[ax.nedge[k]];
      const double sg = ax.nsign[k];
      s.x += sg * re.x;
      s.y += sg * re.y;
    }
    const double2 t = cmul(ax.dninv[nd], s);
    ax.t[nd] = t;
    const double2 st = cmul(s, t);
    v[0] += st.x;
    v[1] += st.y;
    for (int d = 0; d < ax.npi; ++d) {
      double2 sp = make_double2(0.0, 0.0);
      for (int k = ax.nptr[nd]; k < ax.nptr[nd + 1]; ++k) {
        const int e = ax.nedge[k];
        const double2 re = r[e];
        const double w = ax.piw[3 * e + d];
        sp.x += w * re.x;
        sp.y += w * re.y;
      }
      const double2 tp = cmul(ax.dpinv[3 * nd + d], sp);
      ax.tp[3 * nd + d] = tp;
      const double2 spt = cmul(sp, tp);
      v[0] += spt.x;
      v[1] += spt.y;
    }
  }
  double *const dst[2] = {sc + SC_RHO + 2 * P, sc + SC_RHO + 2 * P + 1};
  block_reduce_add<2>(v, dst);
}

__global__ void __launch_bounds__(kBS) cocg_k3(int n, const double2 *__restrict__ dinv,
                                              const double2 *__restrict__ r, double2 *p, double *sc, int P,
                                              const Aux ax, int use_aux, const double2 *__restrict__ zvec) {
  if (stopped(sc)) return;
  const int Q = 1 - P;
  const double rr = sc[SC_RR + P];
  const double iters = sc[SC_ITERS] + 1.0;
  const bool conv = rr <= sc[SC_TOL2] * sc[SC_BB];
  const bool out = iters >= sc[SC_MAXIT];
  const double2 rn = make_double2(sc[SC_RHO + 2 * P], sc[SC_RHO + 2 * P + 1]);
  const double2 ro = make_double2(sc[SC_RHO + 2 * Q], sc[SC_RHO + 2 * Q + 1]);
  const bool brk = (ro.x == 0.0 && ro.y == 0.0) || !(rr == rr);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc[SC_ITERS] = iters;
    sc[SC_LASTRR] = rr;
    sc[SC_PQ + 2 * Q] = 0.0;
    sc[SC_PQ + 2 * Q + 1] = 0.0;
    if (conv) sc[SC_STATUS] = EFGK_CONVERGED;
    else if (brk) sc[SC_STATUS] = EFGK_BREAKDOWN;
    else if (out) sc[SC_STATUS] = EFGK_MAXIT;
  }
  if (conv || out || brk) return;
  const double2 beta = cdiv(rn, ro);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 zi;
    if (zvec) {
      zi = zvec[i];
    } else {
      zi = cmul(dinv[i], r[i]);
      if (use_aux) zi = cadd(zi, aux_term(ax, i));
    }
    p[i] = cfma(beta, p[i], zi);
  }
}

__global__ void __launch_bounds__(kBS) cocg_init(int n, const double2 *__restrict__ b,
                                                const double2 *__restrict__ dinv, double2 *x, double2 *r,
                                                double *sc, int rho_diag) {
  double v[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 bi = b[i];
    x[i] = make_double2(0.0, 0.0);
    r[i] = bi;
    if (rho_diag) {
      const double2 rz = cmul(bi, cmul(dinv[i], bi));
      v[0] += rz.x;
      v[1] += rz.y;
    }
    v[2] += bi.x * bi.x + bi.y * bi.y;
  }
  // rho_0 goes to parity slot 1 (read as rho_k by iteration 0).
  double *const dst[3] = {sc + SC_RHO + 2, sc + SC_RHO + 3, sc + SC_BB};
  block_reduce_add<3>(v, dst);
}

// p = D^-1 r (+ G t)
__global__ void __launch_bounds__(kBS) precond_apply_kernel(int n, const double2 *__restrict__ dinv,
                                                           const double2 *__restrict__ r, double2 *z, const Aux ax,
                                                           int use_aux, const double *sc, int sb_status) {
  if (sc && sc[sb_status] != 0.0) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 zi = cmul(dinv[i], r[i]);
    if (use_aux) zi = cadd(zi, aux_term(ax, i));
    z[i] = zi;
  }
}

__global__ void diag_inverse_kernel(int n, const int *__restrict__ diag, const double2 *__restrict__ vals,
                                    double2 *dinv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 d = vals[diag[i]];
    const double m = d.x * d.x + d.y * d.y;
    dinv[i] = m > 0.0 ? make_double2(d.x / m, -d.y / m) : make_double2(1.0, 0.0);
  }
}

// diag(G^T A G): for edge row e (tail a, head b) and neighbour column c,
// g(c, m) = [head(c) == m] - [tail(c) == m]; dn[a] -= sum_c A[e,c] g(c,a),
// dn[b] += sum_c A[e,c] g(c,b).
// diag(Pi^T A Pi): for edge row e (nodes a, b) and neighbour column c, the
// entry adds w_e,d w_c,d A[e,c] to (n, d) for each end node n of e that is
// also an end node of c.
__global__ void aux_pi_diag_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colidx,
                                   const double2 *__restrict__ vals, const int2 *__restrict__ enodes,
                                   const double *__restrict__ piw, double scale, double2 *dp) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int2 ab = enodes[e];
    if (ab.x < 0) continue;
    double2 ua[3] = {}, ub[3] = {};
    for (int k = rowptr[e]; k < rowptr[e + 1]; ++k) {
      const int c = colidx[k];
      const int2 cn = enodes[c];
      if (cn.x < 0) continue;
      const double2 a = vals[k];
      const bool sa = cn.x == ab.x || cn.y == ab.x, sb = cn.x == ab.y || cn.y == ab.y;
      for (int d = 0; d < 3; ++d) {
        const double ww = scale * piw[3 * e + d] * piw[3 * c + d];
        if (sa) ua[d].x += ww * a.x, ua[d].y += ww * a.y;
        if (sb) ub[d].x += ww * a.x, ub[d].y += ww * a.y;
      }
    }
    for (int d = 0; d < 3; ++d) {
      atomicAdd(&dp[3 * ab.x + d].x, ua[d].x);
      atomicAdd(&dp[3 * ab.x + d].y, ua[d].y);
      atomicAdd(&dp[3 * ab.y + d].x, ub[d].x);
      atomicAdd(&dp[3 * ab.y + d].y, ub[d].y);
    }
  }
}

__global__ void aux_diag_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colidx,
                                const double2 *__restrict__ vals, const int2 *__restrict__ enodes, double2 *dn) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int2 ab = enodes[e];
    if (ab.x < 0) continue;
    double2 ua = make_double2(0, 0), ub = make_double2(0, 0);
    for (int k = rowptr[e]; k < rowptr[e + 1]; ++k) {
      const int2 cn = enodes[colidx[k]];
      if (cn.x < 0) continue;
      const double2 a = vals[k];
      const double ga = (cn.y == ab.x) - (cn.x == ab.x);
      const double gb = (cn.y == ab.y) - (cn.x == ab.y);
      ua.x += ga * a.x;
      ua.y += ga * a.y;
      ub.x += gb * a.x;
      ub.y += gb * a.y;
    }
    atomicAdd(&dn[ab.x].x, -ua.x);
    atomicAdd(&dn[ab.x].y, -ua.y);
    atomicAdd(&dn[ab.y].x, ub.x);
    atomicAdd(&dn[ab.y].y, ub.y);
  }
}

__global__ void recip_kernel(int n, const double2 *__restrict__ d, double2 *out, double rel_floor,
                             const double *__restrict__ dmax) {
  const double floor2 = rel_floor * rel_floor * (*dmax);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 v = d[i];
    const double m = v.x * v.x + v.y * v.y;
    out[i] = m > floor2 && m > 0.0 ? make_double2(v.x / m, -v.y / m) : make_double2(0.0, 0.0);
  }
}

__global__ void absmax2_kernel(int n, const double2 *__restrict__ d, double *out) {
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = fmax(m, d[i].x * d[i].x + d[i].y * d[i].y);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) {
    // non-negative doubles order like their bit patterns
    atomicMax(reinterpret_cast<unsigned long long *>(out), __double_as_longlong(m));
  }
}

// ------------------------------------------------------------ block-Jacobi
// Diagonal blocks of kBJ consecutive rows, inverted once per solve; applied
// as z_I = B_I^-1 r_I.  The preconditioner for matrices without mesh data
// (solve_linear on a CSR matrix given by the caller): on the WR-90 slab
// guide (24x12x60 cells, 10 GHz) COCG needs 3,665 iterations with 16-row
// blocks against 7,120 with Jacobi (CPU study, complex128).
constexpr int kBJ = EFGK_BJ_BS;
static_assert(2 * kBJ == 32, "one lane per column of [B | I]");

__device__ __forceinline__ double2 crecip(double2 a) {
  const double m = a.x * a.x + a.y * a.y;
  return make_double2(a.x / m, -a.y / m);
}

// One warp per block: [B | I] in shared memory, lane j owns column j;
// Gauss-Jordan with partial pivoting leaves B^-1 in the right half.
__global__ void __launch_bounds__(32) bjac_setup_kernel(int n, const int *__restrict__ rowptr,
                                                       const int *__restrict__ colidx,
                                                       const double2 *__restrict__ vals, double2 *binv,
                                                       int *nsing) {
  __shared__ double2 M[kBJ][2 * kBJ];
  const int lane = threadIdx.x;
  const int r0 = blockIdx.x * kBJ;
#pragma unroll
  for (int i = 0; i < kBJ; ++i) M[i][lane] = make_double2(lane == kBJ + i ? 1.0 : 0.0, 0.0);
  __syncwarp();
  double2 diag = make_double2(1.0, 0.0);  // lane i < kBJ: A[r0+i][r0+i] (1 for padding rows)
  if (lane < kBJ) {
    const int row = r0 + lane;
    if (row < n) {
      diag = make_double2(0.0, 0.0);
      for (int k = __ldg(rowptr + row); k < __ldg(rowptr + row + 1); ++k) {
        const int c = __ldg(colidx + k) - r0;
        if (c >= 0 && c < kBJ) {
          const double2 v = __ldg(vals + k);
          M[lane][c] = v;
          if (c == lane) diag = v;
        }
      }
    } else {
      M[lane][lane] = make_double2(1.0, 0.0);
    }
  }
  __syncwarp();
  bool singular = false;
  for (int k = 0; k < kBJ; ++k) {
    int piv = k;
    double best = -1.0;
    for (int i = k; i < kBJ; ++i) {
      const double2 v = M[i][k];
      const double m = v.x * v.x + v.y * v.y;
      if (m > best) best = m, piv = i;
    }
    if (!(best > 0.0) || !isfinite(best)) {  // same shared data in every lane: uniform
      singular = true;
      break;
    }
    if (piv != k) {
      const double2 a = M[k][lane];
      M[k][lane] = M[piv][lane];
      M[piv][lane] = a;
    }
    __syncwarp();
    const double2 pinv = crecip(M[k][k]);
    double2 f[kBJ];
#pragma unroll
    for (int i = 0; i < kBJ; ++i) f[i] = M[i][k];
    __syncwarp();
    const double2 mk = cmul(M[k][lane], pinv);
#pragma unroll
    for (int i = 0; i < kBJ; ++i) M[i][lane] = i == k ? mk : csub(M[i][lane], cmul(f[i], mk));
    __syncwarp();
  }
  // lane kBJ + j writes column j of the inverse (column-major per block)
  double2 dj = make_double2(__shfl_sync(0xffffffffu, diag.x, lane & (kBJ - 1)),
                            __shfl_sync(0xffffffffu, diag.y, lane & (kBJ - 1)));
  if (dj.x == 0.0 && dj.y == 0.0) dj = make_double2(1.0, 0.0);
  if (lane >= kBJ) {
    const int j = lane - kBJ;
    double2 *out = binv + (static_cast<long long>(blockIdx.x) * kBJ + j) * kBJ;
    if (!singular) {
#pragma unroll
      for (int i = 0; i < kBJ; ++i) out[i] = M[i][lane];
    } else {
      const double2 dinv = crecip(dj);
#pragma unroll
      for (int i = 0; i < kBJ; ++i) out[i] = i == j ? dinv : make_double2(0.0, 0.0);
    }
  }
  if (singular && lane == 0) atomicAdd(nsing, 1);
}

// z = B^-1 r per block (half a warp per block, lane i = row i); with
// rho_slot >= 0 also r^T z into sc[rho_slot], sc[rho_slot + 1].  Skips
// when sc[status] != 0 (status < 0: no check).
__global__ void __launch_bounds__(kBS) bjac_apply_kernel(int n, const double2 *__restrict__ binv,
                                                        const double2 *__restrict__ r, double2 *z, double *sc,
                                                        int rho_slot, int status) {
  if (status >= 0) {
    __shared__ int s_stop;
    if (threadIdx.x == 0) s_stop = sc[status] != 0.0;
    __syncthreads();
    if (s_stop) return;
  }
  const int nb = (n + kBJ - 1) / kBJ;
  const int half = (threadIdx.x >> 4) & 1, i = threadIdx.x & (kBJ - 1);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double v[2] = {0.0, 0.0};
  for (int base = 2 * warp; base < nb; base += 2 * nwarps) {  // uniform trip count per warp
    const int blk = base + half;
    const int row = blk * kBJ + i;
    const bool live = blk < nb && row < n;
    const double2 ri = live ? r[row] : make_double2(0.0, 0.0);
    double2 zi = make_double2(0.0, 0.0);
    const double2 *col = binv + static_cast<long long>(blk < nb ? blk : 0) * kBJ * kBJ + i;
#pragma unroll 4
    for (int j = 0; j < kBJ; ++j) {
      const double2 rj = make_double2(__shfl_sync(0xffffffffu, ri.x, (half << 4) + j),
                                      __shfl_sync(0xffffffffu, ri.y, (half << 4) + j));
      if (blk < nb) zi = cfma(__ldg(col + j * kBJ), rj, zi);
    }
    if (live) {
      z[row] = zi;
      const double2 rz = cmul(ri, zi);
      v[0] += rz.x;
      v[1] += rz.y;
    }
  }
  if (rho_slot >= 0) {
    double *const dst[2] = {sc + rho_slot, sc + rho_slot + 1};
    block_reduce_add<2>(v, dst);
  }
}

// ---------------------------------------------------------------- BiCGStab
// Scalar phases run in a single thread between vector phases.
__global__ void bicg_init(int n, const double2 *__restrict__ b, double2 *x, double2 *r, double2 *rhat,
                          double2 *p, double2 *v, double *sc) {
  double a[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 bi = b[i];
    x[i] = make_double2(0, 0);
    r[i] = bi;
    rhat[i] = bi;
    p[i] = make_double2(0, 0);
    v[i] = make_double2(0, 0);
    a[0] += bi.x * bi.x + bi.y * bi.y;  // rhat^H r = |b|^2
  }
  a[2] = a[0];
  double *const dst[3] = {sc + SB_RHR, nullptr, sc + SB_BB};
  block_reduce_add<3>(a, dst);
}

// p = r + beta (p - omega v)
__global__ void bicg_p(int n, const double2 *__restrict__ r, double2 *p, const double2 *__restrict__ v,
                       const double *sc) {
  if (sc[SB_STATUS] != 0.0) return;
  const double2 beta = make_double2(sc[SB_BETA], sc[SB_BETA + 1]);
  const double2 om = make_double2(sc[SB_OMEGA], sc[SB_OMEGA + 1]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 pi = csub(p[i], cmul(om, v[i]));
    p[i] = cfma(beta, pi, r[i]);
  }
}

// y = A x and acc += sum conj(w) y (and |y|^2 into acc2 if non-null)
__global__ void __launch_bounds__(kBS) bicg_spmv_dot(int n, const int *__restrict__ rowptr,
                                                    const int *__restrict__ colidx,
                                                    const double2 *__restrict__ vals,
                                                    const double2 *__restrict__ x, double2 *__restrict__ y,
                                                    const double2 *__restrict__ w, double *acc, double *acc2,
                                                    const double *sc) {
  if (sc[SB_STATUS] != 0.0) return;
  const int lane = threadIdx.x % kL;
  double a[3] = {0.0, 0.0, 0.0};
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) / kL; row < n; row += gridDim.x * blockDim.x / kL) {
    const double2 s = row_dot<kL>(row, lane, rowptr, colidx, vals, x);
    if (lane == 0) {
      y[row] = s;
      const double2 d = cconjmul(w[row], s);
      a[0] += d.x;
      a[1] += d.y;
      a[2] += s.x * s.x + s.y * s.y;
    }
  }
  double *const dst[3] = {acc, acc + 1, acc2};
  block_reduce_add<3>(a, dst);
}

__global__ void bicg_s(int n, const double2 *__restrict__ r, const double2 *__restrict__ v, double2 *s,
                       const double *sc) {
  if (sc[SB_STATUS] != 0.0) return;
  const double2 al = make_double2(sc[SB_ALPHA], sc[SB_ALPHA + 1]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s[i] = cfma(make_double2(-al.x, -al.y), v[i], r[i]);
}

__global__ void __launch_bounds__(kBS) bicg_xr(int n, double2 *x, double2 *r, const double2 *__restrict__ rhat,
                                              const double2 *__restrict__ phat,
                                              const double2 *__restrict__ shat, const double2 *__restrict__ s,
                                              const double2 *__restrict__ t, double *sc) {
  if (sc[SB_STATUS] != 0.0) return;
  const double2 al = make_double2(sc[SB_ALPHA], sc[SB_ALPHA + 1]);
  const double2 om = make_double2(sc[SB_OMEGA], sc[SB_OMEGA + 1]);
  double a[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 xi = cfma(al, phat[i], x[i]);
    x[i] = cfma(om, shat[i], xi);
    const double2 ri = cfma(make_double2(-om.x, -om.y), t[i], s[i]);
    r[i] = ri;
    const double2 d = cconjmul(rhat[i], ri);
    a[0] += d.x;
    a[1] += d.y;
    a[2] += ri.x * ri.x + ri.y * ri.y;
  }
  double *const dst[3] = {sc + SB_RHR, sc + SB_RHR + 1, sc + SB_RR};
  block_reduce_add<3>(a, dst);
}

// Scalar phases.  phase 0: before bicg_p (beta); 1: after v (alpha);
// 2: after t (omega); 3: after x/r (convergence).
__global__ void bicg_scalar(double *sc, int phase) {
  if (sc[SB_STATUS] != 0.0) return;
  auto ld = [&](int k) { return make_double2(sc[k], sc[k + 1]); };
  auto st = [&](int k, double2 v) {
    sc[k] = v.x;
    sc[k + 1] = v.y;
  };
  if (phase == 0) {
    const double2 rho_new = ld(SB_RHR), rho = ld(SB_RHO), al = ld(SB_ALPHA), om = ld(SB_OMEGA);
    if ((rho.x == 0 && rho.y == 0) || (om.x == 0 && om.y == 0)) {
      sc[SB_STATUS] = EFGK_BREAKDOWN;
      return;
    }
    st(SB_BETA, cmul(cdiv(rho_new, rho), cdiv(al, om)));
    st(SB_RHO, rho_new);
    sc[SB_RHR] = sc[SB_RHR + 1] = 0.0;
    sc[SB_RV] = sc[SB_RV + 1] = 0.0;
  } else if (phase == 1) {
    const double2 rv = ld(SB_RV), rho = ld(SB_RHO);
    if (rv.x == 0 && rv.y == 0) {
      sc[SB_STATUS] = EFGK_BREAKDOWN;
      return;
    }
    st(SB_ALPHA, cdiv(rho, rv));
    sc[SB_TS] = sc[SB_TS + 1] = sc[SB_TT] = 0.0;
  } else if (phase == 2) {
    const double tt = sc[SB_TT];
    if (tt == 0.0) {
      sc[SB_STATUS] = EFGK_BREAKDOWN;
      return;
    }
    // SB_TS holds sum conj(s) t = conj(t^H s).
    st(SB_OMEGA, make_double2(sc[SB_TS] / tt, -sc[SB_TS + 1] / tt));
    sc[SB_RR] = 0.0;
  } else {
    sc[SB_ITERS] += 1.0;
    const double rr = sc[SB_RR];
    sc[SB_LASTRR] = rr;
    if (rr <= sc[SB_TOL2] * sc[SB_BB]) sc[SB_STATUS] = EFGK_CONVERGED;
    else if (!(rr == rr)) sc[SB_STATUS] = EFGK_BREAKDOWN;
    else if (sc[SB_ITERS] >= sc[SB_MAXIT]) sc[SB_STATUS] = EFGK_MAXIT;
  }
}

// Node pass for a preconditioner application inside BiCGStab (no scalars).
__global__ void __launch_bounds__(kBS) aux_node_plain(const Aux ax, const double2 *__restrict__ r,
                                                     const double *sc) {
  if (sc && sc[SB_STATUS] != 0.0) return;
  for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < ax.nn; nd += gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int k = ax.nptr[nd]; k < ax.nptr[nd + 1]; ++k) {
      const double2 re = r[ax.nedge[k]];
      const double sg = ax.nsign[k];
      s.x += sg * re.x;
      s.y += sg * re.y;
    }
    ax.t[nd] = cmul(ax.dninv[nd], s);
  }
}

__global__ void port_overlap_kernel(const int *__restrict__ off, const int *__restrict__ idx,
                                    const double2 *__restrict__ c, const double2 *__restrict__ x, double2 *out) {
  const int list = blockIdx.x;
  double a[2] = {0.0, 0.0};
  for (int k = off[list] + threadIdx.x; k < off[list + 1]; k += blockDim.x) {
    const double2 d = cmul(c[k], x[idx[k]]);
    a[0] += d.x;
    a[1] += d.y;
  }
  __shared__ double sh[2][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < 2; ++k)
    for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
  if (lane == 0) {
    sh[0][warp] = a[0];
    sh[1][warp] = a[1];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0, s1 = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
      s0 += sh[0][w];
      s1 += sh[1][w];
    }
    out[list] = make_double2(s0, s1);
  }
}

inline const double2 *C2(const double *p) { return reinterpret_cast<const double2 *>(p); }
inline double2 *M2(double *p) { return reinterpret_cast<double2 *>(p); }

// Fixed grid: enough blocks to fill the GPU a few times over, no more (each
// block adds its partial sums with one atomic per accumulator).
int grid_for(long long work_items) {
  static int sms = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 132;
  }();
  const long long need = (work_items + kBS - 1) / kBS;
  const long long cap = 8LL * sms;
  return static_cast<int>(need < 1 ? 1 : (need < cap ? need : cap));
}

Aux make_aux(const EfgkAux *a) {
  Aux ax{};
  if (!a) return ax;
  ax.enodes = reinterpret_cast<const int2 *>(a->enodes);
  ax.nptr = a->nptr;
  ax.nedge = a->nedge;
  ax.nsign = reinterpret_cast<const signed char *>(a->nsign);
  ax.dninv = C2(a->dninv);
  ax.t = M2(a->t);
  ax.nn = a->nn;
  ax.npi = a->npi;
  ax.piw = a->piw;
  ax.dpinv = C2(a->dpinv);
  ax.tp = M2(a->tp);
  ax.bjinv = C2(a->bj_inv);
  ax.z = M2(a->z);
  ax.bs = a->bj_bs;
  return ax;
}

inline bool use_bjac(const EfgkAux *a) { return a && a->bj_bs > 0 && a->bj_inv && a->z; }
inline bool use_nodes(const EfgkAux *a) { return a && !use_bjac(a) && a->nn > 0; }

int bjac_grid(int n) {
  const long long warps = ((static_cast<long long>(n) + kBJ - 1) / kBJ + 1) / 2;
  return grid_for(warps * 32);
}

}  // namespace

extern "C" int efgk_spmv64(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                           const double *x, double *y, efgk_stream_t stream) {
  if (n <= 0) return 0;
  spmv64_kernel<<<grid_for(static_cast<long long>(n) * kL), kBS, 0, stream>>>(n, rowptr, colidx, C2(vals), C2(x),
                                                                             M2(y));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_spmv32(int32_t n, const int32_t *rowptr, const int32_t *colidx, const float *vals,
                           const float *x, float *y, efgk_stream_t stream) {
  if (n <= 0) return 0;
  // One wave of resident blocks (grid-stride over the rows beyond it).
  static const int wave = [] {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, spmv32_kernel, kBS, 0);
    return (sms > 0 ? sms : 132) * (per_sm > 0 ? per_sm : 4);
  }();
  const long long need = (static_cast<long long>(n) * kL32 + kBS - 1) / kBS;
  const int grid = static_cast<int>(need < wave ? need : wave);
  spmv32_kernel<<<grid, kBS, 0, stream>>>(n, rowptr, colidx, reinterpret_cast<const float2 *>(vals),
                                          reinterpret_cast<const float2 *>(x), reinterpret_cast<float2 *>(y));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_diag_inverse64(int32_t n, const int32_t *diag_slot, const double *vals, double *dinv,
                                   efgk_stream_t stream) {
  if (n <= 0) return 0;
  diag_inverse_kernel<<<grid_for(n), kBS, 0, stream>>>(n, diag_slot, C2(vals), M2(dinv));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_aux_diag64(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                               const int32_t *enodes, double *dn, efgk_stream_t stream) {
  if (n <= 0) return 0;
  aux_diag_kernel<<<grid_for(n), kBS, 0, stream>>>(n, rowptr, colidx, C2(vals),
                                                  reinterpret_cast<const int2 *>(enodes), M2(dn));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_aux_pi_diag64(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                                  const int32_t *enodes, const double *piw, double scale, double *dp,
                                  efgk_stream_t stream) {
  if (n <= 0) return 0;
  aux_pi_diag_kernel<<<grid_for(n), kBS, 0, stream>>>(n, rowptr, colidx, C2(vals),
                                                     reinterpret_cast<const int2 *>(enodes), piw, scale, M2(dp));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_aux_recip64(int32_t nn, const double *dn, double rel_floor, double *scratch, double *dninv,
                                efgk_stream_t stream) {
  if (nn <= 0) return 0;
  cudaMemsetAsync(scratch, 0, sizeof(double), stream);
  absmax2_kernel<<<grid_for(nn), kBS, 0, stream>>>(nn, C2(dn), scratch);
  recip_kernel<<<grid_for(nn), kBS, 0, stream>>>(nn, C2(dn), M2(dninv), rel_floor, scratch);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_bjacobi_setup64(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                                    double *binv, int32_t *nsingular, efgk_stream_t stream) {
  if (n <= 0) return 0;
  bjac_setup_kernel<<<(n + kBJ - 1) / kBJ, 32, 0, stream>>>(n, rowptr, colidx, C2(vals), M2(binv), nsingular);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_cocg64_init(int32_t n, const double *b, const double *dinv, double *x, double *r, double *p,
                                double *sc, const struct EfgkAux *aux, efgk_stream_t stream) {
  const bool bj = use_bjac(aux);
  cocg_init<<<grid_for(n), kBS, 0, stream>>>(n, C2(b), C2(dinv), M2(x), M2(r), sc, bj ? 0 : 1);
  const Aux ax = make_aux(aux);
  if (bj) {
    // p = B^-1 r, rho_0 = r^T p into parity slot 1
    bjac_apply_kernel<<<bjac_grid(n), kBS, 0, stream>>>(n, ax.bjinv, C2(r), M2(p), sc, SC_RHO + 2, -1);
    return static_cast<int>(cudaGetLastError());
  }
  if (use_nodes(aux)) aux_node_kernel<<<grid_for(aux->nn), kBS, 0, stream>>>(ax, C2(r), sc, 1, 0);
  precond_apply_kernel<<<grid_for(n), kBS, 0, stream>>>(n, C2(dinv), C2(r), M2(p), ax, use_nodes(aux), nullptr, 0);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_cocg64_step(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                                const double *dinv, double *x, double *r, double *p, double *q, double *sc,
                                int parity, const struct EfgkAux *aux, efgk_stream_t stream) {
  const Aux ax = make_aux(aux);
  const bool bj = use_bjac(aux);
  cocg_k1<<<grid_for(static_cast<long long>(n) * kL), kBS, 0, stream>>>(n, rowptr, colidx, C2(vals), C2(p), M2(q),
                                                                        sc, parity);
  cocg_k2<<<grid_for(n), kBS, 0, stream>>>(n, C2(dinv), M2(x), M2(r), C2(p), C2(q), sc, parity, bj ? 0 : 1);
  if (bj)
    bjac_apply_kernel<<<bjac_grid(n), kBS, 0, stream>>>(n, ax.bjinv, C2(r), ax.z, sc, SC_RHO + 2 * parity,
                                                        SC_STATUS);
  else if (use_nodes(aux))
    aux_node_kernel<<<grid_for(aux->nn), kBS, 0, stream>>>(ax, C2(r), sc, parity, 1);
  cocg_k3<<<grid_for(n), kBS, 0, stream>>>(n, C2(dinv), C2(r), M2(p), sc, parity, ax, use_nodes(aux),
                                           bj ? ax.z : nullptr);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_bicgstab64_init(int32_t n, const double *b, double *x, double *r, double *rhat, double *p,
                                    double *v, double *sc, efgk_stream_t stream) {
  bicg_init<<<grid_for(n), kBS, 0, stream>>>(n, C2(b), M2(x), M2(r), M2(rhat), M2(p), M2(v), sc);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_bicgstab64_step(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                                    const double *dinv, double *x, double *r, const double *rhat, double *p,
                                    double *v, double *s, double *t, double *phat, double *shat, double *sc,
                                    const struct EfgkAux *aux, efgk_stream_t stream) {
  const int gv = grid_for(n), gm = grid_for(static_cast<long long>(n) * kL);
  const Aux ax = make_aux(aux);
  const bool bj = use_bjac(aux);
  const int ua = use_nodes(aux);
  auto precond = [&](const double *in, double *out) {
    if (bj) {
      bjac_apply_kernel<<<bjac_grid(n), kBS, 0, stream>>>(n, ax.bjinv, C2(in), M2(out), sc, -1, SB_STATUS);
      return;
    }
    if (ua) aux_node_plain<<<grid_for(aux->nn), kBS, 0, stream>>>(ax, C2(in), sc);
    precond_apply_kernel<<<gv, kBS, 0, stream>>>(n, C2(dinv), C2(in), M2(out), ax, ua, sc, SB_STATUS);
  };
  bicg_scalar<<<1, 1, 0, stream>>>(sc, 0);
  bicg_p<<<gv, kBS, 0, stream>>>(n, C2(r), M2(p), C2(v), sc);
  precond(p, phat);
  bicg_spmv_dot<<<gm, kBS, 0, stream>>>(n, rowptr, colidx, C2(vals), C2(phat), M2(v), C2(rhat), sc + SB_RV, nullptr,
                                        sc);
  bicg_scalar<<<1, 1, 0, stream>>>(sc, 1);
  bicg_s<<<gv, kBS, 0, stream>>>(n, C2(r), C2(v), M2(s), sc);
  precond(s, shat);
  // t = A shat with sum conj(s) t and |t|^2.
  bicg_spmv_dot<<<gm, kBS, 0, stream>>>(n, rowptr, colidx, C2(vals), C2(shat), M2(t), C2(s), sc + SB_TS, sc + SB_TT,
                                        sc);
  bicg_scalar<<<1, 1, 0, stream>>>(sc, 2);
  bicg_xr<<<gv, kBS, 0, stream>>>(n, M2(x), M2(r), C2(rhat), C2(phat), C2(shat), C2(s), C2(t), sc);
  bicg_scalar<<<1, 1, 0, stream>>>(sc, 3);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_port_overlaps64(int32_t nlists, const int32_t *offsets, const int32_t *idx, const double *c,
                                    const double *x, int64_t x_stride, double *out, efgk_stream_t stream) {
  (void)x_stride;
  if (nlists <= 0) return 0;
  port_overlap_kernel<<<nlists, 256, 0, stream>>>(offsets, idx, C2(c), C2(x), M2(out));
  return static_cast<int>(cudaGetLastError());
}
