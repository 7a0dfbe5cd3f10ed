// Batched complex64 COCG kernels with FP64 residual replacement.
//
// All right-hand sides of one row (every frequency x active port of one mesh
// instance) are contiguous, so one pass over a matrix row serves all of them:
// the CSR column index and the K (real FP32) and M (complex FP32) values are
// read once per row and re-used R times, and the x gather of a column is one
// contiguous R*8-byte segment.  The operator is formed on the fly,
//   (K - k0_f^2 M) x  +  port-face terms  (see batch_layout.h),
// so no per-frequency matrix is ever stored.
//
// Per iteration (parity P = k & 1):
//   spmm      q = A p               + per-(instance, rhs) p^T q
//   update    x_c += alpha p, r -= alpha q, rho' = r^T D^-1 r, |r|^2
//   pupdate   p = D^-1 r + beta p   (+ convergence test on refinement steps)
// and on refinement steps, between update and pupdate,
//   flush     x64 += x_c, x_c = 0
//   residual  r = b - A x64 in FP64 (true residual), rho' and |r|^2 again
#include <cuda_runtime.h>

#include "batch_layout.h"
#include "edgefem_gb300_kernels.h"

namespace {

constexpr int kBS = 256;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 crecipf(float2 d) {
  const float m = d.x * d.x + d.y * d.y;
  return m > 0.f ? make_float2(d.x / m, -d.y / m) : make_float2(1.f, 0.f);
}
__device__ __forceinline__ double2 cdivd(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

template <int V>
struct CVec {
  float2 v[V];
};

template <int V>
__device__ __forceinline__ CVec<V> ldv(const float2 *p) {
  CVec<V> o;
  if constexpr (V == 4) {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
    const float4 b = __ldg(reinterpret_cast<const float4 *>(p) + 1);
    o.v[0] = make_float2(a.x, a.y);
    o.v[1] = make_float2(a.z, a.w);
    o.v[2] = make_float2(b.x, b.y);
    o.v[3] = make_float2(b.z, b.w);
  } else if constexpr (V == 2) {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
    o.v[0] = make_float2(a.x, a.y);
    o.v[1] = make_float2(a.z, a.w);
  } else {
#pragma unroll
    for (int i = 0; i < V; ++i) o.v[i] = __ldg(p + i);
  }
  return o;
}
// Plain (non-read-only-path) load for data written earlier in the same kernel sequence.
template <int V>
__device__ __forceinline__ CVec<V> ldv_rw(const float2 *p) {
  CVec<V> o;
  if constexpr (V == 4) {
    const float4 a = reinterpret_cast<const float4 *>(p)[0];
    const float4 b = reinterpret_cast<const float4 *>(p)[1];
    o.v[0] = make_float2(a.x, a.y);
    o.v[1] = make_float2(a.z, a.w);
    o.v[2] = make_float2(b.x, b.y);
    o.v[3] = make_float2(b.z, b.w);
  } else if constexpr (V == 2) {
    const float4 a = reinterpret_cast<const float4 *>(p)[0];
    o.v[0] = make_float2(a.x, a.y);
    o.v[1] = make_float2(a.z, a.w);
  } else {
#pragma unroll
    for (int i = 0; i < V; ++i) o.v[i] = p[i];
  }
  return o;
}
template <int V>
__device__ __forceinline__ void stv(float2 *p, const CVec<V> &o) {
  if constexpr (V == 4) {
    reinterpret_cast<float4 *>(p)[0] = make_float4(o.v[0].x, o.v[0].y, o.v[1].x, o.v[1].y);
    reinterpret_cast<float4 *>(p)[1] = make_float4(o.v[2].x, o.v[2].y, o.v[3].x, o.v[3].y);
  } else if constexpr (V == 2) {
    reinterpret_cast<float4 *>(p)[0] = make_float4(o.v[0].x, o.v[0].y, o.v[1].x, o.v[1].y);
  } else {
#pragma unroll
    for (int i = 0; i < V; ++i) p[i] = o.v[i];
  }
}

// Zero a per-(instance, rhs) accumulator array of `count` doubles from one block.
__device__ __forceinline__ void block_zero(double *a, int count) {
  for (int i = threadIdx.x; i < count; i += blockDim.x) a[i] = 0.0;
}

// Jacobi diagonal of A_bf at row for rhs.
__device__ __forceinline__ float2 diag32(const EfgkBatch &bt, int row, int rhs, int b) {
  const float kd = __ldg(bt.kd32 + row);
  const float2 md = __ldg(bt.md32 + row);
  const float k2 = __ldg(bt.k0sq32 + rhs);
  float2 d = make_float2(kd - k2 * md.x, -k2 * md.y);
  const int s = __ldg(bt.sidx + row);
  if (s >= 0) {
    for (int p = 0; p < bt.P; ++p) {
      const float sd = __ldg(bt.sdiag32 + s * bt.P + p);
      if (sd != 0.f) {
        const float2 c = __ldg(bt.scoef32 + (b * bt.P + p) * bt.R + rhs);
        d.x += c.x * sd;
        d.y += c.y * sd;
      }
    }
  }
  return d;
}

// ------------------------------------------------------------------ SpMM
template <int V>
__global__ void __launch_bounds__(kBS) batch_spmm_kernel(const EfgkBatch bt, const int P) {
  const int R = bt.R;
  const int G = R / V;  // lanes per row group (divides 32)
  const int chunk = blockIdx.x;
  const int b = bt.chunk_inst[chunk], r0 = bt.chunk_begin[chunk], r1 = bt.chunk_end[chunk];
  const int BR = bt.B * R;
  if (blockIdx.x == 0) {
    block_zero(bt.rho + P * 2 * BR, 2 * BR);
    block_zero(bt.rr + P * BR, BR);
  }
  const int group = threadIdx.x / G, lane = threadIdx.x % G, ngroups = kBS / G;
  const int rhs0 = lane * V;
  float k2[V];
#pragma unroll
  for (int v = 0; v < V; ++v) k2[v] = __ldg(bt.k0sq32 + rhs0 + v);
  float dot[2][V];
#pragma unroll
  for (int v = 0; v < V; ++v) dot[0][v] = dot[1][v] = 0.f;

  for (int base = r0; ; base += ngroups) {
    const int row = base + group;
    const bool active = row < r1;
    if (__all_sync(kFull, !active)) break;
    int kb = 0, ke = 0;
    if (active) {
      kb = __ldg(bt.rowptr + row);
      ke = __ldg(bt.rowptr + row + 1);
    }
    const int nnz = ke - kb;
    const int maxnnz = __reduce_max_sync(kFull, nnz);
    CVec<V> acc;
#pragma unroll
    for (int v = 0; v < V; ++v) acc.v[v] = make_float2(0.f, 0.f);
    for (int k0 = 0; k0 < maxnnz; k0 += G) {
      int c = 0;
      float kv = 0.f, mx = 0.f, my = 0.f;
      if (k0 + lane < nnz) {
        const int k = kb + k0 + lane;
        c = __ldg(bt.colidx + k);
        kv = __ldg(bt.K32 + k);
        const float2 m = __ldg(bt.M32 + k);
        mx = m.x;
        my = m.y;
      }
      const int cnt = nnz - k0;
      const int jmax = min(G, maxnnz - k0);
#pragma unroll 4
      for (int j = 0; j < jmax; ++j) {
        const int cj = __shfl_sync(kFull, c, j, G);
        const float kj = __shfl_sync(kFull, kv, j, G);
        const float mjx = __shfl_sync(kFull, mx, j, G);
        const float mjy = __shfl_sync(kFull, my, j, G);
        if (j < cnt) {
          const CVec<V> xv = ldv<V>(bt.p + static_cast<long long>(cj) * R + rhs0);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const float ar = fmaf(-k2[v], mjx, kj), ai = -k2[v] * mjy;
            acc.v[v].x = fmaf(ar, xv.v[v].x, fmaf(-ai, xv.v[v].y, acc.v[v].x));
            acc.v[v].y = fmaf(ar, xv.v[v].y, fmaf(ai, xv.v[v].x, acc.v[v].y));
          }
        }
      }
    }
    if (active) {
      const int s = __ldg(bt.sidx + row);
      if (s >= 0) {
        for (int e = __ldg(bt.sptr + s); e < __ldg(bt.sptr + s + 1); ++e) {
          const int cj = __ldg(bt.scol + e);
          const float val = __ldg(bt.sval32 + e);
          const int ci = __ldg(bt.scidx + e);
          const CVec<V> xv = ldv<V>(bt.p + static_cast<long long>(cj) * R + rhs0);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const float2 cf = __ldg(bt.scoef32 + ci * R + rhs0 + v);
            const float2 t = cmulf(make_float2(cf.x * val, cf.y * val), xv.v[v]);
            acc.v[v].x += t.x;
            acc.v[v].y += t.y;
          }
        }
      }
      stv<V>(bt.q + static_cast<long long>(row) * R + rhs0, acc);
      const CVec<V> pv = ldv<V>(bt.p + static_cast<long long>(row) * R + rhs0);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const float2 d = cmulf(pv.v[v], acc.v[v]);
        dot[0][v] += d.x;
        dot[1][v] += d.y;
      }
    }
  }
  // Block reduction: groups share rhs slots.
  __shared__ float sh[2][kBS * 4];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    sh[0][threadIdx.x * V + v] = dot[0][v];
    sh[1][threadIdx.x * V + v] = dot[1][v];
  }
  __syncthreads();
  for (int rhs = threadIdx.x; rhs < R; rhs += blockDim.x) {
    // thread t slot v holds rhs (t % G) * V + v  -> flat index t*V + v
    double sre = 0.0, sim = 0.0;
    const int l = rhs / V, v = rhs % V;
    for (int g = 0; g < ngroups; ++g) {
      const int t = g * G + l;
      sre += sh[0][t * V + v];
      sim += sh[1][t * V + v];
    }
    double *dst = bt.pq + P * 2 * BR + 2 * (static_cast<long long>(b) * R + rhs);
    atomicAdd(dst, sre);
    atomicAdd(dst + 1, sim);
  }
}

// ------------------------------------------------------------ vector phases
// Thread owns W = 4 consecutive right-hand sides of one row; R % 4 == 0 and
// (kBS * 4) % R == 0, so a thread's rhs set is fixed across its rows.
constexpr int W = 4;

__device__ __forceinline__ int chunk_elems(const EfgkBatch &bt, int r0, int r1) { return (r1 - r0) * bt.R; }

__global__ void __launch_bounds__(kBS) batch_update_kernel(const EfgkBatch bt, const int P) {
  const int R = bt.R, BR = bt.B * R;
  const int chunk = blockIdx.x;
  const int b = bt.chunk_inst[chunk], r0 = bt.chunk_begin[chunk], r1 = bt.chunk_end[chunk];
  const int Q = 1 - P;
  const int rhs0 = (threadIdx.x * W) % R;
  float2 alpha[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const long long i = static_cast<long long>(b) * R + rhs0 + w;
    const double2 rho = make_double2(bt.rho[Q * 2 * BR + 2 * i], bt.rho[Q * 2 * BR + 2 * i + 1]);
    const double2 pq = make_double2(bt.pq[P * 2 * BR + 2 * i], bt.pq[P * 2 * BR + 2 * i + 1]);
    double2 a = cdivd(rho, pq);
    if (bt.status[i] != 0 || !(isfinite(a.x) && isfinite(a.y))) a = make_double2(0.0, 0.0);
    alpha[w] = make_float2(static_cast<float>(a.x), static_cast<float>(a.y));
  }
  float part[3][W];
#pragma unroll
  for (int w = 0; w < W; ++w) part[0][w] = part[1][w] = part[2][w] = 0.f;
  const long long base = static_cast<long long>(r0) * R;
  const int total = chunk_elems(bt, r0, r1);
  for (int e = threadIdx.x * W; e < total; e += kBS * W) {
    const int row = r0 + e / R;
    const long long o = base + e;
    const CVec<4> pv = ldv_rw<4>(bt.p + o), qv = ldv_rw<4>(bt.q + o);
    CVec<4> xv = ldv_rw<4>(bt.xc + o), rv = ldv_rw<4>(bt.r + o);
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const float2 ap = cmulf(alpha[w], pv.v[w]), aq = cmulf(alpha[w], qv.v[w]);
      xv.v[w].x += ap.x;
      xv.v[w].y += ap.y;
      rv.v[w].x -= aq.x;
      rv.v[w].y -= aq.y;
      const float2 z = cmulf(crecipf(diag32(bt, row, rhs0 + w, b)), rv.v[w]);
      const float2 rz = cmulf(rv.v[w], z);
      part[0][w] += rz.x;
      part[1][w] += rz.y;
      part[2][w] += rv.v[w].x * rv.v[w].x + rv.v[w].y * rv.v[w].y;
    }
    stv<4>(bt.xc + o, xv);
    stv<4>(bt.r + o, rv);
  }
  __shared__ float sh[3][kBS * W];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int w = 0; w < W; ++w) sh[k][threadIdx.x * W + w] = part[k][w];
  __syncthreads();
  for (int rhs = threadIdx.x; rhs < R; rhs += blockDim.x) {
    double s0 = 0, s1 = 0, s2 = 0;
    for (int i = rhs; i < kBS * W; i += R) {
      s0 += sh[0][i];
      s1 += sh[1][i];
      s2 += sh[2][i];
    }
    const long long idx = static_cast<long long>(b) * R + rhs;
    atomicAdd(bt.rho + P * 2 * BR + 2 * idx, s0);
    atomicAdd(bt.rho + P * 2 * BR + 2 * idx + 1, s1);
    atomicAdd(bt.rr + P * BR + idx, s2);
  }
}

__global__ void __launch_bounds__(kBS) batch_pupdate_kernel(const EfgkBatch bt, const int P, const int check) {
  const int R = bt.R, BR = bt.B * R;
  const int chunk = blockIdx.x;
  const int b = bt.chunk_inst[chunk], r0 = bt.chunk_begin[chunk], r1 = bt.chunk_end[chunk];
  const int Q = 1 - P;
  if (blockIdx.x == 0) {
    block_zero(bt.pq + Q * 2 * BR, 2 * BR);
    const int it = bt.it_count[0] + 1;
    for (int i = threadIdx.x; i < BR; i += blockDim.x) {
      if (bt.status[i] != 0) continue;
      const double rr = bt.rr[P * BR + i];
      const double2 rn = make_double2(bt.rho[P * 2 * BR + 2 * i], bt.rho[P * 2 * BR + 2 * i + 1]);
      if (check && rr <= bt.tol2 * bt.bb[i]) {
        bt.status[i] = 1;
        bt.iters[i] = it;
      } else if (!(isfinite(rr) && isfinite(rn.x) && isfinite(rn.y))) {
        bt.status[i] = 2;
        bt.iters[i] = it;
      } else if (it >= bt.max_iters) {
        bt.status[i] = 3;
        bt.iters[i] = it;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) bt.it_count[0] = it;
  }
  const int rhs0 = (threadIdx.x * W) % R;
  float2 beta[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const long long i = static_cast<long long>(b) * R + rhs0 + w;
    const double2 rn = make_double2(bt.rho[P * 2 * BR + 2 * i], bt.rho[P * 2 * BR + 2 * i + 1]);
    const double2 ro = make_double2(bt.rho[Q * 2 * BR + 2 * i], bt.rho[Q * 2 * BR + 2 * i + 1]);
    double2 be = cdivd(rn, ro);
    if (!(isfinite(be.x) && isfinite(be.y))) be = make_double2(0.0, 0.0);
    beta[w] = make_float2(static_cast<float>(be.x), static_cast<float>(be.y));
  }
  const long long base = static_cast<long long>(r0) * R;
  const int total = chunk_elems(bt, r0, r1);
  for (int e = threadIdx.x * W; e < total; e += kBS * W) {
    const int row = r0 + e / R;
    const long long o = base + e;
    const CVec<4> rv = ldv_rw<4>(bt.r + o);
    CVec<4> pv = ldv_rw<4>(bt.p + o);
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const float2 z = cmulf(crecipf(diag32(bt, row, rhs0 + w, b)), rv.v[w]);
      const float2 bp = cmulf(beta[w], pv.v[w]);
      pv.v[w] = make_float2(z.x + bp.x, z.y + bp.y);
    }
    stv<4>(bt.p + o, pv);
  }
}

// x64 += xc, xc = 0 (and clear the accumulators the residual pass refills).
__global__ void __launch_bounds__(kBS) batch_flush_kernel(const EfgkBatch bt, const int P) {
  const int R = bt.R, BR = bt.B * R;
  if (blockIdx.x == 0 && P >= 0) {
    block_zero(bt.rho + P * 2 * BR, 2 * BR);
    block_zero(bt.rr + P * BR, BR);
  }
  const long long total = static_cast<long long>(bt.N) * R;
  for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float2 c = bt.xc[e];
    double2 x = bt.x64[e];
    x.x += c.x;
    x.y += c.y;
    bt.x64[e] = x;
    bt.xc[e] = make_float2(0.f, 0.f);
  }
}

// True residual in FP64: r = b - A x64, stored as complex64; rho' = r^T D^-1 r
// and |r|^2 (FP64) into parity slot P.  One lane per right-hand side, R/G
// lanes per row group as in the SpMM (G = min(R, 32)).
__global__ void __launch_bounds__(kBS) batch_residual_kernel(const EfgkBatch bt, const int P) {
  const int R = bt.R, BR = bt.B * R;
  const int G = R < 32 ? R : 32;
  const int VR = R / G;  // rhs per lane
  const int chunk = blockIdx.x;
  const int b = bt.chunk_inst[chunk], r0 = bt.chunk_begin[chunk], r1 = bt.chunk_end[chunk];
  const int group = threadIdx.x / G, lane = threadIdx.x % G, ngroups = kBS / G;
  double acc_rz[2][4], acc_rr[4];
  for (int v = 0; v < 4; ++v) acc_rz[0][v] = acc_rz[1][v] = acc_rr[v] = 0.0;
  for (int row = r0 + group; row < r1; row += ngroups) {
    const int kb = __ldg(bt.rowptr + row), ke = __ldg(bt.rowptr + row + 1);
    const int s = __ldg(bt.sidx + row);
    for (int v = 0; v < VR; ++v) {
      const int rhs = lane + v * G;
      const double k2 = __ldg(bt.k0sq64 + rhs);
      double ax = 0.0, ay = 0.0;
      for (int k = kb; k < ke; ++k) {
        const int c = __ldg(bt.colidx + k);
        const double kv = __ldg(bt.K64 + k);
        const double2 m = __ldg(bt.M64 + k);
        const double2 x = bt.x64[static_cast<long long>(c) * R + rhs];
        const double ar = kv - k2 * m.x, ai = -k2 * m.y;
        ax += ar * x.x - ai * x.y;
        ay += ar * x.y + ai * x.x;
      }
      double bx = 0.0, by = 0.0;
      if (s >= 0) {
        for (int e = __ldg(bt.sptr + s); e < __ldg(bt.sptr + s + 1); ++e) {
          const int c = __ldg(bt.scol + e);
          const double val = __ldg(bt.sval64 + e);
          const double2 cf = __ldg(bt.scoef64 + __ldg(bt.scidx + e) * R + rhs);
          const double2 x = bt.x64[static_cast<long long>(c) * R + rhs];
          ax += val * (cf.x * x.x - cf.y * x.y);
          ay += val * (cf.x * x.y + cf.y * x.x);
        }
        // b = 2 * coef(b, a, f) * c_a[row] for active port a = rhs % P
        if (rhs < bt.F * bt.P) {
          const int a = rhs % bt.P;
          const double2 cf = __ldg(bt.scoef64 + (b * bt.P + a) * R + rhs);
          const double2 cv = __ldg(bt.cval + s * bt.P + a);
          bx = 2.0 * (cf.x * cv.x - cf.y * cv.y);
          by = 2.0 * (cf.x * cv.y + cf.y * cv.x);
        }
      }
      const double rx = bx - ax, ry = by - ay;
      const float2 r32 = make_float2(static_cast<float>(rx), static_cast<float>(ry));
      bt.r[static_cast<long long>(row) * R + rhs] = r32;
      const float2 z = cmulf(crecipf(diag32(bt, row, rhs, b)), r32);
      const float2 rz = cmulf(r32, z);
      acc_rz[0][v] += rz.x;
      acc_rz[1][v] += rz.y;
      acc_rr[v] += rx * rx + ry * ry;
    }
  }
  __shared__ double sh[3][kBS * 4];
  for (int v = 0; v < 4; ++v) {
    sh[0][threadIdx.x * 4 + v] = acc_rz[0][v];
    sh[1][threadIdx.x * 4 + v] = acc_rz[1][v];
    sh[2][threadIdx.x * 4 + v] = acc_rr[v];
  }
  __syncthreads();
  for (int rhs = threadIdx.x; rhs < R; rhs += blockDim.x) {
    const int l = rhs % G, v = rhs / G;
    double s0 = 0, s1 = 0, s2 = 0;
    for (int g = 0; g < ngroups; ++g) {
      const int t = g * G + l;
      s0 += sh[0][t * 4 + v];
      s1 += sh[1][t * 4 + v];
      s2 += sh[2][t * 4 + v];
    }
    const long long idx = static_cast<long long>(b) * R + rhs;
    atomicAdd(bt.rho + P * 2 * BR + 2 * idx, s0);
    atomicAdd(bt.rho + P * 2 * BR + 2 * idx + 1, s1);
    atomicAdd(bt.rr + P * BR + idx, s2);
  }
}

// After the first residual pass: |b|^2, p = D^-1 r, status.
__global__ void __launch_bounds__(kBS) batch_init_finish_kernel(const EfgkBatch bt) {
  const int R = bt.R, BR = bt.B * R;
  const int chunk = blockIdx.x;
  const int b = bt.chunk_inst[chunk], r0 = bt.chunk_begin[chunk], r1 = bt.chunk_end[chunk];
  if (blockIdx.x == 0) {
    for (int i = threadIdx.x; i < BR; i += blockDim.x) {
      bt.bb[i] = bt.rr[1 * BR + i];
      bt.status[i] = bt.bb[i] > 0.0 ? 0 : 1;
      bt.iters[i] = 0;
    }
    if (threadIdx.x == 0) bt.it_count[0] = 0;
  }
  const int rhs0 = (threadIdx.x * W) % R;
  const long long base = static_cast<long long>(r0) * R;
  const int total = chunk_elems(bt, r0, r1);
  for (int e = threadIdx.x * W; e < total; e += kBS * W) {
    const int row = r0 + e / R;
    const long long o = base + e;
    const CVec<4> rv = ldv_rw<4>(bt.r + o);
    CVec<4> pv;
#pragma unroll
    for (int w = 0; w < W; ++w) pv.v[w] = cmulf(crecipf(diag32(bt, row, rhs0 + w, b)), rv.v[w]);
    stv<4>(bt.p + o, pv);
  }
}

// S_acc[b][j][rhs] += sum over port rows of conj(c_j[row]) * x64[row][rhs].
__global__ void __launch_bounds__(kBS) batch_overlap_kernel(const EfgkBatch bt, const int rows_per_block) {
  const int R = bt.R;
  const int s0 = blockIdx.x * rows_per_block;
  const int s1 = min(bt.n_srows, s0 + rows_per_block);
  for (int rhs = threadIdx.x; rhs < R; rhs += blockDim.x) {
    for (int j = 0; j < bt.P; ++j) {
      double ax = 0.0, ay = 0.0;
      int cur = -1;
      for (int s = s0; s < s1; ++s) {
        const int inst = bt.srow_inst[s];
        if (inst != cur) {
          if (cur >= 0) {
            double *d = bt.S_acc + 2 * ((static_cast<long long>(cur) * bt.P + j) * R + rhs);
            atomicAdd(d, ax);
            atomicAdd(d + 1, ay);
          }
          cur = inst;
          ax = ay = 0.0;
        }
        const double2 c = bt.cval[s * bt.P + j];
        if (c.x == 0.0 && c.y == 0.0) continue;
        const double2 x = bt.x64[static_cast<long long>(bt.srow_row[s]) * R + rhs];
        ax += c.x * x.x + c.y * x.y;  // conj(c) * x
        ay += c.x * x.y - c.y * x.x;
      }
      if (cur >= 0) {
        double *d = bt.S_acc + 2 * ((static_cast<long long>(cur) * bt.P + j) * R + rhs);
        atomicAdd(d, ax);
        atomicAdd(d + 1, ay);
      }
    }
  }
}

}  // namespace

extern "C" int efgk_batch_spmm(const EfgkBatch *bt, int parity, efgk_stream_t stream) {
  const int V = bt->R >= 32 ? bt->R / 32 : 1;
  switch (V) {
    case 1: batch_spmm_kernel<1><<<bt->n_chunks, kBS, 0, stream>>>(*bt, parity); break;
    case 2: batch_spmm_kernel<2><<<bt->n_chunks, kBS, 0, stream>>>(*bt, parity); break;
    case 4: batch_spmm_kernel<4><<<bt->n_chunks, kBS, 0, stream>>>(*bt, parity); break;
    default: return static_cast<int>(cudaErrorInvalidValue);
  }
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_update(const EfgkBatch *bt, int parity, efgk_stream_t stream) {
  batch_update_kernel<<<bt->n_chunks, kBS, 0, stream>>>(*bt, parity);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_pupdate(const EfgkBatch *bt, int parity, efgk_stream_t stream) {
  // parity bit 1 carries the "check convergence" flag
  batch_pupdate_kernel<<<bt->n_chunks, kBS, 0, stream>>>(*bt, parity & 1, parity >> 1);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_flush_residual(const EfgkBatch *bt, int parity, efgk_stream_t stream) {
  batch_flush_kernel<<<1024, kBS, 0, stream>>>(*bt, parity);
  batch_residual_kernel<<<bt->n_chunks, kBS, 0, stream>>>(*bt, parity);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_init(const EfgkBatch *bt, efgk_stream_t stream) {
  // x64 = xc = 0 is done by the host (memset); r = b via the residual pass
  // into parity slot 1, then |b|^2, p = D^-1 r.
  batch_residual_kernel<<<bt->n_chunks, kBS, 0, stream>>>(*bt, 1);
  batch_init_finish_kernel<<<bt->n_chunks, kBS, 0, stream>>>(*bt);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_finish(const EfgkBatch *bt, efgk_stream_t stream) {
  batch_flush_kernel<<<1024, kBS, 0, stream>>>(*bt, -1);
  const int rpb = 64;
  const int nb = (bt->n_srows + rpb - 1) / rpb;
  if (nb > 0) batch_overlap_kernel<<<nb, kBS, 0, stream>>>(*bt, rpb);
  return static_cast<int>(cudaGetLastError());
}

namespace {
__global__ void batch_pack_kernel(long long nnz, const double2 *__restrict__ K, const double2 *__restrict__ M,
                                  float *K32, float2 *M32, double *K64, double2 *M64) {
  for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < nnz;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double kv = K[k].x;
    const double2 mv = M[k];
    K32[k] = static_cast<float>(kv);
    K64[k] = kv;
    M32[k] = make_float2(static_cast<float>(mv.x), static_cast<float>(mv.y));
    M64[k] = mv;
  }
}
__global__ void batch_diag_kernel(int n, const int *__restrict__ diag, const double *__restrict__ K64,
                                  const double2 *__restrict__ M64, float *kd32, float2 *md32, double *kd64,
                                  double2 *md64) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const double kv = K64[diag[r]];
  const double2 mv = M64[diag[r]];
  kd64[r] = kv;
  md64[r] = mv;
  kd32[r] = static_cast<float>(kv);
  md32[r] = make_float2(static_cast<float>(mv.x), static_cast<float>(mv.y));
}
}  // namespace

extern "C" int efgk_batch_pack(int64_t nnz, const double *K, const double *M, float *K32, float *M32, double *K64,
                               double *M64, efgk_stream_t stream) {
  if (nnz <= 0) return 0;
  batch_pack_kernel<<<1024, kBS, 0, stream>>>(nnz, reinterpret_cast<const double2 *>(K),
                                              reinterpret_cast<const double2 *>(M), K32,
                                              reinterpret_cast<float2 *>(M32), K64,
                                              reinterpret_cast<double2 *>(M64));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_diag(int32_t n, const int32_t *diag_slot, const double *K64, const double *M64,
                               float *kd32, float *md32, double *kd64, double *md64, efgk_stream_t stream) {
  if (n <= 0) return 0;
  batch_diag_kernel<<<(n + 255) / 256, 256, 0, stream>>>(n, diag_slot, K64, reinterpret_cast<const double2 *>(M64),
                                                         kd32, reinterpret_cast<float2 *>(md32), kd64,
                                                         reinterpret_cast<double2 *>(md64));
  return static_cast<int>(cudaGetLastError());
}
