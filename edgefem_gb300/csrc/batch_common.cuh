// Device helpers shared by the batched engines: launch shape, partial
// sums per right-hand side, and the Jacobi / nodal diagonals formed on the
// fly from their per-row / per-node components (see batch_layout.h).
#pragma once

#include <cuda_runtime.h>

#include "batch_layout.h"
#include "dd.cuh"

namespace efg_batch {

constexpr int kBS = 256;

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// 1/d with one correctly rounded reciprocal (rcp.rn): a fixed function of
// d, so the preconditioner stays one linear operator.
__device__ __forceinline__ float2 crecipf(float2 d) {
  const float m = d.x * d.x + d.y * d.y;
  const float im = __frcp_rn(m);
  return m > 0.f ? make_float2(d.x * im, -d.y * im) : make_float2(0.f, 0.f);
}
__device__ __forceinline__ double2 cdivd(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// 32-byte accesses of two consecutive float4 (the 256-bit global loads and
// stores of sm_100+).  A warp whose lanes each take two consecutive complex
// dd entries then moves its 1 KB in 8 L1 wavefronts; two 16-byte accesses
// at a 32-byte lane stride take 16.  p must be 32-byte aligned: the vectors
// are separate allocations whose rows hold a power-of-two count of float4,
// and lanes start on even columns.
__device__ __forceinline__ void ldg_pair(const float4 *p, float4 &a, float4 &b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}
// Coherent form, for arrays the kernel also writes (each entry read before
// its own thread writes it, never after).
__device__ __forceinline__ void ld_pair(const float4 *p, float4 &a, float4 &b) {
  asm volatile("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
               : "l"(p)
               : "memory");
}
__device__ __forceinline__ void st_pair(float4 *p, float4 a, float4 b) {
  asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
               :
               : "l"(p), "f"(a.x), "f"(a.y), "f"(a.z), "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
               : "memory");
}
// V consecutive entries from p (read-only for the kernel), in pairs where V
// is even.
template <int V>
__device__ __forceinline__ void ldg_cols(const float4 *p, float4 (&v)[V]) {
  if constexpr (V % 2 == 0) {
#pragma unroll
    for (int i = 0; i < V; i += 2) ldg_pair(p + i, v[i], v[i + 1]);
  } else {
#pragma unroll
    for (int i = 0; i < V; ++i) v[i] = __ldg(p + i);
  }
}
template <int V>
__device__ __forceinline__ void ld_cols(const float4 *p, float4 (&v)[V]) {
  if constexpr (V % 2 == 0) {
#pragma unroll
    for (int i = 0; i < V; i += 2) ld_pair(p + i, v[i], v[i + 1]);
  } else {
#pragma unroll
    for (int i = 0; i < V; ++i) v[i] = p[i];
  }
}
template <int V>
__device__ __forceinline__ void st_cols(float4 *p, const float4 (&v)[V]) {
  if constexpr (V % 2 == 0) {
#pragma unroll
    for (int i = 0; i < V; i += 2) st_pair(p + i, v[i], v[i + 1]);
  } else {
#pragma unroll
    for (int i = 0; i < V; ++i) p[i] = v[i];
  }
}

__device__ __forceinline__ void block_zero(double *a, int count) {
  for (int i = threadIdx.x; i < count; i += blockDim.x) a[i] = 0.0;
}

// Contiguous chunk range of this block.
__device__ __forceinline__ void my_chunks(int n_chunks, int &c0, int &c1) {
  c0 = static_cast<int>((static_cast<long long>(n_chunks) * blockIdx.x) / gridDim.x);
  c1 = static_cast<int>((static_cast<long long>(n_chunks) * (blockIdx.x + 1)) / gridDim.x);
}

// Jacobi diagonal of A_bf at row for rhs.
__device__ __forceinline__ float2 diag32(const EfgkBatch &bt, int row, int rhs, int b) {
  const float kd = __ldg(bt.kd32 + row);
  const float2 md = __ldg(bt.md32 + row);
  const float k2 = __ldg(bt.k0sq32 + rhs);
  float2 d = make_float2(kd - k2 * md.x, -k2 * md.y);
  if (bt.has_md) {
    const float mdd = __ldg(bt.mdd32 + row);
    const float2 ka = __ldg(bt.kappa32 + rhs);
    d.x -= ka.x * mdd;
    d.y -= ka.y * mdd;
  }
  const int s = __ldg(bt.sidx + row);
  if (s >= 0) {
    for (int c = 0; c < bt.C; ++c) {
      const float sd = __ldg(bt.sdiag32 + s * bt.C + c);
      if (sd != 0.f) {
        const float2 cf = __ldg(bt.scoef32 + (b * bt.C + c) * bt.R + rhs);
        d.x += cf.x * sd;
        d.y += cf.y * sd;
      }
    }
  }
  return d;
}

// Nodal diagonal Dn of A_bf at node for rhs.
__device__ __forceinline__ float2 ndiag32(const EfgkBatch &bt, int node, int rhs, int b) {
  const float kn = __ldg(bt.kn32 + node);
  const float2 mn = __ldg(bt.mn32 + node);
  const float k2 = __ldg(bt.k0sq32 + rhs);
  float2 d = make_float2(kn - k2 * mn.x, -k2 * mn.y);
  if (bt.has_md) {
    const float mnd = __ldg(bt.mnd32 + node);
    const float2 ka = __ldg(bt.kappa32 + rhs);
    d.x -= ka.x * mnd;
    d.y -= ka.y * mnd;
  }
  for (int c = 0; c < bt.C; ++c) {
    const float sd = __ldg(bt.msn32 + static_cast<long long>(node) * bt.C + c);
    if (sd != 0.f) {
      const float2 cf = __ldg(bt.scoef32 + (b * bt.C + c) * bt.R + rhs);
      d.x += cf.x * sd;
      d.y += cf.y * sd;
    }
  }
  return d;
}

// Diagonal of Pi^T A_bf Pi / omega at (node, component d) for rhs.
__device__ __forceinline__ float2 pdiag32(const EfgkBatch &bt, int node, int d, int rhs, int b) {
  const long long i = static_cast<long long>(node) * 3 + d;
  const float kn = __ldg(bt.kpn32 + i);
  const float2 mn = __ldg(bt.mpn32 + i);
  const float k2 = __ldg(bt.k0sq32 + rhs);
  float2 v = make_float2(kn - k2 * mn.x, -k2 * mn.y);
  if (bt.has_md) {
    const float mnd = __ldg(bt.mdpn32 + i);
    const float2 ka = __ldg(bt.kappa32 + rhs);
    v.x -= ka.x * mnd;
    v.y -= ka.y * mnd;
  }
  for (int c = 0; c < bt.C; ++c) {
    const float sd = __ldg(bt.mspn32 + i * bt.C + c);
    if (sd != 0.f) {
      const float2 cf = __ldg(bt.scoef32 + (b * bt.C + c) * bt.R + rhs);
      v.x += cf.x * sd;
      v.y += cf.y * sd;
    }
  }
  return v;
}

// Partial sums of NV quantities for W right-hand-side slots per thread:
// FP32 over a few rows, folded into FP64 every 16 rows.
template <int NV, int W>
struct Partials {
  float f[NV][W];
  double d[NV][W];
  int cnt;
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
      for (int w = 0; w < W; ++w) f[k][w] = 0.f, d[k][w] = 0.0;
    cnt = 0;
  }
  __device__ __forceinline__ void fold() {
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
      for (int w = 0; w < W; ++w) d[k][w] += f[k][w], f[k][w] = 0.f;
    cnt = 0;
  }
  __device__ __forceinline__ void tick() {
    if (++cnt == 16) fold();
  }
  __device__ __forceinline__ double get(int k, int w) const { return d[k][w]; }
};

// Double-float partial sums: dd products added with an exact running
// TwoSum of the high words; the low words and rounding errors collect in a
// float whose own error stays near eps^2 of the sum over a block's rows.
template <int NV, int W>
struct DDPartials {
  efg_dd::Acc a[NV][W];
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
      for (int w = 0; w < W; ++w) a[k][w].zero();
  }
  __device__ __forceinline__ void fold() {}
  __device__ __forceinline__ void tick() {}
  __device__ __forceinline__ double get(int k, int w) const { return a[k][w].to_double(); }
};

// Block reduction of per-thread partials (Partials or DDPartials) and one
// FP64 atomic per (quantity, rhs) into dst[k] + stride_k * (b*R + rhs).
// rhs_of(t, w) maps a thread slot to its right-hand side.  All threads of
// the block must call it.
template <int NV, int W, class PT, class F>
__device__ __forceinline__ void flush_partials(PT &pt, int R, int b, double *const (&dst)[NV],
                                               const int (&stride)[NV], F rhs_of) {
  __shared__ double sh[NV][128];
  pt.fold();
  for (int i = threadIdx.x; i < NV * 128; i += blockDim.x) (&sh[0][0])[i] = 0.0;
  __syncthreads();
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const int rhs = rhs_of(threadIdx.x, w);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double v = pt.get(k, w);
      if (v != 0.0) atomicAdd(&sh[k][rhs], v);
    }
  }
  __syncthreads();
  for (int rhs = threadIdx.x; rhs < R; rhs += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (dst[k] && sh[k][rhs] != 0.0) atomicAdd(dst[k] + static_cast<long long>(stride[k]) * (b * R + rhs), sh[k][rhs]);
  __syncthreads();
  pt.clear();
}

// ------------------------------------------------ scalar phases (one block)
// (internal linkage: each translation unit that launches them has its own)

// Checkpoint decision for each running column, from its recurrence |r|:
//   flag 1 (replace, then decide convergence on the true residual): |r|
//     below the tolerance, not finite, or (replace_on_progress) below delta
//     times its value at the last replacement;
//   flag 2 (replace and restart): no factor-1/delta progress for
//     `stagnation` iterations.
// Without replace_on_progress a factor-1/delta drop only moves the progress
// marker (rmax, last_rep).  Flagged columns get rho[P] and rr[P] cleared for
// the recomputation from the true residual.
static __global__ void batch_flag_kernel(const EfgkBatch bt, const int P, const int iters_done) {
  const int BR = bt.B * bt.R;
  const int it = bt.counters[0] + iters_done;
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < BR; i += blockDim.x) {
    int f = 0;
    if (bt.status[i] == 0) {
      const double rr = bt.rr[P * BR + i];
      const bool progress = rr < bt.delta2 * bt.rmax[i];
      if (progress && !bt.replace_on_progress) {
        bt.rmax[i] = rr;
        bt.last_rep[i] = it;
      }
      f = (rr <= bt.tol2 * bt.bb[i]) || !(rr == rr) || (progress && bt.replace_on_progress) ? 1
          : (it - bt.last_rep[i] >= bt.stagnation)                                          ? 2
                                                                                            : 0;
    }
    bt.flag[i] = f;
    if (f) {
      atomicAdd(&cnt, 1);
      bt.rho[P * 2 * BR + 2 * i] = 0.0;
      bt.rho[P * 2 * BR + 2 * i + 1] = 0.0;
      bt.rr[P * BR + i] = 0.0;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) bt.counters[1] = cnt;
}

// After a replacement: convergence on the true residual, new reference |r|,
// iteration bookkeeping, max-iteration stop.
static __global__ void batch_post_kernel(const EfgkBatch bt, const int P, const int iters_done) {
  const int BR = bt.B * bt.R;
  const int it = bt.counters[0] + iters_done;
  for (int i = threadIdx.x; i < BR; i += blockDim.x) {
    if (bt.status[i] != 0) continue;
    if (bt.flag[i]) {
      const double rr = bt.rr[P * BR + i];
      if (rr <= bt.tol2 * bt.bb[i]) {
        bt.status[i] = 1;
        bt.iters[i] = it;
      } else if (!(rr == rr)) {
        bt.status[i] = 2;
        bt.iters[i] = it;
      }
      bt.rmax[i] = rr;
      bt.last_rep[i] = it;
    }
    if (bt.status[i] == 0 && it >= bt.max_iters) {
      bt.status[i] = 3;
      bt.iters[i] = it;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) bt.counters[0] = it;
}

// After the first residual pass: |b|^2, reference |r|, status.
static __global__ void batch_init_scalars_kernel(const EfgkBatch bt) {
  const int BR = bt.B * bt.R;
  for (int i = threadIdx.x; i < BR; i += blockDim.x) {
    const double rr = bt.rr[1 * BR + i];
    bt.bb[i] = rr;
    bt.rmax[i] = rr;
    bt.status[i] = rr > 0.0 ? 0 : 4;
    bt.iters[i] = 0;
    bt.flag[i] = 0;
    bt.last_rep[i] = 0;
  }
  if (threadIdx.x == 0) bt.counters[0] = bt.counters[1] = 0;
}

}  // namespace efg_batch
