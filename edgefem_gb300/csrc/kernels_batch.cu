// Batched complex64 COCG kernels with the nodal auxiliary-space
// preconditioner and FP64 residual replacement.
//
// All right-hand sides of one row (every frequency x active port of one mesh
// instance) are contiguous, so one pass over a matrix row serves all of them:
// a stored nonzero (column, K, M: 16 bytes) is read once per row with one
// broadcast vector load and re-used R times, and the gather of a column is
// one contiguous R*8-byte segment.  The operator is formed on the fly,
//   (K - k0_f^2 M) x + port-face terms (see batch_layout.h),
// so no per-frequency matrix is ever stored.
//
// Per iteration (parity P = k & 1):
//   spmm      q = A p, p^T q per (instance, rhs)
//   update    x_c += alpha p, r -= alpha q, |r|^2, r^T D^-1 r
//   node      s = G^T r, t = Dn^-1 s, s^T t          (rho' = r^T z complete)
//   [checkpoint: flag rhs whose |r| fell by delta (or below tol);
//    for them x64 += x_c and r = b - A x64 in FP64 (true residual), then
//    |r|^2, r^T D^-1 r and the node pass again; convergence is decided on
//    the true residual only]
//   pupdate   p = D^-1 r + G t + beta p
//
// Launch shape: a fixed grid; block i takes a contiguous range of row chunks
// (chunks never straddle instances) and keeps its partial sums in registers,
// adding them to the per-(instance, rhs) accumulators when the instance
// changes and at the end: a few hundred atomics per launch.
#include <cuda_runtime.h>

#include "batch_common.cuh"
#include "edgefem_gb300_kernels.h"

namespace {

using namespace efg_batch;

template <int V>
struct CVec {
  float2 v[V];
};

template <int V>
__device__ __forceinline__ CVec<V> ldg_v(const float2 *p) {
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
template <int V>
__device__ __forceinline__ CVec<V> ld_v(const float2 *p) {
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
__device__ __forceinline__ void st_v(float2 *p, const CVec<V> &o) {
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

// ------------------------------------------------------------------ SpMM
// A group of LW = min(32, R/V) lanes computes one row for a tile of LW*V
// right-hand sides (V per lane); T = R/(LW*V) tiles cover a row, so with
// V < R/32 several warps share a row and each holds fewer registers and
// keeps more gathers in flight.  V is chosen by the autotuner.
template <int V>
__global__ void __launch_bounds__(kBS) batch_spmm_kernel(const EfgkBatch bt, const int P) {
  const int R = bt.R;
  const int LW = R / V < 32 ? R / V : 32;
  const int T = R / (LW * V);
  const int BR = bt.B * R;
  if (blockIdx.x == 0) {
    block_zero(bt.rho + P * 2 * BR, 2 * BR);
    block_zero(bt.rr + P * BR, BR);
  }
  const int g = threadIdx.x / LW, lane = threadIdx.x % LW;
  const int tile = g % T, group = g / T, ngroups = kBS / LW / T;
  const int rhs0 = tile * LW * V + lane * V;
  float k2[V];
#pragma unroll
  for (int v = 0; v < V; ++v) k2[v] = __ldg(bt.k0sq32 + rhs0 + v);
  Partials<2, V> pt;
  pt.clear();
  auto rhs_of = [LW, T](int t, int w) { return ((t / LW) % T) * LW * V + (t % LW) * V + w; };
  double *const dst[2] = {bt.pq + P * 2 * BR, bt.pq + P * 2 * BR + 1};
  const int stride[2] = {2, 2};
  int c0, c1;
  my_chunks(bt.n_chunks, c0, c1);
  int cur = c0 < c1 ? bt.chunk_inst[c0] : -1;
  for (int c = c0; c < c1; ++c) {
    const int b = bt.chunk_inst[c];
    if (b != cur) {
      flush_partials<2, V>(pt, R, cur, dst, stride, rhs_of);
      cur = b;
    }
    const int r1 = bt.chunk_end[c];
    for (int row = bt.chunk_begin[c] + group; row < r1; row += ngroups) {
      const int kb = __ldg(bt.rowptr + row), ke = __ldg(bt.rowptr + row + 1);
      CVec<V> acc;
#pragma unroll
      for (int v = 0; v < V; ++v) acc.v[v] = make_float2(0.f, 0.f);
#pragma unroll 4
      for (int k = kb; k < ke; ++k) {
        const int4 raw = __ldg(reinterpret_cast<const int4 *>(bt.nz) + k);
        const int cj = raw.x;
        const float kj = __int_as_float(raw.y), mjx = __int_as_float(raw.z), mjy = __int_as_float(raw.w);
        const CVec<V> xv = ldg_v<V>(bt.p + static_cast<long long>(cj) * R + rhs0);
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const float ar = fmaf(-k2[v], mjx, kj), ai = -k2[v] * mjy;
          acc.v[v].x = fmaf(ar, xv.v[v].x, fmaf(-ai, xv.v[v].y, acc.v[v].x));
          acc.v[v].y = fmaf(ar, xv.v[v].y, fmaf(ai, xv.v[v].x, acc.v[v].y));
        }
      }
      const int s = __ldg(bt.sidx + row);
      if (s >= 0) {
        for (int e = __ldg(bt.sptr + s); e < __ldg(bt.sptr + s + 1); ++e) {
          const int cj = __ldg(bt.scol + e);
          const float val = __ldg(bt.sval32 + e);
          const int ci = __ldg(bt.scidx + e);
          const CVec<V> xv = ldg_v<V>(bt.p + static_cast<long long>(cj) * R + rhs0);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const float2 cf = __ldg(bt.scoef32 + ci * R + rhs0 + v);
            const float2 t = cmulf(make_float2(cf.x * val, cf.y * val), xv.v[v]);
            acc.v[v].x += t.x;
            acc.v[v].y += t.y;
          }
        }
      }
      st_v<V>(bt.q + static_cast<long long>(row) * R + rhs0, acc);
      const CVec<V> pv = ldg_v<V>(bt.p + static_cast<long long>(row) * R + rhs0);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const float2 d = cmulf(pv.v[v], acc.v[v]);
        pt.f[0][v] += d.x;
        pt.f[1][v] += d.y;
      }
      pt.tick();
    }
  }
  if (cur >= 0) flush_partials<2, V>(pt, R, cur, dst, stride, rhs_of);
}

// ------------------------------------------------------------ vector phases
// A thread owns W = 4 consecutive right-hand sides of one row; R % 4 == 0 and
// (kBS * 4) % R == 0, so its rhs set is the same on every row it visits.
constexpr int W = 4;

__device__ __forceinline__ void load_alpha(const EfgkBatch &bt, int b, int rhs0, int P, float2 (&alpha)[W]) {
  const int R = bt.R, BR = bt.B * R, Q = 1 - P;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const long long i = static_cast<long long>(b) * R + rhs0 + w;
    const double2 rho = make_double2(bt.rho[Q * 2 * BR + 2 * i], bt.rho[Q * 2 * BR + 2 * i + 1]);
    const double2 pq = make_double2(bt.pq[P * 2 * BR + 2 * i], bt.pq[P * 2 * BR + 2 * i + 1]);
    double2 a = cdivd(rho, pq);
    if (bt.status[i] != 0 || !(isfinite(a.x) && isfinite(a.y))) a = make_double2(0.0, 0.0);
    alpha[w] = make_float2(static_cast<float>(a.x), static_cast<float>(a.y));
  }
}

__global__ void __launch_bounds__(kBS) batch_update_kernel(const EfgkBatch bt, const int P) {
  const int R = bt.R, BR = bt.B * R;
  const int rhs0 = (threadIdx.x * W) % R;
  Partials<3, W> pt;
  pt.clear();
  auto rhs_of = [R](int t, int w) { return (t * W + w) % R; };
  double *const dst[3] = {bt.rho + P * 2 * BR, bt.rho + P * 2 * BR + 1, bt.rr + P * BR};
  const int stride[3] = {2, 2, 1};
  int c0, c1;
  my_chunks(bt.n_chunks, c0, c1);
  int cur = c0 < c1 ? bt.chunk_inst[c0] : -1;
  float2 alpha[W];
  if (cur >= 0) load_alpha(bt, cur, rhs0, P, alpha);
  for (int c = c0; c < c1; ++c) {
    const int b = bt.chunk_inst[c];
    if (b != cur) {
      flush_partials<3, W>(pt, R, cur, dst, stride, rhs_of);
      cur = b;
      load_alpha(bt, cur, rhs0, P, alpha);
    }
    const int r0 = bt.chunk_begin[c], r1 = bt.chunk_end[c];
    const long long base = static_cast<long long>(r0) * R;
    const int total = (r1 - r0) * R;
    for (int e = threadIdx.x * W; e < total; e += kBS * W) {
      const int row = r0 + e / R;
      const long long o = base + e;
      const CVec<4> pv = ld_v<4>(bt.p + o), qv = ld_v<4>(bt.q + o);
      CVec<4> xv = ld_v<4>(bt.xc + o), rv = ld_v<4>(bt.r + o);
#pragma unroll
      for (int w = 0; w < W; ++w) {
        const float2 ap = cmulf(alpha[w], pv.v[w]), aq = cmulf(alpha[w], qv.v[w]);
        xv.v[w].x += ap.x;
        xv.v[w].y += ap.y;
        rv.v[w].x -= aq.x;
        rv.v[w].y -= aq.y;
        const float2 rz = cmulf(rv.v[w], cmulf(crecipf(diag32(bt, row, rhs0 + w, b)), rv.v[w]));
        pt.f[0][w] += rz.x;
        pt.f[1][w] += rz.y;
        pt.f[2][w] += rv.v[w].x * rv.v[w].x + rv.v[w].y * rv.v[w].y;
      }
      st_v<4>(bt.xc + o, xv);
      st_v<4>(bt.r + o, rv);
      pt.tick();
    }
  }
  if (cur >= 0) flush_partials<3, W>(pt, R, cur, dst, stride, rhs_of);
}

// Node pass: t = Dn^-1 G^T r and s^T t into rho[P].  only_flagged: restrict
// to right-hand sides flagged for replacement (their t is recomputed from
// the new residual; the others keep theirs) and skip if none is flagged.
template <int V>
__global__ void __launch_bounds__(kBS) batch_node_kernel(const EfgkBatch bt, const int P, const int only_flagged) {
  if (only_flagged && bt.counters[1] == 0) return;
  const int R = bt.R, BR = bt.B * R;
  const int G = R / V;
  const int group = threadIdx.x / G, lane = threadIdx.x % G, ngroups = kBS / G;
  const int rhs0 = lane * V;
  Partials<2, V> pt;
  pt.clear();
  auto rhs_of = [G](int t, int w) { return (t % G) * V + w; };
  double *const dst[2] = {bt.rho + P * 2 * BR, bt.rho + P * 2 * BR + 1};
  const int stride[2] = {2, 2};
  int c0, c1;
  my_chunks(bt.n_nchunks, c0, c1);
  int cur = c0 < c1 ? bt.nchunk_inst[c0] : -1;
  bool act[V];
  for (int c = c0; c < c1; ++c) {
    const int b = bt.nchunk_inst[c];
    if (b != cur) {
      flush_partials<2, V>(pt, R, cur, dst, stride, rhs_of);
      cur = b;
    }
#pragma unroll
    for (int v = 0; v < V; ++v) act[v] = !only_flagged || bt.flag[b * R + rhs0 + v] != 0;
    const int n1 = bt.nchunk_end[c];
    for (int node = bt.nchunk_begin[c] + group; node < n1; node += ngroups) {
      CVec<V> s;
#pragma unroll
      for (int v = 0; v < V; ++v) s.v[v] = make_float2(0.f, 0.f);
      for (int k = __ldg(bt.nptr + node); k < __ldg(bt.nptr + node + 1); ++k) {
        const int e = __ldg(bt.nedge + k);
        const float sg = __ldg(bt.nsign + k);
        const CVec<V> rv = ld_v<V>(bt.r + static_cast<long long>(e) * R + rhs0);
#pragma unroll
        for (int v = 0; v < V; ++v) {
          s.v[v].x = fmaf(sg, rv.v[v].x, s.v[v].x);
          s.v[v].y = fmaf(sg, rv.v[v].y, s.v[v].y);
        }
      }
      float2 *tp = bt.t + static_cast<long long>(node) * R + rhs0;
      CVec<V> tv = ld_v<V>(tp);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        if (!act[v]) continue;
        const float2 t = cmulf(crecipf(ndiag32(bt, node, rhs0 + v, b)), s.v[v]);
        tv.v[v] = t;
        const float2 st = cmulf(s.v[v], t);
        pt.f[0][v] += st.x;
        pt.f[1][v] += st.y;
      }
      st_v<V>(tp, tv);
      pt.tick();
    }
  }
  if (cur >= 0) flush_partials<2, V>(pt, R, cur, dst, stride, rhs_of);
}

// restart: this iteration ran a checkpoint; right-hand sides whose residual
// was just replaced restart their search direction (p = z), which keeps the
// FP32 recurrence consistent with the new FP64 residual.
__global__ void __launch_bounds__(kBS) batch_pupdate_kernel(const EfgkBatch bt, const int P, const int restart) {
  const int R = bt.R, BR = bt.B * R;
  const int Q = 1 - P;
  if (blockIdx.x == 0) block_zero(bt.pq + Q * 2 * BR, 2 * BR);
  const int rhs0 = (threadIdx.x * W) % R;
  int c0, c1;
  my_chunks(bt.n_chunks, c0, c1);
  int cur = -1;
  float2 beta[W];
  for (int c = c0; c < c1; ++c) {
    const int b = bt.chunk_inst[c];
    if (b != cur) {
      cur = b;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        const long long i = static_cast<long long>(b) * R + rhs0 + w;
        const double2 rn = make_double2(bt.rho[P * 2 * BR + 2 * i], bt.rho[P * 2 * BR + 2 * i + 1]);
        const double2 ro = make_double2(bt.rho[Q * 2 * BR + 2 * i], bt.rho[Q * 2 * BR + 2 * i + 1]);
        double2 be = cdivd(rn, ro);
        // Stopped right-hand sides restart from p = z so p stays bounded
        // (their x and r no longer change: alpha is 0 for them).
        if (bt.status[i] != 0 || (restart && bt.flag[i]) || !(isfinite(be.x) && isfinite(be.y)))
          be = make_double2(0.0, 0.0);
        beta[w] = make_float2(static_cast<float>(be.x), static_cast<float>(be.y));
      }
    }
    const int r0 = bt.chunk_begin[c], r1 = bt.chunk_end[c];
    const long long base = static_cast<long long>(r0) * R;
    const int total = (r1 - r0) * R;
    for (int e = threadIdx.x * W; e < total; e += kBS * W) {
      const int row = r0 + e / R;
      const long long o = base + e;
      const CVec<4> rv = ld_v<4>(bt.r + o);
      CVec<4> pv = ld_v<4>(bt.p + o);
      const int2 en = __ldg(bt.enodes + row);
      CVec<4> ta, tb;
      if (en.x >= 0) {
        ta = ld_v<4>(bt.t + static_cast<long long>(en.x) * R + rhs0);
        tb = ld_v<4>(bt.t + static_cast<long long>(en.y) * R + rhs0);
      }
#pragma unroll
      for (int w = 0; w < W; ++w) {
        float2 z = cmulf(crecipf(diag32(bt, row, rhs0 + w, b)), rv.v[w]);
        if (en.x >= 0) {
          z.x += tb.v[w].x - ta.v[w].x;
          z.y += tb.v[w].y - ta.v[w].y;
        }
        const float2 bp = cmulf(beta[w], pv.v[w]);
        pv.v[w] = make_float2(z.x + bp.x, z.y + bp.y);
      }
      st_v<4>(bt.p + o, pv);
    }
  }
}

// x64 += x_c, x_c = 0 for flagged right-hand sides (all with flush_all).
__global__ void __launch_bounds__(kBS) batch_flush_kernel(const EfgkBatch bt, const int flush_all) {
  if (!flush_all && bt.counters[1] == 0) return;
  const int R = bt.R;
  int c0, c1;
  my_chunks(bt.n_chunks, c0, c1);
  for (int c = c0; c < c1; ++c) {
    const int b = bt.chunk_inst[c];
    const long long base = static_cast<long long>(bt.chunk_begin[c]) * R;
    const int total = (bt.chunk_end[c] - bt.chunk_begin[c]) * R;
    for (int e = threadIdx.x; e < total; e += kBS) {
      const int rhs = e % R;
      if (!flush_all && !bt.flag[b * R + rhs]) continue;
      const long long o = base + e;
      const float2 cx = bt.xc[o];
      double2 x = bt.x64[o];
      x.x += cx.x;
      x.y += cx.y;
      bt.x64[o] = x;
      bt.xc[o] = make_float2(0.f, 0.f);
    }
  }
}

// True residual in FP64 for flagged right-hand sides (all with do_all):
// r = b - A x64 stored as complex64; |r|^2 (FP64) and r^T D^-1 r into slot P.
// One lane per right-hand side, G = min(R, 32) lanes per row group.
__global__ void __launch_bounds__(kBS) batch_residual_kernel(const EfgkBatch bt, const int P, const int do_all) {
  if (!do_all && bt.counters[1] == 0) return;
  const int R = bt.R, BR = bt.B * R;
  const int G = R < 32 ? R : 32;
  const int VR = R / G;
  const int group = threadIdx.x / G, lane = threadIdx.x % G, ngroups = kBS / G;
  Partials<3, 4> pt;
  pt.clear();
  auto rhs_of = [G](int t, int w) { return (t % G) + w * G; };
  double *const dst[3] = {bt.rho + P * 2 * BR, bt.rho + P * 2 * BR + 1, bt.rr + P * BR};
  const int stride[3] = {2, 2, 1};
  int c0, c1;
  my_chunks(bt.n_chunks, c0, c1);
  int cur = c0 < c1 ? bt.chunk_inst[c0] : -1;
  bool act[4] = {false, false, false, false};
  for (int c = c0; c < c1; ++c) {
    const int b = bt.chunk_inst[c];
    if (b != cur) {
      flush_partials<3, 4>(pt, R, cur, dst, stride, rhs_of);
      cur = b;
    }
    for (int v = 0; v < VR; ++v) act[v] = do_all || bt.flag[b * R + lane + v * G] != 0;
    const int r1 = bt.chunk_end[c];
    for (int row = bt.chunk_begin[c] + group; row < r1; row += ngroups) {
      const int kb = __ldg(bt.rowptr + row), ke = __ldg(bt.rowptr + row + 1);
      const int s = __ldg(bt.sidx + row);
      for (int v = 0; v < VR; ++v) {
        if (!act[v]) continue;
        const int rhs = lane + v * G;
        const double k2 = __ldg(bt.k0sq64 + rhs);
        double ax = 0.0, ay = 0.0;
        for (int k = kb; k < ke; ++k) {
          const int col = __ldg(bt.colidx + k);
          const double kv = __ldg(bt.K64 + k);
          const double2 m = __ldg(bt.M64 + k);
          const double2 x = bt.x64[static_cast<long long>(col) * R + rhs];
          const double ar = kv - k2 * m.x, ai = -k2 * m.y;
          ax += ar * x.x - ai * x.y;
          ay += ar * x.y + ai * x.x;
        }
        double bx = 0.0, by = 0.0;
        if (s >= 0) {
          for (int e = __ldg(bt.sptr + s); e < __ldg(bt.sptr + s + 1); ++e) {
            const int col = __ldg(bt.scol + e);
            const double val = __ldg(bt.sval64 + e);
            const double2 cf = __ldg(bt.scoef64 + __ldg(bt.scidx + e) * R + rhs);
            const double2 x = bt.x64[static_cast<long long>(col) * R + rhs];
            ax += val * (cf.x * x.x - cf.y * x.y);
            ay += val * (cf.x * x.y + cf.y * x.x);
          }
          // b = rcoef(b, a, f) c_a[row] for the active port a = rhs % P
          if (rhs < bt.F * bt.P) {
            const int a = rhs % bt.P;
            const double2 cf = __ldg(bt.rcoef64 + (b * bt.P + a) * R + rhs);
            const double2 cv = __ldg(bt.cval + s * bt.P + a);
            bx = cf.x * cv.x - cf.y * cv.y;
            by = cf.x * cv.y + cf.y * cv.x;
          }
        }
        const double rx = bx - ax, ry = by - ay;
        const float2 r32 = make_float2(static_cast<float>(rx), static_cast<float>(ry));
        bt.r[static_cast<long long>(row) * R + rhs] = r32;
        const float2 rz = cmulf(r32, cmulf(crecipf(diag32(bt, row, rhs, b)), r32));
        pt.d[0][v] += rz.x;
        pt.d[1][v] += rz.y;
        pt.d[2][v] += rx * rx + ry * ry;
      }
    }
  }
  if (cur >= 0) flush_partials<3, 4>(pt, R, cur, dst, stride, rhs_of);
}

// p = D^-1 r + G t (first direction).
__global__ void __launch_bounds__(kBS) batch_pinit_kernel(const EfgkBatch bt) {
  const int R = bt.R;
  const int rhs0 = (threadIdx.x * W) % R;
  int c0, c1;
  my_chunks(bt.n_chunks, c0, c1);
  for (int c = c0; c < c1; ++c) {
    const int b = bt.chunk_inst[c];
    const int r0 = bt.chunk_begin[c], r1 = bt.chunk_end[c];
    const long long base = static_cast<long long>(r0) * R;
    const int total = (r1 - r0) * R;
    for (int e = threadIdx.x * W; e < total; e += kBS * W) {
      const int row = r0 + e / R;
      const long long o = base + e;
      const CVec<4> rv = ld_v<4>(bt.r + o);
      const int2 en = __ldg(bt.enodes + row);
      CVec<4> pv;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        float2 z = cmulf(crecipf(diag32(bt, row, rhs0 + w, b)), rv.v[w]);
        if (en.x >= 0) {
          const float2 ta = bt.t[static_cast<long long>(en.x) * R + rhs0 + w];
          const float2 tb = bt.t[static_cast<long long>(en.y) * R + rhs0 + w];
          z.x += tb.x - ta.x;
          z.y += tb.y - ta.y;
        }
        pv.v[w] = z;
      }
      st_v<4>(bt.p + o, pv);
    }
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

__global__ void batch_pack_kernel(long long nnz, const int *__restrict__ col_local, int col_off,
                                  const double2 *__restrict__ K, const double2 *__restrict__ M, EfgkNz *nz,
                                  int *colidx, double *K64, double2 *M64) {
  for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < nnz;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double kv = K[k].x;
    const double2 mv = M[k];
    const int c = col_local[k] + col_off;
    EfgkNz e;
    e.col = c;
    e.k = static_cast<float>(kv);
    e.mre = static_cast<float>(mv.x);
    e.mim = static_cast<float>(mv.y);
    nz[k] = e;
    colidx[k] = c;
    K64[k] = kv;
    M64[k] = mv;
  }
}

__global__ void batch_diag_kernel(int n, const int *__restrict__ diag, const double *__restrict__ K64,
                                  const double2 *__restrict__ M64, float *kd32, float2 *md32) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  kd32[r] = static_cast<float>(K64[diag[r]]);
  const double2 mv = M64[diag[r]];
  md32[r] = make_float2(static_cast<float>(mv.x), static_cast<float>(mv.y));
}

int g_grid = 0;
int grid() {
  if (!g_grid) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_grid = (sms > 0 ? sms : 132) * 4;
  }
  return g_grid;
}
inline int grid_for(int chunks) { return chunks < grid() ? (chunks > 0 ? chunks : 1) : grid(); }

template <template <int> class Kern, class... A>
int launch_v(int R, int grid_blocks, cudaStream_t s, A... args) {
  const int V = R >= 32 ? R / 32 : 1;
  switch (V) {
    case 1: Kern<1>::go(grid_blocks, s, args...); break;
    case 2: Kern<2>::go(grid_blocks, s, args...); break;
    case 4: Kern<4>::go(grid_blocks, s, args...); break;
    default: return static_cast<int>(cudaErrorInvalidValue);
  }
  return static_cast<int>(cudaGetLastError());
}
template <int V>
struct SpmmL {
  static void go(int g, cudaStream_t s, const EfgkBatch &bt, int P) { batch_spmm_kernel<V><<<g, kBS, 0, s>>>(bt, P); }
};
template <int V>
struct NodeL {
  static void go(int g, cudaStream_t s, const EfgkBatch &bt, int P, int only) {
    batch_node_kernel<V><<<g, kBS, 0, s>>>(bt, P, only);
  }
};

}  // namespace

extern "C" int efgk_batch_spmm(const EfgkBatch *bt, int parity, efgk_stream_t stream) {
  return launch_v<SpmmL>(bt->R, grid_for(bt->n_chunks), stream, *bt, parity);
}

extern "C" int efgk_batch_spmm_grid(const EfgkBatch *bt, int parity, int grid_blocks, int rhs_per_lane,
                                    efgk_stream_t stream) {
  if (rhs_per_lane <= 0) return launch_v<SpmmL>(bt->R, grid_blocks, stream, *bt, parity);
  // R and rhs_per_lane are powers of two; the tile width LW*V must divide R.
  if (bt->R % rhs_per_lane != 0) return static_cast<int>(cudaErrorInvalidValue);
  switch (rhs_per_lane) {
    case 1: SpmmL<1>::go(grid_blocks, stream, *bt, parity); break;
    case 2: SpmmL<2>::go(grid_blocks, stream, *bt, parity); break;
    case 4: SpmmL<4>::go(grid_blocks, stream, *bt, parity); break;
    default: return static_cast<int>(cudaErrorInvalidValue);
  }
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_update(const EfgkBatch *bt, int parity, efgk_stream_t stream) {
  batch_update_kernel<<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt, parity);
  int err = static_cast<int>(cudaGetLastError());
  if (err) return err;
  return launch_v<NodeL>(bt->R, grid_for(bt->n_nchunks), stream, *bt, parity, 0);
}

extern "C" int efgk_batch_checkpoint(const EfgkBatch *bt, int parity, int iters_done, efgk_stream_t stream) {
  batch_flag_kernel<<<1, 1024, 0, stream>>>(*bt, parity, iters_done);
  batch_flush_kernel<<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt, 0);
  batch_residual_kernel<<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt, parity, 0);
  int err = launch_v<NodeL>(bt->R, grid_for(bt->n_nchunks), stream, *bt, parity, 1);
  if (err) return err;
  batch_post_kernel<<<1, 1024, 0, stream>>>(*bt, parity, iters_done);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_pupdate(const EfgkBatch *bt, int parity, efgk_stream_t stream) {
  // bit 1 of `parity`: a checkpoint ran in this iteration
  batch_pupdate_kernel<<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt, parity & 1, (parity >> 1) & 1);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_init(const EfgkBatch *bt, efgk_stream_t stream) {
  // x64 = x_c = t = 0 and all accumulators zeroed by the host beforehand.
  // r = b (true residual of x = 0) into parity slot 1, then |b|^2, t, p.
  batch_residual_kernel<<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt, 1, 1);
  batch_init_scalars_kernel<<<1, 1024, 0, stream>>>(*bt);
  int err = launch_v<NodeL>(bt->R, grid_for(bt->n_nchunks), stream, *bt, 1, 0);
  if (err) return err;
  batch_pinit_kernel<<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_finish(const EfgkBatch *bt, efgk_stream_t stream) {
  batch_flush_kernel<<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt, 1);
  const int rpb = 64;
  const int nb = (bt->n_srows + rpb - 1) / rpb;
  if (nb > 0) batch_overlap_kernel<<<nb, kBS, 0, stream>>>(*bt, rpb);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_pack(int64_t nnz, const int32_t *col_local, int32_t col_off, const double *K,
                               const double *M, void *nz, int32_t *colidx, double *K64, double *M64,
                               efgk_stream_t stream) {
  if (nnz <= 0) return 0;
  batch_pack_kernel<<<1024, kBS, 0, stream>>>(nnz, col_local, col_off, reinterpret_cast<const double2 *>(K),
                                              reinterpret_cast<const double2 *>(M), static_cast<EfgkNz *>(nz),
                                              colidx, K64, reinterpret_cast<double2 *>(M64));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_diag(int32_t n, const int32_t *diag_slot, const double *K64, const double *M64,
                               float *kd32, float *md32, efgk_stream_t stream) {
  if (n <= 0) return 0;
  batch_diag_kernel<<<(n + 255) / 256, 256, 0, stream>>>(n, diag_slot, K64, reinterpret_cast<const double2 *>(M64),
                                                         kd32, reinterpret_cast<float2 *>(md32));
  return static_cast<int>(cudaGetLastError());
}
