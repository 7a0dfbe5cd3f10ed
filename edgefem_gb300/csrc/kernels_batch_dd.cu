// Batched COCG in double-float ("dd") arithmetic.
//
// Same algorithm, layout and launch shape as the complex64 engine
// (kernels_batch.cu): all right-hand sides of a row contiguous, operator
// (K - k0_f^2 M) p + port-face terms formed on the fly, nodal
// auxiliary-space preconditioner, per-(instance, rhs) FP64 scalars, FP64
// true-residual replacement at checkpoints.  The difference is precision:
// the Krylov vectors x, r, p, q, t are complex dd (float4: re_hi, re_lo,
// im_hi, im_lo, about 48 bits), K and M are applied with their low words
// (nzlo) in dd arithmetic, the scalars alpha and beta are dd, and dot
// products are summed exactly per element in dd.  On this indefinite,
// ill-conditioned system the complex64 recurrences lose conjugacy and need
// several times the FP64 iteration count; in dd the count stays near
// FP64's, while every operation runs on the FP32 pipes (GB300's FP64 rate is
// a small fraction of its FP32 rate).
//
// Only the port-face rows (a few hundred per instance) use FP64 arithmetic.
//
// Launch shape: block i of a G-block grid takes row chunks i, i + G, ...,
// so at any moment the grid works on one window of consecutive rows and the
// rows of p (x, r, t) gathered around it - the mesh neighbours, up to one
// z-layer of the hex grid away - are re-read from L2 rather than HBM.
#include <cuda_runtime.h>

#include "batch_common.cuh"
#include "edgefem_gb300_kernels.h"

namespace {

using namespace efg_batch;
using efg_dd::Acc;
using efg_dd::Acc2;
using efg_dd::f2;
using efg_dd::hi2;
using efg_dd::lo2;
using efg_dd::rmul;
using efg_dd::swap2;
using efg_dd::cadd;
using efg_dd::cjoin;
using efg_dd::cmul;
using efg_dd::cmul_f;
using efg_dd::cneg;
using efg_dd::csplit;
using efg_dd::dot_add;
using efg_dd::from_acc;

__device__ __forceinline__ float4 zero4() { return make_float4(0.f, 0.f, 0.f, 0.f); }

// True when no right-hand side of this warp is still running in instance b
// (each lane passes its own n consecutive rhs from rhs0).  Stopped right-hand
// sides keep x and r (alpha = 0), so a warp whose right-hand sides have all
// stopped can skip the rows: low frequencies converge first, and their warps
// then cost nothing.  Call with the whole warp converged on the loop.
__device__ __forceinline__ bool warp_done(const EfgkBatch &bt, int b, int rhs0, int n) {
  bool run = false;
  for (int v = 0; v < n; ++v) run |= bt.status[b * bt.R + rhs0 + v] == 0;
  return !__any_sync(0xffffffffu, run);
}

// ------------------------------------------------------------------ SpMM
// q = A p and p^T q per (instance, rhs).  Lane layout as in the complex64
// SpMM: LW = min(32, R/V) lanes per row tile, V right-hand sides per lane.
// MM = 1: M applied with its low words in dd; MM = 0: M in FP32 on the
// high words of p (K always in dd); MM = 2: as MM = 1, but the coefficient
// a = K - k0^2 M is formed once in dd and shared by the two right-hand sides
// of a lane that belong to one frequency (V and P even: rhs = f*P + port),
// which saves a fifth of the arithmetic; MM = 3: the same per right-hand
// side (odd P: every column its own frequency), which still takes the
// real-coefficient shortcut (two real products instead of four, against
// the six to eight of MM = 1) wherever the entry touches no lossy or
// dispersive material.  The coefficient's final
// renormalisation uses FastTwoSum: its second operand is a low-word
// correction (about 2^-24 of K), so where s = K - k0^2 M cancels below it
// the subtraction was exact (Sterbenz) and the error term is off by at most
// about 2^-48 of K.
//
// Work order: with TM (tile-major) every warp of a block works on the same
// column tile (LW * V right-hand sides) and the grid sweeps all row chunks
// of tile 0, then of tile 1, ...: the p rows gathered while a tile is swept
// are 1/T of a full row wide, so the window of p the grid is gathering
// from fits L2 better, at the price of reading the matrix entries once per
// tile.  Without TM the T tiles of a row are taken by different warps of
// one block at the same time.
template <int V, int MM, bool TM>
// Register budget: 64 per thread for V <= 2 with the shared coefficient
// (four blocks, 32 warps per SM; 3 blocks where the per-column forms keep
// more accumulators): the kernel waits mostly on its p gathers, so
// resident warps matter more than the registers a deeper schedule would use.
__global__ void __launch_bounds__(kBS, V <= 2 ? (MM == 2 || MM == 0 ? 4 : 3) : 2)
    dd_spmm_kernel(const EfgkBatch bt, const int P) {
  constexpr int S = MM == 2 ? 2 : 1;  // right-hand sides sharing one coefficient
  const int R = bt.R;
  const int LW = R / V < 32 ? R / V : 32;
  const int T = R / (LW * V);
  const int BR = bt.B * R;
  if (blockIdx.x == 0) {
    block_zero(bt.rho + P * 2 * BR, 2 * BR);
    block_zero(bt.rr + P * BR, BR);
  }
  const int g = threadIdx.x / LW, lane = threadIdx.x % LW;
  const int group = TM ? g : g / T, ngroups = TM ? kBS / LW : kBS / LW / T;
  const int n_items = TM ? bt.n_chunks * T : bt.n_chunks;
  int cur = -1, cur_tile = -1, rhs0 = 0;
  float k2h[V], k2l[V];
  // kappa = k0^2 eps_D(f) of the Debye region (zero without one)
  float4 kap[V];
  // per-thread constants of the right-hand sides rhs0 .. rhs0 + V - 1
  auto load_consts = [&]() {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      efg_dd::split(__ldg(bt.k0sq64 + rhs0 + v), k2h[v], k2l[v]);
      const double2 ka = bt.has_md ? __ldg(bt.kappa64 + rhs0 + v) : make_double2(0.0, 0.0);
      kap[v] = csplit(ka.x, ka.y);
    }
  };
  DDPartials<2, V> pt;
  pt.clear();
  auto rhs_of = [&](int t, int w) {
    return (TM ? cur_tile : (t / LW) % T) * LW * V + (t % LW) * V + w;
  };
  double *const dst[2] = {bt.pq + P * 2 * BR, bt.pq + P * 2 * BR + 1};
  const int stride[2] = {2, 2};
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int c = TM ? it % bt.n_chunks : it;
    const int tl = TM ? it / bt.n_chunks : g % T;
    const int b = bt.chunk_inst[c];
    if (b != cur || tl != cur_tile) {  // uniform over the block
      if (cur >= 0) flush_partials<2, V>(pt, R, cur, dst, stride, rhs_of);
      cur = b;
      cur_tile = tl;
      rhs0 = tl * LW * V + lane * V;
      load_consts();
    }
    if (warp_done(bt, b, rhs0, V)) continue;
    const int r1 = bt.chunk_end[c];
    for (int row = bt.chunk_begin[c] + group; row < r1; row += ngroups) {
      const int kb = __ldg(bt.rowptr + row), ke = __ldg(bt.rowptr + row + 1);
      // (real, imaginary) lanes of (K - k0^2 M) p, or of K p, M p, MD p
      // separately (MM < 2), for every right-hand side of the lane
      Acc2 acc[V], macc[V], dacc[V];
      float2 m32[V];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        acc[v].zero(), macc[v].zero(), dacc[v].zero();
        m32[v] = make_float2(0.f, 0.f);
      }
#pragma unroll 2
      for (int k = kb; k < ke; ++k) {
        const int4 raw = __ldg(reinterpret_cast<const int4 *>(bt.nz) + k);
        const float4 lo = __ldg(bt.nzlo + k);
        const int cj = raw.x;
        const float kh = __int_as_float(raw.y), mrh = __int_as_float(raw.z), mih = __int_as_float(raw.w);
        const float4 *pp = bt.pd + static_cast<long long>(cj) * R + rhs0;
        float4 pv[V];
        ldg_cols<V>(pp, pv);
        // Debye mass of this entry (nonzero only where it touches the region)
        const float mdh = lo.w;
        const float mdl = mdh != 0.f ? __ldg(bt.mdlo + k) : 0.f;
        if constexpr (MM >= 2) {
          if (mih == 0.f && lo.z == 0.f && mdh == 0.f) {
            // Real M (no lossy material on this entry): a = K - k0^2 M is
            // real and scales the real and imaginary lanes alike.  The test
            // is the same for every lane (one nonzero), so the branch does
            // not diverge.
#pragma unroll
            for (int v = 0; v < V; v += S) {
              float p, e, s, t, arh, arl;
              efg_dd::prod(k2h[v], k2l[v], mrh, lo.y, p, e);
              efg_dd::two_sum(kh, -p, s, t);
              efg_dd::fast_two_sum(s, (lo.x - e) + t, arh, arl);
              const float2 ah = f2(arh), ahn = f2(-arh), al = f2(arl);
#pragma unroll
              for (int u = 0; u < S; ++u) acc[v + u].add_prod(ahn, ah, al, hi2(pv[v + u]), lo2(pv[v + u]));
            }
          } else {
#pragma unroll
            for (int v = 0; v < V; v += S) {
              float p, e, s, t, arh, arl, aih, ail;
              efg_dd::prod(k2h[v], k2l[v], mrh, lo.y, p, e);
              efg_dd::two_sum(kh, -p, s, t);
              efg_dd::fast_two_sum(s, (lo.x - e) + t, arh, arl);
              efg_dd::prod(k2h[v], k2l[v], mih, lo.z, p, e);
              efg_dd::fast_two_sum(-p, -e, aih, ail);
              if (mdh != 0.f) {
                // a -= kappa * MD (kappa complex, MD real)
                efg_dd::prod(kap[v].x, kap[v].z, mdh, mdl, p, e);
                efg_dd::two_sum(arh, -p, s, t);
                efg_dd::two_sum(s, (arl - e) + t, arh, arl);
                efg_dd::prod(kap[v].y, kap[v].w, mdh, mdl, p, e);
                efg_dd::two_sum(aih, -p, s, t);
                efg_dd::two_sum(s, (ail - e) + t, aih, ail);
              }
              // (re, im) += (ar, ar)(x.re, x.im) + (-ai, ai)(x.im, x.re)
              const float2 rh = f2(arh), rhn = f2(-arh), rl = f2(arl);
              const float2 ih = make_float2(-aih, aih), ihn = make_float2(aih, -aih), il = make_float2(-ail, ail);
#pragma unroll
              for (int u = 0; u < S; ++u) {
                const float2 xh = hi2(pv[v + u]), xl = lo2(pv[v + u]);
                acc[v + u].add_prod(rhn, rh, rl, xh, xl);
                acc[v + u].add_prod(ihn, ih, il, swap2(xh), swap2(xl));
              }
            }
          }
        } else {
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const float2 xh = hi2(pv[v]), xl = lo2(pv[v]);
            acc[v].add_prod(f2(kh), f2(lo.x), xh, xl);
            if constexpr (MM == 1) {
              macc[v].add_prod(f2(mrh), f2(lo.y), xh, xl);
              if (mih != 0.f || lo.z != 0.f)  // same for every lane: no divergence
                macc[v].add_prod(make_float2(-mih, mih), make_float2(-lo.z, lo.z), swap2(xh), swap2(xl));
              if (mdh != 0.f) dacc[v].add_prod(f2(mdh), f2(mdl), xh, xl);
            } else {
              m32[v] = efg_dd::fma2(f2(mrh), xh, efg_dd::fma2(make_float2(-mih, mih), swap2(xh), m32[v]));
            }
          }
        }
      }
      float4 q[V];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        if constexpr (MM >= 2) {
          q[v] = acc[v].value();
        } else {
          const float4 mp = MM == 1 ? macc[v].value() : make_float4(m32[v].x, m32[v].y, 0.f, 0.f);
          q[v] = cadd(acc[v].value(), cneg(rmul(mp, k2h[v], k2l[v])));
          if (MM == 1 && bt.has_md) q[v] = cadd(q[v], cneg(cmul(dacc[v].value(), kap[v])));
        }
      }
      const int s = __ldg(bt.sidx + row);
      if (s >= 0) {
        double2 sacc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) sacc[v] = make_double2(0.0, 0.0);
        for (int e = __ldg(bt.sptr + s); e < __ldg(bt.sptr + s + 1); ++e) {
          const int cj = __ldg(bt.scol + e);
          const double val = __ldg(bt.sval64 + e);
          const int ci = __ldg(bt.scidx + e);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const double2 cf = __ldg(bt.scoef64 + ci * R + rhs0 + v);
            const double2 x = cjoin(__ldg(bt.pd + static_cast<long long>(cj) * R + rhs0 + v));
            sacc[v].x += val * (cf.x * x.x - cf.y * x.y);
            sacc[v].y += val * (cf.x * x.y + cf.y * x.x);
          }
        }
#pragma unroll
        for (int v = 0; v < V; ++v) q[v] = cadd(q[v], csplit(sacc[v].x, sacc[v].y));
      }
      float4 pr[V];
      ldg_cols<V>(bt.pd + static_cast<long long>(row) * R + rhs0, pr);
      st_cols<V>(bt.qd + static_cast<long long>(row) * R + rhs0, q);
#pragma unroll
      for (int v = 0; v < V; ++v) dot_add(pt.a[0][v], pt.a[1][v], pr[v], q[v]);
      pt.tick();
    }
  }
  if (cur >= 0) flush_partials<2, V>(pt, R, cur, dst, stride, rhs_of);
}

// Preconditioned residual z = D^-1 r + G t0 (+ Pi t) of one (edge, rhs):
// t0 and t_d gathered at the edge's end nodes (layout [node][1 + NPI][R]),
// pw the edge's NPI vector-nodal weights.  NPI is a compile-time count so
// that the 2 + 2 NPI gathers are issued together rather than one vector-
// nodal component after the other.
template <int NPI>
__device__ __forceinline__ float4 precond_z(const EfgkBatch &bt, int row, int rhs, int b, int2 en, float4 r,
                                            const float (&pw)[NPI > 0 ? NPI : 1]) {
  float4 z = cmul_f(r, crecipf(diag32(bt, row, rhs, b)));
  if (en.x < 0) return z;
  constexpr int NT = 1 + NPI;
  const long long R = bt.R;
  const float4 *ta = bt.td + static_cast<long long>(en.x) * NT * R + rhs;
  const float4 *tb = bt.td + static_cast<long long>(en.y) * NT * R + rhs;
  float4 ga[NT], gb[NT];
#pragma unroll
  for (int d = 0; d < NT; ++d) {
    ga[d] = __ldg(ta + d * R);
    gb[d] = __ldg(tb + d * R);
  }
  z = cadd(z, cadd(gb[0], cneg(ga[0])));
#pragma unroll
  for (int d = 0; d < NPI; ++d) z = cadd(z, rmul(cadd(ga[1 + d], gb[1 + d]), pw[d], 0.f));
  return z;
}

template <int NPI>
__device__ __forceinline__ void load_piw(const EfgkBatch &bt, int row, float (&pw)[NPI > 0 ? NPI : 1]) {
#pragma unroll
  for (int d = 0; d < NPI; ++d) pw[d] = __ldg(bt.piw + 3 * static_cast<long long>(row) + d);
}

// ------------------------------------------------------------ vector phases
// A thread owns W = 2 consecutive right-hand sides of one row; R % 2 == 0 and
// (kBS * 2) % R == 0, so its rhs set is the same on every row it visits.
// Two (rather than four) keep these kernels near 64 registers, so enough
// warps are resident to cover the memory latency of their loads.
constexpr int W = 2;

template <int N>
__device__ __forceinline__ void load_alpha_dd(const EfgkBatch &bt, int b, int rhs0, int P, float4 (&alpha)[N]) {
  const int R = bt.R, BR = bt.B * R, Q = 1 - P;
#pragma unroll
  for (int w = 0; w < N; ++w) {
    const long long i = static_cast<long long>(b) * R + rhs0 + w;
    const double2 rho = make_double2(bt.rho[Q * 2 * BR + 2 * i], bt.rho[Q * 2 * BR + 2 * i + 1]);
    const double2 pq = make_double2(bt.pq[P * 2 * BR + 2 * i], bt.pq[P * 2 * BR + 2 * i + 1]);
    double2 a = cdivd(rho, pq);
    if (bt.status[i] != 0 || !(isfinite(a.x) && isfinite(a.y))) a = make_double2(0.0, 0.0);
    alpha[w] = csplit(a.x, a.y);
  }
}

// r -= alpha q (and x += alpha p when do_x); r^T D^-1 r (dd) and |r|^2.
// Between checkpoints x is advanced by the p-update pass instead, which
// reads p anyway: this pass then moves 48 instead of 96 bytes per entry.
template <bool DO_X>
__global__ void __launch_bounds__(kBS, 3) dd_update_kernel(const EfgkBatch bt, const int P) {
  const int R = bt.R, BR = bt.B * R;
  const int rhs0 = (threadIdx.x * W) % R;
  DDPartials<3, W> pt;
  pt.clear();
  auto rhs_of = [R](int t, int w) { return (t * W + w) % R; };
  double *const dst[3] = {bt.rho + P * 2 * BR, bt.rho + P * 2 * BR + 1, bt.rr + P * BR};
  const int stride[3] = {2, 2, 1};
  int cur = static_cast<int>(blockIdx.x) < bt.n_chunks ? bt.chunk_inst[blockIdx.x] : -1;
  float4 alpha[W];
  if (cur >= 0) load_alpha_dd(bt, cur, rhs0, P, alpha);
  for (int c = blockIdx.x; c < bt.n_chunks; c += gridDim.x) {
    const int b = bt.chunk_inst[c];
    if (b != cur) {
      flush_partials<3, W>(pt, R, cur, dst, stride, rhs_of);
      cur = b;
      load_alpha_dd(bt, cur, rhs0, P, alpha);
    }
    if (warp_done(bt, b, rhs0, W)) continue;
    const int r0 = bt.chunk_begin[c], r1 = bt.chunk_end[c];
    const long long base = static_cast<long long>(r0) * R;
    const int total = (r1 - r0) * R;
    for (int e = threadIdx.x * W; e < total; e += kBS * W) {
      const int row = r0 + e / R;
      const long long o = base + e;
      // All loads first: the stores below may alias them as far as the
      // compiler knows, and issuing them together keeps 256 B in flight.
      float4 pv[W], qv[W], xv[W], rv[W];
      if (DO_X) ldg_cols<W>(bt.pd + o, pv);
      ldg_cols<W>(bt.qd + o, qv);
      if (DO_X) ld_cols<W>(bt.xd + o, xv);
      ld_cols<W>(bt.rd + o, rv);
#pragma unroll
      for (int w = 0; w < W; ++w) {
        if (DO_X) xv[w] = cadd(xv[w], cmul(alpha[w], pv[w]));
        rv[w] = cadd(rv[w], cneg(cmul(alpha[w], qv[w])));
        const float4 z = cmul_f(rv[w], crecipf(diag32(bt, row, rhs0 + w, b)));
        dot_add(pt.a[0][w], pt.a[1][w], rv[w], z);
        pt.a[2][w].add(efg_dd::cabs2_hi(rv[w]), 0.f);
      }
      if (DO_X) st_cols<W>(bt.xd + o, xv);
      st_cols<W>(bt.rd + o, rv);
    }
  }
  if (cur >= 0) flush_partials<3, W>(pt, R, cur, dst, stride, rhs_of);
}

// Node pass: t0 = Dn^-1 G^T r and, with NPI = 3, t_d = omega Dp^-1 (Pi^T r)_d
// (d = x, y, z), stored per node as [1 + NPI][R]; s^T t of every space into
// rho[P].  only_flagged restricts it to right-hand sides flagged for
// replacement.
template <int V, int NPI>
__global__ void __launch_bounds__(kBS, NPI ? 3 : 4) dd_node_kernel(const EfgkBatch bt, const int P, const int only_flagged) {
  if (only_flagged && bt.counters[1] == 0) return;
  constexpr int NT = 1 + NPI;
  // incidences per load batch: 2 where the vector-nodal sums already hold
  // 12 accumulators per lane (4 measured the same, at more registers)
  constexpr int KU = NPI && V > 1 ? 2 : 4;
  const int R = bt.R, BR = bt.B * R;
  const int G = R / V;
  const int group = threadIdx.x / G, lane = threadIdx.x % G, ngroups = kBS / G;
  const int rhs0 = lane * V;
  DDPartials<2, V> pt;
  pt.clear();
  auto rhs_of = [G](int t, int w) { return (t % G) * V + w; };
  double *const dst[2] = {bt.rho + P * 2 * BR, bt.rho + P * 2 * BR + 1};
  const int stride[2] = {2, 2};
  int cur = static_cast<int>(blockIdx.x) < bt.n_nchunks ? bt.nchunk_inst[blockIdx.x] : -1;
  bool act[V];
  for (int c = blockIdx.x; c < bt.n_nchunks; c += gridDim.x) {
    const int b = bt.nchunk_inst[c];
    if (b != cur) {
      flush_partials<2, V>(pt, R, cur, dst, stride, rhs_of);
      cur = b;
    }
#pragma unroll
    for (int v = 0; v < V; ++v) act[v] = !only_flagged || bt.flag[b * R + rhs0 + v] != 0;
    bool any = false;
#pragma unroll
    for (int v = 0; v < V; ++v) any |= act[v];
    if (!any) continue;  // no flagged right-hand side in this lane's set
    const int n1 = bt.nchunk_end[c];
    for (int node = bt.nchunk_begin[c] + group; node < n1; node += ngroups) {
      float4 s[V];
      Acc2 pacc[V][NPI > 0 ? NPI : 1];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        s[v] = zero4();
#pragma unroll
        for (int d = 0; d < NPI; ++d) pacc[v][d].zero();
      }
      const int k1 = __ldg(bt.nptr + node + 1);
      // KU incidences at a time: their records, then their rows of r, are
      // loaded together, so each group keeps KU gathers in flight instead
      // of waiting out one record-then-row latency per incidence.
      for (int k0 = __ldg(bt.nptr + node); k0 < k1; k0 += KU) {
        // one 16-byte record per incidence: edge (bit-inverted at its tail)
        // and the edge's three vector-nodal weights
        int4 inc[KU];
#pragma unroll
        for (int u = 0; u < KU; ++u) inc[u] = k0 + u < k1 ? __ldg(bt.ninc + k0 + u) : make_int4(0, 0, 0, 0);
        float4 rv[KU][V];
#pragma unroll
        for (int u = 0; u < KU; ++u) {
          const int e = inc[u].x < 0 ? ~inc[u].x : inc[u].x;
          if (k0 + u < k1) {
            ldg_cols<V>(bt.rd + static_cast<long long>(e) * R + rhs0, rv[u]);
          } else {
#pragma unroll
            for (int v = 0; v < V; ++v) rv[u][v] = zero4();
          }
        }
#pragma unroll
        for (int u = 0; u < KU; ++u) {
          const bool neg = inc[u].x < 0;
          const float w[3] = {__int_as_float(inc[u].y), __int_as_float(inc[u].z), __int_as_float(inc[u].w)};
#pragma unroll
          for (int v = 0; v < V; ++v) {
            s[v] = cadd(s[v], neg ? cneg(rv[u][v]) : rv[u][v]);
#pragma unroll
            for (int d = 0; d < NPI; ++d) pacc[v][d].add_prod(f2(w[d]), f2(0.f), hi2(rv[u][v]), lo2(rv[u][v]));
          }
        }
      }
      float4 *tp = bt.td + static_cast<long long>(node) * NT * R + rhs0;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        if (!act[v]) continue;
        const float4 t = cmul_f(s[v], crecipf(ndiag32(bt, node, rhs0 + v, b)));
        tp[v] = t;
        dot_add(pt.a[0][v], pt.a[1][v], s[v], t);
#pragma unroll
        for (int d = 0; d < NPI; ++d) {
          const float4 sd = pacc[v][d].value();
          const float4 td = cmul_f(sd, crecipf(pdiag32(bt, node, d, rhs0 + v, b)));
          tp[(1 + d) * R + v] = td;
          dot_add(pt.a[0][v], pt.a[1][v], sd, td);
        }
      }
      pt.tick();
    }
  }
  if (cur >= 0) flush_partials<2, V>(pt, R, cur, dst, stride, rhs_of);
}

// The p-update pass waits on its gathers of t, so resident warps matter
// more than the registers of a deeper schedule: one right-hand side per
// thread (where kBS % R == 0) and three blocks per SM, 72-80 registers
// without spills, 24 resident warps.  On the 24x12x60 guide (R = 128) a
// launch takes 326 us against 348 us for two right-hand sides per thread at
// two blocks per SM (114 registers) and 348 us for one per thread at four
// blocks (64 registers, spilling).
constexpr int kPupWP = 1;
constexpr int kPupMinBlocks = 3;

// x += alpha p (when DO_X: the iterations without a checkpoint), then
// p = D^-1 r + G t + beta p.  restart (checkpoint iterations): right-hand
// sides whose residual was replaced because they stagnated restart their
// direction (beta = 0); after an ordinary replacement the direction is kept.
// WP consecutive right-hand sides per thread ((kBS * WP) % R == 0).
template <bool DO_X, int NPI, int WP>
__global__ void __launch_bounds__(kBS, kPupMinBlocks) dd_pupdate_kernel(const EfgkBatch bt, const int P, const int restart) {
  const int R = bt.R, BR = bt.B * R;
  const int Q = 1 - P;
  // pq[Q] is the next iteration's SpMM accumulator (alpha reads pq[P])
  if (blockIdx.x == 0) block_zero(bt.pq + Q * 2 * BR, 2 * BR);
  const int rhs0 = (threadIdx.x * WP) % R;
  int cur = -1;
  float4 beta[WP], alpha[WP];
  for (int c = blockIdx.x; c < bt.n_chunks; c += gridDim.x) {
    const int b = bt.chunk_inst[c];
    if (b != cur) {
      cur = b;
      if (DO_X) load_alpha_dd<WP>(bt, cur, rhs0, P, alpha);
#pragma unroll
      for (int w = 0; w < WP; ++w) {
        const long long i = static_cast<long long>(b) * R + rhs0 + w;
        const double2 rn = make_double2(bt.rho[P * 2 * BR + 2 * i], bt.rho[P * 2 * BR + 2 * i + 1]);
        const double2 ro = make_double2(bt.rho[Q * 2 * BR + 2 * i], bt.rho[Q * 2 * BR + 2 * i + 1]);
        double2 be = cdivd(rn, ro);
        // Stopped right-hand sides restart from p = z so p stays bounded.
        if (bt.status[i] != 0 || (restart && bt.flag[i] == 2) || !(isfinite(be.x) && isfinite(be.y)))
          be = make_double2(0.0, 0.0);
        beta[w] = csplit(be.x, be.y);
      }
    }
    if (warp_done(bt, b, rhs0, WP)) continue;
    const int r0 = bt.chunk_begin[c], r1 = bt.chunk_end[c];
    const long long base = static_cast<long long>(r0) * R;
    const int total = (r1 - r0) * R;
    for (int e = threadIdx.x * WP; e < total; e += kBS * WP) {
      const int row = r0 + e / R;
      const long long o = base + e;
      const int2 en = __ldg(bt.enodes + row);
      float pw[NPI > 0 ? NPI : 1];
      load_piw<NPI>(bt, row, pw);
      float4 rv[WP], pv[WP], xv[WP];
#pragma unroll
      for (int w = 0; w < WP; ++w) {
        rv[w] = __ldg(bt.rd + o + w);
        pv[w] = bt.pd[o + w];
        if (DO_X) xv[w] = bt.xd[o + w];
      }
      if (DO_X) {
#pragma unroll
        for (int w = 0; w < WP; ++w) bt.xd[o + w] = cadd(xv[w], cmul(alpha[w], pv[w]));
      }
#pragma unroll
      for (int w = 0; w < WP; ++w)
        pv[w] = cadd(precond_z<NPI>(bt, row, rhs0 + w, b, en, rv[w], pw), cmul(beta[w], pv[w]));
#pragma unroll
      for (int w = 0; w < WP; ++w) bt.pd[o + w] = pv[w];
    }
  }
}

// p = D^-1 r + G t (first direction).
template <int NPI>
__global__ void __launch_bounds__(kBS) dd_pinit_kernel(const EfgkBatch bt) {
  const int R = bt.R;
  const int rhs0 = (threadIdx.x * W) % R;
  for (int c = blockIdx.x; c < bt.n_chunks; c += gridDim.x) {
    const int b = bt.chunk_inst[c];
    const int r0 = bt.chunk_begin[c], r1 = bt.chunk_end[c];
    const long long base = static_cast<long long>(r0) * R;
    const int total = (r1 - r0) * R;
    for (int e = threadIdx.x * W; e < total; e += kBS * W) {
      const int row = r0 + e / R;
      const long long o = base + e;
      const int2 en = __ldg(bt.enodes + row);
      float pw[NPI > 0 ? NPI : 1];
      load_piw<NPI>(bt, row, pw);
#pragma unroll
      for (int w = 0; w < W; ++w) bt.pd[o + w] = precond_z<NPI>(bt, row, rhs0 + w, b, en, bt.rd[o + w], pw);
    }
  }
}

// ------------------------------------------------------- residual replacement
// True residual r = b - A x for flagged right-hand sides (all with do_all),
// in dd arithmetic with the operator's low words (K and M to about 48 bits
// of their FP64 values; port-face rows in FP64): r stored as dd, r^T D^-1 r
// and |r|^2 into slot P.  Lane layout as in the SpMM; a lane whose right-hand
// sides are all unflagged skips the rows, so a checkpoint costs in
// proportion to the flagged fraction.
template <int V>
__global__ void __launch_bounds__(kBS) dd_resid_kernel(const EfgkBatch bt, const int P, const int do_all) {
  if (!do_all && bt.counters[1] == 0) return;
  const int R = bt.R;
  const int LW = R / V < 32 ? R / V : 32;
  const int T = R / (LW * V);
  const int BR = bt.B * R;
  const int g = threadIdx.x / LW, lane = threadIdx.x % LW;
  const int tile = g % T, group = g / T, ngroups = kBS / LW / T;
  const int rhs0 = tile * LW * V + lane * V;
  float k2h[V], k2l[V];
#pragma unroll
  for (int v = 0; v < V; ++v) efg_dd::split(__ldg(bt.k0sq64 + rhs0 + v), k2h[v], k2l[v]);
  float4 kap[V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const double2 ka = bt.has_md ? __ldg(bt.kappa64 + rhs0 + v) : make_double2(0.0, 0.0);
    kap[v] = csplit(ka.x, ka.y);
  }
  DDPartials<3, V> pt;
  pt.clear();
  auto rhs_of = [LW, T](int t, int w) { return ((t / LW) % T) * LW * V + (t % LW) * V + w; };
  double *const dst[3] = {bt.rho + P * 2 * BR, bt.rho + P * 2 * BR + 1, bt.rr + P * BR};
  const int stride[3] = {2, 2, 1};
  int cur = static_cast<int>(blockIdx.x) < bt.n_chunks ? bt.chunk_inst[blockIdx.x] : -1;
  bool act[V];
  for (int c = blockIdx.x; c < bt.n_chunks; c += gridDim.x) {
    const int b = bt.chunk_inst[c];
    if (b != cur) {
      flush_partials<3, V>(pt, R, cur, dst, stride, rhs_of);
      cur = b;
    }
    bool any = false;
#pragma unroll
    for (int v = 0; v < V; ++v) any |= (act[v] = do_all || bt.flag[b * R + rhs0 + v] != 0);
    if (!any) continue;
    const int r1 = bt.chunk_end[c];
    for (int row = bt.chunk_begin[c] + group; row < r1; row += ngroups) {
      const int kb = __ldg(bt.rowptr + row), ke = __ldg(bt.rowptr + row + 1);
      Acc2 kacc[V], macc[V], dacc[V];
#pragma unroll
      for (int v = 0; v < V; ++v) kacc[v].zero(), macc[v].zero(), dacc[v].zero();
      for (int k = kb; k < ke; ++k) {
        const int4 raw = __ldg(reinterpret_cast<const int4 *>(bt.nz) + k);
        const float4 lo = __ldg(bt.nzlo + k);
        const float kh = __int_as_float(raw.y), mrh = __int_as_float(raw.z), mih = __int_as_float(raw.w);
        const float mdh = lo.w;
        const float mdl = mdh != 0.f ? __ldg(bt.mdlo + k) : 0.f;
        const float4 *xp = bt.xd + static_cast<long long>(raw.x) * R + rhs0;
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const float4 x = xp[v];
          const float2 xh = hi2(x), xl = lo2(x);
          kacc[v].add_prod(f2(kh), f2(lo.x), xh, xl);
          macc[v].add_prod(f2(mrh), f2(lo.y), xh, xl);
          macc[v].add_prod(make_float2(-mih, mih), make_float2(-lo.z, lo.z), swap2(xh), swap2(xl));
          if (mdh != 0.f) dacc[v].add_prod(f2(mdh), f2(mdl), xh, xl);
        }
      }
      float4 ax[V];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        ax[v] = cadd(kacc[v].value(), cneg(rmul(macc[v].value(), k2h[v], k2l[v])));
        if (bt.has_md) ax[v] = cadd(ax[v], cneg(cmul(dacc[v].value(), kap[v])));
      }
      const int s = __ldg(bt.sidx + row);
      if (s >= 0) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const int rhs = rhs0 + v;
          double px = 0.0, py = 0.0;
          for (int e = __ldg(bt.sptr + s); e < __ldg(bt.sptr + s + 1); ++e) {
            const double val = __ldg(bt.sval64 + e);
            const double2 cf = __ldg(bt.scoef64 + __ldg(bt.scidx + e) * R + rhs);
            const double2 x = cjoin(bt.xd[static_cast<long long>(__ldg(bt.scol + e)) * R + rhs]);
            px += val * (cf.x * x.x - cf.y * x.y);
            py += val * (cf.x * x.y + cf.y * x.x);
          }
          // minus b = rcoef(b, a, f) c_a[row] for the active port a = rhs % P
          if (rhs < bt.F * bt.P) {
            const int a = rhs % bt.P;
            const double2 cf = __ldg(bt.rcoef64 + (b * bt.P + a) * R + rhs);
            const double2 cv = __ldg(bt.cval + s * bt.P + a);
            px -= cf.x * cv.x - cf.y * cv.y;
            py -= cf.x * cv.y + cf.y * cv.x;
          }
          ax[v] = cadd(ax[v], csplit(px, py));
        }
      }
      float4 *rp = bt.rd + static_cast<long long>(row) * R + rhs0;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        if (!act[v]) continue;
        const float4 r = cneg(ax[v]);  // r = b - A x
        rp[v] = r;
        const float4 z = cmul_f(r, crecipf(diag32(bt, row, rhs0 + v, b)));
        dot_add(pt.a[0][v], pt.a[1][v], r, z);
        pt.a[2][v].add(efg_dd::cabs2_hi(r), 0.f);
      }
    }
  }
  if (cur >= 0) flush_partials<3, V>(pt, R, cur, dst, stride, rhs_of);
}

// Initial residual of x = 0: r = b (nonzero on port rows only), stored as
// dd; |b|^2 and b^T D^-1 b into slot P.  One lane per right-hand side,
// G = min(R, 32) lanes per row.  (Restarts from a nonzero x use the
// double-float true residual, dd_resid_kernel.)
__global__ void __launch_bounds__(kBS) dd_residual_kernel(const EfgkBatch bt, const int P) {
  const int R = bt.R, BR = bt.B * R;
  const int G = R < 32 ? R : 32;
  const int VR = R / G;
  const int group = threadIdx.x / G, lane = threadIdx.x % G, ngroups = kBS / G;
  Partials<3, 4> pt;
  pt.clear();
  auto rhs_of = [G](int t, int w) { return (t % G) + w * G; };
  double *const dst[3] = {bt.rho + P * 2 * BR, bt.rho + P * 2 * BR + 1, bt.rr + P * BR};
  const int stride[3] = {2, 2, 1};
  int cur = static_cast<int>(blockIdx.x) < bt.n_chunks ? bt.chunk_inst[blockIdx.x] : -1;
  for (int c = blockIdx.x; c < bt.n_chunks; c += gridDim.x) {
    const int b = bt.chunk_inst[c];
    if (b != cur) {
      flush_partials<3, 4>(pt, R, cur, dst, stride, rhs_of);
      cur = b;
    }
    const int r1 = bt.chunk_end[c];
    for (int row = bt.chunk_begin[c] + group; row < r1; row += ngroups) {
      const int s = __ldg(bt.sidx + row);
      for (int v = 0; v < VR; ++v) {
        const int rhs = lane + v * G;
        double bx = 0.0, by = 0.0;
        // b = rcoef(b, a, f) c_a[row] for the active port a = rhs % P
        if (s >= 0 && rhs < bt.F * bt.P) {
          const int a = rhs % bt.P;
          const double2 cf = __ldg(bt.rcoef64 + (b * bt.P + a) * R + rhs);
          const double2 cv = __ldg(bt.cval + s * bt.P + a);
          bx = cf.x * cv.x - cf.y * cv.y;
          by = cf.x * cv.y + cf.y * cv.x;
        }
        const float4 r = csplit(bx, by);
        bt.rd[static_cast<long long>(row) * R + rhs] = r;
        if (s < 0) continue;  // r = 0 off the port rows
        const double2 z = cjoin(cmul_f(r, crecipf(diag32(bt, row, rhs, b))));
        pt.d[0][v] += bx * z.x - by * z.y;
        pt.d[1][v] += bx * z.y + by * z.x;
        pt.d[2][v] += bx * bx + by * by;
      }
    }
  }
  if (cur >= 0) flush_partials<3, 4>(pt, R, cur, dst, stride, rhs_of);
}

// S_acc[b][j][rhs] += sum over port rows of conj(c_j[row]) * x[row][rhs].
__global__ void __launch_bounds__(kBS) dd_overlap_kernel(const EfgkBatch bt, const int rows_per_block) {
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
        const double2 x = cjoin(bt.xd[static_cast<long long>(bt.srow_row[s]) * R + rhs]);
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

// out[row][c] = in[row][map[c]] (0 where map[c] < 0): repacks the kept
// right-hand-side columns of a [rows][r_old] dd vector into [rows][r_new].
__global__ void gather_cols_kernel(long long rows, int r_old, int r_new, const int *__restrict__ map,
                                   const float4 *__restrict__ in, float4 *out) {
  const long long total = rows * r_new;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long row = i / r_new;
    const int m = __ldg(map + static_cast<int>(i - row * r_new));
    out[i] = m >= 0 ? __ldg(in + row * r_old + m) : zero4();
  }
}

__global__ void dd_pack_md_kernel(long long nnz, const double *__restrict__ md, float4 *nzlo, float *mdlo) {
  for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < nnz;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double v = md[k];
    const float h = static_cast<float>(v);
    nzlo[k].w = h;
    mdlo[k] = static_cast<float>(v - static_cast<double>(h));
  }
}

// Low words of the packed operator: FP64 master minus its FP32 high word.
__global__ void dd_pack_lo_kernel(long long nnz, const EfgkNz *__restrict__ nz, const double *__restrict__ K64,
                                  const double2 *__restrict__ M64, float4 *nzlo) {
  for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < nnz;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const EfgkNz h = nz[k];
    const double2 m = M64[k];
    nzlo[k] = make_float4(static_cast<float>(K64[k] - static_cast<double>(h.k)),
                          static_cast<float>(m.x - static_cast<double>(h.mre)),
                          static_cast<float>(m.y - static_cast<double>(h.mim)), 0.f);
  }
}

int g_grid = 0, g_sms = 0;
int grid() {
  if (!g_grid) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_sms = sms > 0 ? sms : 132;
    g_grid = g_sms * 4;
  }
  return g_grid;
}
inline int grid_for(int chunks) { return chunks < grid() ? (chunks > 0 ? chunks : 1) : grid(); }

// One full wave of a kernel: resident blocks per SM (from its register and
// shared-memory use) times the SM count, capped by the work units.
template <class K>
int wave_grid(K kernel, int units) {
  grid();
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBS, 0) != cudaSuccess || per_sm <= 0)
    per_sm = 2;
  const int g = per_sm * g_sms;
  return units < g ? (units > 0 ? units : 1) : g;
}

// One full wave of resident blocks (a grid of 4 blocks per SM with 3
// resident would run its last quarter as a second, mostly idle wave).
template <int V, int NPI>
void node_launch_v(const EfgkBatch &bt, int P, int only, cudaStream_t s) {
  static int g_wave = 0;
  if (!g_wave) g_wave = wave_grid(dd_node_kernel<V, NPI>, 1 << 30);
  const int g = bt.n_nchunks < g_wave ? (bt.n_nchunks > 0 ? bt.n_nchunks : 1) : g_wave;
  dd_node_kernel<V, NPI><<<g, kBS, 0, s>>>(bt, P, only);
}

int node_launch(const EfgkBatch &bt, int P, int only, cudaStream_t s) {
  if (bt.npi == 3) {
    // the vector-nodal sums hold 12 accumulators per right-hand side: two
    // right-hand sides per lane at most
    if (bt.R >= 64)
      node_launch_v<2, 3>(bt, P, only, s);
    else
      node_launch_v<1, 3>(bt, P, only, s);
    return static_cast<int>(cudaGetLastError());
  }
  const int V = bt.R >= 32 ? bt.R / 32 : 1;
  switch (V) {
    case 1: node_launch_v<1, 0>(bt, P, only, s); break;
    case 2: node_launch_v<2, 0>(bt, P, only, s); break;
    case 4: node_launch_v<4, 0>(bt, P, only, s); break;
    default: return static_cast<int>(cudaErrorInvalidValue);
  }
  return static_cast<int>(cudaGetLastError());
}

template <int NPI, int WP>
void pupdate_launch(const EfgkBatch &bt, int P, int restart, bool do_x, cudaStream_t s) {
  static int g_wave = 0;
  if (!g_wave) g_wave = wave_grid(dd_pupdate_kernel<true, NPI, WP>, 1 << 30);
  const int g = bt.n_chunks < g_wave ? (bt.n_chunks > 0 ? bt.n_chunks : 1) : g_wave;
  if (do_x)
    dd_pupdate_kernel<true, NPI, WP><<<g, kBS, 0, s>>>(bt, P, restart);
  else
    dd_pupdate_kernel<false, NPI, WP><<<g, kBS, 0, s>>>(bt, P, restart);
}

int resid_launch(const EfgkBatch &bt, int P, int do_all, int g, int V, cudaStream_t s) {
  switch (V) {
    case 1: dd_resid_kernel<1><<<g, kBS, 0, s>>>(bt, P, do_all); break;
    case 2: dd_resid_kernel<2><<<g, kBS, 0, s>>>(bt, P, do_all); break;
    case 4: dd_resid_kernel<4><<<g, kBS, 0, s>>>(bt, P, do_all); break;
    default: return static_cast<int>(cudaErrorInvalidValue);
  }
  return static_cast<int>(cudaGetLastError());
}

template <int MM, bool TM>
int spmm_launch(const EfgkBatch &bt, int P, int g, int V, cudaStream_t s) {
  switch (V) {
    case 1: dd_spmm_kernel<1, MM == 2 ? 3 : MM, TM><<<g, kBS, 0, s>>>(bt, P); break;
    case 2: dd_spmm_kernel<2, MM, TM><<<g, kBS, 0, s>>>(bt, P); break;
    case 4: dd_spmm_kernel<4, MM, TM><<<g, kBS, 0, s>>>(bt, P); break;
    default: return static_cast<int>(cudaErrorInvalidValue);
  }
  return static_cast<int>(cudaGetLastError());
}
template <int MM>
int spmm_launch(const EfgkBatch &bt, int P, int g, int V, bool tm, cudaStream_t s) {
  return tm ? spmm_launch<MM, true>(bt, P, g, V, s) : spmm_launch<MM, false>(bt, P, g, V, s);
}

}  // namespace

extern "C" int efgk_batch_dd_spmm(const EfgkBatch *bt, int parity, int grid_blocks, int rhs_per_lane, int m_mode,
                                  efgk_stream_t stream) {
  const int g = grid_blocks > 0 ? grid_blocks : grid_for(bt->n_chunks);
  int V = rhs_per_lane;
  if (V <= 0) V = bt->R >= 32 ? bt->R / 32 : 1;
  if (bt->R % V != 0) return static_cast<int>(cudaErrorInvalidValue);
  const bool tm = (m_mode & 16) != 0;  // tile-major work order
  m_mode &= 15;
  if (m_mode == 2 && bt->P % 2 != 0) m_mode = 3;  // shared coefficient needs port pairs
  if (m_mode == 3) return spmm_launch<3>(*bt, parity, g, V, tm, stream);
  if (m_mode == 2) return spmm_launch<2>(*bt, parity, g, V, tm, stream);
  return m_mode ? spmm_launch<1>(*bt, parity, g, V, tm, stream) : spmm_launch<0>(*bt, parity, g, V, tm, stream);
}

extern "C" int efgk_batch_dd_update(const EfgkBatch *bt, int parity, efgk_stream_t stream) {
  // bit 1 of `parity`: advance x here (checkpoint iterations); otherwise the
  // p-update pass does it
  static int g_upd = 0;
  if (!g_upd) g_upd = wave_grid(dd_update_kernel<true>, 1 << 30);
  const int g = bt->n_chunks < g_upd ? bt->n_chunks : g_upd;
  if (parity & 2)
    dd_update_kernel<true><<<g, kBS, 0, stream>>>(*bt, parity & 1);
  else
    dd_update_kernel<false><<<g, kBS, 0, stream>>>(*bt, parity & 1);
  const int err = static_cast<int>(cudaGetLastError());
  if (err) return err;
  return node_launch(*bt, parity & 1, 0, stream);
}

extern "C" int efgk_batch_dd_checkpoint(const EfgkBatch *bt, int parity, int iters_done, efgk_stream_t stream) {
  batch_flag_kernel<<<1, 1024, 0, stream>>>(*bt, parity, iters_done);
  int err = resid_launch(*bt, parity, 0, grid_for(bt->n_chunks), bt->R >= 32 ? bt->R / 32 : 1, stream);
  if (err) return err;
  err = node_launch(*bt, parity, 1, stream);
  if (err) return err;
  batch_post_kernel<<<1, 1024, 0, stream>>>(*bt, parity, iters_done);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_dd_pupdate(const EfgkBatch *bt, int parity, efgk_stream_t stream) {
  // bit 1 of `parity`: restart the directions of replaced right-hand sides;
  // bit 2: advance x here (x += alpha p with the old p)
  const int P = parity & 1, restart = (parity >> 1) & 1;
  if (bt->npi != 0 && bt->npi != 3) return static_cast<int>(cudaErrorInvalidValue);
  if (bt->npi == 3) {
    if (kBS % bt->R == 0)
      pupdate_launch<3, kPupWP>(*bt, P, restart, (parity & 4) != 0, stream);
    else
      pupdate_launch<3, 2>(*bt, P, restart, (parity & 4) != 0, stream);
  } else {
    if (kBS % bt->R == 0)
      pupdate_launch<0, kPupWP>(*bt, P, restart, (parity & 4) != 0, stream);
    else
      pupdate_launch<0, 2>(*bt, P, restart, (parity & 4) != 0, stream);
  }
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_dd_init(const EfgkBatch *bt, efgk_stream_t stream) {
  // x = t = 0 and all accumulators zeroed by the host beforehand.  r = b
  // (true residual of x = 0) into parity slot 1, then |b|^2, t, p.
  dd_residual_kernel<<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt, 1);
  batch_init_scalars_kernel<<<1, 1024, 0, stream>>>(*bt);
  const int err = node_launch(*bt, 1, 0, stream);
  if (err) return err;
  if (bt->npi == 3)
    dd_pinit_kernel<3><<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt);
  else if (bt->npi == 0)
    dd_pinit_kernel<0><<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt);
  else
    return static_cast<int>(cudaErrorInvalidValue);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_dd_restart(const EfgkBatch *bt, efgk_stream_t stream) {
  const long long BR = static_cast<long long>(bt->B) * bt->R;
  cudaMemsetAsync(bt->rho + 2 * BR, 0, 2 * BR * sizeof(double), stream);
  cudaMemsetAsync(bt->rr + BR, 0, BR * sizeof(double), stream);
  int err = resid_launch(*bt, 1, 1, grid_for(bt->n_chunks), bt->R >= 32 ? bt->R / 32 : 1, stream);
  if (err) return err;
  err = node_launch(*bt, 1, 0, stream);
  if (err) return err;
  if (bt->npi == 3)
    dd_pinit_kernel<3><<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt);
  else if (bt->npi == 0)
    dd_pinit_kernel<0><<<grid_for(bt->n_chunks), kBS, 0, stream>>>(*bt);
  else
    return static_cast<int>(cudaErrorInvalidValue);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_dd_finish(const EfgkBatch *bt, efgk_stream_t stream) {
  const int rpb = 64;
  const int nb = (bt->n_srows + rpb - 1) / rpb;
  if (nb > 0) dd_overlap_kernel<<<nb, kBS, 0, stream>>>(*bt, rpb);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_gather_cols(int64_t rows, int32_t r_old, int32_t r_new, const int32_t *map,
                                      const void *in, void *out, efgk_stream_t stream) {
  if (rows <= 0 || r_new <= 0) return 0;
  if (in == out) return static_cast<int>(cudaErrorInvalidValue);
  gather_cols_kernel<<<4 * grid(), kBS, 0, stream>>>(rows, r_old, r_new, map, static_cast<const float4 *>(in),
                                                     static_cast<float4 *>(out));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_pack_md(int64_t nnz, const double *MD64, void *nzlo, float *mdlo, efgk_stream_t stream) {
  if (nnz <= 0) return 0;
  dd_pack_md_kernel<<<1024, kBS, 0, stream>>>(nnz, MD64, static_cast<float4 *>(nzlo), mdlo);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_batch_pack_lo(int64_t nnz, const void *nz, const double *K64, const double *M64, void *nzlo,
                                  efgk_stream_t stream) {
  if (nnz <= 0) return 0;
  dd_pack_lo_kernel<<<1024, kBS, 0, stream>>>(nnz, static_cast<const EfgkNz *>(nz), K64,
                                              reinterpret_cast<const double2 *>(M64), static_cast<float4 *>(nzlo));
  return static_cast<int>(cudaGetLastError());
}
