// Reduced-basis initial guesses for a frequency sweep (FP64).
//
// The solutions x(f) of one mesh over a band lie close to a space of low
// dimension: the converged solutions at a few sample frequencies, made
// orthonormal (Q, n x k), reproduce the solution at any frequency of the
// band through the Galerkin system (Q^T A(f) Q) y = Q^T b(f), x0 = Q y, to
// about the accuracy of the samples.  These kernels build Q by classical
// Gram-Schmidt with one reorthogonalisation pass, the k x k products
// Q^T K Q, Q^T M Q, Q^T M_D Q of the engine's FP64 operator, and x0 = Q Y
// for every column of the sweep (written as complex double-float into the
// batched engine's x).  The engine then starts its Krylov iteration from
// x0 with the true residual b - A x0, so the tolerance it reports holds
// whatever the quality of x0.
//
// Layout: Q, W row-major [n][ld] complex FP64 (double2), one row per edge
// row of the instance; the engine's x is [N][R] float4 (re_hi, im_hi,
// re_lo, im_lo).
#include <cuda_runtime.h>

#include "batch_common.cuh"
#include "edgefem_gb300_kernels.h"

namespace {

using efg_batch::kBS;
using efg_dd::cjoin;
using efg_dd::csplit;

__device__ __forceinline__ double2 cmad(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
// conj(a) * b + c
__device__ __forceinline__ double2 cmadc(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}

int g_blocks = 0;
int blocks() {
  if (!g_blocks) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_blocks = 4 * (sms > 0 ? sms : 132);
  }
  return g_blocks;
}

// out[row][map[c]] = in[row][c] wherever map[c] >= 0; other columns of out
// are left as they are.
__global__ void scatter_cols_kernel(long long rows, int r_in, int r_out, const int *__restrict__ map,
                                    const float4 *__restrict__ in, float4 *out) {
  const long long total = rows * r_in;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long row = i / r_in;
    const int m = __ldg(map + static_cast<int>(i - row * r_in));
    if (m >= 0) out[row * r_out + m] = in[i];
  }
}

// v[row] = x[row0 + row][col] joined to FP64; |v|^2 into *nrm.
__global__ void load_col_kernel(long long n, const float4 *__restrict__ x, int r, long long row0, int col,
                                double2 *v, double *nrm) {
  __shared__ double sh[kBS / 32];
  double s = 0.0;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double2 a = cjoin(x[(row0 + i) * r + col]);
    v[i] = a;
    s += a.x * a.x + a.y * a.y;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kBS / 32; ++w) t += sh[w];
    atomicAdd(nrm, t);
  }
}

// Contiguous row range of warp gw of nw warps.
__device__ __forceinline__ void warp_rows(long long n, long long &r0, long long &r1) {
  const long long nw = static_cast<long long>(gridDim.x) * (kBS / 32);
  const long long gw = static_cast<long long>(blockIdx.x) * (kBS / 32) + (threadIdx.x >> 5);
  const long long per = (n + nw - 1) / nw;
  r0 = gw * per < n ? gw * per : n;
  r1 = r0 + per < n ? r0 + per : n;
}

// h[t] += sum_row conj(Q[row][t]) v[row], t < k <= 32 U: each warp takes a
// contiguous range of rows, four at a time (their loads issued together),
// lane t, t + 32, ... of each row.
template <int U>
__global__ void proj_kernel(long long n, const double2 *__restrict__ Q, int ld, int k,
                            const double2 *__restrict__ v, double *h) {
  constexpr int RU = 4;
  __shared__ double2 sh[kBS / 32][32 * U];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double2 acc[U];
#pragma unroll
  for (int u = 0; u < U; ++u) acc[u] = make_double2(0.0, 0.0);
  long long r0, r1;
  warp_rows(n, r0, r1);
  for (long long row = r0; row < r1; row += RU) {
    double2 vr[RU], q[RU][U];
#pragma unroll
    for (int j = 0; j < RU; ++j) {
      const bool ok = row + j < r1;
      vr[j] = ok ? __ldg(v + row + j) : make_double2(0.0, 0.0);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int t = lane + 32 * u;
        q[j][u] = ok && t < k ? __ldg(Q + (row + j) * ld + t) : make_double2(0.0, 0.0);
      }
    }
#pragma unroll
    for (int j = 0; j < RU; ++j)
#pragma unroll
      for (int u = 0; u < U; ++u) acc[u] = cmadc(q[j][u], vr[j], acc[u]);
  }
#pragma unroll
  for (int u = 0; u < U; ++u) sh[warp][lane + 32 * u] = acc[u];
  __syncthreads();
  for (int t = threadIdx.x; t < k; t += blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int w = 0; w < kBS / 32; ++w) s.x += sh[w][t].x, s.y += sh[w][t].y;
    atomicAdd(h + 2 * t, s.x);
    atomicAdd(h + 2 * t + 1, s.y);
  }
}

// v[row] -= sum_t Q[row][t] h[t]: a thread per row, h in shared memory
// (a warp's 32 rows share the L1 lines of Q as t advances).
__global__ void update_kernel(long long n, const double2 *__restrict__ Q, int ld, int k,
                              const double2 *__restrict__ h, double2 *v) {
  __shared__ double2 sh[128];
  for (int t = threadIdx.x; t < k; t += blockDim.x) sh[t] = h[t];
  __syncthreads();
  for (long long row = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; row < n;
       row += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double2 *q = Q + row * ld;
    double2 s0 = make_double2(0.0, 0.0), s1 = make_double2(0.0, 0.0);
    int t = 0;
    for (; t + 1 < k; t += 2) {
      s0 = cmad(__ldg(q + t), sh[t], s0);
      s1 = cmad(__ldg(q + t + 1), sh[t + 1], s1);
    }
    if (t < k) s0 = cmad(__ldg(q + t), sh[t], s0);
    const double2 a = v[row];
    v[row] = make_double2(a.x - s0.x - s1.x, a.y - s0.y - s1.y);
  }
}

__global__ void norm2_kernel(long long n, const double2 *__restrict__ v, double *nrm) {
  __shared__ double sh[kBS / 32];
  double s = 0.0;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double2 a = v[i];
    s += a.x * a.x + a.y * a.y;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kBS / 32; ++w) t += sh[w];
    atomicAdd(nrm, t);
  }
}

__global__ void set_col_kernel(long long n, const double2 *__restrict__ v, double scale, double2 *Q, int ld, int j) {
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double2 a = v[i];
    Q[i * ld + j] = make_double2(a.x * scale, a.y * scale);
  }
}

// W[row][t] = sum over the row's entries of A(row, col) Q[col - row0][t]
// for A = K (kind 0, real), M (kind 1, complex) or M_D (kind 2, real); a
// warp per row (contiguous rows per warp), lanes over t, four entries'
// gathers issued together.
template <int U>
__global__ void apply_kernel(long long n, long long row0, const int *__restrict__ rowptr,
                             const int *__restrict__ colidx, const double *__restrict__ a64, int kind,
                             const double2 *__restrict__ Q, int ld, int k, double2 *W) {
  constexpr int EU = 4;
  const int lane = threadIdx.x & 31;
  long long r0, r1;
  warp_rows(n, r0, r1);
  for (long long row = r0; row < r1; ++row) {
    double2 acc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) acc[u] = make_double2(0.0, 0.0);
    const int kb = __ldg(rowptr + row0 + row), ke = __ldg(rowptr + row0 + row + 1);
    for (int e0 = kb; e0 < ke; e0 += EU) {
      double2 av[EU], q[EU][U];
#pragma unroll
      for (int j = 0; j < EU; ++j) {
        const int e = e0 + j;
        long long c = e < ke ? __ldg(colidx + e) - row0 : -1;
        if (c >= n) c = -1;  // instances are decoupled: never taken
        av[j] = c < 0 ? make_double2(0.0, 0.0)
                      : (kind == 1 ? __ldg(reinterpret_cast<const double2 *>(a64) + e)
                                   : make_double2(__ldg(a64 + e), 0.0));
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int t = lane + 32 * u;
          q[j][u] = c >= 0 && t < k ? __ldg(Q + c * ld + t) : make_double2(0.0, 0.0);
        }
      }
#pragma unroll
      for (int j = 0; j < EU; ++j)
#pragma unroll
        for (int u = 0; u < U; ++u) acc[u] = cmad(av[j], q[j][u], acc[u]);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = lane + 32 * u;
      if (t < k) W[row * ld + t] = acc[u];
    }
  }
}

// G[i][j] += sum_row Q[row][i] W[row][j] (bilinear, no conjugate), i, j < k
// <= 64: 16-row tiles of Q and W staged in shared memory, each thread owns
// k*k/256 (rounded up) of the (i, j) pairs.
constexpr int kTile = 16;
constexpr int kMaxK = 64;
__global__ void gram_kernel(long long n, const double2 *__restrict__ Q, const double2 *__restrict__ W, int ld,
                            int k, double *G) {
  constexpr int U = kMaxK * kMaxK / kBS;
  __shared__ double2 sq[kTile][kMaxK], sw[kTile][kMaxK];
  double2 acc[U];
#pragma unroll
  for (int u = 0; u < U; ++u) acc[u] = make_double2(0.0, 0.0);
  const long long tiles = (n + kTile - 1) / kTile;
  for (long long tl = blockIdx.x; tl < tiles; tl += gridDim.x) {
    __syncthreads();
    for (int i = threadIdx.x; i < kTile * k; i += blockDim.x) {
      const int r = i / k, c = i % k;
      const long long row = tl * kTile + r;
      sq[r][c] = row < n ? __ldg(Q + row * ld + c) : make_double2(0.0, 0.0);
      sw[r][c] = row < n ? __ldg(W + row * ld + c) : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int p = threadIdx.x + kBS * u;
      if (p >= k * k) break;
      const int i = p / k, j = p % k;
      double2 a = acc[u];
#pragma unroll 4
      for (int r = 0; r < kTile; ++r) a = cmad(sq[r][i], sw[r][j], a);
      acc[u] = a;
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int p = threadIdx.x + kBS * u;
    if (p >= k * k) break;
    atomicAdd(G + 2 * p, acc[u].x);
    atomicAdd(G + 2 * p + 1, acc[u].y);
  }
}

// x[row0 + row][c] = sum_t Q[row][t] Y[t][c] for c < r (complex dd out),
// Y (k x r) in dynamic shared memory; thread per (row, column).
__global__ void combine_kernel(long long n, const double2 *__restrict__ Q, int ld, int k,
                               const double2 *__restrict__ Y, int r, float4 *x, long long row0) {
  extern __shared__ double2 sy[];
  for (int i = threadIdx.x; i < k * r; i += blockDim.x) sy[i] = Y[i];
  __syncthreads();
  const long long total = n * r;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long row = i / r;
    const int c = static_cast<int>(i - row * r);
    const double2 *q = Q + row * ld;
    double2 s = make_double2(0.0, 0.0);
    for (int t = 0; t < k; ++t) s = cmad(__ldg(q + t), sy[t * r + c], s);
    x[(row0 + row) * r + c] = csplit(s.x, s.y);
  }
}

// out[i][t] = Q[idx[i]][t], t < k.
__global__ void gather_rows_kernel(int m, const int *__restrict__ idx, const double2 *__restrict__ Q, int ld, int k,
                                   double2 *out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m * k; i += gridDim.x * blockDim.x) {
    const int r = i / k, t = i % k;
    out[i] = Q[static_cast<long long>(__ldg(idx + r)) * ld + t];
  }
}

}  // namespace

extern "C" int efgk_batch_scatter_cols(int64_t rows, int32_t r_in, int32_t r_out, const int32_t *map,
                                       const void *in, void *out, efgk_stream_t stream) {
  if (rows <= 0 || r_in <= 0) return 0;
  if (in == out) return static_cast<int>(cudaErrorInvalidValue);
  scatter_cols_kernel<<<blocks(), kBS, 0, stream>>>(rows, r_in, r_out, map, static_cast<const float4 *>(in),
                                                    static_cast<float4 *>(out));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_rb_load_col(int64_t n, const void *x, int32_t r, int64_t row0, int32_t col, double *v,
                                double *nrm, efgk_stream_t stream) {
  if (n <= 0) return 0;
  load_col_kernel<<<blocks(), kBS, 0, stream>>>(n, static_cast<const float4 *>(x), r, row0, col,
                                                reinterpret_cast<double2 *>(v), nrm);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_rb_orth_step(int64_t n, const double *Q, int32_t ld, int32_t k, double *v, double *h,
                                 efgk_stream_t stream) {
  if (n <= 0 || k <= 0) return 0;
  if (k > 128) return static_cast<int>(cudaErrorInvalidValue);
  cudaMemsetAsync(h, 0, static_cast<size_t>(k) * 16, stream);
  const auto *q = reinterpret_cast<const double2 *>(Q);
  auto *vv = reinterpret_cast<double2 *>(v);
  const auto *hh = reinterpret_cast<const double2 *>(h);
  if (k <= 32)
    proj_kernel<1><<<blocks(), kBS, 0, stream>>>(n, q, ld, k, vv, h);
  else if (k <= 64)
    proj_kernel<2><<<blocks(), kBS, 0, stream>>>(n, q, ld, k, vv, h);
  else
    proj_kernel<4><<<blocks(), kBS, 0, stream>>>(n, q, ld, k, vv, h);
  update_kernel<<<blocks(), kBS, 0, stream>>>(n, q, ld, k, hh, vv);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_rb_norm2(int64_t n, const double *v, double *nrm, efgk_stream_t stream) {
  if (n <= 0) return 0;
  norm2_kernel<<<blocks(), kBS, 0, stream>>>(n, reinterpret_cast<const double2 *>(v), nrm);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_rb_set_col(int64_t n, const double *v, double scale, double *Q, int32_t ld, int32_t j,
                               efgk_stream_t stream) {
  if (n <= 0) return 0;
  set_col_kernel<<<blocks(), kBS, 0, stream>>>(n, reinterpret_cast<const double2 *>(v), scale,
                                               reinterpret_cast<double2 *>(Q), ld, j);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_rb_apply(int64_t n, int64_t row0, const int32_t *rowptr, const int32_t *colidx,
                             const double *a64, int32_t kind, const double *Q, int32_t ld, int32_t k, double *W,
                             efgk_stream_t stream) {
  if (n <= 0 || k <= 0) return 0;
  if (k > 128 || kind < 0 || kind > 2) return static_cast<int>(cudaErrorInvalidValue);
  const auto *q = reinterpret_cast<const double2 *>(Q);
  auto *w = reinterpret_cast<double2 *>(W);
  if (k <= 32)
    apply_kernel<1><<<blocks(), kBS, 0, stream>>>(n, row0, rowptr, colidx, a64, kind, q, ld, k, w);
  else if (k <= 64)
    apply_kernel<2><<<blocks(), kBS, 0, stream>>>(n, row0, rowptr, colidx, a64, kind, q, ld, k, w);
  else
    apply_kernel<4><<<blocks(), kBS, 0, stream>>>(n, row0, rowptr, colidx, a64, kind, q, ld, k, w);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_rb_gram(int64_t n, const double *Q, const double *W, int32_t ld, int32_t k, double *G,
                            efgk_stream_t stream) {
  if (n <= 0 || k <= 0) return 0;
  if (k > kMaxK) return static_cast<int>(cudaErrorInvalidValue);
  cudaMemsetAsync(G, 0, static_cast<size_t>(k) * k * 16, stream);
  gram_kernel<<<blocks(), kBS, 0, stream>>>(n, reinterpret_cast<const double2 *>(Q),
                                            reinterpret_cast<const double2 *>(W), ld, k, G);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_rb_combine(int64_t n, const double *Q, int32_t ld, int32_t k, const double *Y, int32_t r,
                               void *x, int64_t row0, efgk_stream_t stream) {
  if (n <= 0 || r <= 0) return 0;
  const size_t smem = static_cast<size_t>(k) * r * 16;
  if (k <= 0 || smem > 200 * 1024) return static_cast<int>(cudaErrorInvalidValue);
  cudaFuncSetAttribute(combine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  combine_kernel<<<blocks(), kBS, smem, stream>>>(n, reinterpret_cast<const double2 *>(Q), ld, k,
                                                  reinterpret_cast<const double2 *>(Y), r, static_cast<float4 *>(x),
                                                  row0);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_rb_gather_rows(int32_t m, const int32_t *idx, const double *Q, int32_t ld, int32_t k,
                                   double *out, efgk_stream_t stream) {
  if (m <= 0 || k <= 0) return 0;
  gather_rows_kernel<<<(m * k + kBS - 1) / kBS, kBS, 0, stream>>>(m, idx, reinterpret_cast<const double2 *>(Q), ld,
                                                                  k, reinterpret_cast<double2 *>(out));
  return static_cast<int>(cudaGetLastError());
}
