// Complex64 SpMV on a sliced-ELLPACK copy of the CSR matrix.
//
// Layout (SELL-32 with rows sorted by length inside windows of 1024 rows):
// sorted position p = 32 s + lane holds row perm[p]; slice s stores its 32
// rows' entries column-major, entry j of the row at sorted position p at
// slice_ptr[s] + 32 j + lane, padded to the longest row of the slice with a
// zero value (column 0).  A warp computes one slice: lane = row, and every
// load of column indices and values is one contiguous 128 / 256-byte line
// for the warp, so the matrix streams at full width with no shuffles and no
// per-row bounds.  Sorting inside a window keeps a slice's rows (and the x
// entries they gather) close in the mesh and leaves 0.6% padding on the
// WR-90 edge matrices (19% unsorted).  The copy is built once on the device
// from the CSR arrays; y is written back in row order through perm.
#include <cuda_runtime.h>

#include "edgefem_gb300_kernels.h"

namespace {

constexpr int kSlice = 32;
constexpr int kWindow = 1024;
constexpr int kBS = 256;

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

// perm inside each window: rows by decreasing length, ties by row index
// (deterministic).  One block per window.
__global__ void rank_kernel(int n, const int *__restrict__ rowptr, int *perm) {
  __shared__ int len[kWindow];
  const int w0 = blockIdx.x * kWindow;
  const int m = n - w0 < kWindow ? n - w0 : kWindow;
  for (int i = threadIdx.x; i < m; i += blockDim.x) len[i] = rowptr[w0 + i + 1] - rowptr[w0 + i];
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const int li = len[i];
    int rank = 0;
    for (int j = 0; j < m; ++j) rank += (len[j] > li) || (len[j] == li && j < i);
    perm[w0 + rank] = w0 + i;
  }
}

// slice_ptr[s + 1] = 32 * (longest row of slice s); slice_ptr[0] = 0 is set
// by the scan.
__global__ void slice_len_kernel(int n, int n_slices, const int *__restrict__ rowptr, const int *__restrict__ perm,
                                 long long *slice_ptr) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_slices; s += gridDim.x * blockDim.x) {
    int mx = 0;
    for (int l = 0; l < kSlice; ++l) {
      const int p = s * kSlice + l;
      if (p >= n) break;
      const int r = perm[p];
      const int L = rowptr[r + 1] - rowptr[r];
      mx = L > mx ? L : mx;
    }
    slice_ptr[s + 1] = static_cast<long long>(mx) * kSlice;
  }
}

// In-place inclusive scan of a[1..m] (a[0] = 0) by one block.
__global__ void scan_kernel(long long *a, int m) {
  __shared__ long long part[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int per = (m + T - 1) / T;
  const int i0 = 1 + t * per, i1 = (1 + (t + 1) * per) < (m + 1) ? 1 + (t + 1) * per : m + 1;
  long long s = 0;
  for (int i = i0; i < i1; ++i) s += a[i];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    long long acc = 0;
    for (int k = 0; k < T; ++k) {
      const long long v = part[k];
      part[k] = acc;
      acc += v;
    }
    a[0] = 0;
  }
  __syncthreads();
  long long acc = part[t];
  for (int i = i0; i < i1; ++i) {
    acc += a[i];
    a[i] = acc;
  }
}

__global__ void fill_kernel(int n, int n_slices, const int *__restrict__ rowptr, const int *__restrict__ colidx,
                            const float2 *__restrict__ vals, const int *__restrict__ perm,
                            const long long *__restrict__ slice_ptr, int *scol, float2 *sval) {
  const long long total = static_cast<long long>(n_slices) * kSlice;
  for (long long p = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; p < total;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int s = static_cast<int>(p / kSlice), lane = static_cast<int>(p % kSlice);
    const long long base = slice_ptr[s];
    const int L = static_cast<int>((slice_ptr[s + 1] - base) / kSlice);
    int b = 0, len = 0;
    if (p < n) {
      const int r = perm[p];
      b = rowptr[r];
      len = rowptr[r + 1] - b;
    }
    for (int j = 0; j < L; ++j) {
      const long long o = base + static_cast<long long>(j) * kSlice + lane;
      scol[o] = j < len ? colidx[b + j] : 0;
      sval[o] = j < len ? vals[b + j] : make_float2(0.f, 0.f);
    }
  }
}

// y[perm[p]] = sum_j val * x[col] for the row at sorted position p: a warp
// per slice, four entries' loads in flight per lane.
__global__ void __launch_bounds__(kBS) spmv_sell_kernel(int n, int n_slices, const int *__restrict__ perm,
                                                        const long long *__restrict__ slice_ptr,
                                                        const int *__restrict__ scol,
                                                        const float2 *__restrict__ sval,
                                                        const float2 *__restrict__ x, float2 *__restrict__ y) {
  constexpr int U = 4;
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (kBS / 32);
  for (int s = blockIdx.x * (kBS / 32) + (threadIdx.x >> 5); s < n_slices; s += nw) {
    const long long base = __ldg(slice_ptr + s);
    const int L = static_cast<int>((__ldg(slice_ptr + s + 1) - base) / kSlice);
    const int *cp = scol + base + lane;
    const float2 *vp = sval + base + lane;
    float2 acc = make_float2(0.f, 0.f);
    int j = 0;
    for (; j + U <= L; j += U) {
      int c[U];
      float2 v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        c[u] = __ldg(cp + (j + u) * kSlice);
        v[u] = __ldg(vp + (j + u) * kSlice);
      }
      float2 xv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) xv[u] = __ldg(x + c[u]);
#pragma unroll
      for (int u = 0; u < U; ++u) acc = cfma(v[u], xv[u], acc);
    }
    for (; j < L; ++j) acc = cfma(__ldg(vp + j * kSlice), __ldg(x + __ldg(cp + j * kSlice)), acc);
    const int p = s * kSlice + lane;
    if (p < n) y[__ldg(perm + p)] = acc;
  }
}

int sm_blocks(const void *kernel) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kBS, 0);
  return (sms > 0 ? sms : 132) * (per > 0 ? per : 4);
}

}  // namespace

extern "C" int efgk_sell32_plan(int32_t n, const int32_t *rowptr, int32_t *perm, int64_t *slice_ptr,
                                int64_t *entries, efgk_stream_t stream) {
  if (n <= 0 || !entries) return static_cast<int>(cudaErrorInvalidValue);
  const int n_slices = (n + kSlice - 1) / kSlice;
  rank_kernel<<<(n + kWindow - 1) / kWindow, kBS, 0, stream>>>(n, rowptr, perm);
  slice_len_kernel<<<(n_slices + kBS - 1) / kBS, kBS, 0, stream>>>(n, n_slices, rowptr, perm,
                                                                     reinterpret_cast<long long *>(slice_ptr));
  scan_kernel<<<1, 1024, 0, stream>>>(reinterpret_cast<long long *>(slice_ptr), n_slices);
  cudaError_t e = cudaMemcpyAsync(entries, slice_ptr + n_slices, sizeof(int64_t), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return static_cast<int>(e);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_sell32_fill(int32_t n, const int32_t *rowptr, const int32_t *colidx, const float *vals,
                                const int32_t *perm, const int64_t *slice_ptr, int32_t *sell_col, float *sell_val,
                                efgk_stream_t stream) {
  if (n <= 0) return 0;
  const int n_slices = (n + kSlice - 1) / kSlice;
  fill_kernel<<<sm_blocks(reinterpret_cast<const void *>(fill_kernel)), kBS, 0, stream>>>(
      n, n_slices, rowptr, colidx, reinterpret_cast<const float2 *>(vals), perm,
      reinterpret_cast<const long long *>(slice_ptr), sell_col, reinterpret_cast<float2 *>(sell_val));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_spmv32_sell(int32_t n, const int32_t *perm, const int64_t *slice_ptr, const int32_t *sell_col,
                                const float *sell_val, const float *x, float *y, efgk_stream_t stream) {
  if (n <= 0) return 0;
  const int n_slices = (n + kSlice - 1) / kSlice;
  static const int wave = sm_blocks(reinterpret_cast<const void *>(spmv_sell_kernel));
  const int need = (n_slices + kBS / 32 - 1) / (kBS / 32);
  spmv_sell_kernel<<<need < wave ? need : wave, kBS, 0, stream>>>(
      n, n_slices, perm, reinterpret_cast<const long long *>(slice_ptr), sell_col,
      reinterpret_cast<const float2 *>(sell_val), reinterpret_cast<const float2 *>(x), reinterpret_cast<float2 *>(y));
  return static_cast<int>(cudaGetLastError());
}
