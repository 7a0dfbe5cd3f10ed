// Complex64 CSR SpMV with the matrix streamed through shared memory by bulk
// asynchronous copies (cp.async.bulk, the TMA engine's one-dimensional form)
// and FP32 accumulation: y = A x for the single-right-hand-side FP32 Krylov
// form (the complex FP32 form of the Eigen SpMV inside BiCGSTAB,
// src/solver.cpp:54-99).
//
// The product is bound by HBM: 12 bytes per stored entry (8-byte complex64
// value, 4-byte column) against 8 FP32 operations.  A thread-per-entry
// kernel keeps too few bytes in flight to reach the copy bandwidth; here
// each CTA streams tiles of kTileRows rows: one thread issues two bulk
// copies per tile (values and columns of the tile's entry range) into one
// of two shared-memory stages, the copy engine moves them while the CTA
// multiplies the previous tile, and an mbarrier with a transaction count
// tells the CTA when a stage has landed.  Two threads share a row: they
// read its entries from shared memory, gather x (L2-resident after first
// touch: a row's columns lie within a few mesh layers of the row) and add
// their halves with one shuffle.
//
// Bulk copies need 16-byte aligned addresses and sizes: a tile's copied
// range is its entry range rounded out to multiples of 4 entries and
// clamped to the last multiple of 4 below nnz; entries outside the copied
// range (at most three at the very end, or a tile longer than a stage) are
// read from global memory directly.  Every wait on an mbarrier is bounded:
// when it gives up (which only a fault elsewhere can cause) the kernel sets
// *status and stops, after a bounded wait for its own copies still in
// flight.
#include <cuda_runtime.h>

#include <cstdint>

#include "edgefem_gb300_kernels.h"

namespace {

constexpr int kTileRows = 128;   // rows per tile
constexpr int kThreads = 256;    // two threads per row
constexpr int kStageCap = 3072;  // entries per stage (24 per row on average)
constexpr long long kSpinLimit = 1LL << 26;

struct __align__(16) Stage {
  float2 vals[kStageCap];
  int cols[kStageCap];
};
constexpr int kSmemBytes = 2 * static_cast<int>(sizeof(Stage));

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Arrive once, announcing `bytes` of asynchronous copy to land on the barrier.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (long long i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

// Per-stage copy description, written by thread 0 before its arrive.
struct StageInfo {
  int base;  // first entry held (multiple of 4)
  int lim;   // one past the last entry held (base when nothing was copied)
};

__global__ void __launch_bounds__(kThreads) spmv32_bulk_kernel(int n, int nnz, const int *__restrict__ rowptr,
                                                              const int *__restrict__ colidx,
                                                              const float2 *__restrict__ vals,
                                                              const float2 *__restrict__ x, float2 *__restrict__ y,
                                                              int *status) {
  extern __shared__ __align__(128) unsigned char smem[];
  Stage *st = reinterpret_cast<Stage *>(smem);
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ StageInfo info[2];
  __shared__ int s_fail;
  const int ntiles = (n + kTileRows - 1) / kTileRows;
  const int nnz4 = nnz & ~3;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
    s_fail = 0;
  }
  __syncthreads();

  // Thread 0: start the copy of tile t into stage s (row bounds k0, k1).
  auto issue = [&](int s, int k0, int k1) {
    const int a0 = k0 & ~3;
    int a1 = (k1 + 3) & ~3;
    if (a1 > nnz4) a1 = nnz4;
    if (a1 > a0 && a1 - a0 <= kStageCap) {
      info[s].base = a0;
      info[s].lim = a1;
      const uint32_t m = static_cast<uint32_t>(a1 - a0);
      mbar_arrive_expect_tx(&bar[s], m * 12u);
      bulk_g2s(st[s].vals, vals + a0, m * 8u, &bar[s]);
      bulk_g2s(st[s].cols, colidx + a0, m * 4u, &bar[s]);
    } else {
      info[s].base = a0;
      info[s].lim = a0;  // nothing staged: every entry from global memory
      mbar_arrive(&bar[s]);
    }
  };
  const int G = gridDim.x;
  int t = blockIdx.x;
  // Thread 0 loads the row bounds of the next tile of each stage early
  // (stage 0: a0/a1, stage 1: b0/b1), so issuing a copy never waits on them.
  int a0 = 0, a1 = 0, b0 = 0, b1 = 0;
  auto bounds = [&](int tile, int &k0, int &k1) {
    if (tile < ntiles) k0 = __ldg(rowptr + tile * kTileRows), k1 = __ldg(rowptr + min(n, (tile + 1) * kTileRows));
  };
  if (tid == 0) {
    for (int j = 0; j < 2; ++j) {
      const int tj = t + j * G;
      if (tj < ntiles)
        issue(j, __ldg(rowptr + tj * kTileRows), __ldg(rowptr + min(n, (tj + 1) * kTileRows)));
    }
    bounds(t + 2 * G, a0, a1);
    bounds(t + 3 * G, b0, b1);
  }
  const int half = tid & 1;
  for (int j = 0; t < ntiles; ++j, t += G) {
    const int s = j & 1;
    if (!mbar_wait(&bar[s], static_cast<uint32_t>((j >> 1) & 1))) {
      s_fail = 1;  // benign race: every writer stores 1
    }
    __syncthreads();
    if (s_fail) break;
    const int base = info[s].base, lim = info[s].lim;
    const int row = t * kTileRows + (tid >> 1);
    float2 acc = make_float2(0.f, 0.f);
    if (row < n) {
      const int kb = __ldg(rowptr + row), ke = __ldg(rowptr + row + 1);
      int k = kb + half;
      // four entries of this thread at a time: gathers issued together
      for (; k + 6 < ke; k += 8) {
        float2 a[4];
        int c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int kk = k + 2 * u;
          const bool in = kk >= base && kk < lim;
          a[u] = in ? st[s].vals[kk - base] : __ldg(vals + kk);
          c[u] = in ? st[s].cols[kk - base] : __ldg(colidx + kk);
        }
        float2 xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) xv[u] = __ldg(x + c[u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) acc = cfma(a[u], xv[u], acc);
      }
      for (; k < ke; k += 2) {
        const bool in = k >= base && k < lim;
        const float2 a = in ? st[s].vals[k - base] : __ldg(vals + k);
        const int c = in ? st[s].cols[k - base] : __ldg(colidx + k);
        acc = cfma(a, __ldg(x + c), acc);
      }
    }
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 1);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 1);
    if (row < n && half == 0) y[row] = acc;
    __syncthreads();  // stage s fully read
    if (tid == 0) {
      const int t2 = t + 2 * G;  // the next tile of stage s
      if (t2 < ntiles) {
        if (s == 0) {
          issue(0, a0, a1);
          bounds(t2 + 2 * G, a0, a1);
        } else {
          issue(1, b0, b1);
          bounds(t2 + 2 * G, b0, b1);
        }
      }
    }
  }
  if (s_fail) {
    // A stage never completed.  Record it, and wait (bounded) for the copies
    // this CTA may still have in flight before its shared memory goes away.
    if (tid == 0) {
      atomicExch(status, 1);
      for (int j = 0; j < 2; ++j) mbar_wait(&bar[j], 0), mbar_wait(&bar[j], 1);
    }
    __syncthreads();
  }
}

int g_grid = 0;

}  // namespace

extern "C" int efgk_spmv32_bulk(int32_t n, int32_t nnz, const int32_t *rowptr, const int32_t *colidx,
                                const float *vals, const float *x, float *y, int32_t *status, efgk_stream_t stream) {
  if (n <= 0) return 0;
  if ((reinterpret_cast<uintptr_t>(colidx) | reinterpret_cast<uintptr_t>(vals)) & 15u)
    return static_cast<int>(cudaErrorMisalignedAddress);
  if (!g_grid) {
    cudaError_t e = cudaFuncSetAttribute(spmv32_bulk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return static_cast<int>(e);
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, spmv32_bulk_kernel, kThreads, kSmemBytes);
    g_grid = (sms > 0 ? sms : 132) * (per_sm > 0 ? per_sm : 1);
  }
  const int ntiles = (n + kTileRows - 1) / kTileRows;
  const int grid = ntiles < g_grid ? ntiles : g_grid;
  spmv32_bulk_kernel<<<grid, kThreads, kSmemBytes, stream>>>(n, nnz, rowptr, colidx,
                                                             reinterpret_cast<const float2 *>(vals),
                                                             reinterpret_cast<const float2 *>(x),
                                                             reinterpret_cast<float2 *>(y), status);
  return static_cast<int>(cudaGetLastError());
}

