// Mesh ingest on the device: global edge numbering without a hash table.
//
// The numbering is the reference's (src/mesh_gmsh.cpp:104-147,
// include/edgefem/mesh.hpp:56-60): edges numbered in order of first
// appearance while scanning the tetrahedra's local pairs (0,1),(0,2),(0,3),
// (1,2),(1,3),(2,3) and then the triangles' (0,1),(1,2),(2,0); a local edge
// has orientation +1 iff the id of its first node is the smaller.
//
// An "occurrence" is one local edge of one element, numbered in scan order:
// o = 6 t + e for tetrahedron t, 6 T + 3 s + e for triangle s.  An edge is
// identified by its node pair (i < j, dense node indices), so:
//   1. occurrences are bucketed by their smaller node i (count, exclusive
//      scan, scatter with per-node cursors);
//   2. each bucket (a few dozen occurrences on a tetrahedral mesh) is sorted
//      by (j, o) by one thread; the head of every run of equal j is the
//      edge's first occurrence, and every occurrence records that head;
//   3. an exclusive scan of the head flags over o gives each edge its rank
//      among first occurrences, which is its id in first-appearance order;
//   4. occurrences take the id of their head, orientations come from the
//      node ids, and each head writes its edge's node pair.
// The scatter order inside a bucket depends on atomics, the sort makes the
// result independent of it.  Every kernel is a grid-stride loop; there are
// no waits between blocks.
#include <cuda_runtime.h>

#include <cstdint>

#include "edgefem_gb300_kernels.h"

namespace {

constexpr int kBS = 256;
constexpr int kScanPT = 8;                    // elements per thread in a scan
constexpr int kScanChunk = kBS * kScanPT;     // elements per scan block

// Local pair tables as nibbles: pair e of a tetrahedron is
// ((kTet0 >> 4e) & 15, (kTet1 >> 4e) & 15), likewise for a triangle.
constexpr unsigned kTet0 = 0x211000u, kTet1 = 0x332321u;
constexpr unsigned kTri0 = 0x210u, kTri1 = 0x021u;

__device__ __forceinline__ void occ_nodes(long long o, long long T, const int *__restrict__ tet,
                                          const int *__restrict__ tri, int &a, int &b) {
  if (o < 6 * T) {
    const long long t = o / 6;
    const int e = static_cast<int>(o - 6 * t);
    a = __ldg(tet + 4 * t + ((kTet0 >> (4 * e)) & 15u));
    b = __ldg(tet + 4 * t + ((kTet1 >> (4 * e)) & 15u));
  } else {
    const long long q = o - 6 * T;
    const long long s = q / 3;
    const int e = static_cast<int>(q - 3 * s);
    a = __ldg(tri + 3 * s + ((kTri0 >> (4 * e)) & 15u));
    b = __ldg(tri + 3 * s + ((kTri1 >> (4 * e)) & 15u));
  }
}

long long grid_for(long long items) {
  const long long need = (items + kBS - 1) / kBS;
  const long long cap = 8LL * 152;
  return need < 1 ? 1 : (need < cap ? need : cap);
}

// --------------------------------------------------------------- scan
__device__ __forceinline__ int block_exclusive_scan(int v, int &total) {
  __shared__ int warp_sums[kBS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < kBS / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    if (lane < kBS / 32) warp_sums[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  const int before = warp == 0 ? 0 : warp_sums[warp - 1];
  total = warp_sums[kBS / 32 - 1];
  __syncthreads();  // warp_sums is reused by the next call
  return before + x - v;
}

// bsum[blk] = sum of chunk blk of data[0..n).
__global__ void __launch_bounds__(kBS) scan_sums_kernel(const int *__restrict__ data, long long n, int *bsum) {
  const long long base = static_cast<long long>(blockIdx.x) * kScanChunk + threadIdx.x * kScanPT;
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanPT; ++k)
    if (base + k < n) s += data[base + k];
  int total = 0;
  block_exclusive_scan(s, total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// Exclusive scan of bsum[0..nb) in place by one block; the grand total to
// *total_out.
__global__ void __launch_bounds__(kBS) scan_bsum_kernel(int *bsum, int nb, int *total_out) {
  int carry = 0;
  for (int base = 0; base < nb; base += kBS) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? bsum[i] : 0;
    int chunk = 0;
    const int ex = block_exclusive_scan(v, chunk);
    if (i < nb) bsum[i] = carry + ex;
    carry += chunk;
  }
  if (threadIdx.x == 0) *total_out = carry;
}

// data[i] = bsum[chunk] + sum of data[chunk start .. i) (in place).
__global__ void __launch_bounds__(kBS) scan_apply_kernel(int *data, long long n, const int *__restrict__ bsum) {
  const long long base = static_cast<long long>(blockIdx.x) * kScanChunk + threadIdx.x * kScanPT;
  int v[kScanPT];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanPT; ++k) {
    v[k] = base + k < n ? data[base + k] : 0;
    s += v[k];
  }
  int total = 0;
  int run = bsum[blockIdx.x] + block_exclusive_scan(s, total);
#pragma unroll
  for (int k = 0; k < kScanPT; ++k) {
    if (base + k < n) data[base + k] = run;
    run += v[k];
  }
}

// Exclusive scan of data[0..n) in place, total to data[n].  bsum: room for
// ceil(n / kScanChunk) ints.
int exclusive_scan(int *data, long long n, int *bsum, cudaStream_t s) {
  const long long nb = (n + kScanChunk - 1) / kScanChunk;
  if (nb > 0) scan_sums_kernel<<<static_cast<unsigned>(nb), kBS, 0, s>>>(data, n, bsum);
  scan_bsum_kernel<<<1, kBS, 0, s>>>(bsum, static_cast<int>(nb), data + n);
  if (nb > 0) scan_apply_kernel<<<static_cast<unsigned>(nb), kBS, 0, s>>>(data, n, bsum);
  return static_cast<int>(cudaGetLastError());
}

// ------------------------------------------------------------ numbering
struct Scratch {
  unsigned long long *bucket;  // [m] (j << 32) | o, bucketed by i
  int *cnt;                    // [nn + 1] bucket sizes -> offsets, total
  int *cur;                    // [nn] scatter cursors
  int *first;                  // [m] first occurrence of the occurrence's edge (-1: skipped)
  int *flag;                   // [m + 1] head flags -> ranks, edge count
  int *bsum;                   // scan block sums
  int *err;                    // [1] out-of-range node index seen
};

long long align256(long long b) { return (b + 255) / 256 * 256; }

Scratch carve(void *p, long long m, int nn) {
  char *c = static_cast<char *>(p);
  Scratch s{};
  s.bucket = reinterpret_cast<unsigned long long *>(c);
  c += align256(8 * m);
  s.cnt = reinterpret_cast<int *>(c);
  c += align256(4LL * (nn + 1));
  s.cur = reinterpret_cast<int *>(c);
  c += align256(4LL * nn);
  s.first = reinterpret_cast<int *>(c);
  c += align256(4 * m);
  s.flag = reinterpret_cast<int *>(c);
  c += align256(4 * (m + 1));
  s.err = reinterpret_cast<int *>(c);
  c += 256;
  s.bsum = reinterpret_cast<int *>(c);
  return s;
}

long long bsum_len(long long m, int nn) {
  const long long n = m > nn ? m : nn;
  return (n + kScanChunk - 1) / kScanChunk + 1;
}

__global__ void __launch_bounds__(kBS) count_kernel(long long m, long long T, const int *__restrict__ tet,
                                                    const int *__restrict__ tri, int nn, Scratch s) {
  for (long long o = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; o < m;
       o += static_cast<long long>(gridDim.x) * blockDim.x) {
    int a, b;
    occ_nodes(o, T, tet, tri, a, b);
    if (a < 0 || a >= nn || b < 0 || b >= nn) {
      *s.err = 1;
      s.first[o] = -1;
      s.flag[o] = 0;
      continue;
    }
    atomicAdd(s.cnt + (a < b ? a : b), 1);
  }
}

__global__ void __launch_bounds__(kBS) scatter_kernel(long long m, long long T, const int *__restrict__ tet,
                                                      const int *__restrict__ tri, int nn, Scratch s) {
  for (long long o = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; o < m;
       o += static_cast<long long>(gridDim.x) * blockDim.x) {
    int a, b;
    occ_nodes(o, T, tet, tri, a, b);
    if (a < 0 || a >= nn || b < 0 || b >= nn) continue;
    const int i = a < b ? a : b, j = a < b ? b : a;
    const int pos = s.cnt[i] + atomicAdd(s.cur + i, 1);
    s.bucket[pos] = (static_cast<unsigned long long>(j) << 32) | static_cast<unsigned>(o);
  }
}

// One thread per node: insertion sort of its bucket, then the run heads.
__global__ void __launch_bounds__(kBS) bucket_kernel(int nn, Scratch s) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
    const int b0 = s.cnt[i], b1 = s.cnt[i + 1];
    unsigned long long *v = s.bucket;
    for (int p = b0 + 1; p < b1; ++p) {
      const unsigned long long key = v[p];
      int q = p - 1;
      while (q >= b0 && v[q] > key) {
        v[q + 1] = v[q];
        --q;
      }
      v[q + 1] = key;
    }
    int head = -1;
    unsigned prev_j = 0xffffffffu;
    for (int p = b0; p < b1; ++p) {
      const unsigned j = static_cast<unsigned>(v[p] >> 32);
      const int o = static_cast<int>(v[p] & 0xffffffffu);
      const bool first = j != prev_j;
      if (first) head = o, prev_j = j;
      s.flag[o] = first ? 1 : 0;
      s.first[o] = head;
    }
  }
}

__global__ void __launch_bounds__(kBS) finish_kernel(long long m, long long T, const int *__restrict__ tet,
                                                     const int *__restrict__ tri, const long long *__restrict__ ids,
                                                     Scratch s, int *occ_edge, signed char *occ_orient,
                                                     int *edge_nodes, int *n_edges) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *n_edges = *s.err ? -1 : s.flag[m];
  for (long long o = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; o < m;
       o += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int h = s.first[o];
    if (h < 0) {
      occ_edge[o] = -1;
      occ_orient[o] = 0;
      continue;
    }
    int a, b;
    occ_nodes(o, T, tet, tri, a, b);
    const int id = s.flag[h];
    const bool fwd = __ldg(ids + a) < __ldg(ids + b);
    occ_edge[o] = id;
    occ_orient[o] = fwd ? 1 : -1;
    if (h == o) {
      edge_nodes[2LL * id] = fwd ? a : b;
      edge_nodes[2LL * id + 1] = fwd ? b : a;
    }
  }
}

// ------------------------------------------------------------ mesh quality
// validate_mesh: per tetrahedron the signed volume u.(v x w)/6 and the
// ratio of its longest to its shortest edge, with the host's order of
// operations and no fused multiply-adds (explicitly rounded intrinsics), so
// volumes and ratios are bit-identical to the host's.  Block partials of
// (min volume, max ratio) are reduced by one block; min and max are exact,
// so the reduction order does not matter.
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

__global__ void __launch_bounds__(kBS) quality_kernel(long long T, const double *__restrict__ xyz,
                                                      const int *__restrict__ tn, signed char *flag,
                                                      double2 *part, int *counts) {
  __shared__ double s_min[kBS], s_max[kBS];
  double vmin = 1.7976931348623157e308, amax = 0.0;
  int nd = 0, ni = 0;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < T;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    double p[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const long long n = __ldg(tn + 4 * t + k);
#pragma unroll
      for (int d = 0; d < 3; ++d) p[k][d] = __ldg(xyz + 3 * n + d);
    }
    double u[3], v[3], w[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = sub(p[1][d], p[0][d]), v[d] = sub(p[2][d], p[0][d]), w[d] = sub(p[3][d], p[0][d]);
    const double c0 = sub(mul(v[1], w[2]), mul(v[2], w[1]));
    const double c1 = sub(mul(v[0], w[2]), mul(v[2], w[0]));
    const double c2 = sub(mul(v[0], w[1]), mul(v[1], w[0]));
    const double vol = __ddiv_rn(add(sub(mul(u[0], c0), mul(u[1], c1)), mul(u[2], c2)), 6.0);
    double emin = 1.7976931348623157e308, emax = 0.0;
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      const int a = (kTet0 >> (4 * e)) & 15u, b = (kTet1 >> (4 * e)) & 15u;
      const double dx = sub(p[a][0], p[b][0]), dy = sub(p[a][1], p[b][1]), dz = sub(p[a][2], p[b][2]);
      const double len = __dsqrt_rn(add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz)));
      emin = len < emin ? len : emin;
      emax = emax < len ? len : emax;
    }
    const double ar = emin < 2.220446049250313e-16 ? __longlong_as_double(0x7ff0000000000000LL) : __ddiv_rn(emax, emin);
    vmin = vol < vmin ? vol : vmin;
    amax = amax < ar ? ar : amax;
    const signed char f = fabs(vol) < 1e-15 ? 1 : (vol < 0 ? 2 : 0);
    if (flag) flag[t] = f;
    nd += f == 1;
    ni += f == 2;
  }
  s_min[threadIdx.x] = vmin;
  s_max[threadIdx.x] = amax;
  __syncthreads();
  for (int off = kBS / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) {
      const double a = s_min[threadIdx.x + off], b = s_max[threadIdx.x + off];
      if (a < s_min[threadIdx.x]) s_min[threadIdx.x] = a;
      if (s_max[threadIdx.x] < b) s_max[threadIdx.x] = b;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(s_min[0], s_max[0]);
  if (nd) atomicAdd(counts, nd);
  if (ni) atomicAdd(counts + 1, ni);
}

__global__ void __launch_bounds__(kBS) quality_final_kernel(int nb, const double2 *__restrict__ part, double *out) {
  __shared__ double s_min[kBS], s_max[kBS];
  double vmin = 1.7976931348623157e308, amax = 0.0;
  for (int i = threadIdx.x; i < nb; i += kBS) {
    const double2 q = part[i];
    vmin = q.x < vmin ? q.x : vmin;
    amax = amax < q.y ? q.y : amax;
  }
  s_min[threadIdx.x] = vmin;
  s_max[threadIdx.x] = amax;
  __syncthreads();
  for (int off = kBS / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) {
      const double a = s_min[threadIdx.x + off], b = s_max[threadIdx.x + off];
      if (a < s_min[threadIdx.x]) s_min[threadIdx.x] = a;
      if (s_max[threadIdx.x] < b) s_max[threadIdx.x] = b;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = s_min[0], out[1] = s_max[0];
}

}  // namespace

extern "C" int64_t efgk_build_edges_scratch_bytes(int64_t T, int64_t S, int32_t nn) {
  if (T < 0 || S < 0 || nn < 0) return -1;
  const long long m = 6 * T + 3 * S;
  return align256(8 * m) + align256(4LL * (nn + 1)) + align256(4LL * nn) + align256(4 * m) +
         align256(4 * (m + 1)) + 256 + align256(4 * bsum_len(m, nn));
}

extern "C" int efgk_build_edges(int64_t T, const int32_t *tet_nodes, int64_t S, const int32_t *tri_nodes,
                                int32_t nn, const int64_t *node_ids, int32_t *occ_edge, int8_t *occ_orient,
                                int32_t *edge_nodes, int32_t *n_edges, void *scratch, efgk_stream_t stream) {
  if (T < 0 || S < 0 || nn < 0 || 6 * T + 3 * S >= 0x7fffffffLL) return static_cast<int>(cudaErrorInvalidValue);
  const long long m = 6 * T + 3 * S;
  if (!scratch || !n_edges || (m > 0 && (!occ_edge || !occ_orient || !edge_nodes)) ||
      (T > 0 && !tet_nodes) || (S > 0 && !tri_nodes) || (m > 0 && !node_ids))
    return static_cast<int>(cudaErrorInvalidValue);
  const Scratch s = carve(scratch, m, nn);
  int err = static_cast<int>(cudaMemsetAsync(s.cnt, 0, 4LL * (nn + 1), stream));
  if (!err) err = static_cast<int>(cudaMemsetAsync(s.cur, 0, 4LL * nn, stream));
  if (!err) err = static_cast<int>(cudaMemsetAsync(s.err, 0, 4, stream));
  if (err) return err;
  const unsigned g = static_cast<unsigned>(grid_for(m));
  if (m > 0) count_kernel<<<g, kBS, 0, stream>>>(m, T, tet_nodes, tri_nodes, nn, s);
  err = exclusive_scan(s.cnt, nn, s.bsum, stream);
  if (err) return err;
  if (m > 0) scatter_kernel<<<g, kBS, 0, stream>>>(m, T, tet_nodes, tri_nodes, nn, s);
  if (nn > 0) bucket_kernel<<<static_cast<unsigned>(grid_for(nn)), kBS, 0, stream>>>(nn, s);
  err = exclusive_scan(s.flag, m, s.bsum, stream);
  if (err) return err;
  finish_kernel<<<g, kBS, 0, stream>>>(m, T, tet_nodes, tri_nodes, reinterpret_cast<const long long *>(node_ids), s,
                                       occ_edge, reinterpret_cast<signed char *>(occ_orient), edge_nodes, n_edges);
  return static_cast<int>(cudaGetLastError());
}

extern "C" int64_t efgk_validate_mesh_scratch_bytes(int64_t T) {
  if (T < 0) return -1;
  return 256 + align256(16 * grid_for(T));
}

extern "C" int efgk_validate_mesh(int64_t T, const double *xyz, const int32_t *tet_nodes, int8_t *tet_flag,
                                  double *out, int32_t *counts, void *scratch, efgk_stream_t stream) {
  if (T < 0 || !out || !counts || !scratch || (T > 0 && (!xyz || !tet_nodes)))
    return static_cast<int>(cudaErrorInvalidValue);
  const unsigned g = static_cast<unsigned>(grid_for(T));
  double2 *part = reinterpret_cast<double2 *>(static_cast<char *>(scratch) + 256);
  int err = static_cast<int>(cudaMemsetAsync(counts, 0, 2 * sizeof(int32_t), stream));
  if (err) return err;
  quality_kernel<<<g, kBS, 0, stream>>>(T, xyz, tet_nodes, reinterpret_cast<signed char *>(tet_flag), part, counts);
  quality_final_kernel<<<1, kBS, 0, stream>>>(static_cast<int>(g), part, out);
  return static_cast<int>(cudaGetLastError());
}
