// Element assembly and matrix-term kernels (sm_103a, FP64).
//
// One launch per colour: within a colour no two tetrahedra share an edge, so
// no two threads touch the same CSR slot and the scatter is a plain
// read-modify-write.  A warp covers a group of 32 tetrahedra, one per lane;
// each lane forms its tetrahedron's 21 unique curl-curl and mass entries
// from FP64 node coordinates (src/edge_basis.cpp:14-87) and scatters both
// (i, j) and (j, i) with the edge-orientation signs
// (src/assemble_maxwell.cpp:191-204).
#include <cuda_runtime.h>

#include "edgefem_gb300_kernels.h"

namespace {

__device__ __forceinline__ double3 sub3(double3 a, double3 b) {
  return make_double3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ double3 cross3(double3 a, double3 b) {
  return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double dot3(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double3 scale3(double3 a, double s) {
  return make_double3(a.x * s, a.y * s, a.z * s);
}
__device__ __forceinline__ double3 load3(const double *__restrict__ xyz, int i) {
  return make_double3(__ldg(xyz + 3 * i), __ldg(xyz + 3 * i + 1), __ldg(xyz + 3 * i + 2));
}

// Local edge i joins local nodes kPairA(i) and kPairB(i):
// (0,1),(0,2),(0,3),(1,2),(1,3),(2,3) as in src/edge_basis.cpp:9-12.
__device__ __forceinline__ constexpr int kPairA(int i) { return i < 3 ? 0 : (i < 5 ? 1 : 2); }
__device__ __forceinline__ constexpr int kPairB(int i) { return i == 0 ? 1 : (i == 1 || i == 3) ? 2 : 3; }

__global__ void __launch_bounds__(128) assemble_color_kernel(
    const double *__restrict__ xyz, const int4 *__restrict__ tet_nodes,
    const uint8_t *__restrict__ tet_signs, const int *__restrict__ slots,
    const int *__restrict__ color_tets, long long begin, long long end,
    const double2 *__restrict__ cK, const double2 *__restrict__ cM, double2 cK0, double2 cM0,
    double2 *__restrict__ out) {
  const long long k = begin + static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= end) return;
  const int t = __ldg(color_tets + k);
  const int4 nd = tet_nodes[t];
  const double3 v0 = load3(xyz, nd.x), v1 = load3(xyz, nd.y), v2 = load3(xyz, nd.z),
                v3 = load3(xyz, nd.w);
  // B = [v0-v3, v1-v3, v2-v3]; rows of B^{-1} are the gradients g0..g2.
  const double3 c0 = sub3(v0, v3), c1 = sub3(v1, v3), c2 = sub3(v2, v3);
  const double3 x12 = cross3(c1, c2);
  const double det = dot3(c0, x12);
  const double inv = 1.0 / det;
  double3 g[4];
  g[0] = scale3(x12, inv);
  g[1] = scale3(cross3(c2, c0), inv);
  g[2] = scale3(cross3(c0, c1), inv);
  g[3] = make_double3(-(g[0].x + g[1].x + g[2].x), -(g[0].y + g[1].y + g[2].y),
                      -(g[0].z + g[1].z + g[2].z));
  const double V = fabs(det) / 6.0;
  double gg[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = a; b < 4; ++b) {
      gg[a][b] = dot3(g[a], g[b]);
      gg[b][a] = gg[a][b];
    }
  double3 cu[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) cu[i] = scale3(cross3(g[kPairA(i)], g[kPairB(i)]), 2.0);
  const double2 ck = cK ? cK[t] : cK0;
  const double2 cm = cM ? cM[t] : cM0;
  const unsigned sg = tet_signs[t];
  const int *sl = slots + 36LL * t;
  const double v10 = V / 10.0, v20 = V / 20.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const int a = kPairA(i), b = kPairB(i);
#pragma unroll
    for (int j = i; j < 6; ++j) {
      const int c = kPairA(j), d = kPairB(j);
      const double Kij = V * dot3(cu[i], cu[j]);
      const double lac = (a == c) ? v10 : v20, lad = (a == d) ? v10 : v20;
      const double lbc = (b == c) ? v10 : v20, lbd = (b == d) ? v10 : v20;
      const double Mij = gg[b][d] * lac - gg[b][c] * lad - gg[a][d] * lbc + gg[a][c] * lbd;
      const double s = (((sg >> i) ^ (sg >> j)) & 1u) ? -1.0 : 1.0;
      const double re = s * (ck.x * Kij + cm.x * Mij);
      const double im = s * (ck.y * Kij + cm.y * Mij);
      const int s1 = __ldg(sl + 6 * i + j);
      double2 o = out[s1];
      o.x += re;
      o.y += im;
      out[s1] = o;
      if (i != j) {
        const int s2 = __ldg(sl + 6 * j + i);
        double2 p = out[s2];
        p.x += re;
        p.y += im;
        out[s2] = p;
      }
    }
  }
}

// Adjoint sensitivity contraction: out[t] = scale * lam_loc^T M_loc(t) x_loc
// with lam_loc[i] = s_i lam[edge_i], x_loc[j] = s_j x[edge_j].
__global__ void __launch_bounds__(128) adjoint_contract_kernel(
    int T, const double *__restrict__ xyz, const int4 *__restrict__ tet_nodes,
    const uint8_t *__restrict__ tet_signs, const int *__restrict__ tet_edges, const double2 *__restrict__ lam,
    const double2 *__restrict__ x, double scale, double2 *__restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int4 nd = tet_nodes[t];
  const double3 v0 = load3(xyz, nd.x), v1 = load3(xyz, nd.y), v2 = load3(xyz, nd.z),
                v3 = load3(xyz, nd.w);
  const double3 c0 = sub3(v0, v3), c1 = sub3(v1, v3), c2 = sub3(v2, v3);
  const double3 x12 = cross3(c1, c2);
  const double det = dot3(c0, x12);
  const double inv = 1.0 / det;
  double3 g[4];
  g[0] = scale3(x12, inv);
  g[1] = scale3(cross3(c2, c0), inv);
  g[2] = scale3(cross3(c0, c1), inv);
  g[3] = make_double3(-(g[0].x + g[1].x + g[2].x), -(g[0].y + g[1].y + g[2].y),
                      -(g[0].z + g[1].z + g[2].z));
  const double V = fabs(det) / 6.0;
  double gg[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = a; b < 4; ++b) {
      gg[a][b] = dot3(g[a], g[b]);
      gg[b][a] = gg[a][b];
    }
  const unsigned sg = tet_signs[t];
  double2 ll[6], xl[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const int e = tet_edges[6 * t + i];
    const double s = ((sg >> i) & 1u) ? -1.0 : 1.0;
    const double2 a = lam[e], b = x[e];
    ll[i] = make_double2(s * a.x, s * a.y);
    xl[i] = make_double2(s * b.x, s * b.y);
  }
  const double v10 = V / 10.0, v20 = V / 20.0;
  double re = 0.0, im = 0.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const int a = kPairA(i), b = kPairB(i);
    double2 mx = make_double2(0.0, 0.0);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const int c = kPairA(j), d = kPairB(j);
      const double lac = (a == c) ? v10 : v20, lad = (a == d) ? v10 : v20;
      const double lbc = (b == c) ? v10 : v20, lbd = (b == d) ? v10 : v20;
      const double Mij = gg[b][d] * lac - gg[b][c] * lad - gg[a][d] * lbc + gg[a][c] * lbd;
      mx.x += Mij * xl[j].x;
      mx.y += Mij * xl[j].y;
    }
    re += ll[i].x * mx.x - ll[i].y * mx.y;
    im += ll[i].x * mx.y + ll[i].y * mx.x;
  }
  out[t] = make_double2(scale * re, scale * im);
}

__global__ void dirichlet_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colidx,
                                 const uint8_t *__restrict__ is_pec, double2 dv, double2 *values) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const bool prow = is_pec[r] != 0;
  for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) {
    const int c = colidx[k];
    if (prow) {
      values[k] = (c == r) ? dv : make_double2(0.0, 0.0);
    } else if (is_pec[c]) {
      values[k] = make_double2(0.0, 0.0);
    }
  }
}

__global__ void add_terms_kernel(long long count, const int *__restrict__ slot, const int *__restrict__ term,
                                 const double2 *__restrict__ val, const double2 *__restrict__ coef,
                                 double2 *values) {
  const long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const double2 c = coef[term[k]];
  const double2 v = val[k];
  double *dst = reinterpret_cast<double *>(values + slot[k]);
  atomicAdd(dst, c.x * v.x - c.y * v.y);
  atomicAdd(dst + 1, c.x * v.y + c.y * v.x);
}

__global__ void blend_kernel(long long nnz, const double2 *__restrict__ K, const double2 *__restrict__ M,
                             const double2 *__restrict__ M2, double2 a, double2 b, double2 c,
                             double2 *__restrict__ out) {
  const long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const double2 kv = K[k], mv = M[k];
  double re = a.x * kv.x - a.y * kv.y + b.x * mv.x - b.y * mv.y;
  double im = a.x * kv.y + a.y * kv.x + b.x * mv.y + b.y * mv.x;
  if (M2) {
    const double2 m2 = M2[k];
    re += c.x * m2.x - c.y * m2.y;
    im += c.x * m2.y + c.y * m2.x;
  }
  out[k] = make_double2(re, im);
}

// Electric field from the edge solution at query points (one thread per
// point): E(p) = sum_e s_e x[e] (lambda_a(p) grad lambda_b - lambda_b(p)
// grad lambda_a) over the six edges (a, b) of the point's tetrahedron, the
// Whitney interpolant of src/edge_basis.cpp:162-193.  lambda_0..2 =
// B^-1 (p - v3) with B = [v0-v3, v1-v3, v2-v3] (rows of B^-1 are the
// gradients), lambda_3 = 1 - lambda_0 - lambda_1 - lambda_2; without a point
// list the point is the centroid (every lambda 1/4).
__global__ void __launch_bounds__(128) edge_field_kernel(
    long long nq, const double *__restrict__ xyz, const int4 *__restrict__ tet_nodes,
    const uint8_t *__restrict__ tet_signs, const int *__restrict__ tet_edges, const int *__restrict__ tet_of,
    const double *__restrict__ pts, const double2 *__restrict__ x, double2 *__restrict__ E) {
  const long long q = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const int t = tet_of ? __ldg(tet_of + q) : static_cast<int>(q);
  const int4 nd = tet_nodes[t];
  const double3 v0 = load3(xyz, nd.x), v1 = load3(xyz, nd.y), v2 = load3(xyz, nd.z),
                v3 = load3(xyz, nd.w);
  const double3 c0 = sub3(v0, v3), c1 = sub3(v1, v3), c2 = sub3(v2, v3);
  const double3 x12 = cross3(c1, c2);
  const double inv = 1.0 / dot3(c0, x12);
  double3 g[4];
  g[0] = scale3(x12, inv);
  g[1] = scale3(cross3(c2, c0), inv);
  g[2] = scale3(cross3(c0, c1), inv);
  g[3] = make_double3(-(g[0].x + g[1].x + g[2].x), -(g[0].y + g[1].y + g[2].y),
                      -(g[0].z + g[1].z + g[2].z));
  double lam[4] = {0.25, 0.25, 0.25, 0.25};
  if (pts) {
    const double *pq = pts + 3 * q;
    const double3 d = sub3(make_double3(__ldg(pq), __ldg(pq + 1), __ldg(pq + 2)), v3);
    lam[0] = dot3(g[0], d);
    lam[1] = dot3(g[1], d);
    lam[2] = dot3(g[2], d);
    lam[3] = 1.0 - lam[0] - lam[1] - lam[2];
  }
  const unsigned sg = tet_signs[t];
  double2 ex = make_double2(0, 0), ey = make_double2(0, 0), ez = make_double2(0, 0);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const int a = kPairA(i), b = kPairB(i);
    const double3 w = sub3(scale3(g[b], lam[a]), scale3(g[a], lam[b]));
    double2 c = x[__ldg(tet_edges + 6LL * t + i)];
    if ((sg >> i) & 1u) c = make_double2(-c.x, -c.y);
    ex.x += c.x * w.x, ex.y += c.y * w.x;
    ey.x += c.x * w.y, ey.y += c.y * w.y;
    ez.x += c.x * w.z, ez.y += c.y * w.z;
  }
  E[3 * q] = ex;
  E[3 * q + 1] = ey;
  E[3 * q + 2] = ez;
}

inline int blocks_for(long long n, int bs) { return static_cast<int>((n + bs - 1) / bs); }

}  // namespace

extern "C" int efgk_edge_field(int64_t nq, const double *xyz, const int32_t *tet_nodes, const uint8_t *tet_signs,
                               const int32_t *tet_edges, const int32_t *tet_of, const double *pts, const double *x,
                               double *E, efgk_stream_t stream) {
  if (nq <= 0) return 0;
  edge_field_kernel<<<blocks_for(nq, 128), 128, 0, stream>>>(
      nq, xyz, reinterpret_cast<const int4 *>(tet_nodes), tet_signs, tet_edges, tet_of, pts,
      reinterpret_cast<const double2 *>(x), reinterpret_cast<double2 *>(E));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_assemble_color(const double *xyz, const int32_t *tet_nodes, const uint8_t *tet_signs,
                                   const int32_t *slots, const int32_t *color_tets, int64_t begin,
                                   int64_t end, const double *cK, const double *cM,
                                   const double *cK0_host, const double *cM0_host, double *out,
                                   efgk_stream_t stream) {
  if (end <= begin) return 0;
  const double2 ck0 = cK0_host ? make_double2(cK0_host[0], cK0_host[1]) : make_double2(0, 0);
  const double2 cm0 = cM0_host ? make_double2(cM0_host[0], cM0_host[1]) : make_double2(0, 0);
  assemble_color_kernel<<<blocks_for(end - begin, 128), 128, 0, stream>>>(
      xyz, reinterpret_cast<const int4 *>(tet_nodes), tet_signs, slots, color_tets, begin, end,
      reinterpret_cast<const double2 *>(cK), reinterpret_cast<const double2 *>(cM), ck0, cm0,
      reinterpret_cast<double2 *>(out));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_adjoint_contract(int32_t T, const double *xyz, const int32_t *tet_nodes,
                                     const uint8_t *tet_signs, const int32_t *tet_edges, const double *lam,
                                     const double *x, double scale, double *out, efgk_stream_t stream) {
  if (T <= 0) return 0;
  adjoint_contract_kernel<<<blocks_for(T, 128), 128, 0, stream>>>(
      T, xyz, reinterpret_cast<const int4 *>(tet_nodes), tet_signs, tet_edges,
      reinterpret_cast<const double2 *>(lam), reinterpret_cast<const double2 *>(x), scale,
      reinterpret_cast<double2 *>(out));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_dirichlet(int32_t n, const int32_t *rowptr, const int32_t *colidx, const uint8_t *is_pec,
                              double diag_re, double diag_im, double *values, efgk_stream_t stream) {
  if (n <= 0) return 0;
  dirichlet_kernel<<<blocks_for(n, 256), 256, 0, stream>>>(n, rowptr, colidx, is_pec,
                                                          make_double2(diag_re, diag_im),
                                                          reinterpret_cast<double2 *>(values));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_add_terms(int64_t count, const int32_t *slot, const int32_t *term, const double *val,
                              const double *coef, double *values, efgk_stream_t stream) {
  if (count <= 0) return 0;
  add_terms_kernel<<<blocks_for(count, 256), 256, 0, stream>>>(
      count, slot, term, reinterpret_cast<const double2 *>(val), reinterpret_cast<const double2 *>(coef),
      reinterpret_cast<double2 *>(values));
  return static_cast<int>(cudaGetLastError());
}

extern "C" int efgk_blend(int64_t nnz, const double *K, const double *M, const double *M2,
                          const double *a_host, const double *b_host, const double *c_host, double *out,
                          efgk_stream_t stream) {
  if (nnz <= 0) return 0;
  const double2 a = make_double2(a_host[0], a_host[1]);
  const double2 b = make_double2(b_host[0], b_host[1]);
  const double2 c = c_host ? make_double2(c_host[0], c_host[1]) : make_double2(0, 0);
  blend_kernel<<<blocks_for(nnz, 256), 256, 0, stream>>>(
      nnz, reinterpret_cast<const double2 *>(K), reinterpret_cast<const double2 *>(M),
      reinterpret_cast<const double2 *>(M2), a, b, c, reinterpret_cast<double2 *>(out));
  return static_cast<int>(cudaGetLastError());
}
