// Device-resident state for the plain path: per-mesh pattern/topology on
// the GPU, FP64 assembly, and the FP64 Krylov drivers.  Host code only; it
// reaches the GPU through the CUDA runtime (memory, streams, graphs) and the
// kernel-level C-ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "edgefem.hpp"
#include "pattern.hpp"

struct CUstream_st;

namespace edgefem {

// Owning device buffer.
class DevBuf {
 public:
  DevBuf() = default;
  explicit DevBuf(std::size_t bytes) { alloc(bytes); }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr, o.n_ = 0; }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) {
      release();
      p_ = o.p_;
      n_ = o.n_;
      o.p_ = nullptr;
      o.n_ = 0;
    }
    return *this;
  }
  void alloc(std::size_t bytes);
  void release();
  void zero(CUstream_st *s);
  template <class T>
  T *as() const { return static_cast<T *>(p_); }
  std::size_t bytes() const { return n_; }
  void upload(const void *src, std::size_t bytes, CUstream_st *s);
  void download(void *dst, std::size_t bytes, CUstream_st *s) const;

 private:
  void *p_ = nullptr;
  std::size_t n_ = 0;
};

template <class T>
DevBuf to_device(const std::vector<T> &v, CUstream_st *s) {
  DevBuf b(std::max<std::size_t>(v.size() * sizeof(T), 16));
  if (!v.empty()) b.upload(v.data(), v.size() * sizeof(T), s);
  return b;
}

// Transfer accounting for copies made outside DevBuf (pinned staging).
void count_h2d(long long bytes);
void count_d2h(long long bytes);

// Throws std::runtime_error with the CUDA error string if code != 0.
void cuda_check(int code, const char *what);

// The library's CUDA stream (one per process; created on first use).
CUstream_st *stream();

// Per-mesh device topology and pattern.
struct MeshDev {
  std::uint64_t uid = 0;
  std::vector<int> pec_sorted;
  std::vector<std::vector<int>> blocks;
  Pattern pat;
  int n = 0, nnz = 0, T = 0;
  DevBuf xyz, tet_nodes, tet_signs, tet_edges, slots, color_tets, rowptr, colidx, diag, is_pec;
  // Discrete gradient for the auxiliary-space preconditioner: per edge the
  // (tail, head) node index, (-1, -1) for PEC edges; per node the incident
  // non-PEC edges and signs.
  int nn = 0;
  std::vector<int> enodes_h, nptr_h, nedge_h;
  std::vector<signed char> nsign_h;
  DevBuf enodes, nptr, nedge, nsign;
  // vector-nodal space: per edge (x_head - x_tail) / 2 (0 for PEC edges)
  DevBuf piw;
};

// Cached per (mesh, PEC set, dense blocks).  The returned object stays valid
// until the cache evicts it (it keeps the most recent few).
std::shared_ptr<MeshDev> mesh_device(const Mesh &mesh, const BC &bc,
                                     const std::vector<std::vector<int>> &blocks);

// Host-side term list: values[slot] += coef[term] * val.
struct TermList {
  std::vector<int> slot, term;
  VecC val;
  void add(int s, int t, cplx v) {
    slot.push_back(s);
    term.push_back(t);
    val.push_back(v);
  }
};

// FP64 assembly into `values` (nnz complex): sum over tets of
// s_i s_j (cK[t] K_ij + cM[t] M_ij), Dirichlet with diag_value, then terms.
void assemble_device(const MeshDev &md, const VecC &cK, const VecC &cM, cplx diag_value,
                     const TermList *terms, const VecC *coefs, DevBuf &values);

struct KrylovResult {
  int iters = 0;
  double residual = 0;  // |r| / |b|
  bool converged = false;
  std::string status;
};

// Accumulated over krylov64 calls on this thread since the last reset.
struct KrylovTotals {
  long long iters = 0;
  double max_residual = 0;
  int solves = 0;
  double device_ms = 0;
};
KrylovTotals &krylov_totals();

// Preconditioned FP64 solve of A x = b on the device (b, x device, n complex
// each).  method: "cocg" (A complex symmetric) or "bicgstab".  With a mesh
// and aux_level 1 the auxiliary-space preconditioner D^-1 + G Dn^-1 G^T is
// used, with 2 also the vector-nodal term omega Pi Dp^-1 Pi^T, with 0
// Jacobi alone; aux_level 3 selects block-Jacobi on EFGK_BJ_BS-row diagonal
// blocks (no mesh needed).
KrylovResult krylov64(const MeshDev *md, int n, const int *rowptr, const int *colidx, const int *diag_slot,
                      const double *vals, const double *b, double *x, const std::string &method, double tol,
                      int maxit, int aux_level = 0);

// Weight omega of the vector-nodal term omega Pi Dp^-1 Pi^T in the
// auxiliary-space preconditioner (aux_level 2 here, vector_aux in the
// batched engine).  A CPU study on the slab guide (FP64 COCG, 24x12x60 and
// 40x20x100) found 0.5 best among 0.25 ... 1: iterations 1083 -> 744 at
// 12 GHz and 1314 -> 861 at 10 GHz.
constexpr double kVectorAuxWeight = 0.5;

// Per-tet material coefficient vectors for assembly at frequency omega.
void tet_coefficients(const Mesh &mesh, const MaxwellParams &p, double omega, VecC &inv_mu, VecC &eps);

// Port helpers shared by the drivers.
struct PortSurface {  // M_s of one port as (slot, value) and as sparse rows
  std::vector<int> rows, cols;
  std::vector<double> vals;  // real, PEC rows/cols omitted, summed per (row, col)
};
PortSurface port_surface_mass(const Mesh &mesh, int surface_tag, const std::unordered_set<int> &pec);
int port_beta_tet(const Mesh &mesh, int surface_tag);

// Port blocks and ABC terms of the w w^H (driven-port) formulation
// (src/assemble_maxwell.cpp:212-265): per loaded port its non-PEC edges and
// weights, and the non-PEC edges of the absorbing-boundary triangles.
struct WwhTerms {
  std::vector<std::vector<int>> blocks;
  std::vector<std::vector<cplx>> w;
  std::vector<int> port_of_block;
  std::vector<int> abc_edges;
};
WwhTerms wwh_terms(const Mesh &mesh, const MaxwellParams &p, const BC &bc, const std::vector<WavePort> &ports);

}  // namespace edgefem
