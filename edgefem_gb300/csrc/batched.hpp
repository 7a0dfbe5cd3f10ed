// Batched eigenmode engine: set up once (pattern, FP64 assembly packed into
// the solve's operator arrays, gradient topology and nodal diagonals,
// port-face tables, autotuned launch shape), then solve any number of times
// with the inputs resident in device memory.
#pragma once

#include <memory>
#include <utility>
#include <vector>

#include "batch_layout.h"
#include "device.hpp"
#include "edgefem.hpp"

namespace edgefem {

class BatchSolver {
 public:
  BatchSolver(const std::vector<BatchInstance> &inst, const std::vector<double> &freqs, const BatchOptions &opt);
  ~BatchSolver();
  BatchSolver(const BatchSolver &) = delete;
  BatchSolver &operator=(const BatchSolver &) = delete;

  // One full solve from x = 0; S[instance][frequency] (P x P).
  std::vector<std::vector<MatC>> solve(BatchStats *stats);

  EfgkBatch desc() const;
  int rows() const { return N_; }
  int nodes() const { return NN_; }
  long long nnz() const { return nnz_; }
  int rhs() const { return R0_; }  // right-hand sides per row at set-up
  int rows_per_chunk() const { return rows_per_chunk_; }
  int spmm_grid() const { return spmm_grid_; }
  int spmm_rhs_per_lane() const { return spmm_v_; }
  int precision() const { return prec_; }
  double setup_ms() const { return setup_ms_; }
  long long launches() const { return launches_; }
  // (rows per chunk * 100 + blocks per SM, milliseconds per SpMM) candidates
  const std::vector<std::pair<int, float>> &tune_log() const { return tune_log_; }
  // Per (instance, rhs) outcome of the last solve, index b*R + rhs:
  // status (0 running, 1 converged, 2 breakdown, 3 max iterations,
  // 4 inactive padding), iterations, relative true residual at the last
  // replacement.
  const std::vector<int> &last_status() const { return last_status_; }
  const std::vector<int> &last_iters() const { return last_iters_; }
  const std::vector<double> &last_residual() const { return last_residual_; }

 private:
  std::pair<int, int> autotune();
  // Column compaction (double-float engine): keep only the right-hand-side
  // columns `keep` (current column indices, ascending, whole frequencies),
  // repacked into a power-of-two R; results of the dropped columns are
  // harvested first.
  void compact(const std::vector<int> &keep);
  // Overlap of the current x into the host results for the current columns
  // c with take[c] != 0.
  void harvest(const std::vector<char> &take);
  void upload_tables();
  // Reduced-basis phase: x of every current column (R_ == R0_) set to the
  // Galerkin solution on the orthonormalised solutions of `coarse` (which
  // kept its converged x); returns the smallest basis size over instances.
  int rb_warm_start(const BatchSolver &coarse);
  void set_chunks(int rows_per_chunk);
  void build_graph(int chunk_iters);
  int launch_iteration(const EfgkBatch &bt, int k, int chunk_iters, CUstream_st *s, bool record);

  BatchOptions opt_;
  std::vector<double> freqs_;
  int B_ = 0, F_ = 0, P_ = 0, R_ = 0, N_ = 0, NN_ = 0, n_chunks_ = 0, n_nchunks_ = 0, n_srows_ = 0;
  int rows_per_chunk_ = 0, spmm_grid_ = 0, spmm_v_ = 0;
  bool spmm_tm_ = false;  // tile-major SpMM work order
  int prec_ = 2;  // BatchOptions::precision (0 complex64, 1/2 double-float)
  bool driven_ = false, has_md_ = false, use_pi_ = false;
  int C_ = 0;     // side-term coefficient rows per instance
  std::vector<cplx> sqrt_z0_;  // [B][P], driven ports
  long long nnz_ = 0;
  std::vector<int> row_off_, node_off_;
  std::vector<char> evanescent_;
  // Original right-hand-side count and per-column tables (column = f*P + a),
  // the original column held by each current column (-1: padding), and the
  // per (instance, original column) results of the last solve.
  int R0_ = 0, tuned_v_ = 0;
  std::vector<float> k2f_h_;
  std::vector<double> k2d_h_;
  std::vector<std::complex<float>> scf_h_;
  std::vector<cplx> scd_h_, rcd_h_, kap_h_;
  std::vector<int> col_orig_;
  std::vector<cplx> res_S_;  // [B][P][R0]
  std::vector<int> res_status_, res_iters_;
  std::vector<double> res_resid_;
  long long compactions_ = 0;
  DevBuf d_rowptr_, d_nz_, d_colidx_, d_K64_, d_M64_, d_kd32_, d_md32_;
  DevBuf d_enodes_, d_nptr_, d_nedge_, d_nsign_, d_kn32_, d_mn32_, d_msn32_;
  DevBuf d_piw_, d_kpn32_, d_mpn32_, d_mdpn32_, d_mspn32_, d_ninc_;
  DevBuf d_sidx_, d_sptr_, d_scol_, d_sval32_, d_sval64_, d_scidx_, d_sdiag32_, d_cval_, d_srow_inst_,
      d_srow_row_;
  DevBuf d_k2f_, d_k2d_, d_scf_, d_scd_, d_rcd_, d_kap64_, d_kap32_, d_MD64_, d_mdlo_, d_mdd32_, d_mnd32_;
  DevBuf d_xc_, d_r_, d_p_, d_q_, d_t_, d_x64_;
  DevBuf d_xd_, d_rd_, d_pd_, d_qd_, d_td_, d_nzlo_;
  DevBuf d_rho_, d_pq_, d_rr_, d_bb_, d_rmax_, d_status_, d_flag_, d_iters_, d_last_rep_, d_counters_, d_Sacc_;
  DevBuf d_ci_, d_cb_, d_ce_, d_nci_, d_ncb_, d_nce_;
  void *exec_ = nullptr;
  int graph_iters_ = 0;
  double setup_ms_ = 0, solve_ms_ = 0, device_ms_ = 0, spmm_ms_ = 0;
  long long launches_ = 0, kernel_launches_ = 0, spmm_timed_ = 0;
  std::vector<void *> events_;
  std::vector<std::pair<int, float>> tune_log_;
  std::vector<int> last_status_, last_iters_;
  std::vector<double> last_residual_;
  // Reduced-basis phase: the sample-frequency engine and the indices of its
  // frequencies in freqs_; keep_x_ makes harvest() copy converged columns of
  // x into d_xkeep_ ([N][R0] complex dd, column = original column).
  std::unique_ptr<BatchSolver> coarse_;
  std::vector<int> coarse_f_;
  bool keep_x_ = false;
  DevBuf d_xkeep_;
  // host copies of the port-face side CSR (global rows and columns)
  std::vector<int> hs_ptr_, hs_col_, hs_cidx_, hs_row_, hs_inst_;
  std::vector<double> hs_val_;
  std::vector<cplx> hs_cval_;
};

}  // namespace edgefem
