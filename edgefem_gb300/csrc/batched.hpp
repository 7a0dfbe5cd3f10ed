// Batched eigenmode engine: set up once (pattern, FP64 assembly packed into
// FP32/FP64 operator arrays, port-face tables, autotuned chunking), then
// solve any number of times with the inputs resident in device memory.
#pragma once

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
  long long nnz() const { return nnz_; }
  int rhs() const { return R_; }
  int rows_per_chunk() const { return rows_per_chunk_; }
  double setup_ms() const { return setup_ms_; }
  long long launches() const { return launches_; }
  const std::vector<std::pair<int, float>> &tune_log() const { return tune_log_; }

 private:
  int autotune();
  void set_chunks(int rows_per_chunk);
  void build_graph(int chunk_iters);

  BatchOptions opt_;
  std::vector<double> freqs_;
  int B_ = 0, F_ = 0, P_ = 0, R_ = 0, N_ = 0, n_chunks_ = 0, n_srows_ = 0, rows_per_chunk_ = 0;
  long long nnz_ = 0;
  std::vector<int> row_off_;
  std::vector<char> evanescent_;
  DevBuf d_rowptr_, d_colidx_, d_K32_, d_M32_, d_K64_, d_M64_, d_kd32_, d_md32_, d_kd64_, d_md64_;
  DevBuf d_sidx_, d_sptr_, d_scol_, d_sval32_, d_sval64_, d_scidx_, d_sdiag32_, d_sdiag64_, d_cval_,
      d_srow_inst_, d_srow_row_;
  DevBuf d_k2f_, d_k2d_, d_scf_, d_scd_;
  DevBuf d_xc_, d_r_, d_p_, d_q_, d_x64_;
  DevBuf d_rho_, d_pq_, d_rr_, d_bb_, d_status_, d_iters_, d_itc_, d_Sacc_;
  DevBuf d_ci_, d_cb_, d_ce_;
  void *exec_ = nullptr;
  int graph_iters_ = 0;
  double setup_ms_ = 0, solve_ms_ = 0;
  long long launches_ = 0;
  std::vector<std::pair<int, float>> tune_log_;
};

}  // namespace edgefem
