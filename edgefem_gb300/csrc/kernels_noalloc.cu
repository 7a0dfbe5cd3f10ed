// Allocation-free Jacobi-COCG solve on caller-owned device arrays.
//
// For callers that cannot call cudaMalloc (a host that owns every device
// allocation through its own pool, or code running where allocation is not
// allowed), this entry point runs the FP64 COCG of efg_solve_linear with
// the Jacobi preconditioner (efg_solve_linear's preconditioner 0: it has no
// mesh data), but its work vectors and scalar block live in one fixed,
// file-scope device array instead of fresh allocations.
//
// Scratch layout (kNoAllocBytes, 256-byte aligned):
//   [0, 256)      scalar block (SC_SIZE doubles, sc_layout.h; the last
//                 double flags a row without a diagonal entry)
//   then r, p, q, dinv: kNoAllocMaxRows complex doubles each.
// Nothing in it has to start at zero: every call first rewrites the scalar
// block and the Jacobi diagonal, and the COCG initialisation writes x, r
// and p before they are read.
//
// Set-up: every call looks up the array's address on the current device
// with cudaGetSymbolAddress (no allocation; the address is not cached, so
// a context torn down and created again, e.g. by cudaDeviceReset, is
// picked up).  The first lookup on a device may load this file's module,
// which places the array in device memory: make the first call before any
// stream capture on the device.  Calls that overlap on one device (other
// threads or streams) share the array and race: serialise them.
#include <cuda_runtime.h>

#include <string>

#include "edgefem_gb300.h"
#include "edgefem_gb300_kernels.h"
#include "sc_layout.h"

namespace edgefem {
void set_last_error(const std::string &msg);
}

namespace {

constexpr int kNoAllocMaxRows = EFG_NOALLOC_MAX_ROWS;
constexpr size_t kScalarBytes = 256;
constexpr size_t kVecBytes = static_cast<size_t>(kNoAllocMaxRows) * 16;
constexpr size_t kNoAllocBytes = kScalarBytes + 4 * kVecBytes;
static_assert(SC_SIZE * sizeof(double) < kScalarBytes, "scalar block and flag must fit their slot");
constexpr int kScalarSlots = static_cast<int>(kScalarBytes / sizeof(double));
constexpr int kMissingDiag = kScalarSlots - 1;  // > 0: 1 + a row without a diagonal entry

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

__global__ void noalloc_scalars_kernel(double *sc, double tol2, double maxit) {
  for (int i = threadIdx.x; i < kScalarSlots; i += blockDim.x) sc[i] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    sc[SC_TOL2] = tol2;
    sc[SC_MAXIT] = maxit;
  }
}

// Inverse Jacobi diagonal found by scanning each row for its diagonal
// column; a zero diagonal gives 1 (no scaling), as in the allocating solve.
// A row without a diagonal entry (which the allocating solve rejects)
// records 1 + its index in sc[kMissingDiag] (any one such row).
__global__ void noalloc_dinv_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colidx,
                                    const double2 *__restrict__ vals, double2 *dinv, double *sc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 d = make_double2(0.0, 0.0);
    bool found = false;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (colidx[k] == i) {
        d = vals[k];
        found = true;
        break;
      }
    if (!found) sc[kMissingDiag] = 1.0 + i;
    const double m = d.x * d.x + d.y * d.y;
    dinv[i] = m > 0.0 ? make_double2(d.x / m, -d.y / m) : make_double2(1.0, 0.0);
  }
}

int fail(const std::string &msg) {
  edgefem::set_last_error("efg_solve_linear_device_noalloc: " + msg);
  return -1;
}

int cuda_fail(const char *what, cudaError_t e) {
  return fail(std::string(what) + ": " + cudaGetErrorString(e));
}

// Device address of the scratch array on the current device, looked up on
// every call (a host-side lookup that allocates nothing).
cudaError_t scratch_address(unsigned char **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<unsigned char *>(p);
  return cudaSuccess;
}

}  // namespace

extern "C" int efg_solve_linear_device_noalloc(int32_t n, const int32_t *rowptr, const int32_t *colidx,
                                               const double *vals, const double *b, double *x, double tolerance,
                                               int32_t max_iterations, void *stream, int32_t *iterations,
                                               double *residual, int32_t *converged) {
  edgefem::set_last_error("");
  if (n < 0) return fail("n must be >= 0");
  if (n > kNoAllocMaxRows)
    return fail("n = " + std::to_string(n) + " rows exceeds the fixed scratch capacity of " +
                std::to_string(kNoAllocMaxRows) + " rows (EFG_NOALLOC_MAX_ROWS); use efg_solve_linear");
  if (!(tolerance > 0.0)) return fail("tolerance must be > 0");
  if (max_iterations <= 0) return fail("max_iterations must be > 0");
  if (n > 0 && (!rowptr || !colidx || !vals || !b || !x)) return fail("null array pointer");
  if (iterations) *iterations = 0;
  if (residual) *residual = 0.0;
  if (converged) *converged = 1;
  if (n == 0) return 0;

  unsigned char *base = nullptr;
  cudaError_t e = scratch_address(&base);
  if (e != cudaSuccess) return cuda_fail("cudaGetSymbolAddress", e);
  double *sc = reinterpret_cast<double *>(base);
  double *r = reinterpret_cast<double *>(base + kScalarBytes);
  double *p = reinterpret_cast<double *>(base + kScalarBytes + kVecBytes);
  double *q = reinterpret_cast<double *>(base + kScalarBytes + 2 * kVecBytes);
  double *dinv = reinterpret_cast<double *>(base + kScalarBytes + 3 * kVecBytes);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  noalloc_scalars_kernel<<<1, 32, 0, s>>>(sc, tolerance * tolerance, static_cast<double>(max_iterations));
  noalloc_dinv_kernel<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, s>>>(
      n, rowptr, colidx, reinterpret_cast<const double2 *>(vals), reinterpret_cast<double2 *>(dinv), sc);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail("set-up launch", e);
  double missing = 0.0;
  e = cudaMemcpyAsync(&missing, sc + kMissingDiag, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail("set-up read", e);
  if (missing > 0.0)
    return fail("row " + std::to_string(static_cast<long long>(missing) - 1) +
                " has no diagonal entry (every row must store its diagonal)");
  int err = efgk_cocg64_init(n, b, dinv, x, r, p, sc, nullptr, s);
  if (err) return cuda_fail("cocg init", static_cast<cudaError_t>(err));

  // Chunks of 16 iterations; the device stops updating once its status
  // leaves "running", so a chunk may overrun the stop harmlessly.
  const int chunk = 16;
  const int max_chunks = max_iterations / chunk + 2;
  double hs[SC_SIZE];
  for (int c = 0; c < max_chunks; ++c) {
    for (int k = 0; k < chunk; ++k) {
      err = efgk_cocg64_step(n, rowptr, colidx, vals, dinv, x, r, p, q, sc, k & 1, nullptr, s);
      if (err) return cuda_fail("cocg step", static_cast<cudaError_t>(err));
    }
    e = cudaMemcpyAsync(hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail("status read", e);
    if (hs[SC_STATUS] != EFGK_RUNNING) break;
  }
  const double bb = hs[SC_BB];
  const bool ok = bb == 0.0 || hs[SC_STATUS] == EFGK_CONVERGED;
  if (iterations) *iterations = static_cast<int32_t>(hs[SC_ITERS]);
  if (residual) *residual = bb > 0.0 ? sqrt(hs[SC_LASTRR] / bb) : 0.0;
  if (converged) *converged = ok ? 1 : 0;
  if (!ok) {
    edgefem::set_last_error(hs[SC_STATUS] == EFGK_BREAKDOWN ? "efg_solve_linear_device_noalloc: breakdown"
                                                           : "efg_solve_linear_device_noalloc: not converged");
    return 1;
  }
  return 0;
}
