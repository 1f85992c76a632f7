// solve_noalloc.cu — an allocation-free 3-column solve L x = b for callers that cannot allocate.
//
// Some callers cannot call cudaMalloc at the point where they need a solve: a host engine that
// hands out device memory only from its own pool, a real-time loop where allocation is banned,
// or a JNI / plugin host that owns the device heap. pd_solve_noalloc serves them: the caller
// passes the factor, b and x in its own device memory, and the solve's only workspace (the
// permuted right-hand side, 3 doubles per vertex) lives in the file-scope array below, which
// every GPU that loads this library holds until the process exits.
//
// Arithmetic follows the reference's solve exactly (EigenDirectSolver.cpp:411-448): forward
// sweep column by column in scatter form, then D⁻¹, then the backward sweep gathering each
// column in ascending row order — so the result is bit-identical to pd_sim_solve on a handle in
// the FP64_EXACT mode (whose solve follows the same order).
#include <cuda_runtime.h>

#include <atomic>
#include <string>

#include "../../include/pd_gb300.h"

namespace pdg {
void setLastError(const std::string& msg);
}

namespace {

// The shared workspace: 3 doubles per vertex, at most PD_NOALLOC_MAX_VERTICES vertices (1.5 MiB).
static __device__ __align__(256) double g_noallocScratch[3 * PD_NOALLOC_MAX_VERTICES];

// The workspace's device address per device ordinal, looked up by the first call on that device.
// Atomic: two host threads making their first call together both store the same address. The
// address belongs to the device's primary context; after that context is reset (cudaDeviceReset)
// the library must be reloaded before the next call, which this cache does not detect.
constexpr int kMaxDevices = 64;
std::atomic<double*> g_scratchAddr[kMaxDevices] = {};

// One warp per x/y/z component; the three components never touch each other's entries.
__global__ void __launch_bounds__(96) solveNoAllocKernel(int n, const int32_t* __restrict__ perm,
                                                        const int32_t* __restrict__ colptr,
                                                        const int32_t* __restrict__ rowidx,
                                                        const double* __restrict__ val,
                                                        const double* __restrict__ dinv,
                                                        const double* __restrict__ b, double* __restrict__ x,
                                                        double* __restrict__ w) {
  const int c = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  for (int k = lane; k < n; k += 32) w[3 * k + c] = b[3 * perm[k] + c];
  __syncwarp();
  // forward: y_k final when column k is reached; push −L_ik·y_k to every row i > k
  for (int k = 0; k < n; ++k) {
    const double yk = w[3 * k + c];
    for (int p = colptr[k] + lane; p < colptr[k + 1]; p += 32) {
      const int i = rowidx[p];
      w[3 * i + c] = __dsub_rn(w[3 * i + c], __dmul_rn(val[p], yk));
    }
    __syncwarp();
  }
  // backward: x_k = y_k·D⁻¹_k − Σ_{i>k} L_ik·x_i, terms subtracted in ascending i
  for (int k = n - 1; k >= 0; --k) {
    if (lane == 0) {
      double acc = __dmul_rn(w[3 * k + c], dinv[k]);
      for (int p = colptr[k]; p < colptr[k + 1]; ++p) acc = __dsub_rn(acc, __dmul_rn(val[p], w[3 * rowidx[p] + c]));
      w[3 * k + c] = acc;
    }
    __syncwarp();
  }
  for (int k = lane; k < n; k += 32) x[3 * perm[k] + c] = w[3 * k + c];
}

}  // namespace

extern "C" int pd_solve_noalloc(int32_t n, const int32_t* perm, const int32_t* colptr, const int32_t* rowidx,
                                const double* val, const double* dinv, const double* b, double* x,
                                void* stream) {
  if (n <= 0 || !perm || !colptr || !dinv || !b || !x || (n > 1 && (!rowidx || !val))) {
    pdg::setLastError("pd_solve_noalloc: null pointer or non-positive vertex count");
    return PD_ERR_INVALID_ARGUMENT;
  }
  if (n > PD_NOALLOC_MAX_VERTICES) {
    pdg::setLastError("pd_solve_noalloc: " + std::to_string(n) + " vertices exceed the fixed workspace of " +
                      std::to_string(PD_NOALLOC_MAX_VERTICES) + " vertices");
    return PD_ERR_INVALID_ARGUMENT;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    pdg::setLastError(std::string("pd_solve_noalloc: no usable current device: ") + cudaGetErrorString(e));
    return PD_ERR_CUDA;
  }
  // Set-up, once per device, with that device current: the array's host-side name is only a
  // stand-in, so the kernel must be given the device address.
  double* scratch = g_scratchAddr[dev].load(std::memory_order_acquire);
  if (scratch == nullptr) {
    e = cudaGetSymbolAddress(reinterpret_cast<void**>(&scratch), g_noallocScratch);
    if (e != cudaSuccess || scratch == nullptr) {
      pdg::setLastError(std::string("pd_solve_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      return PD_ERR_CUDA;
    }
    g_scratchAddr[dev].store(scratch, std::memory_order_release);
  }
  solveNoAllocKernel<<<1, 96, 0, static_cast<cudaStream_t>(stream)>>>(n, perm, colptr, rowidx, val, dinv, b, x,
                                                                       scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    pdg::setLastError(std::string("pd_solve_noalloc: launch failed: ") + cudaGetErrorString(e));
    return PD_ERR_CUDA;
  }
  return PD_OK;
}
