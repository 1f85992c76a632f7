// state_copy.cu — positions and velocities of a whole batch moved between the caller's host arrays
// and the device arena by one kernel launch each way.
//
// The reference steps SimContext::mesh.positions / velocities in host memory (core/sim/Scene.h:
// 154-178, core/sim/Integrator.cpp:312-797); pd_sim_step_host keeps that contract. When every
// bound array is page-locked (cudaHostAlloc / cudaHostRegister), the GPU reads and writes it
// directly over the host link: one gather before the substeps and one scatter after them, grid
// (chunks, instances), instead of four cudaMemcpyAsync calls per cloth. Both report into a status
// word in mapped host memory, so the host reads them after the stream synchronises without a copy:
// word 0 — the gather saw a non-finite position (the check pd_sim_set_state makes on the host);
// word 1 — the scatter saw an instance's team-exchange error flag set.
#include <cuda_runtime.h>

#include <cstdint>

#include "device.cuh"

namespace pdg {

namespace {

constexpr int kCopyThreads = 256;
constexpr int kCopyMaxChunks = 64;  // blocks per instance along x

// 16-byte accesses when all four arrays of an instance allow them (the arena always does;
// page-locked host allocations normally do), else 8-byte ones.
__device__ __forceinline__ bool aligned16(const HostStateDev& s) {
  return ((reinterpret_cast<uintptr_t>(s.hx) | reinterpret_cast<uintptr_t>(s.hv) | reinterpret_cast<uintptr_t>(s.dx) |
           reinterpret_cast<uintptr_t>(s.dv)) & 15u) == 0;
}

__global__ void __launch_bounds__(kCopyThreads) gatherStateKernel(const HostStateDev* __restrict__ t,
                                                                  volatile int* status) {
  const HostStateDev s = t[blockIdx.y];
  const int total = 3 * s.n;
  const int stride = gridDim.x * blockDim.x, first = blockIdx.x * blockDim.x + threadIdx.x;
  bool bad = false;
  int k0 = 0;
  if (aligned16(s)) {
    const int pairs = total >> 1;
    const double2* hx = reinterpret_cast<const double2*>(s.hx);
    const double2* hv = reinterpret_cast<const double2*>(s.hv);
    double2* dx = reinterpret_cast<double2*>(s.dx);
    double2* dv = reinterpret_cast<double2*>(s.dv);
    for (int k = first; k < pairs; k += stride) {
      const double2 x = hx[k], v = hv[k];
      bad |= !isfinite(x.x) || !isfinite(x.y);
      dx[k] = x;
      dv[k] = v;
    }
    k0 = 2 * pairs;  // the odd last double, if any
  }
  for (int k = k0 + first; k < total; k += stride) {
    const double x = s.hx[k];
    bad |= !isfinite(x);
    s.dx[k] = x;
    s.dv[k] = s.hv[k];
  }
  if (bad) status[0] = 1;
}

__global__ void __launch_bounds__(kCopyThreads) scatterStateKernel(const HostStateDev* __restrict__ t,
                                                                   volatile int* status) {
  const HostStateDev s = t[blockIdx.y];
  if (blockIdx.x == 0 && threadIdx.x == 0 && s.err && *s.err) status[1] = 1;
  const int total = 3 * s.n;
  const int stride = gridDim.x * blockDim.x, first = blockIdx.x * blockDim.x + threadIdx.x;
  int k0 = 0;
  if (aligned16(s)) {
    const int pairs = total >> 1;
    double2* hx = reinterpret_cast<double2*>(s.hx);
    double2* hv = reinterpret_cast<double2*>(s.hv);
    const double2* dx = reinterpret_cast<const double2*>(s.dx);
    const double2* dv = reinterpret_cast<const double2*>(s.dv);
    for (int k = first; k < pairs; k += stride) {
      hx[k] = dx[k];
      hv[k] = dv[k];
    }
    k0 = 2 * pairs;
  }
  for (int k = k0 + first; k < total; k += stride) {
    s.hx[k] = s.dx[k];
    s.hv[k] = s.dv[k];
  }
}

dim3 copyGrid(int count, int maxN) {
  const int chunks = (3 * maxN + kCopyThreads - 1) / kCopyThreads;
  return dim3(static_cast<unsigned>(chunks < 1 ? 1 : chunks > kCopyMaxChunks ? kCopyMaxChunks : chunks),
              static_cast<unsigned>(count));
}

}  // namespace

int launchGatherState(const HostStateDev* dTable, int count, int maxN, int* status, void* stream) {
  if (count <= 0 || count > 65535) return static_cast<int>(cudaErrorInvalidValue);
  gatherStateKernel<<<copyGrid(count, maxN), kCopyThreads, 0, static_cast<cudaStream_t>(stream)>>>(dTable, status);
  return static_cast<int>(cudaGetLastError());
}

int launchScatterState(const HostStateDev* dTable, int count, int maxN, int* status, void* stream) {
  if (count <= 0 || count > 65535) return static_cast<int>(cudaErrorInvalidValue);
  scatterStateKernel<<<copyGrid(count, maxN), kCopyThreads, 0, static_cast<cudaStream_t>(stream)>>>(dTable, status);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace pdg
