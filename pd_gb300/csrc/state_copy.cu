// state_copy.cu — positions and velocities of a whole batch moved between the caller's host arrays
// and the device arena by one kernel launch each way.
//
// The reference steps SimContext::mesh.positions / velocities in host memory (core/sim/Scene.h:
// 154-178, core/sim/Integrator.cpp:312-797); pd_sim_step_host keeps that contract. When every
// bound array is page-locked (cudaHostAlloc / cudaHostRegister), the GPU reads and writes it
// directly over the host link: one gather before the substeps and one scatter after them, grid
// (chunks, instances), instead of four cudaMemcpyAsync calls per cloth. The gather also flags a
// non-finite position, the check pd_sim_set_state makes on the host.
#include <cuda_runtime.h>

#include "device.cuh"

namespace pdg {

namespace {

constexpr int kCopyThreads = 256;
constexpr int kCopyMaxChunks = 64;  // blocks per instance along x

__global__ void __launch_bounds__(kCopyThreads) gatherStateKernel(const HostStateDev* __restrict__ t,
                                                                  int* __restrict__ nonFinite) {
  const HostStateDev s = t[blockIdx.y];
  const int total = 3 * s.n;
  bool bad = false;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    const double x = s.hx[k];
    bad |= !isfinite(x);
    s.dx[k] = x;
    s.dv[k] = s.hv[k];
  }
  if (bad) atomicOr(nonFinite, 1);
}

__global__ void __launch_bounds__(kCopyThreads) scatterStateKernel(const HostStateDev* __restrict__ t) {
  const HostStateDev s = t[blockIdx.y];
  const int total = 3 * s.n;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
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

int launchGatherState(const HostStateDev* dTable, int count, int maxN, int* dNonFinite, void* stream) {
  if (count <= 0 || count > 65535) return static_cast<int>(cudaErrorInvalidValue);
  gatherStateKernel<<<copyGrid(count, maxN), kCopyThreads, 0, static_cast<cudaStream_t>(stream)>>>(dTable,
                                                                                                  dNonFinite);
  return static_cast<int>(cudaGetLastError());
}

int launchScatterState(const HostStateDev* dTable, int count, int maxN, void* stream) {
  if (count <= 0 || count > 65535) return static_cast<int>(cudaErrorInvalidValue);
  scatterStateKernel<<<copyGrid(count, maxN), kCopyThreads, 0, static_cast<cudaStream_t>(stream)>>>(dTable);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace pdg
