// refactor.cu — numeric LDLᵀ refactorization on the device when Ã's values change but its pattern
// does not (a stiffness, mass or dt change: the reference refactorizes on such a stamp change,
// core/sim/Integrator.cpp:341-372, core/assemble/Assembler.cpp:111-174).
//
// The symbolic structure (ordering, pattern of L in CSR and CSC, nested-dissection supernodes)
// stays what the host built. Columns are computed left-looking in the dot-product form
//   L(i,j)·d_j = Ã(i,j) − Σ_{k<j} L(i,k)·L(j,k)·d_k,   d_j = Ã(j,j) − Σ_{k<j} L(j,k)²·d_k,
// where the k run over the columns both rows i and j hold (a merge of two sorted CSR rows), in
// ascending order, by one thread per entry: no atomics, the same bits on every run. Row j's
// products L(j,k)·d_k sit in shared memory for the column. Supernodes of one tree level are
// independent (a column depends only on its descendants in the elimination tree, which lie in
// its supernode or in the supernodes below it), so a launch runs one level with one CTA per
// supernode and its columns in order. Then the dense inverses of the unit-lower diagonal blocks
// (one thread per block column, forward substitution in the host's order) and the FP32 copies.
#include <cuda_runtime.h>

#include <cstdint>

#include "device.cuh"

namespace pdg {

namespace {

constexpr int kRefactorThreads = 256;

__global__ void __launch_bounds__(kRefactorThreads) ldltLevelKernel(RefactorDev r, const int32_t* __restrict__ sns) {
  extern __shared__ double sv[];                   // L(j,k)·d_k of row j
  int32_t* sk = reinterpret_cast<int32_t*>(sv + r.maxRowLen);  // k of row j
  __shared__ double sd;
  const int s = sns[blockIdx.x];
  const int s0 = r.snStart[s], s1 = r.snStart[s + 1];
  for (int j = s0; j < s1; ++j) {
    const int rb = r.rowptr[j], len2 = r.rowptr[j + 1] - rb;
    for (int t = threadIdx.x; t < len2; t += blockDim.x) {
      const int k = r.colidx[rb + t];
      sk[t] = k;
      sv[t] = r.rowval[rb + t] * r.d[k];
    }
    __syncthreads();
    const int cb = r.colptr[j], ce = r.colptr[j + 1];
    for (int p = static_cast<int>(threadIdx.x) - 1; p < ce - cb; p += blockDim.x) {
      const int i = p < 0 ? j : r.rowidx[cb + p];
      const int ap = p < 0 ? r.aPosDiag[j] : r.aPosCsc[cb + p];
      double acc = ap >= 0 ? r.Aval[ap] : 0.0;
      int a = r.rowptr[i], b = 0;
      const int ae = r.rowptr[i + 1];
      while (a < ae && b < len2) {  // row i's columns below j against row j's, both ascending
        const int ka = r.colidx[a];
        if (ka >= j) break;
        const int kb = sk[b];
        if (ka == kb) {
          acc -= r.rowval[a] * sv[b];
          ++a;
          ++b;
        } else if (ka < kb) {
          ++a;
        } else {
          ++b;
        }
      }
      if (p < 0) sd = acc;
      else r.colval[cb + p] = acc;  // unscaled until d_j is known
    }
    __syncthreads();
    const double dj = sd;
    if (threadIdx.x == 0) {
      r.d[j] = dj;
      r.dinv[j] = 1.0 / dj;
      if (dj == 0.0 || !isfinite(dj)) atomicCAS(r.status, 0, j + 1);
    }
    for (int q = cb + threadIdx.x; q < ce; q += blockDim.x) {
      const double l = r.colval[q] / dj;
      r.colval[q] = l;
      r.rowval[r.cscToCsr[q]] = l;
    }
    __syncthreads();  // row values of column j are read by the next column
  }
}

// Packed rows of L_SS⁻¹ (row-major lower, r(r+1)/2 + c) and of its transpose (row r: c = r..sz−1).
__global__ void __launch_bounds__(kRefactorThreads) blockInverseKernel(RefactorDev r) {
  const int s = blockIdx.x;
  const int s0 = r.snStart[s], sz = r.snStart[s + 1] - s0;
  double* lo = r.invL + r.snInvOff[s];
  double* up = r.invLT + r.snInvOff[s];
  for (int c = threadIdx.x; c < sz; c += blockDim.x) {  // column c by forward substitution
    lo[static_cast<int64_t>(c) * (c + 1) / 2 + c] = 1.0;
    for (int rr = c + 1; rr < sz; ++rr) {
      const int i = s0 + rr;
      double acc = 0.0;
      for (int p = r.offEnd[i]; p < r.rowptr[i + 1]; ++p) {  // the block part of row i, columns ascending
        const int t = r.colidx[p] - s0;
        if (t < c) continue;
        acc += r.rowval[p] * lo[static_cast<int64_t>(t) * (t + 1) / 2 + c];
      }
      lo[static_cast<int64_t>(rr) * (rr + 1) / 2 + c] = -acc;
    }
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  for (int rr = warp; rr < sz; rr += warps) {
    const int64_t off = static_cast<int64_t>(rr) * sz - static_cast<int64_t>(rr) * (rr - 1) / 2;
    for (int c = rr + lane; c < sz; c += 32) up[off + (c - rr)] = lo[static_cast<int64_t>(c) * (c + 1) / 2 + rr];
  }
}

__global__ void convertKernel(RefactorDev r) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t first = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  for (int64_t q = first; q < r.nnz; q += stride) {
    r.rowval32[q] = static_cast<float>(r.rowval[q]);
    r.colval32[q] = static_cast<float>(r.colval[q]);
  }
  for (int64_t q = first; q < r.nInv; q += stride) {
    r.invL32[q] = static_cast<float>(r.invL[q]);
    r.invLT32[q] = static_cast<float>(r.invLT[q]);
  }
  for (int64_t q = first; q < r.n; q += stride) r.dinv32[q] = static_cast<float>(r.dinv[q]);
}

}  // namespace

int refactorSmemBytes(int maxRowLen) { return maxRowLen * 12 + 8; }

int launchRefactor(const RefactorDev& r, const int32_t* dSnByLevel, const int32_t* snLevelPtr, int levels, int ns,
                   void* stream) {
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int smem = refactorSmemBytes(r.maxRowLen);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(ldltLevelKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return static_cast<int>(e);
  }
  for (int l = 0; l < levels; ++l) {
    const int count = snLevelPtr[l + 1] - snLevelPtr[l];
    if (count <= 0) continue;
    ldltLevelKernel<<<count, kRefactorThreads, smem, st>>>(r, dSnByLevel + snLevelPtr[l]);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return static_cast<int>(e);
  }
  if (ns > 0) blockInverseKernel<<<ns, kRefactorThreads, 0, st>>>(r);
  convertKernel<<<4 * 152, 256, 0, st>>>(r);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace pdg
