// refactor.cu — numeric LDLᵀ refactorization on the device when Ã's values change but its pattern
// does not (a stiffness, mass or dt change: the reference refactorizes on such a stamp change,
// core/sim/Integrator.cpp:341-372, core/assemble/Assembler.cpp:111-174).
//
// The symbolic structure (ordering, pattern of L in CSR and CSC, nested-dissection supernodes)
// stays what the host built. Columns are computed left-looking in the dot-product form
//   L(i,j)·d_j = Ã(i,j) − Σ_{k<j} L(i,k)·L(j,k)·d_k,   d_j = Ã(j,j) − Σ_{k<j} L(j,k)²·d_k,
// where the k run over the columns both rows i and j hold (a merge of two sorted CSR rows), in
// ascending order, by one thread per entry: no atomics, the same bits on every run. Row j's
// products L(j,k)·d_k sit in shared memory for the column. A column depends only on its
// descendants in the elimination tree, which lie in its supernode or in the supernodes below it,
// so each tree level is two launches: part A subtracts the contributions of the supernodes below
// for every column of the level at once (one CTA per column), part B runs each supernode's
// columns in order for the contributions from inside the supernode (one CTA per supernode) —
// the sequential chain then only merges rows over the supernode's own columns. Then the dense
// inverses of the unit-lower diagonal blocks (one thread per block column, forward substitution in
// the host's order) and the FP32 copies.
#include <cuda_runtime.h>

#include <cstdint>

#include "device.cuh"

namespace pdg {

namespace {

constexpr int kRefactorThreads = 256;

// Σ over the columns k both rows hold, k in [klo, khi), ascending, of L(i,k)·(L(j,k)·d_k), with
// row j's part staged as (sk, sv)[0, len): row i's entries from position a on.
__device__ __forceinline__ double mergeDot(const RefactorDev& r, int a, int ae, int khi, const int32_t* sk,
                                           const double* sv, int len) {
  double acc = 0.0;
  int b = 0;
  while (a < ae && b < len) {
    const int ka = r.colidx[a];
    if (ka >= khi) break;
    const int kb = sk[b];
    if (ka == kb) {
      acc += r.rowval[a] * sv[b];
      ++a;
      ++b;
    } else if (ka < kb) {
      ++a;
    } else {
      ++b;
    }
  }
  return acc;
}

// Part A, every column j of the level at once (one CTA per column): the contributions of the
// columns below j's supernode, Ã(i,j) − Σ_{k<s0} L(i,k)·d_k·L(j,k), into colval (and d_j's into d).
__global__ void __launch_bounds__(kRefactorThreads) ldltExternalKernel(RefactorDev r, const int32_t* __restrict__ cols) {
  extern __shared__ double sv[];
  int32_t* sk = reinterpret_cast<int32_t*>(sv + r.maxRowLen);
  const int j = cols[blockIdx.x];
  const int s0 = r.snStart[r.rowSn[j]];
  const int rb = r.rowptr[j], len = r.offEnd[j] - rb;  // row j's columns below s0
  for (int t = threadIdx.x; t < len; t += blockDim.x) {
    const int k = r.colidx[rb + t];
    sk[t] = k;
    sv[t] = r.rowval[rb + t] * r.d[k];
  }
  __syncthreads();
  const int cb = r.colptr[j], ce = r.colptr[j + 1];
  for (int p = static_cast<int>(threadIdx.x) - 1; p < ce - cb; p += blockDim.x) {
    const int i = p < 0 ? j : r.rowidx[cb + p];
    const int ap = p < 0 ? r.aPosDiag[j] : r.aPosCsc[cb + p];
    const double a = ap >= 0 ? r.Aval[ap] : 0.0;
    const double v = a - mergeDot(r, r.rowptr[i], r.rowptr[i + 1], s0, sk, sv, len);
    if (p < 0) r.d[j] = v;
    else r.colval[cb + p] = v;
  }
}

// First CSR position of row i at a column ≥ s0 (binary search; rows are sorted).
__device__ __forceinline__ int rowFrom(const RefactorDev& r, int i, int s0) {
  int lo = r.rowptr[i], hi = r.rowptr[i + 1];
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (r.colidx[mid] < s0) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Part B, one CTA per supernode, its columns in order: the contributions of the supernode's own
// earlier columns, then d_j and L(i,j) = (…)/d_j, written to both the CSC and the CSR copy.
__global__ void __launch_bounds__(kRefactorThreads) ldltInternalKernel(RefactorDev r, const int32_t* __restrict__ sns) {
  extern __shared__ double sv[];
  int32_t* sk = reinterpret_cast<int32_t*>(sv + r.maxRowLen);
  __shared__ double sd;
  const int s = sns[blockIdx.x];
  const int s0 = r.snStart[s], s1 = r.snStart[s + 1];
  for (int j = s0; j < s1; ++j) {
    const int rb = r.offEnd[j], len = r.rowptr[j + 1] - rb;  // row j's columns in [s0, j)
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      const int k = r.colidx[rb + t];
      sk[t] = k;
      sv[t] = r.rowval[rb + t] * r.d[k];
    }
    __syncthreads();
    const int cb = r.colptr[j], ce = r.colptr[j + 1];
    for (int p = static_cast<int>(threadIdx.x) - 1; p < ce - cb; p += blockDim.x) {
      const int i = p < 0 ? j : r.rowidx[cb + p];
      const int a0 = i < s1 ? r.offEnd[i] : rowFrom(r, i, s0);
      const int w = j - s0;
      double dot;
      if (len == w && a0 + w <= r.rowptr[i + 1] && (w == 0 || (r.colidx[a0] == s0 && r.colidx[a0 + w - 1] == j - 1))) {
        // rows i and j both hold every column of [s0, j) (a filled separator block): the same
        // terms in the same order as the merge, read directly
        dot = 0.0;
#pragma unroll 8
        for (int t = 0; t < w; ++t) dot += r.rowval[a0 + t] * sv[t];
      } else {
        dot = mergeDot(r, a0, r.rowptr[i + 1], j, sk, sv, len);
      }
      const double v = (p < 0 ? r.d[j] : r.colval[cb + p]) - dot;
      if (p < 0) sd = v;
      else r.colval[cb + p] = v;  // unscaled until d_j is known
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
// CTA (s, chunk): one thread per block column c = chunk·blockDim + lane, the column kept in shared
// memory while it is built by forward substitution in the host's order (rows of the block part
// of L ascending); grid (supernodes, most chunks), chunks past a supernode's size exit.
__global__ void blockInverseKernel(RefactorDev r, int maxSn) {
  extern __shared__ double xs[];  // blockDim × maxSn: column of thread t at xs[t·maxSn]
  const int s = blockIdx.x;
  const int s0 = r.snStart[s], sz = r.snStart[s + 1] - s0;
  const int c = blockIdx.y * blockDim.x + threadIdx.x;
  if (static_cast<int>(blockIdx.y * blockDim.x) >= sz) return;  // the whole CTA: no barrier below
  if (c >= sz) return;
  double* x = xs + static_cast<size_t>(threadIdx.x) * maxSn;
  double* lo = r.invL + r.snInvOff[s];
  double* up = r.invLT + r.snInvOff[s];
  for (int t = c; t < sz; ++t) x[t] = 0.0;
  x[c] = 1.0;
  for (int rr = c + 1; rr < sz; ++rr) {
    const int i = s0 + rr;
    const int pb = r.offEnd[i], pe = r.rowptr[i + 1];
    double acc = 0.0;
    if (pe - pb == rr) {  // row i holds every column of the block before it: read directly
#pragma unroll 8
      for (int t = c; t < rr; ++t) acc += r.rowval[pb + t] * x[t];
    } else {
      for (int p = pb; p < pe; ++p) {  // the block part of row i, columns ascending
        const int t = r.colidx[p] - s0;
        if (t < c) continue;
        acc += r.rowval[p] * x[t];
      }
    }
    x[rr] = -acc;
  }
  for (int rr = c; rr < sz; ++rr) lo[static_cast<int64_t>(rr) * (rr + 1) / 2 + c] = x[rr];
  const int64_t off = static_cast<int64_t>(c) * sz - static_cast<int64_t>(c) * (c - 1) / 2;
  for (int rr = c; rr < sz; ++rr) up[off + (rr - c)] = x[rr];
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

int launchRefactor(const RefactorDev& r, const int32_t* dSnByLevel, const int32_t* snLevelPtr, const int32_t* dLvlRows,
                   const int32_t* lvlRowPtr, int levels, int ns, int maxSn, void* stream) {
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int smem = refactorSmemBytes(r.maxRowLen);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(ldltExternalKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(ldltInternalKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return static_cast<int>(e);
  }
  for (int l = 0; l < levels; ++l) {
    const int cols = lvlRowPtr[l + 1] - lvlRowPtr[l], sns = snLevelPtr[l + 1] - snLevelPtr[l];
    if (cols > 0) ldltExternalKernel<<<cols, kRefactorThreads, smem, st>>>(r, dLvlRows + lvlRowPtr[l]);
    if (sns > 0) ldltInternalKernel<<<sns, kRefactorThreads, smem, st>>>(r, dSnByLevel + snLevelPtr[l]);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return static_cast<int>(e);
  }
  if (ns > 0 && maxSn > 0) {
    // columns per CTA: as many as fit in shared memory (at most 32), so that the root block's
    // columns run on several SMs
    int w = 32;
    while (w > 1 && static_cast<size_t>(w) * maxSn * sizeof(double) > 200 * 1024) w >>= 1;
    const size_t bytes = static_cast<size_t>(w) * maxSn * sizeof(double);
    if (bytes > 200 * 1024) return static_cast<int>(cudaErrorInvalidValue);
    if (bytes > 48 * 1024) {
      const cudaError_t e = cudaFuncSetAttribute(blockInverseKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 static_cast<int>(bytes));
      if (e != cudaSuccess) return static_cast<int>(e);
    }
    const dim3 grid(ns, (maxSn + w - 1) / w);
    blockInverseKernel<<<grid, w, bytes, st>>>(r, maxSn);
  }
  convertKernel<<<4 * 152, 256, 0, st>>>(r);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace pdg
