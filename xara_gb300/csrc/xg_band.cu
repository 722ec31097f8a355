// xg_band.cu -- `system ProfileSPD` for a model made of many small
// disconnected parts (a batch of frames): every part's LDL' in its own band,
// one block per part, all parts in one launch.  The reference runs each such
// model alone with ProfileSPDLinDirectSolver (system_of_eqn/linearSOE/
// profileSPD/ProfileSPDLinDirectSolver.cpp:100-256); its pivot checks are
// applied per part (the part's first pivot must be positive, later ones
// non-zero and above minDiagTol in magnitude).
//
// Storage: part c, local row i holds the entries (i, i-k), k = 0..b_c, at
// band[boff[c] + i*(b_c+1) + k] (b_c: the part's envelope width).  Factor:
// right-looking, column j scales the b_c entries below the pivot and updates
// the trailing triangle of the band; the column below the pivot is staged in
// shared memory.  Solve: one warp per part walks the rows forward and back,
// the band's dot products reduced with shuffles.
#include <cuda_runtime.h>

#include <algorithm>

#include "xg_internal.h"

namespace xg {

namespace {

constexpr int kBandThreads = 128;
constexpr int kBandMaxWidth = 255;      // b_c + 1 <= 256 staged column entries

__global__ void __launch_bounds__(kBandThreads) k_band_factor(BandSystem S) {
  const int c = blockIdx.x;
  if (c >= S.ncomp) return;
  const int e0 = S.cstart[c], n = S.cstart[c + 1] - e0, b = S.bw[c], ld = b + 1;
  double *B = S.band + S.boff[c];
  __shared__ double col[kBandMaxWidth + 1], lcol[kBandMaxWidth + 1];
  __shared__ double sinv;
  __shared__ int bad;
  // fill the band from the CSR rows of the part (lower triangle)
  for (long k = threadIdx.x; k < (long)n * ld; k += blockDim.x) B[k] = 0.0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int row = e0 + i;
    for (int q = S.rowptr[row]; q < S.rowptr[row + 1]; q++) {
      const int j = S.colidx[q] - e0;
      if (j <= i) B[(long)i * ld + (i - j)] = S.vals[q];
    }
  }
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < n; j++) {
    const int m = min(b, n - 1 - j);          // rows below the pivot in the band
    if (threadIdx.x == 0) {
      const double d = B[(long)j * ld];
      // ProfileSPDLinDirectSolver.cpp:134-138 (first pivot), :189-199
      const bool fail = (j == 0) ? !(d > 0.0) : (d == 0.0 || fabs(d) <= S.min_diag_tol);
      if (fail && !bad) {
        bad = 1;
        S.flags[1] = e0 + j;
        S.flags[0] = 3;
      }
      sinv = 1.0 / d;
      S.invD[e0 + j] = sinv;
    }
    for (int t = threadIdx.x; t < m; t += blockDim.x) col[t] = B[(long)(j + 1 + t) * ld + (1 + t)];
    __syncthreads();
    const double inv = sinv;
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
      const double l = col[t] * inv;
      lcol[t] = l;
      B[(long)(j + 1 + t) * ld + (1 + t)] = l;
    }
    __syncthreads();
    // trailing triangle: rows i = j+1+ti, columns k = j+1+tk, tk <= ti < m
    const int tri = m * (m + 1) / 2;
    for (int q = threadIdx.x; q < tri; q += blockDim.x) {
      int ti = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
      while (ti * (ti + 1) / 2 > q) ti--;
      while ((ti + 1) * (ti + 2) / 2 <= q) ti++;
      const int tk = q - ti * (ti + 1) / 2;
      double *a = B + (long)(j + 1 + ti) * ld + (ti - tk);
      *a = fma(-lcol[ti], col[tk], *a);
    }
    __syncthreads();
    if (bad) return;
  }
}

// one warp per part: forward (unit lower), diagonal, backward (unit upper)
__global__ void k_band_solve(BandSystem S, int nrhs, double *x, int ldx) {
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= S.ncomp) return;
  const int e0 = S.cstart[c], n = S.cstart[c + 1] - e0, b = S.bw[c], ld = b + 1;
  const double *B = S.band + S.boff[c];
  for (int q = 0; q < nrhs; q++) {
    double *xq = x + (long)q * ldx + e0;
    for (int i = 0; i < n; i++) {
      const int kmax = min(b, i);
      double s = 0.0;
      for (int k = 1 + lane; k <= kmax; k += 32) s += B[(long)i * ld + k] * xq[i - k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) xq[i] -= s;
      __syncwarp();
    }
    for (int i = lane; i < n; i += 32) xq[i] *= S.invD[e0 + i];
    __syncwarp();
    for (int i = n - 1; i >= 0; i--) {
      const int kmax = min(b, n - 1 - i);
      double s = 0.0;
      for (int k = 1 + lane; k <= kmax; k += 32) s += B[(long)(i + k) * ld + k] * xq[i + k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) xq[i] -= s;
      __syncwarp();
    }
  }
}

}  // namespace

int band_plan(int neq, const int *rowptr, const int *colidx, const std::vector<int> &cstart,
              std::vector<int> &bw, std::vector<long> &boff) {
  const int ncomp = (int)cstart.size() - 1;
  bw.assign(ncomp, 0);
  boff.assign(ncomp + 1, 0);
  for (int c = 0; c < ncomp; c++) {
    int w = 0;
    for (int i = cstart[c]; i < cstart[c + 1]; i++) {
      const int j = colidx[rowptr[i]];
      if (j < cstart[c]) return XG_EINVAL;        // coupled to another part
      w = std::max(w, i - j);
    }
    if (w > kBandMaxWidth) return XG_EINVAL;
    bw[c] = w;
    boff[c + 1] = boff[c] + (long)(cstart[c + 1] - cstart[c]) * (w + 1);
  }
  (void)neq;
  return 0;
}

int band_factor(const BandSystem &S, cudaStream_t s, int *bad_eq) {
  if (S.ncomp == 0) return 0;
  if (cudaMemsetAsync(S.flags, 0, 4 * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  k_band_factor<<<S.ncomp, kBandThreads, 0, s>>>(S);
  if (cudaGetLastError() != cudaSuccess) return XG_ECUDA;
  int hflags[4];
  if (cudaMemcpyAsync(hflags, S.flags, sizeof hflags, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return XG_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return XG_ECUDA;
  if (bad_eq) *bad_eq = hflags[0] == 3 ? hflags[1] : -1;
  return hflags[0] != 0 ? XG_ESOLVE : 0;
}

int band_solve(const BandSystem &S, int nrhs, double *x, int ldx, cudaStream_t s) {
  if (S.ncomp == 0) return 0;
  const int warps = 4;
  k_band_solve<<<(S.ncomp + warps - 1) / warps, 32 * warps, 0, s>>>(S, nrhs, x, ldx);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

}  // namespace xg
