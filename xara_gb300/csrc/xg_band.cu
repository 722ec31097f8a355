// xg_band.cu -- `system ProfileSPD` for a model made of many small
// disconnected parts (a batch of frames): every part's LDL' in its own band,
// one block per part, all parts in one launch.  The reference runs each such
// model alone with ProfileSPDLinDirectSolver (system_of_eqn/linearSOE/
// profileSPD/ProfileSPDLinDirectSolver.cpp:100-256); its pivot checks are
// applied per part (the part's first pivot must be positive, later ones
// non-zero and above minDiagTol in magnitude).
//
// Storage: part c, local row i holds the entries (i, i-k), k = 0..b_c, at
// band[boff[c] + i*(b_c+1) + k] (b_c: the part's envelope width).
//
// Factor (k_band_factor_win): right-looking.  The rows column j touches,
// j..j+b, live in a ring of shared-memory rows; the rows beyond them are
// fetched kBandAhead columns early with cp.async, and a finished row goes
// back to the band.  Column j takes two barriers: the threads below the
// pivot scale the column (l = a / d) and apply it to the right-hand sides,
// then the trailing triangle takes one FMA per entry, and the threads that
// finish column j+1's entries hand them (and the next pivot's reciprocal) to
// the next column through a second buffer.  The forward substitution and
// the diagonal scaling of up to four right-hand sides run inside the
// factorisation; the backward substitution (k_band_back) is one warp per
// part walking the band's rows upwards (x_i final, then the rows above take
// one FMA each from row i of L), rows prefetched the same way.
#include <cuda_runtime.h>

#include <algorithm>

#include "xg_internal.h"
#include "xg_rcp.h"

namespace xg {

namespace {

constexpr int kBandWorkers = 96;        // warps 1-3
constexpr int kBandThreads = kBandWorkers + 32;
constexpr int kBandMaxWidth = 255;      // widest envelope band_plan accepts
constexpr int kBandAhead = 8;           // rows fetched ahead of use
constexpr int kBandMaxRhs = 4;
constexpr int kBackWarps = 4;

// reciprocal on the pivot chain (xg_rcp.h); the stored reciprocals are the
// correctly rounded ones
__device__ __forceinline__ double chain_rcp(double d) { return chain_reciprocal(d); }

__device__ __forceinline__ void cp_async8(double *dst, const double *src) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// the part's band from its CSR rows (lower triangle)
__device__ void band_fill(const BandSystem &S, int e0, int n, int ld, double *B) {
  for (long k = threadIdx.x; k < (long)n * ld; k += blockDim.x) B[k] = 0.0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int row = e0 + i;
    for (int q = S.rowptr[row]; q < S.rowptr[row + 1]; q++) {
      const int j = S.colidx[q] - e0;
      if (j <= i) B[(long)i * ld + (i - j)] = S.vals[q];
    }
  }
  __syncthreads();
}

// ProfileSPDLinDirectSolver.cpp:134-138 (first pivot), :189-199
__device__ __forceinline__ bool pivot_fails(const BandSystem &S, int j, double d) {
  return (j == 0) ? !(d > 0.0) : (d == 0.0 || fabs(d) <= S.min_diag_tol);
}

// Shared memory (doubles): W[R*ldm] ring rows, Y[R*kBandMaxRhs] ring of the
// right-hand sides, col[2*ldm], lcol[ldm].  ldm = bmax + 1, R = the power of
// two at or above ldm + kBandAhead (ring slot = row & (R-1)).
// Warps 1-3 scale the columns and update the trailing triangles; warp 0
// carries the pivot chain (the next pivot's last update right after the
// column is scaled, its reciprocal while the others update), the
// right-hand sides (forward substitution) and their ring.  Every worker
// owns up to K entries (ti, tk) of the width-b trailing triangle, fixed for
// the whole factorisation (entry q = worker + 96 k, row-major); a column
// loads all its entries' operands before their FMAs.
template <int K>
__global__ void __launch_bounds__(kBandThreads) k_band_factor_win(BandSystem S, int nrhs,
                                                                   double *x, int ldx, int R) {
  extern __shared__ double sm[];
  const int c = blockIdx.x;
  if (c >= S.ncomp) return;
  const int e0 = S.cstart[c], n = S.cstart[c + 1] - e0, b = S.bw[c], ld = b + 1;
  const int ldm = S.bmax + 1, Rm = R - 1;
  double *W = sm;
  double *Y = W + (size_t)R * ldm;
  double *colb = Y + (size_t)R * kBandMaxRhs;
  double *lcol = colb + 2 * ldm;
  __shared__ double sinv[2], pivv;
  __shared__ int bad;
  const int tid = threadIdx.x;
  const bool worker = tid >= 32;
  const int wid = tid - 32;                     // worker index
  double *B = S.band + S.boff[c];
  band_fill(S, e0, n, ld, B);
  // this worker's entries: q = wid + 96 k of the row-major lower triangle
  // of width b, without entry 0 (the pivot, warp 0's), as (ti << 16) | tk
  int ent[K];
  const int trib = b * (b + 1) / 2;
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int q = wid + kBandWorkers * k;
    ent[k] = -1;
    if (worker && q > 0 && q < trib) {
      int ti = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
      while (ti * (ti + 1) / 2 > q) ti--;
      while ((ti + 1) * (ti + 2) / 2 <= q) ti++;
      ent[k] = (ti << 16) | (q - ti * (ti + 1) / 2);
    }
  }
  // the first R rows and their right-hand sides directly
  const int n0 = min(n, R);
  for (int k = tid; k < n0 * ld; k += blockDim.x) W[(k / ld) * ldm + k % ld] = B[k];
  for (int k = tid; k < n0 * nrhs; k += blockDim.x)
    Y[(k / nrhs) * kBandMaxRhs + k % nrhs] = x[(long)(k % nrhs) * ldx + e0 + k / nrhs];
  if (tid == 0) bad = 0;
  __syncthreads();
  // column 0's entries and pivot
  for (int t = tid; t < min(b, n - 1); t += blockDim.x) colb[t] = W[(1 + t) * ldm + 1 + t];
  if (tid == 0 && n > 0) {
    const double d = W[0];
    if (pivot_fails(S, 0, d)) {
      bad = 1;
      S.flags[1] = e0;
      S.flags[0] = 3;
    }
    sinv[0] = chain_rcp(d);
  }
  __syncthreads();
  for (int j = 0; j < n; j++) {
    const int m = min(b, n - 1 - j);
    const int sj = j & Rm, s1 = (j + 1) & Rm;
    const double *cl = colb + (j & 1) * ldm;
    double *cn = colb + ((j + 1) & 1) * ldm;
    double *Wj = W + sj * ldm;
    const double inv = sinv[j & 1];
    if (worker) {
      // scale the column
      for (int t = wid; t < m; t += kBandWorkers) {
        const double l = cl[t] * inv;
        lcol[t] = l;
        W[((s1 + t) & Rm) * ldm + 1 + t] = l;
      }
    } else if (tid == 0 && m > 0) {
      // the next pivot's last update (the arithmetic of the trailing
      // triangle's entry (0, 0), which the workers leave out)
      const double l0 = cl[0] * inv;
      double *a = W + s1 * ldm;
      pivv = fma(-l0, cl[0], *a);
      *a = pivv;
    }
    // row j+b+1, fetched kBandAhead columns ago, is complete for everyone
    // after this barrier
    cp_async_wait<kBandAhead - 1>();
    __syncthreads();
    if (worker) {
      // trailing triangle (rows and columns j+1..j+m), one FMA per entry
      double *ap[K];
      double lv[K], cv[K], av[K];
#pragma unroll
      for (int k = 0; k < K; k++) {
        const int e = ent[k];
        const int ti = e >> 16, tk = e & 0xffff;
        if (e >= 0 && ti < m) {
          ap[k] = W + ((s1 + ti) & Rm) * ldm + (ti - tk);
          lv[k] = lcol[ti];
          cv[k] = cl[tk];
          av[k] = *ap[k];
        }
      }
#pragma unroll
      for (int k = 0; k < K; k++) {
        const int e = ent[k];
        const int ti = e >> 16, tk = e & 0xffff;
        if (e >= 0 && ti < m) {
          const double v = fma(-lv[k], cv[k], av[k]);
          *ap[k] = v;
          if (tk == 0) cn[ti - 1] = v;
        }
      }
      // row j is final: back to the band; its ring row then takes band row
      // j+R (each entry is read and refilled by the same thread)
      const bool refill = j + R < n;
      for (int t = wid; t < ld; t += kBandWorkers) {
        B[(long)j * ld + t] = Wj[t];
        if (refill) cp_async8(Wj + t, B + (long)(j + R) * ld + t);
      }
    } else {
      if (tid == 0 && m > 0) {
        const double v = pivv;
        if (pivot_fails(S, j + 1, v) && atomicCAS(&bad, 0, 1) == 0) {
          S.flags[1] = e0 + j + 1;
          S.flags[0] = 3;
        }
        sinv[(j + 1) & 1] = chain_rcp(v);
      }
      // forward substitution: the right-hand sides below row j take the
      // column (its entries in lcol, complete after the barrier above)
      const double *yj = Y + sj * kBandMaxRhs;
      for (int t = tid; t < m; t += 32) {
        double *yr = Y + ((s1 + t) & Rm) * kBandMaxRhs;
        const double l = lcol[t];
        for (int r = 0; r < nrhs; r++) yr[r] = fma(-l, yj[r], yr[r]);
      }
      __syncwarp();
      if (tid == 0) {
        // row j's forward-substituted right-hand sides (scaled by the
        // reciprocal pivots after the loop); the ring row takes row j+R
        double *yw = Y + sj * kBandMaxRhs;
        for (int r = 0; r < nrhs; r++) {
          x[(long)r * ldx + e0 + j] = yw[r];
          if (j + R < n) cp_async8(yw + r, x + (long)r * ldx + e0 + j + R);
        }
      }
      if (b > 0 && j + b + 1 < n && tid == 1)   // column j+1's entry in row j+b+1
        cn[b - 1] = W[((s1 + b) & Rm) * ldm + b];
    }
    cp_async_commit();
    __syncthreads();
    if (bad) break;
  }
  cp_async_wait<0>();
  __syncthreads();
  // the correctly rounded reciprocal pivots, and the diagonal scaling
  if (!bad) {
    for (int i = tid; i < n; i += blockDim.x) {
      const double inv = __drcp_rn(B[(long)i * ld]);
      S.invD[e0 + i] = inv;
      for (int r = 0; r < nrhs; r++) x[(long)r * ldx + e0 + i] *= inv;
    }
  }
}

// Backward substitution, one warp per part: x_i = z_i once every row below
// has been applied, then z_{i-1-t} -= L(i, i-1-t) x_i for t < b (row i of
// the band, contiguous).  The band rows come through a ring of kBandAhead
// rows fetched ahead (one row per sweep step, over all right-hand sides in
// turn); z sits in shared memory when the part has at most zcap equations.
__global__ void __launch_bounds__(32 * kBackWarps) k_band_back(BandSystem S, int nrhs, double *x,
                                                               int ldx, int zcap) {
  extern __shared__ double sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * kBackWarps + w;
  const int ldm = S.bmax + 1;
  double *rows = sm + (size_t)w * (kBandAhead * ldm + zcap);
  double *zs = rows + kBandAhead * ldm;
  if (c >= S.ncomp) return;
  const int e0 = S.cstart[c], n = S.cstart[c + 1] - e0, b = S.bw[c], ld = b + 1;
  const double *B = S.band + S.boff[c];
  const long T = (long)nrhs * n;           // sweep steps: rhs k / n, row n-1 - k % n
  for (long k = 0; k < kBandAhead; k++) {
    if (k < T) {
      const long i = n - 1 - k % n;
      for (int t = lane; t < ld; t += 32) cp_async8(rows + (k % kBandAhead) * ldm + t, B + i * ld + t);
    }
    cp_async_commit();
  }
  const bool in_smem = n <= zcap;
  for (int r = 0; r < nrhs; r++) {
    double *xr = x + (long)r * ldx + e0;
    double *z = in_smem ? zs : xr;
    if (in_smem) {
      for (int i = lane; i < n; i += 32) zs[i] = xr[i];
      __syncwarp();
    }
    for (int i = n - 1; i >= 0; i--) {
      const long k = (long)r * n + (n - 1 - i);
      cp_async_wait<kBandAhead - 1>();
      __syncwarp();
      const double *Li = rows + (k % kBandAhead) * ldm;
      const double xi = z[i];
      const int m = min(b, i);
      for (int t = lane; t < m; t += 32) z[i - 1 - t] = fma(-Li[1 + t], xi, z[i - 1 - t]);
      __syncwarp();
      // this ring row takes the row of sweep step k + kBandAhead
      const long kn = k + kBandAhead;
      if (kn < T) {
        const long in = n - 1 - kn % n;
        for (int t = lane; t < ld; t += 32) cp_async8(rows + (k % kBandAhead) * ldm + t, B + in * ld + t);
      }
      cp_async_commit();
    }
    if (in_smem) {
      __syncwarp();
      for (int i = lane; i < n; i += 32) xr[i] = zs[i];
      __syncwarp();
    }
  }
  cp_async_wait<0>();
}

// Forward substitution and diagonal scaling on factors already in the band
// (solves after the factorisation): one warp per part, y_i = b_i - L(i,:) y
// reduced over the lanes.
__global__ void k_band_forward(BandSystem S, int nrhs, double *x, int ldx) {
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
  }
}

int ring_rows(int bmax) {
  int R = 1;
  while (R < bmax + 1 + kBandAhead) R <<= 1;
  return R;
}

size_t factor_smem(int bmax) {
  const size_t ldm = bmax + 1, R = ring_rows(bmax);
  return (R * ldm + R * kBandMaxRhs + 3 * ldm) * sizeof(double);
}

// trailing entries per worker for the widest band, rounded up to a kernel
// instance
int entries_per_worker(int bmax) {
  const int tri = bmax * (bmax + 1) / 2;
  const int k = (tri + kBandWorkers - 1) / kBandWorkers;
  for (int c : {3, 6, 9, 12, 16, 20, 24, 32})
    if (k <= c) return c;
  return -1;
}

template <int K>
void launch_factor(const BandSystem &S, int nrhs, double *x, int ldx, size_t smem, int R,
                   cudaStream_t s, int *err) {
  if (cudaFuncSetAttribute(k_band_factor_win<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess) {
    *err = XG_ECUDA;
    return;
  }
  k_band_factor_win<K><<<S.ncomp, kBandThreads, smem, s>>>(S, nrhs, x, ldx, R);
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
  // the factorisation's ring of rows must fit in one block's shared memory,
  // and each worker's entries in its registers
  const int bmax = ncomp ? *std::max_element(bw.begin(), bw.end()) : 0;
  if (factor_smem(bmax) > 200 * 1024 || entries_per_worker(bmax) < 0) return XG_EINVAL;
  return 0;
}

int band_factor_async(const BandSystem &S, cudaStream_t s, int nrhs, double *x, int ldx) {
  if (S.ncomp == 0) return 0;
  if (nrhs < 0 || nrhs > kBandMaxRhs) return XG_EINVAL;
  if (cudaMemsetAsync(S.flags, 0, 4 * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  const size_t smem = factor_smem(S.bmax);
  const int R = ring_rows(S.bmax);
  int err = 0;
  switch (entries_per_worker(S.bmax)) {
    case 3: launch_factor<3>(S, nrhs, x, ldx, smem, R, s, &err); break;
    case 6: launch_factor<6>(S, nrhs, x, ldx, smem, R, s, &err); break;
    case 9: launch_factor<9>(S, nrhs, x, ldx, smem, R, s, &err); break;
    case 12: launch_factor<12>(S, nrhs, x, ldx, smem, R, s, &err); break;
    case 16: launch_factor<16>(S, nrhs, x, ldx, smem, R, s, &err); break;
    case 20: launch_factor<20>(S, nrhs, x, ldx, smem, R, s, &err); break;
    case 24: launch_factor<24>(S, nrhs, x, ldx, smem, R, s, &err); break;
    case 32: launch_factor<32>(S, nrhs, x, ldx, smem, R, s, &err); break;
    default: return XG_EINVAL;
  }
  if (err || cudaGetLastError() != cudaSuccess) return XG_ECUDA;
  return 0;
}

int band_factor(const BandSystem &S, cudaStream_t s, int *bad_eq, int nrhs, double *x, int ldx) {
  if (S.ncomp == 0) return 0;
  const int r = band_factor_async(S, s, nrhs, x, ldx);
  if (r) return r;
  int hflags[4];
  if (cudaMemcpyAsync(hflags, S.flags, sizeof hflags, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return XG_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return XG_ECUDA;
  if (bad_eq) *bad_eq = hflags[0] == 3 ? hflags[1] : -1;
  return hflags[0] != 0 ? XG_ESOLVE : 0;
}

int band_solve(const BandSystem &S, int nrhs, double *x, int ldx, cudaStream_t s, bool forward) {
  if (S.ncomp == 0) return 0;
  if (forward) {
    const int warps = 4;
    k_band_forward<<<(S.ncomp + warps - 1) / warps, 32 * warps, 0, s>>>(S, nrhs, x, ldx);
  }
  // z in shared memory for parts of up to 2,048 equations
  const int zcap = S.nmax <= 2048 ? S.nmax : 0;
  const size_t smem = (size_t)kBackWarps * (kBandAhead * (S.bmax + 1) + zcap) * sizeof(double);
  if (cudaFuncSetAttribute(k_band_back, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return XG_ECUDA;
  k_band_back<<<(S.ncomp + kBackWarps - 1) / kBackWarps, 32 * kBackWarps, smem, s>>>(S, nrhs, x,
                                                                                      ldx, zcap);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

}  // namespace xg
