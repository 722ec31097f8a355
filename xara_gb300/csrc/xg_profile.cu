// xg_profile.cu -- the `system ProfileSPD` path on the device: LDL' of the
// symmetric tangent without pivoting, then forward / diagonal / backward
// substitution, FP64 (ProfileSPDLinDirectSolver::solve, system_of_eqn/
// linearSOE/profileSPD/ProfileSPDLinDirectSolver.cpp:100-256).
//
// Storage: the lower triangle of the envelope (row i holds columns
// first(i)..i, first(i) = the first column of row i in the CSR pattern) in
// dense 32 x 32 tiles.  Tile row I keeps the tiles of columns J = I-W..I
// (W = the widest envelope in tiles), so tile (I, J) lives at offset
// (I*(W+1) + I-J) * 1024, row-major inside the tile; tiles left of the
// envelope (J < ftile[I]) stay zero and are skipped.  Right-looking LDL':
// for every tile column J,
//   A  the diagonal tile is factored by one block (pivots d, unit lower L);
//   B  every tile below it becomes W_IJ = A_IJ L_JJ^-T (kept in a scratch
//      slot) and L_IJ = W_IJ D^-1 (stored in place);
//   C  every trailing tile pair loses W_IJ L_KJ' (one 32^3 product each).
// One cooperative launch runs all columns; phases meet at a grid barrier
// whose wait is bounded by the global timer.  The block that updates the
// next diagonal tile in phase C factors it right away, so a column costs
// two barriers.  Pivot checks follow the reference: the first pivot must be
// positive, later ones only non-zero and above minDiagTol in magnitude.
//
// The substitutions stream the tiles through one block: every step reads
// one tile row (forward) or tile column (backward), accumulates it against
// the known part of the solution and solves the diagonal tile with warp
// shuffles.  Up to four right-hand sides share the tile loads.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "xg_internal.h"

namespace xg {

namespace {

constexpr int kT = 32;                 // tile edge
constexpr int kTT = kT * kT;
constexpr int kFactorThreads = 256;
constexpr int kSolveThreads = 512;
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Sense-reversing grid barrier: bar[0] arrivals, bar[1] generation.  Returns
// false on timeout (flags[0] = 2) or when a block raised flags[0].
__device__ bool prof_barrier(unsigned int *bar, volatile int *flags) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned int *vgen = bar + 1;
    const unsigned int gen = *vgen;
    __threadfence();
    const unsigned int arrived = atomicAdd(bar, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const unsigned long long t0 = global_ns();
      while (*vgen == gen) {
        if (flags[0] != 0) { ok = 0; break; }
        if (global_ns() - t0 > kBarrierTimeoutNs) { flags[0] = 2; ok = 0; break; }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (flags[0] != 0) ok = 0;
  }
  __syncthreads();
  return ok != 0;
}

__device__ __forceinline__ double *tile_at(const ProfileSystem &S, int I, int o) {
  return S.L + ((size_t)I * (S.W + 1) + o) * kTT;
}

// Envelope of the CSR values into the tiles (the tiles were zeroed); rows
// past n get a unit pivot so the padded system solves to zero there.
__global__ void k_prof_fill(ProfileSystem S) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int npad = S.nt * kT;
  if (warp >= npad) return;
  const int i = warp, I = i / kT, r = i % kT;
  if (i >= S.n) {
    if (lane == 0) tile_at(S, I, 0)[r * kT + r] = 1.0;
    return;
  }
  for (int k = S.rowptr[i] + lane; k < S.rowptr[i + 1]; k += 32) {
    const int j = S.colidx[k];
    if (j > i) continue;
    const int J = j / kT;
    tile_at(S, I, I - J)[r * kT + (j % kT)] = S.vals[k];
  }
}

// LDL' of diagonal tile J in shared memory (block-wide); returns false and
// records the equation when a pivot fails the reference's checks.
__device__ bool factor_diag(const ProfileSystem &S, int J, double (*sA)[kT + 1], double *col,
                            volatile int *flags) {
  double *g = tile_at(S, J, 0);
  for (int k = threadIdx.x; k < kTT; k += blockDim.x) sA[k / kT][k % kT] = g[k];
  __syncthreads();
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  for (int c = 0; c < kT; c++) {
    const double d = sA[c][c];
    const int eq = J * kT + c;
    if (threadIdx.x == 0 && eq < S.n) {
      // ProfileSPDLinDirectSolver.cpp:134-138 (first pivot), :189-199
      const bool fail = (eq == 0) ? !(d > 0.0) : (d == 0.0 || fabs(d) <= S.min_diag_tol);
      if (fail && !bad) {
        bad = 1;
        flags[1] = eq;
        flags[0] = 3;
      }
    }
    const double inv = 1.0 / d;
    for (int r = c + 1 + threadIdx.x; r < kT; r += blockDim.x) col[r] = sA[r][c];
    __syncthreads();
    // trailing update of the tile: a_rs -= (a_rc / d) a_sc for c < s <= r
    const int m = kT - 1 - c;
    for (int k = threadIdx.x; k < m * m; k += blockDim.x) {
      const int r = c + 1 + k / m, s = c + 1 + k % m;
      if (s <= r) sA[r][s] -= (col[r] * inv) * col[s];
    }
    for (int r = c + 1 + threadIdx.x; r < kT; r += blockDim.x) sA[r][c] = col[r] * inv;
    if (threadIdx.x == 0) S.invD[eq] = inv;
    __syncthreads();
  }
  for (int k = threadIdx.x; k < kTT; k += blockDim.x) g[k] = sA[k / kT][k % kT];
  __syncthreads();
  return bad == 0;
}

// Phase B on tile (I = J+o, J): W = A L_JJ^-T by rows, L = W D^-1.  Eight
// threads share a row: w_c = a_c - sum_{k<c} w_k l_ck, the sum split by k
// mod 8 and reduced with shuffles inside the eight lanes.
__device__ void panel_solve(const ProfileSystem &S, int J, int o, double (*sA)[kT + 1],
                            double (*sB)[kT + 1]) {
  const double *Ljj = tile_at(S, J, 0);
  double *g = tile_at(S, J + o, o);
  for (int k = threadIdx.x; k < kTT; k += blockDim.x) {
    sB[k / kT][k % kT] = Ljj[k];
    sA[k / kT][k % kT] = g[k];
  }
  __syncthreads();
  {
    const int r = threadIdx.x >> 3, q = threadIdx.x & 7;   // blockDim.x == 256
    for (int c = 1; c < kT; c++) {
      double part = 0.0;
      for (int k = q; k < c; k += 8) part += sA[r][k] * sB[c][k];
      part += __shfl_xor_sync(0xffffffffu, part, 4);
      part += __shfl_xor_sync(0xffffffffu, part, 2);
      part += __shfl_xor_sync(0xffffffffu, part, 1);
      if (q == 0) sA[r][c] -= part;
      __syncwarp();
    }
  }
  __syncthreads();
  double *wt = S.Wt + (size_t)(o - 1) * kTT;
  const double *invD = S.invD + (size_t)J * kT;
  for (int k = threadIdx.x; k < kTT; k += blockDim.x) {
    const double w = sA[k / kT][k % kT];
    wt[k] = w;
    g[k] = w * invD[k % kT];
  }
  __syncthreads();
}

// Phase C on pair (I = J+a, K = J+b), b <= a: A_IK -= W_IJ L_KJ'.
__device__ void pair_update(const ProfileSystem &S, int J, int a, int b, double (*sA)[kT + 1],
                            double (*sB)[kT + 1]) {
  const double *wt = S.Wt + (size_t)(a - 1) * kTT;
  const double *lk = tile_at(S, J + b, b);
  for (int k = threadIdx.x; k < kTT; k += blockDim.x) {
    sA[k / kT][k % kT] = wt[k];
    sB[k / kT][k % kT] = lk[k];
  }
  __syncthreads();
  double *out = tile_at(S, J + a, a - b);
  for (int k = threadIdx.x; k < kTT; k += blockDim.x) {
    const int r = k / kT, s = k % kT;
    double acc = 0.0;
#pragma unroll 8
    for (int c = 0; c < kT; c++) acc += sA[r][c] * sB[s][c];
    out[k] -= acc;
  }
  __syncthreads();
}

__device__ __forceinline__ void decode_pair(int p, int &a, int &b) {
  // p = a(a-1)/2 + (b-1), 1 <= b <= a
  int aa = (int)((1.0 + sqrt(1.0 + 8.0 * (double)p)) * 0.5);
  while (aa * (aa - 1) / 2 > p) aa--;
  while ((aa + 1) * aa / 2 <= p) aa++;
  a = aa;
  b = p - aa * (aa - 1) / 2 + 1;
}

__global__ void __launch_bounds__(kFactorThreads) k_prof_factor(ProfileSystem S) {
  __shared__ double sA[kT][kT + 1], sB[kT][kT + 1];
  __shared__ double col[kT];
  volatile int *flags = S.flags;
  const int nb = gridDim.x;
  if (blockIdx.x == 0) factor_diag(S, 0, sA, col, flags);
  if (!prof_barrier(S.barrier, flags)) return;
  const int npairs = S.W * (S.W + 1) / 2;
  for (int J = 0; J < S.nt; J++) {
    const int omax = min(S.W, S.nt - 1 - J);
    for (int o = 1 + blockIdx.x; o <= omax; o += nb)
      if (S.ftile[J + o] <= J) panel_solve(S, J, o, sA, sB);
    if (!prof_barrier(S.barrier, flags)) return;
    for (int p = blockIdx.x; p < npairs; p += nb) {
      int a, b;
      decode_pair(p, a, b);
      if (a > omax) continue;
      if (S.ftile[J + a] > J || S.ftile[J + b] > J) continue;
      pair_update(S, J, a, b, sA, sB);
    }
    // pair 0 is (J+1, J+1): its block factors the next diagonal tile now
    if (blockIdx.x == 0 && J + 1 < S.nt) factor_diag(S, J + 1, sA, col, flags);
    if (!prof_barrier(S.barrier, flags)) return;
  }
}

// Forward (L y = b), diagonal (z = D^-1 y) and backward (L' x = z)
// substitution in one block; x[r * ldx + i] for right-hand side r.  Every
// thread issues its loads of a whole tile row (column) before it uses them,
// so a step costs about one memory latency plus the diagonal solve.
__global__ void __launch_bounds__(kSolveThreads) k_prof_solve(ProfileSystem S, int nrhs,
                                                               double *x, int ldx) {
  __shared__ double red[kSolveThreads / 32][4][kT];
  __shared__ double sL[kT][kT + 1];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  constexpr int nw = kSolveThreads / 32;
  const int nt = S.nt, W = S.W;
  // ---- forward: t = b_J - sum_o L(J, J-o) y_{J-o}; then unit-lower solve
  {
    const int r = tid >> 4, g = tid & 15;      // row of the tile, column group
    for (int J = 0; J < nt; J++) {
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      const int ohi = min(W, J - S.ftile[J]);
#pragma unroll 4
      for (int o = 1; o <= ohi; o++) {
        const double *Lt = tile_at(S, J, o) + r * kT;
        const double l0 = Lt[g], l1 = Lt[g + 16];
        const double *xc = x + (J - o) * kT;
        for (int q = 0; q < nrhs; q++)
          acc[q] += l0 * xc[(size_t)q * ldx + g] + l1 * xc[(size_t)q * ldx + g + 16];
      }
      for (int q = 0; q < nrhs; q++) {
        double v = acc[q];
        v += __shfl_xor_sync(0xffffffffu, v, 8);
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        v += __shfl_xor_sync(0xffffffffu, v, 2);
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        if (g == 0) red[0][q][r] = v;
      }
      {
        const double *L = tile_at(S, J, 0);
        for (int k = tid; k < kTT; k += kSolveThreads) sL[k / kT][k % kT] = L[k];
      }
      __syncthreads();
      if (w < nrhs) {
        const int q = w;
        double v = x[(size_t)q * ldx + J * kT + lane] - red[0][q][lane];
        for (int c = 0; c < kT - 1; c++) {
          const double yc = __shfl_sync(0xffffffffu, v, c);
          if (lane > c) v -= sL[lane][c] * yc;
        }
        x[(size_t)q * ldx + J * kT + lane] = v;
      }
      __syncthreads();
    }
  }
  // ---- diagonal
  for (int q = 0; q < nrhs; q++)
    for (int i = tid; i < nt * kT; i += kSolveThreads) x[(size_t)q * ldx + i] *= S.invD[i];
  __syncthreads();
  // ---- backward: t = z_J - sum_o L(J+o, J)' x_{J+o}; then unit-upper solve
  {
    const int c = lane, g = w;                 // column of the tile, row group
    for (int J = nt - 1; J >= 0; J--) {
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      const int ohi = min(W, nt - 1 - J);
#pragma unroll 4
      for (int o = 1; o <= ohi; o++) {
        if (S.ftile[J + o] > J) continue;
        const double *Lt = tile_at(S, J + o, o);
        const double l0 = Lt[g * kT + c], l1 = Lt[(g + nw) * kT + c];
        const double *xr = x + (J + o) * kT;
        for (int q = 0; q < nrhs; q++)
          acc[q] += l0 * xr[(size_t)q * ldx + g] + l1 * xr[(size_t)q * ldx + g + nw];
      }
      for (int q = 0; q < nrhs; q++) red[g][q][c] = acc[q];
      {
        const double *L = tile_at(S, J, 0);
        for (int k = tid; k < kTT; k += kSolveThreads) sL[k / kT][k % kT] = L[k];
      }
      __syncthreads();
      if (w < nrhs) {
        const int q = w;
        double s = 0.0;
        for (int h = 0; h < nw; h++) s += red[h][q][lane];
        double v = x[(size_t)q * ldx + J * kT + lane] - s;
        // x_c = v_c - sum_{k > c} L[k][c] x_k, from the last row up
        for (int cc = kT - 1; cc > 0; cc--) {
          const double xc = __shfl_sync(0xffffffffu, v, cc);
          if (lane < cc) v -= sL[cc][lane] * xc;
        }
        x[(size_t)q * ldx + J * kT + lane] = v;
      }
      __syncthreads();
    }
  }
}

int g_factor_blocks = -1;

}  // namespace

int profile_plan(int n, const int *rowptr, const int *colidx, std::vector<int> &ftile, int &nt,
                 int &W) {
  nt = (n + kT - 1) / kT;
  ftile.assign(nt > 0 ? nt : 1, 0);
  W = 0;
  for (int I = 0; I < nt; I++) {
    int f = I;
    for (int i = I * kT; i < n && i < (I + 1) * kT; i++) {
      const int j = colidx[rowptr[i]];   // first column of row i (sorted)
      if (j / kT < f) f = j / kT;
    }
    ftile[I] = f;
    if (I - f > W) W = I - f;
  }
  return 0;
}

size_t profile_tile_doubles(int nt, int W) { return (size_t)nt * (W + 1) * kTT; }
int profile_tile_edge() { return kT; }

int profile_factor(const ProfileSystem &S, cudaStream_t s, int *bad_eq) {
  if (S.n == 0) return 0;
  if (cudaMemsetAsync(S.L, 0, profile_tile_doubles(S.nt, S.W) * sizeof(double), s) != cudaSuccess)
    return XG_ECUDA;
  const int fill_threads = 256;
  const long warps = (long)S.nt * kT;
  k_prof_fill<<<(int)((warps * 32 + fill_threads - 1) / fill_threads), fill_threads, 0, s>>>(S);
  if (cudaGetLastError() != cudaSuccess) return XG_ECUDA;
  if (g_factor_blocks < 0) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_prof_factor, kFactorThreads, 0);
    if (per < 1) per = 1;
    g_factor_blocks = sms * per;
  }
  // enough blocks for the widest phase (W panel tiles, W(W+1)/2 pairs)
  long want = (long)S.W * (S.W + 1) / 2;
  if (want < 1) want = 1;
  int nb = (int)(want < g_factor_blocks ? want : g_factor_blocks);
  if (cudaMemsetAsync(S.barrier, 0, 2 * sizeof(unsigned int), s) != cudaSuccess) return XG_ECUDA;
  if (cudaMemsetAsync(S.flags, 0, 4 * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  ProfileSystem Sv = S;
  void *args[] = {(void *)&Sv};
  if (cudaLaunchCooperativeKernel((void *)k_prof_factor, dim3(nb), dim3(kFactorThreads), args, 0,
                                  s) != cudaSuccess)
    return XG_ECUDA;
  int hflags[4];
  if (cudaMemcpyAsync(hflags, S.flags, sizeof hflags, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return XG_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return XG_ECUDA;
  if (bad_eq) *bad_eq = hflags[0] == 3 ? hflags[1] : -1;
  if (hflags[0] == 3) return XG_ESOLVE;   // pivot check failed
  if (hflags[0] != 0) return XG_ESOLVE;   // barrier timeout
  return 0;
}

int profile_solve(const ProfileSystem &S, int nrhs, double *x, int ldx, cudaStream_t s) {
  if (S.n == 0) return 0;
  if (nrhs < 1 || nrhs > 4 || ldx < S.nt * kT) return XG_EINVAL;
  k_prof_solve<<<1, kSolveThreads, 0, s>>>(S, nrhs, x, ldx);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

}  // namespace xg
