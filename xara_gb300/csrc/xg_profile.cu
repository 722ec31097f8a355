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
// The tasks (A: diagonal, B: panel tile in four row parts, C: tile pair of
// one column; for tile (J+1, J) the four panel parts also apply a quarter
// each of the pair (J+1, J+1)'s update, and the chain task of column J
// factors diagonal tile J+1 -- the critical path of the factorisation) run as a dataflow: one persistent launch whose blocks take
// tasks from a list in a fixed order -- for column J: A(J) when no column
// updates it, the C tasks of column J-1 that reach column J+1, the panel
// (J+1, J), the chain task, the other panels B(., J), the C tasks of column
// J that reach column J+1, then the rest of column J-1's trailing update --
// and
// wait (bounded by the global timer) on per-tile counters for the tasks
// each one depends on.  Every dependency sits earlier in the list, so the
// look-ahead is built in: column J+1's diagonal and panels run while the
// rest of column J's trailing update is still going.  C recovers W_IJ as
// L_IJ D_J.  Pivot checks follow the reference: the first pivot must
// be positive, later ones only non-zero and above minDiagTol in magnitude.
//
// The substitutions stream the tiles through one block: every step reads
// one tile row (forward) or tile column (backward), accumulates it against
// the known part of the solution and solves the diagonal tile with warp
// shuffles.  Up to four right-hand sides share the tile loads.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "xg_internal.h"
#include "xg_rcp.h"

namespace xg {

namespace {

constexpr int kT = 32;                 // tile edge
constexpr int kTT = kT * kT;
constexpr int kFactorThreads = 256;
constexpr int kFactorSoloSmem = 120 * 1024;   // more than half an SM's shared memory
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// (row << 5 | column) of the lower triangle of a tile, row by row
struct LowerTable {
  unsigned short rs[kT * (kT + 1) / 2];
  constexpr LowerTable() : rs() {
    int k = 0;
    for (int r = 0; r < kT; r++)
      for (int c = 0; c <= r; c++) rs[k++] = (unsigned short)(r * 32 + c);
  }
};
__device__ const LowerTable kLowerTable{};
#define kLowerRS (kLowerTable.rs)

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
// records the equation when a pivot fails the reference's checks.  Column c:
// the column below the pivot is read and scaled by the reciprocal pivot,
// then every trailing entry takes one FMA; the thread that finishes the
// next pivot takes its reciprocal at once (__drcp_rn: the correctly rounded
// 1/d, the value of the reference's 1.0/aii), so the chain of dependent
// FP64 operations per column stays short.
// 1/d for the elimination (xg_rcp.h); the stored reciprocal pivots are the
// correctly rounded ones.
__device__ __forceinline__ double elim_rcp(double d) { return chain_reciprocal(d); }

__device__ __forceinline__ void named_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void named_arrive(int id, int count) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// LDL' of the diagonal tile in sA (shared memory), as a two-stage pipeline.
// Warp 1 carries the pivot chain: step c applies column c-1 to column c
// (one FMA per row, the factors kept in its registers), takes the pivot's
// reciprocal (FP64 estimate and one cubic Newton step, every lane), scales
// the column (L below the diagonal, the unscaled column in the upper
// triangle for the trailing update).  Warps 0, 2, 3, 4, 6 and 7 apply
// column c to the rest of the trailing triangle (columns c+2 and beyond,
// one FMA per entry, each thread owning up to three fixed entries) while
// the chain goes on with column c+1; warp 5 sits out, so the chain has its
// sub-partition's FP64 pipe to itself.  Hand-offs: named barriers 1-2
// (chain -> trailing, by column parity) and 3-4 (trailing -> chain); the
// chain's step c waits for the trailing update of column c-2 only.  The FMAs
// and their operands are those of the plain right-looking order.
constexpr int kPipeCount = 224;        // the chain warp and six trailing warps

__device__ bool factor_tile(const ProfileSystem &S, int J, double (*sA)[kT + 1],
                            volatile int *flags) {
  double *g = tile_at(S, J, 0);
  __shared__ double sinv[kT];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 1) {
    double lprev = 0.0, uprev = 0.0;
    for (int c = 0; c < kT; c++) {
      if (c >= 2) named_sync(3 + (c & 1), kPipeCount);
      double x = sA[lane][c];
      if (c >= 1) {
        const double ucc = __shfl_sync(0xffffffffu, uprev, c);
        x = fma(-lprev, ucc, x);
      }
      const double d = __shfl_sync(0xffffffffu, x, c);
      const double inv = elim_rcp(d);
      const double l = x * inv;
      if (lane > c) {
        sA[lane][c] = l;
        sA[c][lane] = x;
      } else if (lane == c) {
        sA[c][c] = x;
      }
      lprev = l;
      uprev = x;
      if (c <= kT - 3) named_arrive(1 + (c & 1), kPipeCount);
    }
  } else if (warp != 5) {
    // this thread's entries (r, s), 2 <= s <= r < 32, column-major order
    const int tw = (warp == 0 ? 0 : warp - 1 - (warp > 5)) * 32 + lane;
    int ent[3];
#pragma unroll
    for (int u = 0; u < 3; u++) {
      int e = tw + u * 192;
      ent[u] = -1;
      for (int sc = 2; sc < kT && e >= 0; sc++) {
        if (e < kT - sc) { ent[u] = ((sc + e) << 5) | sc; break; }
        e -= kT - sc;
      }
    }
    for (int c = 0; c < kT - 2; c++) {
      named_sync(1 + (c & 1), kPipeCount);
#pragma unroll
      for (int u = 0; u < 3; u++) {
        const int e = ent[u];
        const int r = e >> 5, sc = e & 31;
        if (e >= 0 && sc >= c + 2) sA[r][sc] = fma(-sA[r][c], sA[c][sc], sA[r][sc]);
      }
      named_arrive(3 + (c & 1), kPipeCount);
    }
  }
  __syncthreads();
  if (tid < kT) sinv[tid] = __drcp_rn(sA[tid][tid]);
  __syncwarp();
  if (tid < kT) {
    const int eq = J * kT + tid;
    const double d = sA[tid][tid];
    S.invD[eq] = sinv[tid];
    S.piv[eq] = d;
    // ProfileSPDLinDirectSolver.cpp:134-138 (first pivot), :189-199; the
    // first failing pivot of the tile is reported
    const bool fail = eq < S.n && ((eq == 0) ? !(d > 0.0)
                                             : (d == 0.0 || fabs(d) <= S.min_diag_tol));
    const unsigned bad = __ballot_sync(0xffffffffu, fail);
    if (bad && tid == 0) {
      flags[1] = J * kT + __ffs(bad) - 1;
      __threadfence();
      flags[0] = 3;
    }
  }
  // the lower triangle (the upper one held the unscaled columns)
  for (int k = tid; k < kTT; k += blockDim.x) {
    const int r = k >> 5, c = k & 31;
    g[k] = c > r ? 0.0 : sA[r][c];
  }
  __syncthreads();
  return flags[0] != 3;
}

__device__ bool factor_diag(const ProfileSystem &S, int J, double (*sA)[kT + 1],
                            volatile int *flags) {
  const double *g = tile_at(S, J, 0);
  for (int k = threadIdx.x; k < kTT; k += blockDim.x) sA[k >> 5][k & 31] = __ldcg(g + k);
  __syncthreads();
  return factor_tile(S, J, sA, flags);
}

// Phase B on rows 8q..8q+7 of tile (I = J+o, J): W = A L_JJ^-T, L = W
// D^-1 (rows are independent, so a tile is four tasks).  A warp per row: once
// column c of W is final (broadcast by shuffle), every later column s loses
// W(r, c) l_sc -- no block barriers inside the sweep.
constexpr int kPanelRows = 8;
constexpr int kPanelParts = kT / kPanelRows;

__device__ void panel_solve(const ProfileSystem &S, int J, int o, int q, double (*sA)[kT + 1],
                            double (*sB)[kT + 1]) {
  (void)sA;
  const double *Ljj = tile_at(S, J, 0);
  double *g = tile_at(S, J + o, o) + q * kPanelRows * kT;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int k = threadIdx.x; k < kTT; k += blockDim.x) sB[k >> 5][k & 31] = __ldcg(Ljj + k);
  // warp w solves row 8q+w: lane s holds W(r, s); column c is final once
  // the columns before it have been applied, then the later columns take it
  double x = w < kPanelRows ? __ldcg(g + w * kT + lane) : 0.0;
  const double inv = __ldcg(S.invD + (size_t)J * kT + lane);
  __syncthreads();
  if (w < kPanelRows) {
    for (int c = 0; c < kT - 1; c++) {
      const double wc = __shfl_sync(0xffffffffu, x, c);
      if (lane > c) x = fma(-wc, sB[lane][c], x);
    }
    g[w * kT + lane] = x * inv;
  }
  __syncthreads();
}

// The panel of tile (J+1, J) in four row parts whose tasks, once all four
// are written, apply a quarter each of that panel's update of diagonal tile
// J+1 (phase C for the pair (J+1, J+1), 132 of its 528 lower entries), so
// the chain task only factors.  The wait for the sibling parts is bounded;
// they sit right after this task in the list, so the blocks that take them
// never wait on this one.
__device__ bool wait_geq_dev(const int *p, int target, volatile int *flags);
__device__ bool panel_update_task(const ProfileSystem &S, int J, int q, double (*sA)[kT + 1],
                                  double (*sB)[kT + 1], volatile int *flags) {
  const int I = J + 1, tid = threadIdx.x;
  panel_solve(S, J, 1, q, sA, sB);
  __shared__ int ok;
  if (tid == 0) {
    __threadfence();
    atomicAdd(S.done + (size_t)I * (S.W + 1) + 1, 1);
    ok = wait_geq_dev(S.done + (size_t)I * (S.W + 1) + 1, kPanelParts, flags) &&
         wait_geq_dev(S.upd + (size_t)I * (S.W + 1), J - S.ftile[I], flags);
    __threadfence();
  }
  __syncthreads();
  if (!ok) return false;
  const double *gp = tile_at(S, I, 1);
  double *gd = tile_at(S, I, 0);
  const double *piv = S.piv + (size_t)J * kT;
  for (int k = tid; k < kTT; k += blockDim.x) {
    const double l = __ldcg(gp + k);
    sB[k >> 5][k & 31] = l;
    sA[k >> 5][k & 31] = l * __ldcg(piv + (k & 31));
  }
  __syncthreads();
  constexpr int kQuarter = kT * (kT + 1) / 2 / kPanelParts;   // 132
  for (int k = q * kQuarter + tid; k < (q + 1) * kQuarter; k += blockDim.x) {
    const int rs = kLowerRS[k], r = rs >> 5, sc = rs & 31;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
#pragma unroll
    for (int c = 0; c < kT; c += 4) {
      a0 = fma(sA[r][c], sB[sc][c], a0);
      a1 = fma(sA[r][c + 1], sB[sc][c + 1], a1);
      a2 = fma(sA[r][c + 2], sB[sc][c + 2], a2);
      a3 = fma(sA[r][c + 3], sB[sc][c + 3], a3);
    }
    gd[r * kT + sc] = __ldcg(gd + r * kT + sc) - ((a0 + a1) + (a2 + a3));
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    atomicAdd(S.upd + (size_t)I * (S.W + 1), 1);
  }
  return true;
}

// For the substitutions, off the factorisation's critical path: W_J =
// L_JJ^-T (rows r of W solve w L_JJ' = e_r, a warp per row as in phase B),
// F_J = W' L_J,J-1, E_J = W' L_J,J-2, G_J = W L_J+1,J', H_J = W L_J+2,J'
// (zero where the tile is outside the envelope), then, once row J-1's task
// has finished, Q_J = E_J - F_J F_J-1 and R_J-1 = H_J-1 - G_J-1 G_J.  With
// them a sweep row depends on the row two back: y_J = c3_J - F_J c_J-1 -
// Q_J y_J-2, c_J = c3_J - E_J y_J-2 (c3_J: W' times the right-hand side
// less rows J-3 and older), and the same backwards with G, H, R.
__device__ void coupling_task(const ProfileSystem &S, int J, double (*sA)[kT + 1],
                              double (*sB)[kT + 1], double (*sC)[kT + 1], volatile int *flags) {
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const size_t off = (size_t)J * kTT;
  const double *Ljj = tile_at(S, J, 0);
  for (int k = tid; k < kTT; k += blockDim.x) sB[k >> 5][k & 31] = __ldcg(Ljj + k);
  __syncthreads();
  // W = I L^-T: warp w takes rows w, w+8, w+16, w+24
  for (int r = w; r < kT; r += blockDim.x / 32) {
    double x = lane == r ? 1.0 : 0.0;
    for (int c = 0; c < kT - 1; c++) {
      const double wc = __shfl_sync(0xffffffffu, x, c);
      if (lane > c) x = fma(-wc, sB[lane][c], x);
    }
    sA[r][lane] = x;
    S.Winv[off + r * kT + lane] = x;
  }
  __syncthreads();
  for (int pass = 0; pass < 4; pass++) {
    // F = W' L_J,J-1, G = W L_J+1,J', E = W' L_J,J-2, H = W L_J+2,J'
    const int o = pass < 2 ? 1 : 2;
    const bool lower = (pass & 1) == 0;      // W' times a tile of row J
    const bool has = lower ? (J >= o && S.ftile[J] <= J - o)
                           : (J + o < S.nt && S.ftile[J + o] <= J);
    double *out = (pass == 0 ? S.F : pass == 1 ? S.G : pass == 2 ? S.E : S.H) + off;
    if (!has) {
      for (int k = tid; k < kTT; k += blockDim.x) out[k] = 0.0;
      continue;
    }
    const double *T = lower ? tile_at(S, J, o) : tile_at(S, J + o, o);
    for (int k = tid; k < kTT; k += blockDim.x) sC[k >> 5][k & 31] = __ldcg(T + k);
    __syncthreads();
    for (int k = tid; k < kTT; k += blockDim.x) {
      const int i = k >> 5, c = k & 31;
      double a0 = 0.0, a1 = 0.0;
      if (lower) {
        for (int q = 0; q < kT; q += 2) {
          a0 = fma(sA[q][i], sC[q][c], a0);
          a1 = fma(sA[q + 1][i], sC[q + 1][c], a1);
        }
      } else {
        for (int q = 0; q < kT; q += 2) {
          a0 = fma(sA[i][q], sC[c][q], a0);
          a1 = fma(sA[i][q + 1], sC[c][q + 1], a1);
        }
      }
      out[k] = a0 + a1;
    }
    __syncthreads();
  }
  // Q_J and R_J-1 need row J-1's matrices (the task before this one)
  __shared__ int ok;
  if (tid == 0) ok = J == 0 || wait_geq_dev(S.cpl + (J - 1), 1, flags);
  __syncthreads();
  if (!ok) return;
  for (int pass = 0; pass < 2; pass++) {
    // pass 0: Q_J = E_J - F_J F_J-1;  pass 1: R_J-1 = H_J-1 - G_J-1 G_J
    if (pass == 1 && J == 0) break;
    const size_t oa = pass == 0 ? off : off - kTT, ob = pass == 0 ? off - kTT : off;
    const double *A = pass == 0 ? S.F + oa : S.G + oa;
    const double *B = pass == 0 ? S.F + ob : S.G + ob;
    const double *C0 = pass == 0 ? S.E + off : S.H + (off - kTT);
    double *out = pass == 0 ? S.Q + off : S.R + (off - kTT);
    if (J == 0) {
      for (int k = tid; k < kTT; k += blockDim.x) out[k] = __ldcg(C0 + k);
      continue;
    }
    for (int k = tid; k < kTT; k += blockDim.x) {
      sA[k >> 5][k & 31] = __ldcg(A + k);
      sC[k >> 5][k & 31] = __ldcg(B + k);
    }
    __syncthreads();
    for (int k = tid; k < kTT; k += blockDim.x) {
      const int i = k >> 5, c = k & 31;
      double a0 = 0.0, a1 = 0.0;
      for (int q = 0; q < kT; q += 2) {
        a0 = fma(sA[i][q], sC[q][c], a0);
        a1 = fma(sA[i][q + 1], sC[q + 1][c], a1);
      }
      out[k] = __ldcg(C0 + k) - (a0 + a1);
    }
    __syncthreads();
  }
  // the last row's R: G_nt-1 is zero, R = H (zero as well)
  if (J == S.nt - 1)
    for (int k = tid; k < kTT; k += blockDim.x) S.R[off + k] = __ldcg(S.H + off + k);
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    atomicExch(S.cpl + J, 1);
  }
}

// Phase C on pair (I = J+a, K = J+b), b <= a: A_IK -= (L_IJ D_J) L_KJ'.
__device__ void pair_update(const ProfileSystem &S, int J, int a, int b, double (*sA)[kT + 1],
                            double (*sB)[kT + 1]) {
  const double *li = tile_at(S, J + a, a);
  const double *lk = tile_at(S, J + b, b);
  const double *piv = S.piv + (size_t)J * kT;
  for (int k = threadIdx.x; k < kTT; k += blockDim.x) {
    sA[k / kT][k % kT] = __ldcg(li + k) * __ldcg(piv + k % kT);
    sB[k / kT][k % kT] = __ldcg(lk + k);
  }
  __syncthreads();
  double *out = tile_at(S, J + a, a - b);
  if (a == b) {
    // a diagonal tile: its lower triangle only (528 entries, packed table)
    for (int k = threadIdx.x; k < kT * (kT + 1) / 2; k += blockDim.x) {
      const int rs = kLowerRS[k], r = rs >> 5, s = rs & 31;
      double acc = 0.0;
#pragma unroll 8
      for (int c = 0; c < kT; c++) acc += sA[r][c] * sB[s][c];
      out[r * kT + s] = __ldcg(out + r * kT + s) - acc;
    }
  } else {
    for (int k = threadIdx.x; k < kTT; k += blockDim.x) {
      const int r = k / kT, s = k % kT;
      double acc = 0.0;
#pragma unroll 8
      for (int c = 0; c < kT; c++) acc += sA[r][c] * sB[s][c];
      out[k] = __ldcg(out + k) - acc;
    }
  }
  __syncthreads();
}

__device__ bool wait_geq(const int *p, int target, volatile int *flags);
__device__ bool wait_geq_dev(const int *p, int target, volatile int *flags) {
  return wait_geq(p, target, flags);
}

__device__ __forceinline__ int slot_of(const ProfileSystem &S, int I, int o) {
  return I * (S.W + 1) + o;
}

// Column J's critical chain: once the four panel-part tasks of tile
// (J+1, J) have applied their quarters of its update of diagonal tile J+1,
// that tile's LDL' in shared memory.
__device__ bool chain_task(const ProfileSystem &S, int J, double (*sC)[kT + 1],
                           volatile int *flags) {
  return factor_diag(S, J + 1, sC, flags);
}

// Wait until *p >= target (thread 0 of a block); false on a raised error
// flag or after kBarrierTimeoutNs (flags[0] = 2).
__device__ bool wait_geq(const int *p, int target, volatile int *flags) {
  const volatile int *vp = p;
  if (*vp >= target) return true;
  const unsigned long long t0 = global_ns();
  while (*vp < target) {
    if (flags[0] != 0) return false;
    if (global_ns() - t0 > kBarrierTimeoutNs) {
      flags[0] = 2;
      return false;
    }
    __nanosleep(20);
  }
  return true;
}

// Dependencies of a task: every update of its tile from earlier columns
// (the count of columns J' < J both tile rows reach), and the diagonal /
// panel tiles it reads.
__device__ bool wait_task(const ProfileSystem &S, int4 t, volatile int *flags) {
  const int type = t.x, I = t.y, K = t.z, J = t.w;
  if (type == 0)
    return wait_geq(S.upd + slot_of(S, J, 0), J - S.ftile[J], flags);
  if (type == 4)
    return wait_geq(S.upd + slot_of(S, I, 0), J - S.ftile[I] + kPanelParts, flags);
  if (type == 5)
    return wait_geq(S.done + slot_of(S, J, 0), 1, flags) &&
           wait_geq(S.upd + slot_of(S, I, 1), J - max(S.ftile[I], S.ftile[J]), flags);
  if (type == 6) {
    if (!wait_geq(S.done + slot_of(S, J, 0), 1, flags)) return false;
    for (int o = 1; o <= 2; o++) {
      if (J >= o && S.ftile[J] <= J - o &&
          !wait_geq(S.done + slot_of(S, J, o), kPanelParts, flags))
        return false;
      if (J + o < S.nt && S.ftile[J + o] <= J &&
          !wait_geq(S.done + slot_of(S, J + o, o), kPanelParts, flags))
        return false;
    }
    return true;
  }
  if (type == 7) {
    // row J's forward step: its coupling matrices and the panel tiles of
    // the row further left (the y values of the rows before it are polled
    // inside the step)
    if (S.fwd_nrhs == 0) return true;
    if (!wait_geq(S.cpl + J, 1, flags)) return false;
    const int ohi = min(S.W, J - S.ftile[J]);
    for (int o = 3; o <= ohi; o++)
      if (!wait_geq(S.done + slot_of(S, J, o), kPanelParts, flags)) return false;
    return true;
  }
  if (type == 1)
    return wait_geq(S.done + slot_of(S, J, 0), 1, flags) &&
           wait_geq(S.upd + slot_of(S, I, I - J), J - max(S.ftile[I], S.ftile[J]), flags);
  return wait_geq(S.done + slot_of(S, I, I - J), kPanelParts, flags) &&
         wait_geq(S.done + slot_of(S, K, K - J), kPanelParts, flags) &&
         wait_geq(S.upd + slot_of(S, I, I - K), J - max(S.ftile[I], S.ftile[K]), flags);
}

// Pipelined substitutions on kPipeBlocks co-resident blocks (cooperative
// launch): block b owns the tile rows J = b, b + P, ... .  Forward, in
// increasing J: c3_J = L_JJ^-1 (b_J minus the contributions of rows J-3 and
// older), then with the factorisation's coupling matrices
//   y_J = c3_J - F_J c_J-1 - Q_J y_J-2,   c_J = c3_J - E_J y_J-2,
// so a row waits for the row two back (and for c_J-1, which its owner
// publishes as soon as y_J-3 is known): the two interleaved chains halve
// the serial length.  Backward, in decreasing J, the same with
// c3'_J = L_JJ^-T (D_J^-1 y_J minus the transposed contributions of rows J+3
// and beyond):  x_J = c3'_J - G_J c'_J+1 - R_J x_J+2,  c'_J = c3'_J -
// H_J x_J+2.  There are no row flags: every solved value is published to a
// scratch vector filled with kUnset beforehand (a NaN pattern that no
// arithmetic result is stored as), and a consumer thread polls exactly the
// values it reads.  Waits are bounded by the global timer.
constexpr int kPipeBlocks = 64;
constexpr int kPipeThreads = 256;
constexpr unsigned long long kUnset = 0xFFFFFFFFFFFFFFFFull;   // byte fill 0xFF

__device__ __forceinline__ double ld_relaxed(const double *p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// *p once its producer has published it; 0 after a failed wait (flags[0]
// is then nonzero and the host reports the solve as failed)
__device__ __forceinline__ double await_value(const double *p, volatile int *flags) {
  double v = ld_relaxed(p);
  if ((unsigned long long)__double_as_longlong(v) != kUnset) return v;
  const unsigned long long t0 = global_ns();
  for (;;) {
    v = ld_relaxed(p);
    if ((unsigned long long)__double_as_longlong(v) != kUnset) return v;
    if (flags[0] != 0) return 0.0;
    if (global_ns() - t0 > kBarrierTimeoutNs) {
      flags[0] = 2;
      return 0.0;
    }
  }
}

// p[0], p[8], p[16], p[24] (the four loads in flight together)
__device__ __forceinline__ void await4(const double *p, double v[4], volatile int *flags) {
  bool ready = true;
#pragma unroll
  for (int m = 0; m < 4; m++) v[m] = ld_relaxed(p + 8 * m);
#pragma unroll
  for (int m = 0; m < 4; m++) ready &= (unsigned long long)__double_as_longlong(v[m]) != kUnset;
  if (!ready)
    for (int m = 0; m < 4; m++) v[m] = await_value(p + 8 * m, flags);
}

__device__ __forceinline__ void publish(double *p, double v) {
  if ((unsigned long long)__double_as_longlong(v) == kUnset)
    v = __longlong_as_double(0x7FF8000000000000ll);   // keep a NaN a NaN
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

// Forward substitution of tile row J for the right-hand sides given to the
// factorisation (S.fwd_nrhs > 0), as a task of the factorisation itself:
// the right-hand sides are known before the tangent is factored (the
// unbalance and the reference load of a Newton iteration), so row J's step
// runs as soon as its coupling matrices are written, a few columns behind
// the factorisation's front, instead of after it.  The step is the pipelined
// sweep's (k_prof_solve_pipe) for one row: c3_J = L_JJ^-1 (b_J minus rows
// J-3 and older), y_J = c3_J - F_J c_J-1 - Q_J y_J-2, c_J = c3_J - E_J
// y_J-2, published to the sweep's scratch (y, c) for the rows after it and
// for the backward sweep.
__device__ bool forward_row(const ProfileSystem &S, int J, double (*rb)[kT],
                            volatile int *flags) {
  const int tid = threadIdx.x;
  const int r = tid >> 3, g = tid & 7;
  const int nrhs = S.fwd_nrhs, ls = S.nt * kT;
  double *ys = S.sweep, *cs = ys + (size_t)nrhs * ls;
  auto group_sum = [](double v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v;
  };
  auto row_of = [&](const double *M, double (&mv)[4]) {
#pragma unroll
    for (int m = 0; m < 4; m++) mv[m] = __ldcg(M + r * kT + g + 8 * m);
  };
  auto row_times = [&](const double (&mv)[4], const double *p) {
    double v[4];
    await4(p + g, v, flags);
    double t = 0.0;
#pragma unroll
    for (int m = 0; m < 4; m++) t = fma(mv[m], v[m], t);
    return group_sum(t);
  };
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const int ohi = min(S.W, J - S.ftile[J]);
  for (int o = ohi; o >= 3; o--) {
    const double *Lt = tile_at(S, J, o) + r * kT + g;
    const double l0 = __ldcg(Lt), l1 = __ldcg(Lt + 8), l2 = __ldcg(Lt + 16), l3 = __ldcg(Lt + 24);
    for (int q = 0; q < nrhs; q++) {
      double y[4];
      await4(ys + (size_t)q * ls + (J - o) * kT + g, y, flags);
      acc[q] += l0 * y[0] + l1 * y[1] + l2 * y[2] + l3 * y[3];
    }
  }
  for (int q = 0; q < nrhs; q++) {
    const double v = group_sum(acc[q]);
    if (g == 0) rb[q][r] = __ldcg(S.fwd_x + (size_t)q * S.fwd_ldx + J * kT + r) - v;
  }
  const double *Wt = S.Winv + (size_t)J * kTT;
  double wv[4];
#pragma unroll
  for (int m = 0; m < 4; m++) wv[m] = __ldcg(Wt + (g + 8 * m) * kT + r);
  const size_t off = (size_t)J * kTT;
  double fv[4], qv[4], ev[4];
  row_of(S.F + off, fv);
  row_of(S.Q + off, qv);
  row_of(S.E + off, ev);
  __syncthreads();
  const bool hasF = J >= 1 && S.ftile[J] <= J - 1;
  for (int q = 0; q < nrhs; q++) {
    double c3 = 0.0;
#pragma unroll
    for (int m = 0; m < 4; m++) c3 = fma(wv[m], rb[q][g + 8 * m], c3);
    c3 = group_sum(c3);
    const size_t vq = (size_t)q * ls;
    double t2 = 0.0, t3 = 0.0;
    if (J >= 2) t3 = row_times(ev, ys + vq + (J - 2) * kT);
    if (g == 0) publish(cs + vq + J * kT + r, c3 - t3);
    if (J >= 2) t2 = row_times(qv, ys + vq + (J - 2) * kT);
    const double t1 = hasF ? row_times(fv, cs + vq + (J - 1) * kT) : 0.0;
    if (g == 0) publish(ys + vq + J * kT + r, (c3 - t1) - t2);
  }
  return flags[0] == 0;
}

__global__ void __launch_bounds__(kFactorThreads) k_prof_factor(ProfileSystem S) {
  __shared__ double sA[kT][kT + 1], sB[kT][kT + 1], sC[kT][kT + 1];
  __shared__ int task, ok;
  volatile int *flags = S.flags;
  while (true) {
    if (threadIdx.x == 0) {
      task = atomicAdd(S.next_task, 1);
      ok = (task < S.ntasks && flags[0] == 0) ? 1 : 0;
      if (ok) ok = wait_task(S, S.tasks[task], flags) ? 1 : 0;
      __threadfence();
    }
    __syncthreads();
    if (!ok) break;
    const int4 t = S.tasks[task];
    bool fine = true;
    if (t.x == 0) {
      fine = factor_diag(S, t.w, sA, flags);
    } else if (t.x == 1) {
      panel_solve(S, t.w, t.y - t.w, t.z, sA, sB);
    } else if (t.x == 2) {
      pair_update(S, t.w, t.y - t.w, t.z - t.w, sA, sB);
    } else if (t.x == 4) {
      fine = chain_task(S, t.w, sC, flags);
    } else if (t.x == 5) {
      fine = panel_update_task(S, t.w, t.z, sA, sB, flags);
    } else if (t.x == 7) {
      if (S.fwd_nrhs > 0) fine = forward_row(S, t.w, reinterpret_cast<double (*)[kT]>(&sA[0][0]),
                                             flags);
    } else {
      coupling_task(S, t.w, sA, sB, sC, flags);
    }
    if (!fine) break;
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      if (t.x == 2) atomicAdd(S.upd + slot_of(S, t.y, t.y - t.z), 1);
      if (t.x == 0 || t.x == 4) atomicExch(S.done + slot_of(S, t.y, 0), 1);
      if (t.x == 1) atomicAdd(S.done + slot_of(S, t.y, t.y - t.w), 1);
    }
    __syncthreads();
  }
}

// Forward (L y = b), diagonal (z = D^-1 y) and backward (L' x = z)
// substitution in one block of 1024 threads; x[r * ldx + i] for right-hand
// side r.  Warp w owns row w of every tile and lane c its column, so a
// tile's 32 x 32 entries come in with one coalesced load per thread; a step
// (one tile row forward, one tile column backward) issues the loads of up
// to kChunk tiles at once, keeps the last W+1 solved tiles of every
// right-hand side in shared memory, and solves the diagonal tile with warp
// shuffles.  A step costs about one L2 latency plus the 32-step solve.
constexpr int kChunk = 24;
constexpr int kSolveBlock = 1024;

__global__ void __launch_bounds__(kSolveBlock) k_prof_solve(ProfileSystem S, int nrhs,
                                                             double *x, int ldx) {
  extern __shared__ double win[];                 // [nrhs][W+1][32]
  __shared__ double red[4][kT][kT + 1];
  __shared__ double sL[kT][kT + 1];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int nt = S.nt, W = S.W, span = W + 1;
  auto ywin = [&](int q, int tile) -> double * { return win + ((size_t)q * span + tile % span) * kT; };
  // ---- forward: t = b_J - sum_o L(J, J-o) y_{J-o}; then unit-lower solve
  for (int J = 0; J < nt; J++) {
    const double dval = __ldg(tile_at(S, J, 0) + w * kT + lane);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int ohi = min(W, J - S.ftile[J]);
    for (int o0 = 1; o0 <= ohi; o0 += kChunk) {
      double l[kChunk];
#pragma unroll
      for (int k = 0; k < kChunk; k++)
        l[k] = (o0 + k <= ohi) ? __ldg(tile_at(S, J, o0 + k) + w * kT + lane) : 0.0;
#pragma unroll
      for (int k = 0; k < kChunk; k++) {
        if (o0 + k > ohi) break;
        for (int q = 0; q < nrhs; q++) acc[q] += l[k] * ywin(q, J - o0 - k)[lane];
      }
    }
    for (int q = 0; q < nrhs; q++) {
      double v = acc[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[q][0][w] = v;
    }
    sL[w][lane] = dval;
    __syncthreads();
    if (w < nrhs) {
      const int q = w;
      double v = x[(size_t)q * ldx + J * kT + lane] - red[q][0][lane];
      for (int c = 0; c < kT - 1; c++) {
        const double yc = __shfl_sync(0xffffffffu, v, c);
        if (lane > c) v -= sL[lane][c] * yc;
      }
      ywin(q, J)[lane] = v;
      x[(size_t)q * ldx + J * kT + lane] = v;
    }
    __syncthreads();
  }
  // ---- diagonal
  for (int q = 0; q < nrhs; q++)
    for (int i = tid; i < nt * kT; i += kSolveBlock) x[(size_t)q * ldx + i] *= S.invD[i];
  __syncthreads();
  // ---- backward: t = z_J - sum_o L(J+o, J)' x_{J+o}; then unit-upper solve
  for (int J = nt - 1; J >= 0; J--) {
    const double dval = __ldg(tile_at(S, J, 0) + w * kT + lane);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int ohi = min(W, nt - 1 - J);
    for (int o0 = 1; o0 <= ohi; o0 += kChunk) {
      double l[kChunk];
#pragma unroll
      for (int k = 0; k < kChunk; k++)
        l[k] = (o0 + k <= ohi && S.ftile[J + o0 + k] <= J)
                   ? __ldg(tile_at(S, J + o0 + k, o0 + k) + w * kT + lane)
                   : 0.0;
      // row w of tile (J+o, J) times x_{J+o}[w]; summed over rows below
#pragma unroll
      for (int k = 0; k < kChunk; k++) {
        if (o0 + k > ohi) break;
        for (int q = 0; q < nrhs; q++) acc[q] += l[k] * ywin(q, J + o0 + k)[w];
      }
    }
    for (int q = 0; q < nrhs; q++) red[q][w][lane] = acc[q];
    sL[w][lane] = dval;
    __syncthreads();
    if (w < nrhs) {
      const int q = w;
      double sum = 0.0;
      for (int h = 0; h < kT; h++) sum += red[q][h][lane];
      double v = x[(size_t)q * ldx + J * kT + lane] - sum;
      // x_c = v_c - sum_{k > c} L[k][c] x_k, from the last row up
      for (int cc = kT - 1; cc > 0; cc--) {
        const double xc = __shfl_sync(0xffffffffu, v, cc);
        if (lane < cc) v -= sL[cc][lane] * xc;
      }
      ywin(q, J)[lane] = v;
      x[(size_t)q * ldx + J * kT + lane] = v;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kPipeThreads) k_prof_solve_pipe(ProfileSystem S, int nrhs,
                                                                  double *x, int ldx,
                                                                  double *ys, double *cs,
                                                                  double *xs, double *ds,
                                                                  int backward_only) {
  __shared__ double rv[2][4][kT];
  volatile int *flags = S.flags;
  const int tid = threadIdx.x;
  const int r = tid >> 3, g = tid & 7;          // tile row, column group (4 columns)
  const int nt = S.nt, W = S.W, P = gridDim.x, ls = nt * kT;
  // reduce over the eight column groups of a row (lanes r*8 .. r*8+7)
  auto group_sum = [](double v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v;
  };
  // this thread's four entries of row r of a 32 x 32 matrix (loaded ahead
  // of the waits), and their product with the vector published at p
  auto row_of = [&](const double *M, double (&mv)[4]) {
#pragma unroll
    for (int m = 0; m < 4; m++) mv[m] = __ldcg(M + r * kT + g + 8 * m);
  };
  auto row_times = [&](const double (&mv)[4], const double *p) {
    double v[4];
    await4(p + g, v, flags);
    double t = 0.0;
#pragma unroll
    for (int m = 0; m < 4; m++) t = fma(mv[m], v[m], t);
    return group_sum(t);
  };
  int it = 0;                                   // rv is double-buffered by iteration
  // ---------------- forward (done by the factorisation when backward_only)
  for (int J = blockIdx.x; J < nt && !backward_only; J += P, it++) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int ohi = min(W, J - S.ftile[J]);
    for (int o = ohi; o >= 3; o--) {
      const double *Lt = tile_at(S, J, o) + r * kT + g;
      const double l0 = __ldcg(Lt), l1 = __ldcg(Lt + 8), l2 = __ldcg(Lt + 16), l3 = __ldcg(Lt + 24);
      for (int q = 0; q < nrhs; q++) {
        double y[4];
        await4(ys + (size_t)q * ls + (J - o) * kT + g, y, flags);
        acc[q] += l0 * y[0] + l1 * y[1] + l2 * y[2] + l3 * y[3];
      }
    }
    double(*rb)[kT] = rv[it & 1];
    for (int q = 0; q < nrhs; q++) {
      const double v = group_sum(acc[q]);
      if (g == 0) rb[q][r] = __ldcg(x + (size_t)q * ldx + J * kT + r) - v;
    }
    const double *Wt = S.Winv + (size_t)J * kTT;
    double wv[4];
#pragma unroll
    for (int m = 0; m < 4; m++) wv[m] = __ldcg(Wt + (g + 8 * m) * kT + r);
    const size_t off = (size_t)J * kTT;
    double fv[4], qv[4], ev[4];
    row_of(S.F + off, fv);
    row_of(S.Q + off, qv);
    row_of(S.E + off, ev);
    __syncthreads();
    const bool hasF = J >= 1 && S.ftile[J] <= J - 1;
    for (int q = 0; q < nrhs; q++) {
      double c3 = 0.0;
#pragma unroll
      for (int m = 0; m < 4; m++) c3 = fma(wv[m], rb[q][g + 8 * m], c3);
      c3 = group_sum(c3);
      const size_t vq = (size_t)q * ls;
      // c_J first: it needs only y_J-2, and row J+1 waits for it
      double t2 = 0.0, t3 = 0.0;
      if (J >= 2) t3 = row_times(ev, ys + vq + (J - 2) * kT);
      if (g == 0) publish(cs + vq + J * kT + r, c3 - t3);
      if (J >= 2) t2 = row_times(qv, ys + vq + (J - 2) * kT);
      const double t1 = hasF ? row_times(fv, cs + vq + (J - 1) * kT) : 0.0;
      if (g == 0) publish(ys + vq + J * kT + r, (c3 - t1) - t2);
    }
  }
  // ---------------- backward
  const int jlast = blockIdx.x + ((nt - 1 - (int)blockIdx.x) / P) * P;
  for (int J = jlast; J >= 0; J -= P, it++) {
    if (J >= nt) continue;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int ohi = min(W, nt - 1 - J);
    // column c = r of the result; rows g, g+8, g+16, g+24 of tile (J+o, J)
    for (int o = ohi; o >= 3; o--) {
      if (S.ftile[J + o] > J) continue;
      const double *Lt = tile_at(S, J + o, o) + r;
      const double l0 = __ldcg(Lt + g * kT), l1 = __ldcg(Lt + (g + 8) * kT);
      const double l2 = __ldcg(Lt + (g + 16) * kT), l3 = __ldcg(Lt + (g + 24) * kT);
      for (int q = 0; q < nrhs; q++) {
        double xv[4];
        await4(xs + (size_t)q * ls + (J + o) * kT + g, xv, flags);
        acc[q] += l0 * xv[0] + l1 * xv[1] + l2 * xv[2] + l3 * xv[3];
      }
    }
    double(*rb)[kT] = rv[it & 1];
    for (int q = 0; q < nrhs; q++) {
      const double v = group_sum(acc[q]);
      // z_J = D^-1 y_J (ProfileSPD divides by the pivots before the back
      // sweep); y_J[r] was published by this same thread in the forward sweep
      if (g == 0)
        rb[q][r] = ld_relaxed(ys + (size_t)q * ls + J * kT + r) * S.invD[J * kT + r] - v;
    }
    const double *Wt = S.Winv + (size_t)J * kTT;
    double wv[4];
#pragma unroll
    for (int m = 0; m < 4; m++) wv[m] = __ldcg(Wt + r * kT + g + 8 * m);
    const size_t off = (size_t)J * kTT;
    double gv[4], rv4[4], hv[4];
    row_of(S.G + off, gv);
    row_of(S.R + off, rv4);
    row_of(S.H + off, hv);
    __syncthreads();
    const bool hasG = J + 1 < nt && S.ftile[J + 1] <= J;
    for (int q = 0; q < nrhs; q++) {
      double c3 = 0.0;
#pragma unroll
      for (int m = 0; m < 4; m++) c3 = fma(wv[m], rb[q][g + 8 * m], c3);
      c3 = group_sum(c3);
      const size_t vq = (size_t)q * ls;
      // c'_J first: it needs only x_J+2, and row J-1 waits for it
      double t2 = 0.0, t3 = 0.0;
      if (J + 2 < nt) t3 = row_times(hv, xs + vq + (J + 2) * kT);
      if (g == 0) publish(ds + vq + J * kT + r, c3 - t3);
      if (J + 2 < nt) t2 = row_times(rv4, xs + vq + (J + 2) * kT);
      const double t1 = hasG ? row_times(gv, ds + vq + (J + 1) * kT) : 0.0;
      if (g == 0) {
        const double xj = (c3 - t1) - t2;
        publish(xs + vq + J * kT + r, xj);
        x[(size_t)q * ldx + J * kT + r] = xj;
      }
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

// The dataflow order of the factor tasks (type, I, K, J): type 0 diagonal
// tile J (I = K = J), 1 rows 8K..8K+7 of panel tile (I, J), 2 update of
// tile (I, K) by
// column J, 3 the update of diagonal tile J+1 by column J followed by its
// factorisation (it is that tile's last update).
void profile_tasks(int nt, int W, const std::vector<int> &ftile, std::vector<int> &tasks) {
  tasks.clear();
  auto emit = [&](int type, int I, int K, int J) {
    tasks.push_back(type); tasks.push_back(I); tasks.push_back(K); tasks.push_back(J);
  };
  // the updates of column J (0 <= J < nt) whose target column is J+b for b
  // in [blo, bhi]
  // (the pair (J+1, J+1) of column J belongs to column J's chain task)
  auto updates = [&](int J, int blo, int bhi) {
    if (J < 0) return;
    const int omax = std::min(W, nt - 1 - J);
    for (int b = blo; b <= std::min(bhi, omax); b++) {
      if (ftile[J + b] > J) continue;
      for (int a = b; a <= omax; a++)
        if (ftile[J + a] <= J && !(a == 1 && b == 1)) emit(2, J + a, J + b, J);
    }
  };
  // Column J: the updates of column J-1 that reach column J+1 (the
  // diagonal's included), the chain task (panel (J+1, J), the last update
  // and the LDL' of diagonal tile J+1), the other panels, column J's
  // updates of column J+1, then the rest of column J-1's trailing update.
  for (int J = 0; J < nt; J++) {
    if (ftile[J] == J) emit(0, J, J, J);   // no column updates this tile
    updates(J - 1, 2, 2);
    const int omax = std::min(W, nt - 1 - J);
    if (omax >= 1 && ftile[J + 1] <= J)
      for (int q = 0; q < kPanelParts; q++) emit(5, J + 1, q, J);
    if (J + 1 < nt && ftile[J + 1] <= J) emit(4, J + 1, J + 1, J);
    for (int o = 2; o <= omax; o++)
      if (ftile[J + o] <= J)
        for (int q = 0; q < kPanelParts; q++) emit(1, J + o, q, J);
    updates(J, 1, 1);
    updates(J - 1, 3, W);
    if (J >= 2) {
      emit(6, J - 2, J - 2, J - 2);
      emit(7, J - 2, J - 2, J - 2);
    }
  }
  updates(nt - 1, 2, W);
  for (int J = std::max(nt - 2, 0); J < nt; J++) {
    emit(6, J, J, J);
    emit(7, J, J, J);
  }
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
    // one block per SM: a block that runs a task on the critical path (a
    // diagonal tile, a panel) must not share its SM's few FP64 units with a
    // bulk tile update; the dynamic shared memory requested below keeps a
    // second block off the SM
    g_factor_blocks = sms;
    cudaFuncSetAttribute(k_prof_factor, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kFactorSoloSmem);
  }
  const size_t nslots = (size_t)S.nt * (S.W + 1);
  if (S.fwd_nrhs > 0) {
    // the forward sweep runs inside: its published values start unset
    if (!profile_pipelined(S) || S.fwd_nrhs > 4 || !S.fwd_x) return XG_EINVAL;
    const size_t ls = (size_t)S.nt * kT;
    if (cudaMemsetAsync(S.sweep, 0xFF, 2 * (size_t)S.fwd_nrhs * ls * sizeof(double), s) !=
        cudaSuccess)
      return XG_ECUDA;
  }
  if (cudaMemsetAsync(S.upd, 0, nslots * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  if (cudaMemsetAsync(S.done, 0, nslots * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  if (cudaMemsetAsync(S.cpl, 0, (size_t)S.nt * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  if (cudaMemsetAsync(S.next_task, 0, sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  if (cudaMemsetAsync(S.flags, 0, 4 * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  const int nb = (int)std::min<long>(g_factor_blocks, std::max(S.ntasks, 1));
  k_prof_factor<<<nb, kFactorThreads, kFactorSoloSmem, s>>>(S);
  if (cudaGetLastError() != cudaSuccess) return XG_ECUDA;
  int hflags[4];
  if (cudaMemcpyAsync(hflags, S.flags, sizeof hflags, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return XG_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return XG_ECUDA;
  if (bad_eq) *bad_eq = hflags[0] == 3 ? hflags[1] : -1;
  if (hflags[0] == 3) return XG_ESOLVE;   // pivot check failed
  if (hflags[0] != 0) return XG_ESOLVE;   // a dependency wait timed out
  return 0;
}

bool profile_pipelined(const ProfileSystem &S) { return S.sweep && S.nt >= 2 * kPipeBlocks; }

int profile_solve(const ProfileSystem &S, int nrhs, double *x, int ldx, cudaStream_t s,
                  bool backward_only) {
  if (S.n == 0) return 0;
  if (nrhs < 1 || nrhs > 4 || ldx < S.nt * kT) return XG_EINVAL;
  if (backward_only && !profile_pipelined(S)) return XG_EINVAL;
  if (profile_pipelined(S)) {
    // pipelined over co-resident blocks (the sweeps' published values are
    // reset to kUnset first; after a factorisation that ran the forward
    // sweep, only the backward sweep's); small systems keep the one-block
    // sweep
    const size_t ls = (size_t)S.nt * kT;
    double *ys = S.sweep, *cs = ys + (size_t)nrhs * ls, *xs = cs + (size_t)nrhs * ls;
    double *ds = xs + (size_t)nrhs * ls;
    double *reset = backward_only ? xs : ys;
    const size_t nreset = (backward_only ? 2 : 4) * (size_t)nrhs * ls;
    if (cudaMemsetAsync(reset, 0xFF, nreset * sizeof(double), s) != cudaSuccess)
      return XG_ECUDA;
    if (cudaMemsetAsync(S.flags, 0, 4 * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
    ProfileSystem Sv = S;
    int bonly = backward_only ? 1 : 0;
    void *args[] = {(void *)&Sv, (void *)&nrhs, (void *)&x,  (void *)&ldx, (void *)&ys,
                    (void *)&cs, (void *)&xs,   (void *)&ds, (void *)&bonly};
    if (cudaLaunchCooperativeKernel((void *)k_prof_solve_pipe, dim3(kPipeBlocks),
                                    dim3(kPipeThreads), args, 0, s) != cudaSuccess)
      return XG_ECUDA;
    int hflag = 0;
    if (cudaMemcpyAsync(&hflag, S.flags, sizeof hflag, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return XG_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return XG_ECUDA;
    return hflag != 0 ? XG_ESOLVE : 0;   // a sweep wait timed out
  }
  const size_t win = (size_t)nrhs * (S.W + 1) * kT * sizeof(double);
  const size_t stat = (4 * kT * (kT + 1) + kT * (kT + 1)) * sizeof(double);
  if (win + stat > 227 * 1024)
    return XG_EINVAL;   // envelope wider than the substitution window
  if (cudaFuncSetAttribute(k_prof_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)win) != cudaSuccess)
    return XG_ECUDA;
  k_prof_solve<<<1, kSolveBlock, win, s>>>(S, nrhs, x, ldx);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

}  // namespace xg
