// xg_pcg.cu -- block-Jacobi preconditioned conjugate gradients, FP64.
//
// The whole solve is one cooperative, persistent launch: every block owns a
// grid-stride share of the rows, SpMV runs warp-per-row over the CSR arrays,
// and the three inner products of an iteration are reduced deterministically
// (fixed-order block partials, then every block sums the partials in the same
// order), so the iterates are bit-identical run to run.  Blocks meet at a
// grid barrier whose wait is bounded by the global timer: a block that waits
// longer than kBarrierTimeoutNs raises flags[0] and every block leaves the
// solve, so a fault can never hang the GPU.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "xg_ff.h"
#include "xg_internal.h"

namespace xg {

namespace {

constexpr int kPcgThreads = 512;
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Sense-reversing grid barrier: bar[0] arrivals, bar[1] generation.
// Returns false (and sets flags[0]) on timeout or when another block did.
__device__ bool grid_barrier(unsigned int *bar, volatile int *flags) {
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
        __nanosleep(64);
      }
    }
    __threadfence();
    if (flags[0] != 0) ok = 0;
  }
  __syncthreads();
  return ok != 0;
}

__device__ double block_reduce(double v, double *smem) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) smem[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = (lane < (int)(blockDim.x >> 5)) ? smem[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// Sum of partials[0..nb) in a fixed order, broadcast to the whole block.
__device__ double sum_partials(const double *partials, int nb, double *smem) {
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partials[i];
  s = block_reduce(s, smem);
  if (threadIdx.x == 0) smem[32] = s;
  __syncthreads();
  const double r = smem[32];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double spmv_row(const PcgSystem &S, int row, const double *x,
                                           int lane) {
  double s = 0.0;
  const int b = S.rowptr[row], e = S.rowptr[row + 1];
  for (int k = b + lane; k < e; k += 32) s += S.vals[k] * x[S.colidx[k]];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  return s;  // lane 0
}

// Row of (A x) from the CSR arrays in FP64, one thread.
__device__ __forceinline__ double csr_row64(const PcgSystem &S, int row, const double *x) {
  double s = 0.0;
  for (int k = S.rowptr[row]; k < S.rowptr[row + 1]; k++) s = fma(S.vals[k], x[S.colidx[k]], s);
  return s;
}

// Sliced ELL copy of the CSR matrix (thread per row): slice s holds rows
// 32s .. 32s+31 column-major over the slice's longest row, entry k of row r
// at sell_off[r/32] + 32k + r%32, so a warp's 32 rows load each entry
// position with one coalesced access.  Each row is summed in its CSR order
// into four interleaved float-float partial sums, a fixed order, against
// p split into (hi, lo) (x2); rows whose values the split cannot hold, or
// every row when fp64 is set, in FP64 against x.
__device__ __forceinline__ double spmv_sell(const PcgSystem &S, int row, const double *x,
                                            const float2 *x2, bool fp64) {
  if (fp64 || !S.row_ff[row]) return csr_row64(S, row, x);
  const int len = S.rowptr[row + 1] - S.rowptr[row];
  const long base = S.sell_off[row >> 5] + (row & 31);
  const int *cp = S.sell_cols + base;
  const float2 *vp = S.sell_vals + base;
  float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f, h3 = 0.f, l3 = 0.f;
  int k = 0;
  for (; k + 4 <= len; k += 4) {
    const int c0 = __ldcs(cp + 32 * k), c1 = __ldcs(cp + 32 * (k + 1));
    const int c2 = __ldcs(cp + 32 * (k + 2)), c3 = __ldcs(cp + 32 * (k + 3));
    const float2 v0 = __ldcs(vp + 32 * k), v1 = __ldcs(vp + 32 * (k + 1));
    const float2 v2 = __ldcs(vp + 32 * (k + 2)), v3 = __ldcs(vp + 32 * (k + 3));
    ff_madd(v0, x2[c0], h0, l0);
    ff_madd(v1, x2[c1], h1, l1);
    ff_madd(v2, x2[c2], h2, l2);
    ff_madd(v3, x2[c3], h3, l3);
  }
  for (; k < len; k++) ff_madd(__ldcs(vp + 32 * k), x2[__ldcs(cp + 32 * k)], h0, l0);
  return (((double)h0 + (double)l0) + ((double)h1 + (double)l1)) +
         (((double)h2 + (double)l2) + ((double)h3 + (double)l3));
}

// f(row, (A x)[row]) for this thread's rows: thread per row over the sliced
// ELL copy (kSell; rows longer than S.sell_cap are left to
// long_row_chunks), else warp per CSR row (lane 0 calls f).
// With kSell: x2 is x split into (hi, lo) for the float-float SpMV, or null
// for FP64 throughout (the initial residual, or a p outside the split's
// range).
template <bool kSell, typename F>
__device__ __forceinline__ void for_rows_Ax(const PcgSystem &S, const double *x,
                                            const float2 *x2, F f) {
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gthreads = gridDim.x * blockDim.x;
  if (kSell) {
    for (int row = gtid; row < S.n; row += gthreads)
      if (S.rowptr[row + 1] - S.rowptr[row] <= S.sell_cap)
        f(row, spmv_sell(S, row, x, x2, x2 == nullptr));
  } else {
    const int lane = threadIdx.x & 31;
    for (int row = gtid >> 5; row < S.n; row += gthreads >> 5) {
      const double ax = spmv_row(S, row, x, lane);
      if (lane == 0) f(row, ax);
    }
  }
}

// Rows longer than S.sell_cap (a node tied to a whole face by a
// multi-point constraint couples to every node of that face) in chunks of
// at most kLongChunk CSR entries, a warp per chunk: g(chunk, row, partial)
// on lane 0.  A warp per row would leave one warp thousands of entries.
constexpr int kLongChunk = 512;
template <typename G>
__device__ __forceinline__ void long_row_chunks(const PcgSystem &S, const double *x, G g) {
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = gtid >> 5; c < S.nchunks; c += nwarps) {
    const int row = S.chunk_row[c];
    const int b = S.chunk_beg[c], e = min(b + kLongChunk, S.rowptr[row + 1]);
    double t = 0.0;
    for (int k = b + lane; k < e; k += 32) t += S.vals[k] * x[S.colidx[k]];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) g(c, row, t);
  }
}

// (A x)[row] of every long row from its chunk partials, in chunk order
// (lane-strided, then a fixed butterfly): h(row, sum) on lane 0 of a warp
// per long row.
template <typename H>
__device__ __forceinline__ void long_row_sums(const PcgSystem &S, H h) {
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = gtid >> 5; i < S.nlong; i += nwarps) {
    double t = 0.0;
    for (int c = S.long_chunk0[i] + lane; c < S.long_chunk0[i + 1]; c += 32) t += S.chunk_part[c];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) h(S.chunk_row[S.long_chunk0[i]], t);
  }
}

// Vector work is done per diagonal block (<= 6 equations of one node), so
// every equation is read and written by exactly one thread in a phase.
struct BlockRange { int b, m; };
__device__ __forceinline__ BlockRange block_range(const PcgSystem &S, int k) {
  BlockRange r;
  r.b = S.blk_start[k];
  r.m = S.blk_start[k + 1] - r.b;
  return r;
}

// z = Binv r on block k
__device__ __forceinline__ void precondition_block(const PcgSystem &S, int k, BlockRange br) {
  const double *B = S.binv + (long)k * 36;
  double rr[6];
  for (int i = 0; i < br.m; i++) rr[i] = S.r[br.b + i];
  for (int i = 0; i < br.m; i++) {
    double t = 0.0;
    for (int j = 0; j < br.m; j++) t += B[6 * i + j] * rr[j];
    S.z[br.b + i] = t;
  }
}

// scalars: [0] rz  [1] bb  [2] rr  [3] iterations  [4] relres
template <bool kSell>
__global__ void __launch_bounds__(kPcgThreads) k_pcg(PcgSystem S, const double *b, double *x,
                                                     double rtol, int maxit) {
  __shared__ double smem[40];
  volatile int *flags = S.flags;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gthreads = gridDim.x * blockDim.x;
  const int nb = gridDim.x;
  double *part = S.partials;          // [3*nb]

  // r = b - A x ; (x is the initial guess)
  for_rows_Ax<kSell>(S, x, nullptr, [&](int row, double ax) { S.r[row] = b[row] - ax; });
  if (kSell) long_row_chunks(S, x, [&](int c, int, double t) { S.chunk_part[c] = t; });
  if (!grid_barrier(S.barrier, flags)) return;
  if (kSell && S.nlong > 0) {
    long_row_sums(S, [&](int row, double ax) { S.r[row] = b[row] - ax; });
    if (!grid_barrier(S.barrier, flags)) return;
  }
  double lrz = 0.0, lbb = 0.0, lrr = 0.0;
  bool p_out = false;                 // an entry of p outside the split's range
  for (int k = gtid; k < S.nblk; k += gthreads) {
    const BlockRange br = block_range(S, k);
    precondition_block(S, k, br);
    for (int i = br.b; i < br.b + br.m; i++) {
      S.p[i] = S.z[i];
      if (kSell) {
        S.p2[i] = split2(S.z[i]);
        p_out |= !ff_range(S.z[i]);
      }
      lrz += S.r[i] * S.z[i];
      lbb += b[i] * b[i];
      lrr += S.r[i] * S.r[i];
    }
  }
  // p = z is read across blocks in the next SpMV: barrier before it
  if (kSell && p_out) flags[2] = 1;   // FP64 SpMV from now on (read after a barrier)
  lrz = block_reduce(lrz, smem);
  if (threadIdx.x == 0) part[blockIdx.x] = lrz;
  lbb = block_reduce(lbb, smem);
  if (threadIdx.x == 0) part[nb + blockIdx.x] = lbb;
  lrr = block_reduce(lrr, smem);
  if (threadIdx.x == 0) part[2 * nb + blockIdx.x] = lrr;
  if (!grid_barrier(S.barrier, flags)) return;
  double rz = sum_partials(part, nb, smem);
  const double bb = sum_partials(part + nb, nb, smem);
  double rr = sum_partials(part + 2 * nb, nb, smem);
  const double bnorm = sqrt(bb);
  int it = 0;
  int status = 0;
  if (bnorm == 0.0 || sqrt(rr) <= rtol * bnorm) {
    status = 1;
  }
  while (status == 0 && it < maxit) {
    // q = A p ; pq = p.q
    if (!grid_barrier(S.barrier, flags)) return;   // partial sums consumed
    double lpq = 0.0;
    for_rows_Ax<kSell>(S, S.p, flags[2] ? nullptr : S.p2, [&](int row, double ap) {
      S.q[row] = ap;
      lpq += ap * S.p[row];
    });
    if (kSell)
      long_row_chunks(S, S.p, [&](int c, int row, double t) {
        S.chunk_part[c] = t;
        lpq += t * S.p[row];
      });
    lpq = block_reduce(lpq, smem);
    if (threadIdx.x == 0) part[blockIdx.x] = lpq;
    if (!grid_barrier(S.barrier, flags)) return;
    const double pq = sum_partials(part, nb, smem);
    if (!(pq > 0.0)) { status = -1; break; }
    const double alpha = rz / pq;
    if (kSell) long_row_sums(S, [&](int row, double ap) { S.q[row] = ap; });
    if (!grid_barrier(S.barrier, flags)) return;   // partial sums consumed, q complete
    lrz = 0.0; lrr = 0.0;
    for (int k = gtid; k < S.nblk; k += gthreads) {
      const BlockRange br = block_range(S, k);
      for (int i = br.b; i < br.b + br.m; i++) {
        x[i] += alpha * S.p[i];
        S.r[i] -= alpha * S.q[i];
      }
      precondition_block(S, k, br);
      for (int i = br.b; i < br.b + br.m; i++) {
        lrz += S.r[i] * S.z[i];
        lrr += S.r[i] * S.r[i];
      }
    }
    lrz = block_reduce(lrz, smem);
    if (threadIdx.x == 0) part[blockIdx.x] = lrz;
    lrr = block_reduce(lrr, smem);
    if (threadIdx.x == 0) part[nb + blockIdx.x] = lrr;
    if (!grid_barrier(S.barrier, flags)) return;
    const double rz_new = sum_partials(part, nb, smem);
    rr = sum_partials(part + nb, nb, smem);
    it++;
    if (sqrt(rr) <= rtol * bnorm) { status = 1; break; }
    const double beta = rz_new / rz;
    rz = rz_new;
    p_out = false;
    for (int k = gtid; k < S.nblk; k += gthreads) {
      const BlockRange br = block_range(S, k);
      for (int i = br.b; i < br.b + br.m; i++) {
        const double pi = S.z[i] + beta * S.p[i];
        S.p[i] = pi;
        if (kSell) {
          S.p2[i] = split2(pi);
          p_out |= !ff_range(pi);
        }
      }
    }
    if (kSell && p_out) flags[2] = 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S.scalars[3] = it;
    S.scalars[4] = bnorm > 0.0 ? sqrt(rr) / bnorm : 0.0;
    S.flags[1] = status;
  }
}

// Diagonal blocks of the CSR matrix, inverted by Gauss-Jordan with partial
// pivoting (blocks are at most 6 x 6: the free dofs of one node).
__global__ void k_factor_blocks(PcgSystem S) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.nblk) return;
  const int b = S.blk_start[k], m = S.blk_start[k + 1] - b;
  double A[6][12];
  for (int i = 0; i < m; i++) {
    for (int j = 0; j < 2 * m; j++) A[i][j] = (j == m + i) ? 1.0 : 0.0;
    const int row = b + i;
    for (int q = S.rowptr[row]; q < S.rowptr[row + 1]; q++) {
      const int c = S.colidx[q];
      if (c >= b && c < b + m) A[i][c - b] = S.vals[q];
    }
  }
  bool singular = false;
  for (int c = 0; c < m; c++) {
    int piv = c;
    double best = fabs(A[c][c]);
    for (int i = c + 1; i < m; i++)
      if (fabs(A[i][c]) > best) { best = fabs(A[i][c]); piv = i; }
    if (best == 0.0) { singular = true; break; }
    if (piv != c)
      for (int j = 0; j < 2 * m; j++) { double t = A[c][j]; A[c][j] = A[piv][j]; A[piv][j] = t; }
    const double inv = 1.0 / A[c][c];
    for (int j = 0; j < 2 * m; j++) A[c][j] *= inv;
    for (int i = 0; i < m; i++) {
      if (i == c) continue;
      const double f = A[i][c];
      if (f != 0.0)
        for (int j = 0; j < 2 * m; j++) A[i][j] -= f * A[c][j];
    }
  }
  double *B = S.binv + (long)k * 36;
  for (int i = 0; i < 36; i++) B[i] = 0.0;
  if (singular) {
    // fall back to the point-Jacobi inverse of whatever diagonal exists
    for (int i = 0; i < m; i++) {
      double d = 0.0;
      const int row = b + i;
      for (int q = S.rowptr[row]; q < S.rowptr[row + 1]; q++)
        if (S.colidx[q] == row) d = S.vals[q];
      B[6 * i + i] = d != 0.0 ? 1.0 / d : 1.0;
    }
    return;
  }
  for (int i = 0; i < m; i++)
    for (int j = 0; j < m; j++) B[6 * i + j] = A[i][m + j];
}

// CSR values into the sliced ELL copy, split into (hi, lo), thread per row;
// row_ff records whether every value of the row lies in the split's range.
__global__ void k_pack_sell(PcgSystem S) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= S.n) return;
  const int b = S.rowptr[row], len = S.rowptr[row + 1] - b;
  if (len > S.sell_cap) return;
  float2 *vp = S.sell_vals + S.sell_off[row >> 5] + (row & 31);
  bool ok = true;
  for (int k = 0; k < len; k++) {
    const double v = S.vals[b + k];
    ok = ok && ff_range(v);
    vp[32 * k] = split2(v);
  }
  S.row_ff[row] = ok ? 1 : 0;
}

int g_max_blocks = -1, g_sell_max_blocks = -1;

int max_coresident(const void *kernel) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kPcgThreads, 0);
  if (per < 1) per = 1;
  return sms * per;
}

}  // namespace

int pcg_max_blocks() {
  if (g_max_blocks < 0) g_max_blocks = max_coresident((const void *)k_pcg<false>);
  return g_max_blocks;
}

int pcg_sell_max_blocks() {
  if (g_sell_max_blocks < 0) g_sell_max_blocks = max_coresident((const void *)k_pcg<true>);
  return g_sell_max_blocks;
}

void sell_layout(int n, const int *rowptr, int cap, std::vector<long> &off,
                 std::vector<int> &chunk_row, std::vector<int> &chunk_beg,
                 std::vector<int> &long_chunk0) {
  const int ns = (n + 31) / 32;
  off.assign((size_t)ns + 1, 0);
  chunk_row.clear();
  chunk_beg.clear();
  long_chunk0.assign(1, 0);
  for (int s = 0; s < ns; s++) {
    int w = 0;
    for (int r = 32 * s; r < std::min(n, 32 * s + 32); r++) {
      const int len = rowptr[r + 1] - rowptr[r];
      if (len <= cap) {
        w = std::max(w, len);
        continue;
      }
      for (int k = rowptr[r]; k < rowptr[r + 1]; k += kLongChunk) {
        chunk_row.push_back(r);
        chunk_beg.push_back(k);
      }
      long_chunk0.push_back((int)chunk_row.size());
    }
    off[s + 1] = off[s] + 32L * w;
  }
}

void sell_columns(int n, const int *rowptr, const int *colidx, int cap,
                  const std::vector<long> &off, std::vector<int> &cols) {
  cols.assign((size_t)off.back(), 0);
  for (int r = 0; r < n; r++) {
    if (rowptr[r + 1] - rowptr[r] > cap) continue;
    for (int k = rowptr[r]; k < rowptr[r + 1]; k++)
      cols[(size_t)off[r / 32] + 32L * (k - rowptr[r]) + r % 32] = colidx[k];
  }
}

int pcg_factor_blocks(const PcgSystem &S, cudaStream_t s) {
  if (S.nblk == 0) return 0;
  k_factor_blocks<<<(S.nblk + 127) / 128, 128, 0, s>>>(S);
  if (cudaGetLastError() != cudaSuccess) return XG_ECUDA;
  if (S.sell_vals && S.n > 0) {
    k_pack_sell<<<(S.n + 255) / 256, 256, 0, s>>>(S);
    if (cudaGetLastError() != cudaSuccess) return XG_ECUDA;
  }
  return 0;
}

int pcg_solve(const PcgSystem &S, const double *b, double *x, double rtol, int maxit,
              int *iters, double *relres, cudaStream_t s, int rows_per_block) {
  if (S.n == 0) {
    if (iters) *iters = 0;
    if (relres) *relres = 0.0;
    return 0;
  }
  // about four rows per warp: SpMV rows are latency-bound chains (row
  // pointer, column index, vector entry), so mid-size systems want many
  // warps; the grid barrier's cost grows slowly with the block count
  const long rpb = rows_per_block > 0 ? rows_per_block : 64;
  long want = ((long)S.n + rpb - 1) / rpb;
  int nb = (int)(want < 1 ? 1 : want);
  const bool sell = S.sell_vals != nullptr;
  const int maxb = sell ? pcg_sell_max_blocks() : pcg_max_blocks();
  if (nb > maxb) nb = maxb;
  if (cudaMemsetAsync(S.barrier, 0, 2 * sizeof(unsigned int), s) != cudaSuccess) return XG_ECUDA;
  if (cudaMemsetAsync(S.flags, 0, 4 * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  PcgSystem Sv = S;
  void *args[] = {(void *)&Sv, (void *)&b, (void *)&x, (void *)&rtol, (void *)&maxit};
  const void *kernel = sell ? (const void *)k_pcg<true> : (const void *)k_pcg<false>;
  cudaError_t err = cudaLaunchCooperativeKernel(kernel, dim3(nb), dim3(kPcgThreads), args, 0, s);
  if (err != cudaSuccess) return XG_ECUDA;
  int hflags[4];
  double hs[8];
  if (cudaMemcpyAsync(hflags, S.flags, sizeof hflags, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return XG_ECUDA;
  if (cudaMemcpyAsync(hs, S.scalars, sizeof hs, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return XG_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return XG_ECUDA;
  if (iters) *iters = (int)hs[3];
  if (relres) *relres = hs[4];
  if (hflags[0] != 0) return XG_ESOLVE;      // barrier timeout
  if (hflags[1] != 1) return XG_ESOLVE;      // breakdown or maxit
  return 0;
}

}  // namespace xg
