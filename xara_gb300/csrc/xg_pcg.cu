// xg_pcg.cu -- block-Jacobi preconditioned conjugate gradients: vectors,
// inner products and the preconditioner in FP64, the SpMV's products in
// float-float over a node-block copy of the matrix (FP64 warp per CSR row
// without one).
//
// The whole solve is one cooperative, persistent launch: every block owns a
// grid-stride share of the node rows (of the rows without the copy), and the
// three inner products of an iteration are reduced deterministically
// (fixed-order block partials, then every block sums the partials in the same
// order), so the iterates are bit-identical run to run.  Blocks meet at a
// grid barrier whose wait is bounded by the global timer: a block that waits
// longer than kBarrierTimeoutNs raises flags[0] and every block leaves the
// solve, so a fault can never hang the GPU.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <iterator>
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

__device__ double block_reduce_max(double v, double *smem) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) smem[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = (lane < (int)(blockDim.x >> 5)) ? smem[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_down_sync(0xffffffffu, t, o));
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// Largest of partials[0..nb) (all >= 0), broadcast to the whole block.
__device__ double max_partials(const double *partials, int nb, double *smem) {
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s = fmax(s, partials[i]);
  s = block_reduce_max(s, smem);
  if (threadIdx.x == 0) smem[32] = s;
  __syncthreads();
  const double r = smem[32];
  __syncthreads();
  return r;
}

// Power-of-two scale of p's split: p2 = p * 2^-s with s the exponent of a
// bound on max |p|, so that every entry of the split lies below 2 whatever
// the size of the residual (p shrinks with it over a solve; a fixed range
// would send the late iterations to FP64).  Entries more than 2^126 below
// the bound fall into the single-precision subnormals or to zero: a change
// of at most 2^-126 of max |p| per entry, below the split's own rounding.
__device__ __forceinline__ int split_exponent(double bound) {
  if (!(bound > 0.0) || !isfinite(bound)) return 0;
  const int e = (int)(((unsigned)__double2hiint(bound) >> 20) & 0x7ff) - 1023;
  return e < -1000 ? -1000 : (e > 1000 ? 1000 : e);
}
__device__ __forceinline__ double pow2(int e) {
  return __hiloint2double((int)((unsigned)(1023 + e) << 20), 0);
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

// Order of the stored inverse diagonal blocks: the node-block order, or 6
// (each block padded to 6 x 6) for a system without a node-block copy.
__device__ __forceinline__ int binv_order(const PcgSystem &S) { return S.kb > 0 ? S.kb : 6; }

// Stride of a node's slots in p2: the block order, 3 rounded up to 4 so that
// a node's entries are one aligned 32-byte sector.
template <int KB>
struct NodeSlots {
  static constexpr int kStride = KB == 3 ? 4 : KB;
};

template <int KB>
__device__ __forceinline__ void load_p2_node(const float2 *p2, int j, float2 *xb) {
  constexpr int KS = NodeSlots<KB>::kStride;
  if constexpr (KS == 1) {
    xb[0] = p2[j];
  } else {
    const float4 *src = reinterpret_cast<const float4 *>(p2 + (long)j * KS);
#pragma unroll
    for (int t = 0; t < KS / 2; t++) {
      const float4 v = src[t];
      xb[2 * t] = make_float2(v.x, v.y);
      xb[2 * t + 1] = make_float2(v.z, v.w);
    }
  }
}

// Node-block sliced ELL copy of the matrix, thread per node row: the
// equations of node i (its diagonal block, m <= KB of them) against the
// nodes j it couples to, each coupling a KB x KB block (zero-padded where a
// node has fewer free dofs).  Slice s holds node rows 32s .. 32s+31; block k
// of node row i has its column node at nb_cols[nb_off[s] + 32k + i%32] and
// entry (a, b) at nb_vals[nb_off[s]*KB*KB + (k*KB*KB + a*KB + b)*32 + i%32],
// so a warp's 32 node rows read each entry position with one coalesced
// access and one column index serves KB*KB values.  p is held split into
// (hi, lo) float pairs, node-major with NodeSlots<KB>::kStride slots per
// node (p2), so a block's KB entries of p are one aligned load.  Each row is
// summed in float-float (xg_ff.h) over the node's blocks in order, even and
// odd blocks into separate partial sums, a fixed order.
template <int KB>
__device__ __forceinline__ void node_row_ff(const PcgSystem &S, int i, double *y) {
  constexpr int KS = NodeSlots<KB>::kStride;
  constexpr int KK = KB * KB;
  const int len = S.nb_len[i];
  const long base = S.nb_off[i >> 5];
  const int *cp = S.nb_cols + base + (i & 31);
  const float2 *vp = S.nb_vals + base * KK + (i & 31);
  float h0[KB], l0[KB], h1[KB], l1[KB];
#pragma unroll
  for (int a = 0; a < KB; a++) h0[a] = l0[a] = h1[a] = l1[a] = 0.f;
  int k = 0;
  for (; k + 2 <= len; k += 2) {
    const int j0 = __ldcs(cp + 32 * k), j1 = __ldcs(cp + 32 * (k + 1));
    float2 x0[KS], x1[KS];
    load_p2_node<KB>(S.p2, j0, x0);
    load_p2_node<KB>(S.p2, j1, x1);
    const float2 *v0 = vp + 32L * KK * k;
    const float2 *v1 = v0 + 32 * KK;
#pragma unroll
    for (int a = 0; a < KB; a++)
#pragma unroll
      for (int b = 0; b < KB; b++) ff_madd(__ldcs(v0 + 32 * (a * KB + b)), x0[b], h0[a], l0[a]);
#pragma unroll
    for (int a = 0; a < KB; a++)
#pragma unroll
      for (int b = 0; b < KB; b++) ff_madd(__ldcs(v1 + 32 * (a * KB + b)), x1[b], h1[a], l1[a]);
  }
  if (k < len) {
    const int j0 = __ldcs(cp + 32 * k);
    float2 x0[KS];
    load_p2_node<KB>(S.p2, j0, x0);
    const float2 *v0 = vp + 32L * KK * k;
#pragma unroll
    for (int a = 0; a < KB; a++)
#pragma unroll
      for (int b = 0; b < KB; b++) ff_madd(__ldcs(v0 + 32 * (a * KB + b)), x0[b], h0[a], l0[a]);
  }
#pragma unroll
  for (int a = 0; a < KB; a++)
    y[a] = ((double)h0[a] + (double)l0[a]) + ((double)h1[a] + (double)l1[a]);
}

// f(row, (A x)[row]) for this thread's rows.  KB > 0: thread per node row
// over the node-block copy (node rows with more than S.nb_cap blocks are
// left to long_row_chunks), in float-float against p2 = x * 2^-s when ff is
// set and the node's values lie in the split's range (the sums times
// scale = 2^s), else each of its rows in FP64 from the CSR arrays against x
// (the initial residual).  KB == 0: warp per CSR row (lane 0 calls f).
template <int KB, typename F>
__device__ __forceinline__ void for_rows_Ax(const PcgSystem &S, const double *x, bool ff,
                                            double scale, F f) {
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gthreads = gridDim.x * blockDim.x;
  if constexpr (KB > 0) {
    for (int i = gtid; i < S.nblk; i += gthreads) {
      if (S.nb_len[i] > S.nb_cap) continue;
      const int b = S.blk_start[i], m = S.blk_start[i + 1] - b;
      if (ff && S.blk_ff[i]) {
        double y[KB];
        node_row_ff<KB>(S, i, y);
#pragma unroll
        for (int a = 0; a < KB; a++)
          if (a < m) f(b + a, y[a] * scale);
      } else {
        for (int a = 0; a < m; a++) f(b + a, csr_row64(S, b + a, x));
      }
    }
  } else {
    const int lane = threadIdx.x & 31;
    for (int row = gtid >> 5; row < S.n; row += gthreads >> 5) {
      const double ax = spmv_row(S, row, x, lane);
      if (lane == 0) f(row, ax);
    }
  }
}

// The rows of node rows with more than S.nb_cap blocks (a node tied to a
// whole face by a multi-point constraint couples to every node of that
// face) in chunks of at most kLongChunk CSR entries, a warp per chunk:
// g(chunk, row, partial) on lane 0.  A warp per row would leave one warp
// thousands of entries.
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

// z = Binv r on block k (MB: the largest block order, so that the block's
// entries of r stay in registers)
template <int MB>
__device__ __forceinline__ void precondition_block(const PcgSystem &S, int k, BlockRange br) {
  const int bo = binv_order(S);
  const double *B = S.binv + (long)k * bo * bo;
  double rr[MB];
#pragma unroll
  for (int i = 0; i < MB; i++) rr[i] = i < br.m ? S.r[br.b + i] : 0.0;
#pragma unroll
  for (int i = 0; i < MB; i++) {
    if (i >= br.m) break;
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < MB; j++)
      if (j < br.m) t += B[bo * i + j] * rr[j];
    S.z[br.b + i] = t;
  }
}

// scalars: [0] rz  [1] bb  [2] rr  [3] iterations  [4] relres
// partials: [0, 3 nb) the inner products' block sums; with KB > 0 also
// [3 nb, 4 nb) the blocks' largest |z| or |p| for the split's scale.
// KB > 0: one 512-thread block per SM with up to 128 registers a thread, so
// that a thread keeps two whole blocks' loads of the SpMV in flight.
template <int KB>
__global__ void __launch_bounds__(kPcgThreads, KB > 0 ? 1 : 2)
    k_pcg(PcgSystem S, const double *b, double *x, double rtol, int maxit) {
  __shared__ double smem[40];
  volatile int *flags = S.flags;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gthreads = gridDim.x * blockDim.x;
  const int nb = gridDim.x;
  double *part = S.partials;
  constexpr int KS = NodeSlots<(KB > 0 ? KB : 1)>::kStride;

  // r = b - A x ; (x is the initial guess)
  for_rows_Ax<KB>(S, x, false, 1.0, [&](int row, double ax) { S.r[row] = b[row] - ax; });
  if (KB > 0) long_row_chunks(S, x, [&](int c, int, double t) { S.chunk_part[c] = t; });
  if (!grid_barrier(S.barrier, flags)) return;
  if (KB > 0 && S.nlong > 0) {
    long_row_sums(S, [&](int row, double ax) { S.r[row] = b[row] - ax; });
    if (!grid_barrier(S.barrier, flags)) return;
  }
  double lrz = 0.0, lbb = 0.0, lrr = 0.0, lmax = 0.0;
  for (int k = gtid; k < S.nblk; k += gthreads) {
    const BlockRange br = block_range(S, k);
    precondition_block<(KB > 0 ? KB : 6)>(S, k, br);
    for (int i = br.b; i < br.b + br.m; i++) {
      S.p[i] = S.z[i];
      lmax = fmax(lmax, fabs(S.z[i]));
      lrz += S.r[i] * S.z[i];
      lbb += b[i] * b[i];
      lrr += S.r[i] * S.r[i];
    }
  }
  lrz = block_reduce(lrz, smem);
  if (threadIdx.x == 0) part[blockIdx.x] = lrz;
  lbb = block_reduce(lbb, smem);
  if (threadIdx.x == 0) part[nb + blockIdx.x] = lbb;
  lrr = block_reduce(lrr, smem);
  if (threadIdx.x == 0) part[2 * nb + blockIdx.x] = lrr;
  if (KB > 0) {
    lmax = block_reduce_max(lmax, smem);
    if (threadIdx.x == 0) part[3 * nb + blockIdx.x] = lmax;
  }
  if (!grid_barrier(S.barrier, flags)) return;
  double rz = sum_partials(part, nb, smem);
  const double bb = sum_partials(part + nb, nb, smem);
  double rr = sum_partials(part + 2 * nb, nb, smem);
  int sp = 0;                         // p2 = p * 2^-sp
  if (KB > 0) {
    const double bound = max_partials(part + 3 * nb, nb, smem);
    if (!isfinite(bound)) flags[2] = 1;   // FP64 SpMV throughout
    sp = split_exponent(bound);
    const double down = pow2(-sp);
    for (int k = gtid; k < S.nblk; k += gthreads) {
      const BlockRange br = block_range(S, k);
      for (int i = br.b; i < br.b + br.m; i++)
        S.p2[(long)k * KS + (i - br.b)] = split2(S.p[i] * down);
    }
  }
  // p and its split are read across blocks in the next SpMV: the barrier at
  // the top of the loop comes first
  const double bnorm = sqrt(bb);
  int it = 0;
  int status = 0;
  if (bnorm == 0.0 || sqrt(rr) <= rtol * bnorm) {
    status = 1;
  }
  while (status == 0 && it < maxit) {
    // q = A p ; pq = p.q
    if (!grid_barrier(S.barrier, flags)) return;   // partial sums consumed, p complete
    double lpq = 0.0, lpmax = 0.0;
    for_rows_Ax<KB>(S, S.p, flags[2] == 0, pow2(sp), [&](int row, double ap) {
      S.q[row] = ap;
      const double pr = S.p[row];
      lpq += ap * pr;
      lpmax = fmax(lpmax, fabs(pr));
    });
    if (KB > 0)
      long_row_chunks(S, S.p, [&](int c, int row, double t) {
        S.chunk_part[c] = t;
        lpq += t * S.p[row];
        lpmax = fmax(lpmax, fabs(S.p[row]));
      });
    lpq = block_reduce(lpq, smem);
    if (threadIdx.x == 0) part[blockIdx.x] = lpq;
    if (KB > 0) {
      lpmax = block_reduce_max(lpmax, smem);
      if (threadIdx.x == 0) part[3 * nb + blockIdx.x] = lpmax;
    }
    if (!grid_barrier(S.barrier, flags)) return;
    const double pq = sum_partials(part, nb, smem);
    const double pmax = KB > 0 ? max_partials(part + 3 * nb, nb, smem) : 0.0;
    if (!(pq > 0.0)) { status = -1; break; }
    const double alpha = rz / pq;
    if (KB > 0) long_row_sums(S, [&](int row, double ap) { S.q[row] = ap; });
    if (!grid_barrier(S.barrier, flags)) return;   // partial sums consumed, q complete
    lrz = 0.0; lrr = 0.0;
    double lzmax = 0.0;
    for (int k = gtid; k < S.nblk; k += gthreads) {
      const BlockRange br = block_range(S, k);
      for (int i = br.b; i < br.b + br.m; i++) {
        x[i] += alpha * S.p[i];
        S.r[i] -= alpha * S.q[i];
      }
      precondition_block<(KB > 0 ? KB : 6)>(S, k, br);
      for (int i = br.b; i < br.b + br.m; i++) {
        lrz += S.r[i] * S.z[i];
        lrr += S.r[i] * S.r[i];
        lzmax = fmax(lzmax, fabs(S.z[i]));
      }
    }
    lrz = block_reduce(lrz, smem);
    if (threadIdx.x == 0) part[blockIdx.x] = lrz;
    lrr = block_reduce(lrr, smem);
    if (threadIdx.x == 0) part[nb + blockIdx.x] = lrr;
    if (KB > 0) {
      lzmax = block_reduce_max(lzmax, smem);
      if (threadIdx.x == 0) part[3 * nb + blockIdx.x] = lzmax;
    }
    if (!grid_barrier(S.barrier, flags)) return;
    const double rz_new = sum_partials(part, nb, smem);
    rr = sum_partials(part + nb, nb, smem);
    const double zmax = KB > 0 ? max_partials(part + 3 * nb, nb, smem) : 0.0;
    it++;
    if (sqrt(rr) <= rtol * bnorm) { status = 1; break; }
    const double beta = rz_new / rz;
    rz = rz_new;
    double down = 1.0;
    if (KB > 0) {
      // |z + beta p| <= max|z| + beta max|p| (beta > 0)
      const double bound = zmax + fabs(beta) * pmax;
      if (!isfinite(bound) && threadIdx.x == 0) flags[2] = 1;
      sp = split_exponent(bound);
      down = pow2(-sp);
    }
    for (int k = gtid; k < S.nblk; k += gthreads) {
      const BlockRange br = block_range(S, k);
      for (int i = br.b; i < br.b + br.m; i++) {
        const double pi = S.z[i] + beta * S.p[i];
        S.p[i] = pi;
        if (KB > 0) S.p2[(long)k * KS + (i - br.b)] = split2(pi * down);
      }
    }
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
  const int bo = binv_order(S);
  double *B = S.binv + (long)k * bo * bo;
  for (int i = 0; i < bo * bo; i++) B[i] = 0.0;
  if (singular) {
    // fall back to the point-Jacobi inverse of whatever diagonal exists
    for (int i = 0; i < m; i++) {
      double d = 0.0;
      const int row = b + i;
      for (int q = S.rowptr[row]; q < S.rowptr[row + 1]; q++)
        if (S.colidx[q] == row) d = S.vals[q];
      B[bo * i + i] = d != 0.0 ? 1.0 / d : 1.0;
    }
    return;
  }
  for (int i = 0; i < m; i++)
    for (int j = 0; j < m; j++) B[bo * i + j] = A[i][m + j];
}

// CSR values into the node-block copy, split into (hi, lo), thread per node
// row (once per matrix); blk_ff records whether every value of the node's
// rows lies in the split's range.  Slots no CSR entry maps to stay zero.
__global__ void k_pack_blocks(PcgSystem S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.nblk) return;
  bool ok = true;
  if (S.nb_len[i] <= S.nb_cap) {
    for (int r = S.blk_start[i]; r < S.blk_start[i + 1]; r++)
      for (int q = S.rowptr[r]; q < S.rowptr[r + 1]; q++) {
        const double v = S.vals[q];
        ok = ok && ff_range(v);
        S.nb_vals[S.nb_pos[q]] = split2(v);
      }
  }
  S.blk_ff[i] = ok ? 1 : 0;
}

int g_max_blocks[5] = {-1, -1, -1, -1, -1};

int kb_index(int kb) { return kb == 1 ? 1 : kb == 2 ? 2 : kb == 3 ? 3 : kb == 6 ? 4 : 0; }

const void *pcg_kernel(int kb) {
  switch (kb) {
    case 1: return (const void *)k_pcg<1>;
    case 2: return (const void *)k_pcg<2>;
    case 3: return (const void *)k_pcg<3>;
    case 6: return (const void *)k_pcg<6>;
    default: return (const void *)k_pcg<0>;
  }
}

int max_coresident(const void *kernel) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kPcgThreads, 0);
  if (per < 1) per = 1;
  return sms * per;
}

int coresident(int kb) {
  int &c = g_max_blocks[kb_index(kb)];
  if (c < 0) c = max_coresident(pcg_kernel(kb));
  return c;
}

}  // namespace

int pcg_max_blocks() {
  int m = 1;
  for (int kb : {0, 1, 2, 3, 6}) m = std::max(m, coresident(kb));
  return m;
}

int block_ell_layout(int n, const int *rowptr, const int *colidx, int nblk, const int *blk_start,
                     int cap, BlockEll &h) {
  h = BlockEll{};
  int maxm = 0;
  for (int i = 0; i < nblk; i++) maxm = std::max(maxm, blk_start[i + 1] - blk_start[i]);
  if (nblk == 0 || maxm < 1 || maxm > 6) return 0;
  const int kb = maxm == 1 ? 1 : maxm == 2 ? 2 : maxm == 3 ? 3 : 6;
  std::vector<int> node_of(n);
  for (int i = 0; i < nblk; i++)
    for (int r = blk_start[i]; r < blk_start[i + 1]; r++) node_of[r] = i;
  // block columns of every node row: the union over its rows (sorted)
  std::vector<long> lptr(nblk + 1, 0);
  std::vector<int> lst, row_l, merged;
  std::vector<int> all;
  all.reserve((size_t)rowptr[n] / (kb * kb) + nblk);
  for (int i = 0; i < nblk; i++) {
    lst.clear();
    for (int r = blk_start[i]; r < blk_start[i + 1]; r++) {
      row_l.clear();
      for (int q = rowptr[r]; q < rowptr[r + 1]; q++) {
        const int j = node_of[colidx[q]];
        if (row_l.empty() || row_l.back() != j) row_l.push_back(j);
      }
      if (r == blk_start[i]) {
        lst.swap(row_l);
      } else if (row_l != lst) {
        merged.clear();
        std::set_union(lst.begin(), lst.end(), row_l.begin(), row_l.end(),
                       std::back_inserter(merged));
        lst.swap(merged);
      }
    }
    all.insert(all.end(), lst.begin(), lst.end());
    lptr[i + 1] = (long)all.size();
  }
  const int ns = (nblk + 31) / 32;
  h.off.assign((size_t)ns + 1, 0);
  h.len.assign(nblk, 0);
  h.chunk_row.clear();
  h.chunk_beg.clear();
  h.long_chunk0.assign(1, 0);
  for (int s = 0; s < ns; s++) {
    int w = 0;
    for (int i = 32 * s; i < std::min(nblk, 32 * s + 32); i++) {
      const int len = (int)(lptr[i + 1] - lptr[i]);
      h.len[i] = len;
      if (len <= cap) {
        w = std::max(w, len);
        continue;
      }
      for (int r = blk_start[i]; r < blk_start[i + 1]; r++) {
        for (int q = rowptr[r]; q < rowptr[r + 1]; q += kLongChunk) {
          h.chunk_row.push_back(r);
          h.chunk_beg.push_back(q);
        }
        h.long_chunk0.push_back((int)h.chunk_row.size());
      }
    }
    h.off[s + 1] = h.off[s] + 32L * w;
  }
  if (h.off.back() * kb * kb >= (long)INT32_MAX) return 0;   // positions as 32-bit ints
  h.cols.assign((size_t)h.off.back(), 0);
  h.pos.assign((size_t)rowptr[n], -1);
  for (int i = 0; i < nblk; i++) {
    const int len = h.len[i];
    if (len > cap) continue;
    const long base = h.off[i / 32];
    const int lane = i % 32;
    const int *L = all.data() + lptr[i];
    for (int k = 0; k < len; k++) h.cols[(size_t)base + 32L * k + lane] = L[k];
    for (int r = blk_start[i]; r < blk_start[i + 1]; r++) {
      const int a = r - blk_start[i];
      int k = 0;
      for (int q = rowptr[r]; q < rowptr[r + 1]; q++) {
        const int j = node_of[colidx[q]];
        while (L[k] != j) k++;
        const int b = colidx[q] - blk_start[j];
        h.pos[q] = (int)(base * kb * kb + ((long)(k * kb + a) * kb + b) * 32 + lane);
      }
    }
  }
  h.kb = kb;
  return kb;
}

size_t block_ell_bytes(const BlockEll &h, int nblk) {
  if (h.kb == 0) return 0;
  const int ks = h.kb == 3 ? 4 : h.kb;
  return (size_t)h.off.back() * (sizeof(int) + sizeof(float2) * h.kb * h.kb) +
         h.pos.size() * sizeof(int) + h.off.size() * sizeof(long) +
         (size_t)nblk * (sizeof(int) + 1 + ks * sizeof(float2));
}

int pcg_factor_blocks(const PcgSystem &S, cudaStream_t s) {
  if (S.nblk == 0) return 0;
  k_factor_blocks<<<(S.nblk + 127) / 128, 128, 0, s>>>(S);
  if (cudaGetLastError() != cudaSuccess) return XG_ECUDA;
  if (S.nb_vals && S.kb > 0) {
    k_pack_blocks<<<(S.nblk + 255) / 256, 256, 0, s>>>(S);
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
  const int kb = (S.nb_vals && S.kb > 0) ? S.kb : 0;
  const int maxb = coresident(kb);
  if (nb > maxb) nb = maxb;
  if (cudaMemsetAsync(S.barrier, 0, 2 * sizeof(unsigned int), s) != cudaSuccess) return XG_ECUDA;
  if (cudaMemsetAsync(S.flags, 0, 4 * sizeof(int), s) != cudaSuccess) return XG_ECUDA;
  PcgSystem Sv = S;
  if (kb == 0) Sv.nb_vals = nullptr;
  void *args[] = {(void *)&Sv, (void *)&b, (void *)&x, (void *)&rtol, (void *)&maxit};
  cudaError_t err =
      cudaLaunchCooperativeKernel(pcg_kernel(kb), dim3(nb), dim3(kPcgThreads), args, 0, s);
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
