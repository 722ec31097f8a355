// xg_noalloc.cu -- a block-Jacobi PCG entry point that allocates nothing.
//
// Some callers cannot allocate device memory when they solve: a host
// application whose device memory is owned by its own pool or by a framework
// allocator (the caching allocator of the Python layer, for one) has no
// spare allocation to give us, and a solver called inside a latency-bound
// loop cannot afford cudaMalloc/cudaFree, which synchronise the whole device
// and stall every other stream.  xg_pcg_solve_noalloc runs the same solver
// as xg_soe_solve on arrays the caller already holds, with its scratch in
// the fixed array below.
//
// The scratch is one file-scope __device__ array of XG_NOALLOC_MAX_DOUBLES
// doubles (32 MiB): every GPU that loads this library holds it until the
// process exits.  In host code the array's name is only a host-side
// stand-in, never a device address, so its device address is looked up with
// cudaGetSymbolAddress, in the current device's context, on every call.  All
// calls share the array and find the previous call's contents
// in it: the solver clears what must start at zero (the grid-barrier counter
// and the status words) and overwrites the rest before reading it.  Calls
// that overlap on the GPU (two streams, two host threads, two devices'
// worth of work on one device) race on the array and must be serialised by
// the caller.
#include <cuda_runtime.h>

#include <cstdio>

#include "xg_internal.h"

namespace {

__device__ __align__(256) double g_noalloc_scratch[XG_NOALLOC_MAX_DOUBLES];

int noalloc_fail(int code, const char *msg) {
  xg::record_error(msg);   // readable through xg_last_error()
  return code;
}

// Device address of the scratch array in the current device's context,
// looked up on every call (a cheap driver query), so that a context
// created again -- after cudaDeviceReset, say -- gets its own address.
double *scratch_for_current_device(int *err) {
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
    *err = XG_ECUDA;
    return nullptr;
  }
  *err = 0;
  return static_cast<double *>(p);
}

// Checks a caller-given block partition: starts at 0, ends at n, every block
// 1..6 equations (the node blocks the factor kernel inverts).
__global__ void k_check_blocks(int n, int nblk, const int *blk_start, int *bad) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0 && (blk_start[0] != 0 || blk_start[nblk] != n)) atomicExch(bad, 1);
  if (k >= nblk) return;
  const int m = blk_start[k + 1] - blk_start[k];
  if (m < 1 || m > 6) atomicExch(bad, 1);
}

// Checks caller-given CSR arrays: rowptr starts at 0 and never decreases,
// every column index lies in [0, n).
__global__ void k_check_csr(int n, const int *rowptr, const int *colidx, int *bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && rowptr[0] != 0) atomicExch(bad, 1);
  if (i >= n) return;
  const int b = rowptr[i], e = rowptr[i + 1];
  if (e < b) {
    atomicExch(bad, 1);
    return;
  }
  for (int k = b; k < e; k++)
    if (colidx[k] < 0 || colidx[k] >= n) {
      atomicExch(bad, 1);
      return;
    }
}

}  // namespace

extern "C" int xg_pcg_solve_noalloc(int n, const int *rowptr, const int *colidx,
                                    const double *vals, int nblk, const int *blk_start,
                                    const double *b, double *x, double rtol, int maxit,
                                    void *stream, int *iters, double *relres) {
  xg::record_error("");
  if (n < 0 || nblk < 1 || nblk > n || !rowptr || !colidx || !vals || !blk_start || !b || !x)
    return noalloc_fail(XG_EINVAL, "xg_pcg_solve_noalloc: bad argument");
  if (!(rtol > 0.0) || maxit < 1)
    return noalloc_fail(XG_EINVAL, "xg_pcg_solve_noalloc: bad tolerance or iteration limit");
  const long long nb = xg::pcg_max_blocks();
  // layout in doubles: binv[36*nblk] | r z p q [4n] | partials[3*nb+8] |
  // scalars[8] | barrier(2 uint) + flags(4 int) + check word [8 doubles]
  const long long need = 36LL * nblk + 4LL * n + 3LL * nb + 8 + 8 + 8;
  if (need > (long long)XG_NOALLOC_MAX_DOUBLES) {
    char msg[256];
    snprintf(msg, sizeof msg,
             "xg_pcg_solve_noalloc: system needs %lld scratch doubles, the fixed array holds "
             "%lld (n=%d equations, %d diagonal blocks)",
             need, (long long)XG_NOALLOC_MAX_DOUBLES, n, nblk);
    return noalloc_fail(XG_EINVAL, msg);
  }
  int err = 0;
  double *s = scratch_for_current_device(&err);
  if (!s) return noalloc_fail(err, "xg_pcg_solve_noalloc: cudaGetSymbolAddress failed");
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  xg::PcgSystem S{};
  S.n = n;
  S.rowptr = rowptr;
  S.colidx = colidx;
  S.vals = vals;
  S.nblk = nblk;
  S.blk_start = blk_start;
  double *q = s;
  S.binv = q;                 q += 36LL * nblk;
  S.r = q;                    q += n;
  S.z = q;                    q += n;
  S.p = q;                    q += n;
  S.q = q;                    q += n;
  S.partials = q;             q += 3 * nb + 8;
  S.scalars = q;              q += 8;
  S.barrier = reinterpret_cast<unsigned int *>(q);
  S.flags = reinterpret_cast<int *>(q + 1);
  int *check = reinterpret_cast<int *>(q + 3);

  // the partition must be safe for the factor kernel before it runs
  if (cudaMemsetAsync(check, 0, sizeof(int), st) != cudaSuccess)
    return noalloc_fail(XG_ECUDA, "xg_pcg_solve_noalloc: cudaMemsetAsync failed");
  k_check_blocks<<<(nblk + 255) / 256, 256, 0, st>>>(n, nblk, blk_start, check);
  k_check_csr<<<(n + 255) / 256, 256, 0, st>>>(n, rowptr, colidx, check);
  int bad = 0;
  if (cudaMemcpyAsync(&bad, check, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return noalloc_fail(XG_ECUDA, "xg_pcg_solve_noalloc: block check failed to run");
  if (bad)
    return noalloc_fail(XG_EINVAL,
                        "xg_pcg_solve_noalloc: blk_start must run from 0 to n in blocks of "
                        "1..6 equations, and every CSR column index must lie in [0, n)");

  if (xg::pcg_factor_blocks(S, st) != 0)
    return noalloc_fail(XG_ECUDA, "xg_pcg_solve_noalloc: block factorisation failed");
  if (cudaMemsetAsync(x, 0, sizeof(double) * (n > 0 ? n : 1), st) != cudaSuccess)
    return noalloc_fail(XG_ECUDA, "xg_pcg_solve_noalloc: cudaMemsetAsync failed");
  int it = 0;
  double rr = 0.0;
  const int r = xg::pcg_solve(S, b, x, rtol, maxit, &it, &rr, st);
  if (iters) *iters = it;
  if (relres) *relres = rr;
  if (r != 0) return noalloc_fail(r, "xg_pcg_solve_noalloc: PCG did not converge");
  return 0;
}
