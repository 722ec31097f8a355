// xg_linsoe.cpp -- a standalone linear system of equations solved on the
// device: the reference's LinearSOE interface (system_of_eqn/linearSOE/
// LinearSOE.h) for callers that keep their own element loop.  The pattern
// comes in as CSR with sorted columns per row; assembly follows
// SparseGenColLinSOE (sparseGEN/SparseGenColLinSOE.cpp:214-350: addA adds
// fact * m(i,j) where both equation numbers are >= 0, locating the column by
// a search of the row; addB / setB likewise) and accumulates in host memory,
// the way the reference's FE_Element loop feeds it; solve() runs the
// block-Jacobi PCG of the model path (node-block sliced ELL SpMV, long node
// rows in chunks)
// on the device and returns X to the host.  With `system ProfileSPD`
// (xg_linsoe_set_system) addA follows ProfileSPDLinSOE instead
// (profileSPD/ProfileSPDLinSOE.cpp:214-269: only the terms with row <= col,
// kept here in the lower triangle's slot (col, row)) and solve() factors
// with the device LDL' once per matrix (the reference's isAfactored), with
// ProfileSPDLinDirectSolver's pivot checks.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "xg_internal.h"

namespace {

int lfail(int code, const char *msg) {
  xg::record_error(msg);
  return code;
}

template <typename T>
struct DevArray {
  T *p = nullptr;
  int alloc(size_t n) {
    if (p) cudaFree(p);
    p = nullptr;
    if (n == 0) return 0;
    return cudaMalloc(&p, n * sizeof(T)) == cudaSuccess ? 0 : XG_ENOMEM;
  }
  int upload(const T *h, size_t n, cudaStream_t s) {
    if (alloc(n)) return XG_ENOMEM;
    if (n && cudaMemcpyAsync(p, h, n * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return XG_ECUDA;
    return 0;
  }
  ~DevArray() {
    if (p) cudaFree(p);
  }
};

}  // namespace

struct xg_linsoe {
  int n = 0;
  std::vector<int> rowptr, colidx, blk;
  std::vector<double> A, B, X;
  // device copies, set up at the first solve
  bool ready = false;
  cudaStream_t stream = nullptr;
  DevArray<int> rp, ci, bs, chunk_row, chunk_beg, long_chunk0, nb_cols, nb_len, nb_pos, flags;
  DevArray<long> nb_off;
  DevArray<unsigned int> barrier;
  DevArray<double> vals, b, x, binv, r, z, p, q, partials, scalars, chunk_part;
  DevArray<float2> nb_vals, p2;
  DevArray<unsigned char> blk_ff;
  xg::PcgSystem S{};
  // `system ProfileSPD`: the device LDL', factored once per matrix
  int system = XG_SYSTEM_BJPCG;
  xg::ProfileSolver prof;
  bool prof_factored = false;
  bool prof_vals_stale = true;

  ~xg_linsoe() {
    if (stream) cudaStreamDestroy(stream);
  }

  // Column slot of (row, col) in the pattern, or -1.
  long slot(int row, int col) const {
    const int *b = colidx.data() + rowptr[row], *e = colidx.data() + rowptr[row + 1];
    const int *it = std::lower_bound(b, e, col);
    return (it != e && *it == col) ? (long)(it - colidx.data()) : -1;
  }

  // Device copies of the pattern for the LDL' (and the envelope tiles).
  int setup_profile() {
    if (prof.ready()) return 0;
    if (!stream && cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess)
      return lfail(XG_ECUDA, "xg_linsoe: stream creation failed");
    const size_t nnz = colidx.size(), nv = std::max(n, 1);
    int e = rp.upload(rowptr.data(), rowptr.size(), stream);
    e |= ci.upload(colidx.data(), nnz, stream);
    e |= vals.alloc(std::max<size_t>(nnz, 1)) | b.alloc(nv) | x.alloc(nv);
    if (e) return lfail(XG_ENOMEM, "xg_linsoe: device allocation failed");
    return prof.setup(n, rowptr.data(), colidx.data(), rp.p, ci.p, vals.p, stream);
  }

  int setup() {
    if (ready) return 0;
    if (!stream && cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess)
      return lfail(XG_ECUDA, "xg_linsoe: stream creation failed");
    const int nblk = (int)blk.size() - 1;
    const size_t nnz = colidx.size(), nv = std::max(n, 1);
    constexpr int kCap = 96;
    xg::BlockEll h;
    xg::block_ell_layout(n, rowptr.data(), colidx.data(), nblk, blk.data(), kCap, h);
    size_t freeb = 0, totalb = 0;
    if (h.kb && (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess ||
                 xg::block_ell_bytes(h, nblk) > freeb / 2))
      h = xg::BlockEll{};
    int e = 0;
    e |= rp.upload(rowptr.data(), rowptr.size(), stream);
    e |= ci.upload(colidx.data(), nnz, stream);
    e |= bs.upload(blk.data(), blk.size(), stream);
    e |= vals.alloc(std::max<size_t>(nnz, 1)) | b.alloc(nv) | x.alloc(nv);
    e |= binv.alloc((size_t)std::max(nblk, 1) * 36);
    e |= r.alloc(nv) | z.alloc(nv) | p.alloc(nv) | q.alloc(nv);
    e |= partials.alloc(4 * (size_t)xg::pcg_max_blocks() + 8);
    e |= scalars.alloc(8) | barrier.alloc(2) | flags.alloc(4);
    size_t nvals = 0, np2 = 0;
    if (h.kb) {
      nvals = std::max<size_t>((size_t)h.off.back() * h.kb * h.kb, 1);
      np2 = (size_t)nblk * (h.kb == 3 ? 4 : h.kb);
      e |= nb_off.upload(h.off.data(), h.off.size(), stream);
      e |= nb_cols.upload(h.cols.data(), h.cols.size(), stream);
      e |= nb_len.upload(h.len.data(), h.len.size(), stream);
      e |= nb_pos.upload(h.pos.data(), h.pos.size(), stream);
      e |= nb_vals.alloc(nvals) | p2.alloc(np2) | blk_ff.alloc(std::max(nblk, 1));
      e |= chunk_row.upload(h.chunk_row.data(), h.chunk_row.size(), stream);
      e |= chunk_beg.upload(h.chunk_beg.data(), h.chunk_beg.size(), stream);
      e |= long_chunk0.upload(h.long_chunk0.data(), h.long_chunk0.size(), stream);
      e |= chunk_part.alloc(std::max<size_t>(h.chunk_row.size(), 1));
    }
    if (e) return lfail(XG_ENOMEM, "xg_linsoe: device allocation failed");
    if (h.kb && (cudaMemsetAsync(nb_vals.p, 0, nvals * sizeof(float2), stream) != cudaSuccess ||
                 cudaMemsetAsync(p2.p, 0, np2 * sizeof(float2), stream) != cudaSuccess))
      return lfail(XG_ECUDA, "xg_linsoe: set-up copies failed");
    S.n = n;
    S.rowptr = rp.p;
    S.colidx = ci.p;
    S.vals = vals.p;
    S.nblk = nblk;
    S.blk_start = bs.p;
    S.binv = binv.p;
    S.r = r.p;
    S.z = z.p;
    S.p = p.p;
    S.q = q.p;
    S.partials = partials.p;
    S.barrier = barrier.p;
    S.flags = flags.p;
    S.scalars = scalars.p;
    S.kb = h.kb;
    if (h.kb) {
      S.nb_off = nb_off.p;
      S.nb_cols = nb_cols.p;
      S.nb_len = nb_len.p;
      S.nb_pos = nb_pos.p;
      S.nb_vals = nb_vals.p;
      S.blk_ff = blk_ff.p;
      S.p2 = p2.p;
      S.nb_cap = kCap;
      S.nlong = (int)h.long_chunk0.size() - 1;
      S.nchunks = (int)h.chunk_row.size();
      S.chunk_row = chunk_row.p;
      S.chunk_beg = chunk_beg.p;
      S.long_chunk0 = long_chunk0.p;
      S.chunk_part = chunk_part.p;
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess)
      return lfail(XG_ECUDA, "xg_linsoe: set-up copies failed");
    ready = true;
    return 0;
  }
};

extern "C" {

int xg_linsoe_create(int n, const int *rowptr, const int *colidx, const int *blk_start, int nblk,
                     xg_linsoe **out) {
  if (!out || n < 0 || !rowptr || (n > 0 && !colidx) || nblk < 0 || (nblk > 0 && !blk_start))
    return lfail(XG_EINVAL, "xg_linsoe_create: bad argument");
  *out = nullptr;
  if (rowptr[0] != 0) return lfail(XG_EINVAL, "xg_linsoe_create: rowptr[0] must be 0");
  for (int i = 0; i < n; i++) {
    if (rowptr[i + 1] < rowptr[i]) return lfail(XG_EINVAL, "xg_linsoe_create: rowptr decreases");
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (colidx[k] < 0 || colidx[k] >= n || (k > rowptr[i] && colidx[k] <= colidx[k - 1]))
        return lfail(XG_EINVAL, "xg_linsoe_create: columns must be sorted, distinct, in range");
  }
  std::vector<int> blk;
  if (nblk > 0) {
    if (blk_start[0] != 0 || blk_start[nblk] != n)
      return lfail(XG_EINVAL, "xg_linsoe_create: blocks must run from 0 to n");
    for (int k = 0; k < nblk; k++)
      if (blk_start[k + 1] - blk_start[k] < 1 || blk_start[k + 1] - blk_start[k] > 6)
        return lfail(XG_EINVAL, "xg_linsoe_create: blocks of 1 to 6 equations");
    blk.assign(blk_start, blk_start + nblk + 1);
  } else {
    blk.resize(n + 1);
    for (int i = 0; i <= n; i++) blk[i] = i;   // point Jacobi
  }
  auto *s = new xg_linsoe;
  s->n = n;
  s->rowptr.assign(rowptr, rowptr + n + 1);
  s->colidx.assign(colidx, colidx + rowptr[n]);
  s->blk = std::move(blk);
  s->A.assign(rowptr[n], 0.0);
  s->B.assign(n, 0.0);
  s->X.assign(n, 0.0);
  *out = s;
  return 0;
}

void xg_linsoe_destroy(xg_linsoe *s) { delete s; }

int xg_linsoe_zero_a(xg_linsoe *s) {
  if (!s) return lfail(XG_EINVAL, "null system");
  std::fill(s->A.begin(), s->A.end(), 0.0);
  s->prof_factored = false;
  s->prof_vals_stale = true;
  return 0;
}

int xg_linsoe_set_system(xg_linsoe *s, int system) {
  if (!s || (system != XG_SYSTEM_BJPCG && system != XG_SYSTEM_PROFILE_SPD))
    return lfail(XG_EINVAL, "xg_linsoe_set_system: XG_SYSTEM_BJPCG or XG_SYSTEM_PROFILE_SPD");
  if (system != s->system) {
    // the two systems keep A in different forms: start from zero
    s->system = system;
    std::fill(s->A.begin(), s->A.end(), 0.0);
  }
  s->prof_factored = false;
  s->prof_vals_stale = true;
  return 0;
}

int xg_linsoe_zero_b(xg_linsoe *s) {
  if (!s) return lfail(XG_EINVAL, "null system");
  std::fill(s->B.begin(), s->B.end(), 0.0);
  return 0;
}

int xg_linsoe_add_a(xg_linsoe *s, const double *m, const int *id, int ndof, double fact) {
  if (!s || ndof < 0 || (ndof && (!m || !id))) return lfail(XG_EINVAL, "bad addA argument");
  if (fact == 0.0) return 0;
  s->prof_factored = false;
  s->prof_vals_stale = true;
  if (s->system == XG_SYSTEM_PROFILE_SPD) {
    // ProfileSPDLinSOE::addA (profileSPD/ProfileSPDLinSOE.cpp:214-269):
    // column-outer, row-inner, A(row, col) += m(row, col) for row <= col
    // only; the entry sits in the lower triangle's slot (col, row), which
    // the LDL' reads.
    for (int j = 0; j < ndof; j++) {
      const int col = id[j];
      if (col < 0 || col >= s->n) continue;
      for (int i = 0; i < ndof; i++) {
        const int row = id[i];
        if (row < 0 || row > col) continue;
        const long k = s->slot(col, row);
        if (k < 0) continue;
        s->A[k] += fact * m[(size_t)i * ndof + j];
      }
    }
    return 0;
  }
  // Column-outer, row-inner, as SparseGenColLinSOE::addA
  // (sparseGEN/SparseGenColLinSOE.cpp:263-313): an ID that names one
  // equation twice (nodes tied by a constraint) then sums the entry's terms
  // in the reference's order.  Equation numbers outside 0..n-1 and entries
  // outside the pattern are skipped, as the reference skips them.
  for (int j = 0; j < ndof; j++) {
    const int col = id[j];
    if (col < 0 || col >= s->n) continue;
    for (int i = 0; i < ndof; i++) {
      const int row = id[i];
      if (row < 0 || row >= s->n) continue;
      const long k = s->slot(row, col);
      if (k < 0) continue;
      s->A[k] += fact * m[(size_t)i * ndof + j];
    }
  }
  return 0;
}

int xg_linsoe_add_b(xg_linsoe *s, const double *v, const int *id, int ndof, double fact) {
  if (!s || ndof < 0 || (ndof && (!v || !id))) return lfail(XG_EINVAL, "bad addB argument");
  if (fact == 0.0) return 0;   // the quick return of SparseGenColLinSOE::addB
  for (int i = 0; i < ndof; i++) {
    // SparseGenColLinSOE::addB (:317-350) skips numbers outside 0..n-1
    if (id[i] < 0 || id[i] >= s->n) continue;
    s->B[id[i]] += fact * v[i];
  }
  return 0;
}

int xg_linsoe_set_b(xg_linsoe *s, const double *v, double fact) {
  if (!s || (s->n && !v)) return lfail(XG_EINVAL, "bad setB argument");
  if (fact == 0.0) return 0;   // SparseGenColLinSOE::setB leaves B as it is
  for (int i = 0; i < s->n; i++) s->B[i] = fact * v[i];
  return 0;
}

int xg_linsoe_get_a(const xg_linsoe *s, double *vals) {
  if (!s || (!vals && !s->A.empty())) return lfail(XG_EINVAL, "bad argument");
  std::copy(s->A.begin(), s->A.end(), vals);
  return 0;
}

// ProfileSPDLinDirectSolver::solve (profileSPD/ProfileSPDLinDirectSolver.cpp:
// 100-256): factor when A changed since the last factorisation, then the
// substitutions; a pivot that fails the reference's checks is XG_ESOLVE.
static int linsoe_solve_profile(xg_linsoe *s, int *iters, double *relres) {
  if (int e = s->setup_profile()) return e;
  cudaStream_t st = s->stream;
  if (s->prof_vals_stale &&
      cudaMemcpyAsync(s->vals.p, s->A.data(), s->A.size() * sizeof(double),
                      cudaMemcpyHostToDevice, st) != cudaSuccess)
    return lfail(XG_ECUDA, "xg_linsoe_solve: copy of A failed");
  s->prof_vals_stale = false;
  if (!s->prof_factored) {
    int bad = -1;
    if (s->prof.factor(st, &bad) != 0) {
      char msg[160];
      if (bad >= 0)
        snprintf(msg, sizeof msg, "xg_linsoe_solve: ProfileSPD pivot %d fails the check (aii == "
                 "0, |aii| <= 1e-12, or a first pivot <= 0)", bad);
      else
        snprintf(msg, sizeof msg, "xg_linsoe_solve: ProfileSPD factorisation wait timed out");
      return lfail(XG_ESOLVE, msg);
    }
    s->prof_factored = true;
  }
  const double *bp = s->b.p;
  double *xp = s->x.p;
  if (cudaMemcpyAsync(s->b.p, s->B.data(), s->B.size() * sizeof(double), cudaMemcpyHostToDevice,
                      st) != cudaSuccess)
    return lfail(XG_ECUDA, "xg_linsoe_solve: copy of B failed");
  if (int e = s->prof.solve(1, &bp, &xp, st)) return lfail(e, "xg_linsoe_solve: substitutions failed");
  if (cudaMemcpyAsync(s->X.data(), s->x.p, s->n * sizeof(double), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return lfail(XG_ECUDA, "xg_linsoe_solve: copy of X failed");
  if (iters) *iters = 0;
  if (relres) *relres = 0.0;
  return 0;
}

int xg_linsoe_solve(xg_linsoe *s, double rtol, int maxit, int *iters, double *relres) {
  if (!s) return lfail(XG_EINVAL, "null system");
  if (s->system == XG_SYSTEM_PROFILE_SPD) {
    if (s->n == 0) return 0;
    return linsoe_solve_profile(s, iters, relres);
  }
  if (!(rtol > 0.0) || maxit < 1) return lfail(XG_EINVAL, "bad solve settings");
  if (s->n == 0) return 0;
  if (int e = s->setup()) return e;
  cudaStream_t st = s->stream;
  if (cudaMemcpyAsync(s->vals.p, s->A.data(), s->A.size() * sizeof(double),
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(s->b.p, s->B.data(), s->B.size() * sizeof(double), cudaMemcpyHostToDevice,
                      st) != cudaSuccess ||
      cudaMemsetAsync(s->x.p, 0, s->n * sizeof(double), st) != cudaSuccess)
    return lfail(XG_ECUDA, "xg_linsoe_solve: copies failed");
  if (xg::pcg_factor_blocks(s->S, st) != 0) return lfail(XG_ECUDA, "xg_linsoe_solve: blocks");
  int it = 0;
  double rr = 0.0;
  const int r = xg::pcg_solve(s->S, s->b.p, s->x.p, rtol, maxit, &it, &rr, st);
  if (cudaMemcpyAsync(s->X.data(), s->x.p, s->n * sizeof(double), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return lfail(XG_ECUDA, "xg_linsoe_solve: copy of X failed");
  if (iters) *iters = it;
  if (relres) *relres = rr;
  if (r) {
    char msg[128];
    snprintf(msg, sizeof msg, "xg_linsoe_solve: PCG did not converge (%d iterations, %.3e)", it,
             rr);
    return lfail(XG_ESOLVE, msg);
  }
  return 0;
}

int xg_linsoe_get_x(const xg_linsoe *s, double *x) {
  if (!s || (!x && s->n)) return lfail(XG_EINVAL, "bad argument");
  std::copy(s->X.begin(), s->X.end(), x);
  return 0;
}

int xg_linsoe_get_b(const xg_linsoe *s, double *b) {
  if (!s || (!b && s->n)) return lfail(XG_EINVAL, "bad argument");
  std::copy(s->B.begin(), s->B.end(), b);
  return 0;
}

}  // extern "C"
