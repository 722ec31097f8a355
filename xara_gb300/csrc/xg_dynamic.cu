// xg_dynamic.cu -- the transient step on the device: Newmark predictor and
// corrector (analysis/integrator/Dynamic/Newmark.cpp), the dynamic
// unbalance with lumped masses, Rayleigh damping and UniformExcitation
// (domain/node/Node.cpp:668-764, element/Element.cpp:284-330,
// domain/pattern/EarthquakePattern.cpp:68-99), the effective tangent, the
// initial stiffness of force-based frames for the betaK0 term, and the
// per-component convergence norms that let disconnected models (a batch of
// frames in one system) converge one by one.
#include <cuda_runtime.h>

#include <algorithm>

#include "xg_internal.h"

namespace xg {

namespace {

// PathSeries::getFactor (domain/pattern/series/PathSeries.cpp:334-356):
// start time 0, factor 1, useLast false.
__device__ __forceinline__ double path_factor(const double *a, int npts, double dt, double t) {
  if (t < 0.0) return 0.0;
  const double incr = t / dt;
  const int i1 = (int)floor(incr), i2 = i1 + 1;
  if (i2 >= npts) return 0.0;
  const double v1 = a[i1], v2 = a[i2];
  return v1 + (v2 - v1) * (incr - i1);
}

// Newmark::newStep (Newmark.cpp:150-170), displacement unknown: from the
// committed state, v = a1 vc + a2 ac and a = a4 ac + a3 vc.
__global__ void k_newmark_predict(DynView d, double a1, double a2, double a3, double a4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.nu || d.eqn[i] < 0) return;
  const double vc = d.Vc[i], ac = d.Ac[i];
  d.V[i] = vc * a1 + ac * a2;
  d.A[i] = ac * a4 + vc * a3;
}

// Newmark::update (Newmark.cpp:432-436): u += du, v += c2 du, a += c3 du.
__global__ void k_newmark_correct(DynView d, const double *dU, double c2, double c3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.nu) return;
  const int e = d.eqn[i];
  if (e < 0) return;
  const double du = dU[e];
  d.U[i] += du;
  d.V[i] += du * c2;
  d.A[i] += du * c3;
}

// velocity on the equations (the first (node, dof) of each equation; dofs
// tied by equalDOF share it)
__global__ void k_vel_eq(DynView d, double *veq) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.neq) return;
  veq[e] = d.V[d.eq_dofs[d.eq_ptr[e]]];
}

// y = A x over the CSR pattern (one warp per row, fixed lane order)
__global__ void k_spmv(int n, const int *rowptr, const int *colidx, const double *vals,
                       const double *x, double *y) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= n) return;
  double s = 0.0;
  for (int k = rowptr[row] + lane; k < rowptr[row + 1]; k += 32) s += vals[k] * x[colidx[k]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = s;
}

// B = F_ext - P_int - betaK0 K0 v + sum over the equation's (node, dof):
// -m (a + alphaM v) - m ag(t) on the excited direction.  The equation's
// (node, dof) list is in node order, so the sum is deterministic.
__global__ void k_dyn_unbalance(DynView d, const double *fext, const double *pint,
                                const double *k0v, double bk0, double am, double t_arg,
                                const double *t_dev, double *B) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.neq) return;
  const double t = t_dev ? *t_dev : t_arg;
  double nodal = 0.0;
  for (int k = d.eq_ptr[e]; k < d.eq_ptr[e + 1]; k++) {
    const int a = d.eq_dofs[k];
    const double m = d.mass[a];
    if (m == 0.0) continue;
    double f = -m * d.A[a];
    const double ama = d.am_node ? d.am_node[a / d.ndf] : am;
    if (ama != 0.0) f -= ama * m * d.V[a];
    if (d.gm_npts > 0 && a % d.ndf == d.gm_dof) {
      const int rec = d.gm_rec ? d.gm_rec[a / d.ndf] : 0;
      f -= m * path_factor(d.gm + (long)rec * d.gm_npts, d.gm_npts, d.gm_dt, t);
    }
    nodal += f;
  }
  double b = fext[e] + nodal - pint[e];
  if (bk0 != 0.0) b -= bk0 * k0v[e];
  B[e] = b;
}

// Newmark::formEleTangent / formNodTangent (Newmark.cpp:262-300):
// c1 Kt + c2 betaK0 K0 on every entry, c2 alphaM m + c3 m on the diagonal
// (meq_am: the equation's alphaM-weighted mass).
__global__ void k_dyn_tangent(DynView d, double *vals, const double *k0vals, double c1,
                              double c2bk0, double c2, double c3) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < d.nnz) {
    double v = vals[k] * c1;
    if (c2bk0 != 0.0) v += c2bk0 * k0vals[k];
    vals[k] = v;
  }
}
__global__ void k_dyn_tangent_diag(DynView d, double *vals, double c2, double c3) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.neq) return;
  const double add = c2 * d.meq_am[e] + c3 * d.meq[e];
  if (add != 0.0) vals[d.diag_pos[e]] += add;
}

// K0 per element scaled by the element's betaK0 before the gather
__global__ void k_scale_blocks(int nblk, int len, const double *scale, double s0, double *x) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)nblk * len) return;
  x[i] *= scale ? scale[i / len] : s0;
}

// sum of x^2 over each component's equation range [cstart[c], cstart[c+1])
__global__ void k_comp_norm2(int ncomp, const int *cstart, const double *x, double *out) {
  const int c = blockIdx.x;
  if (c >= ncomp) return;
  __shared__ double red[32];
  double s = 0.0;
  for (int i = cstart[c] + threadIdx.x; i < cstart[c + 1]; i += blockDim.x) s += x[i] * x[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) out[c] = t;
  }
}

// zero the right-hand side of the components that have converged
__global__ void k_comp_mask(int neq, const int *comp_of, const int *active, double *B) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < neq && !active[comp_of[e]]) B[e] = 0.0;
}

// Start of a captured Newmark step: t += dt on the device, every part
// active, the iteration count cleared.
__global__ void k_step_begin(double *t, double dt, int *stat, int *active, int ncomp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    *t += dt;
    stat[0] = 0;
    stat[1] = 0;
    stat[2] = ncomp;
  }
  if (i < ncomp) active[i] = 1;
}

// End of a captured Newton iteration (CTestNormDispIncr / CTestNormUnbalance
// per part): parts whose norm passed stop; the loop goes on while any part
// is active and fewer than max_iter iterations have run.  stat: [0]
// iterations, [1] 1 converged / 2 not converged, [2] parts still active.
__global__ void k_newton_check(int ncomp, const double *cnorm, double tol, int max_iter,
                               int *active, int *stat, cudaGraphConditionalHandle h) {
  __shared__ int nact;
  if (threadIdx.x == 0) nact = 0;
  __syncthreads();
  int mine = 0;
  for (int c = threadIdx.x; c < ncomp; c += blockDim.x) {
    if (active[c] && sqrt(cnorm[c]) <= tol) active[c] = 0;
    mine += active[c];
  }
  atomicAdd(&nact, mine);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int it = ++stat[0];
    stat[2] = nact;
    unsigned go = 1;
    if (nact == 0) { stat[1] = 1; go = 0; }
    else if (it >= max_iter) { stat[1] = 2; go = 0; }
    cudaGraphSetConditional(h, go);
  }
}

inline int grid(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

int launch_step_begin(double *t, double dt, int *stat, int *active, int ncomp, cudaStream_t s) {
  k_step_begin<<<grid(std::max(ncomp, 1), 256), 256, 0, s>>>(t, dt, stat, active, ncomp);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_newton_check(int ncomp, const double *cnorm, double tol, int max_iter, int *active,
                        int *stat, cudaGraphConditionalHandle h, cudaStream_t s) {
  k_newton_check<<<1, 256, 0, s>>>(ncomp, cnorm, tol, max_iter, active, stat, h);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_newmark_predict(const DynView &d, double a1, double a2, double a3, double a4,
                           cudaStream_t s) {
  if (d.nu == 0) return 0;
  k_newmark_predict<<<grid(d.nu, 256), 256, 0, s>>>(d, a1, a2, a3, a4);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_newmark_correct(const DynView &d, const double *dU, double c2, double c3,
                           cudaStream_t s) {
  if (d.nu == 0) return 0;
  k_newmark_correct<<<grid(d.nu, 256), 256, 0, s>>>(d, dU, c2, c3);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_dyn_unbalance(const DynView &d, const double *fext, const double *pint,
                         const double *k0vals, const int *rowptr, const int *colidx,
                         double bk0, double am, double t, double *veq, double *k0v, double *B,
                         cudaStream_t s, const double *t_dev) {
  if (d.neq == 0) return 0;
  if (bk0 != 0.0) {
    k_vel_eq<<<grid(d.neq, 256), 256, 0, s>>>(d, veq);
    k_spmv<<<grid((long)d.neq * 32, 256), 256, 0, s>>>(d.neq, rowptr, colidx, k0vals, veq, k0v);
  }
  k_dyn_unbalance<<<grid(d.neq, 256), 256, 0, s>>>(d, fext, pint, k0v, bk0, am, t, t_dev, B);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_spmv(int n, const int *rowptr, const int *colidx, const double *vals, const double *x,
                double *y, cudaStream_t s) {
  if (n == 0) return 0;
  k_spmv<<<grid((long)n * 32, 256), 256, 0, s>>>(n, rowptr, colidx, vals, x, y);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_dyn_tangent(const DynView &d, double *vals, const double *k0vals, double c1,
                       double c2bk0, double c2, double c3, cudaStream_t s) {
  if (d.nnz > 0) k_dyn_tangent<<<grid(d.nnz, 256), 256, 0, s>>>(d, vals, k0vals, c1, c2bk0, c2, c3);
  if (d.neq > 0) k_dyn_tangent_diag<<<grid(d.neq, 256), 256, 0, s>>>(d, vals, c2, c3);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_scale_blocks(int nblk, int len, const double *scale, double s0, double *x,
                        cudaStream_t s) {
  if ((long)nblk * len == 0) return 0;
  k_scale_blocks<<<grid((long)nblk * len, 256), 256, 0, s>>>(nblk, len, scale, s0, x);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_comp_norm2(int ncomp, const int *cstart, const double *x, double *out,
                      cudaStream_t s) {
  if (ncomp == 0) return 0;
  k_comp_norm2<<<ncomp, 256, 0, s>>>(ncomp, cstart, x, out);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_comp_mask(int neq, const int *comp_of, const int *active, double *B, cudaStream_t s) {
  if (neq == 0) return 0;
  k_comp_mask<<<grid(neq, 256), 256, 0, s>>>(neq, comp_of, active, B);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

}  // namespace xg
