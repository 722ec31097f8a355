// xg_profile_solver.cpp -- the buffers and call sequence of the tiled
// envelope LDL' (xg_profile.cu): `system ProfileSPD` on the device,
// ProfileSPDLinDirectSolver::factor / solve
// (system_of_eqn/linearSOE/profileSPD/ProfileSPDLinDirectSolver.cpp:100-420)
// for the device model and for the standalone linear system.
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "xg_internal.h"

namespace xg {

template <class T>
int ProfileSolver::Buf<T>::alloc(size_t count) {
  if (p) cudaFree(p);
  p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc(&p, count * sizeof(T)) == cudaSuccess ? 0 : XG_ENOMEM;
}

template <class T>
ProfileSolver::Buf<T>::~Buf() {
  if (p) cudaFree(p);
}

ProfileSolver::~ProfileSolver() = default;

int ProfileSolver::setup(int n, const int *rowptr, const int *colidx, const int *d_rowptr,
                         const int *d_colidx, const double *d_vals, cudaStream_t s) {
  ready_ = false;
  std::vector<int> ftile;
  int nt = 0, W = 0;
  if (int e = profile_plan(n, rowptr, colidx, ftile, nt, W)) return e;
  const size_t tiles = profile_tile_doubles(nt, W);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    record_error("ProfileSPD: cudaMemGetInfo failed");
    return XG_ECUDA;
  }
  if ((tiles + (size_t)nt * 32 * 6) * sizeof(double) > free_b / 2) {
    char msg[160];
    snprintf(msg, sizeof msg,
             "ProfileSPD envelope needs %.1f GB (%d tile rows x %d): use the block-Jacobi PCG "
             "system", tiles * 8e-9, nt, W + 1);
    record_error(msg);
    return XG_ENOMEM;
  }
  std::vector<int> tasks;
  profile_tasks(nt, W, ftile, tasks);
  const size_t nrow = (size_t)nt * 1024, nslot = (size_t)nt * (W + 1);
  int e = 0;
  e |= ftile_.alloc(ftile.size()) | tasks_.alloc(tasks.size());
  e |= L_.alloc(tiles) | Winv_.alloc(nrow) | F_.alloc(nrow) | G_.alloc(nrow);
  e |= E_.alloc(nrow) | H_.alloc(nrow) | Q_.alloc(nrow) | R_.alloc(nrow);
  e |= invD_.alloc((size_t)nt * 32) | piv_.alloc((size_t)nt * 32);
  ldx_ = nt * 32;
  e |= px_.alloc((size_t)ldx_ * 4) | next_.alloc(1) | upd_.alloc(nslot) | done_.alloc(nslot);
  e |= flags_.alloc(4) | cpl_.alloc((size_t)nt) | sweep_.alloc(4 * 4 * (size_t)nt * 32);
  if (e) {
    record_error("ProfileSPD: device allocation failed");
    return XG_ENOMEM;
  }
  if (cudaMemcpyAsync(ftile_.p, ftile.data(), ftile.size() * sizeof(int),
                      cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(tasks_.p, tasks.data(), tasks.size() * sizeof(int), cudaMemcpyHostToDevice,
                      s) != cudaSuccess ||
      cudaMemsetAsync(px_.p, 0, (size_t)ldx_ * 4 * sizeof(double), s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    record_error("ProfileSPD: set-up copies failed");
    return XG_ECUDA;
  }
  S_ = ProfileSystem{};
  S_.n = n; S_.nt = nt; S_.W = W;
  S_.rowptr = d_rowptr; S_.colidx = d_colidx; S_.vals = d_vals;
  S_.ftile = ftile_.p; S_.L = L_.p; S_.invD = invD_.p; S_.piv = piv_.p;
  S_.Winv = Winv_.p; S_.F = F_.p; S_.G = G_.p;
  S_.E = E_.p; S_.H = H_.p; S_.Q = Q_.p; S_.R = R_.p; S_.cpl = cpl_.p;
  S_.sweep = sweep_.p;
  S_.tasks = reinterpret_cast<const int4 *>(tasks_.p);
  S_.ntasks = (int)(tasks.size() / 4);
  S_.next_task = next_.p; S_.upd = upd_.p; S_.done = done_.p;
  S_.flags = flags_.p;
  S_.min_diag_tol = 1.0e-12;   // ProfileSPDLinDirectSolver.h:49 default
  ready_ = true;
  return 0;
}

int ProfileSolver::factor(cudaStream_t s, int *bad_eq) {
  if (!ready_) return XG_ESTATE;
  fwd_nrhs_ = 0;
  return profile_factor(S_, s, bad_eq);
}

int ProfileSolver::solve(int nrhs, const double *const *b, double *const *x, cudaStream_t s) {
  if (!ready_) return XG_ESTATE;
  if (nrhs < 1 || nrhs > 4) return XG_EINVAL;
  const size_t bytes = (size_t)S_.n * sizeof(double);
  for (int r = 0; r < nrhs; r++)
    if (cudaMemcpyAsync(px_.p + (size_t)r * ldx_, b[r], bytes, cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
      return XG_ECUDA;
  if (int e = profile_solve(S_, nrhs, px_.p, ldx_, s)) return e;
  for (int r = 0; r < nrhs; r++)
    if (cudaMemcpyAsync(x[r], px_.p + (size_t)r * ldx_, bytes, cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
      return XG_ECUDA;
  return 0;
}

int ProfileSolver::factor_forward(int nrhs, const double *const *b, cudaStream_t s,
                                  int *bad_eq) {
  if (!ready_) return XG_ESTATE;
  if (nrhs < 1 || nrhs > 4 || !can_fuse()) return XG_EINVAL;
  fwd_nrhs_ = 0;
  const size_t bytes = (size_t)S_.n * sizeof(double);
  for (int r = 0; r < nrhs; r++)
    if (cudaMemcpyAsync(px_.p + (size_t)r * ldx_, b[r], bytes, cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
      return XG_ECUDA;
  ProfileSystem Sf = S_;
  Sf.fwd_nrhs = nrhs;
  Sf.fwd_ldx = ldx_;
  Sf.fwd_x = px_.p;
  if (int e = profile_factor(Sf, s, bad_eq)) return e;
  fwd_nrhs_ = nrhs;
  return 0;
}

int ProfileSolver::solve_backward(int nrhs, double *const *x, cudaStream_t s) {
  if (!ready_) return XG_ESTATE;
  if (nrhs != fwd_nrhs_ || nrhs < 1) return XG_ESTATE;   // no matching forward sweep
  fwd_nrhs_ = 0;
  if (int e = profile_solve(S_, nrhs, px_.p, ldx_, s, true)) return e;
  const size_t bytes = (size_t)S_.n * sizeof(double);
  for (int r = 0; r < nrhs; r++)
    if (cudaMemcpyAsync(x[r], px_.p + (size_t)r * ldx_, bytes, cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
      return XG_ECUDA;
  return 0;
}

}  // namespace xg
