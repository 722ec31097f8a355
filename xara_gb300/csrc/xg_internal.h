// xg_internal.h -- shared declarations of libxara_gpu.so (host C++ and CUDA).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/xara_gpu.h"

namespace xg {

// ---------------------------------------------------------------------------
// device views
// ---------------------------------------------------------------------------

// Continuum element set (quad / brick) with J2 plasticity at every point.
struct ContinuumView {
  int ne, nn, nen, nip, ndf, ndm;
  const int *conn;        // [nen][ne] node indices (SoA)
  const double *crd;      // [ndm][nn] coordinates (SoA)
  const double *U;        // [nn*ndf] trial displacements
  const int *mat;         // [ne] J2 row
  const double *j2;       // [nmat*8]
  double thickness;
  // history, point-major SoA: comp*npts + (e*nip + ip)
  const double *ep_c;     // committed plastic strain (4 comps plane strain: xx yy zz xy; 6 in 3D)
  const double *xi_c;
  double *ep_t, *xi_t;    // trial
  double *sig;            // trial stress (3 plane strain: xx yy xy; 6 in 3D)
  double *tan;            // trial tangent: quad 6 unique D entries; brick a b c n(6)
  int *nfail;             // [1] points whose return map hit the iteration cap
  // element outputs (element-major scratch)
  double *Ke;             // [ne][ned*ned] row-major (quad 64, brick 576); bricks with geo2
                          // write float pairs (hi, lo) there
  double *Re;             // [ne][ned]
  // bricks: shape-function gradients dN_a/dx_i at [(8i+a)*npts + pt] and the
  // Jacobian determinant at [24*npts + pt], formed once (the geometry does
  // not change); null: formed in every kernel that needs them
  const double *geo;
  // bricks: the same dN/dx split into float pairs (hi, lo) at
  // [(pt*3 + i)*8 + a], for the float-float tangent; null: the tangent is
  // formed in FP64
  const float2 *geo2;
};

// CSR system and deterministic gather assembly.
struct GatherMap {
  int nslots;             // nnz or neq
  int nchunks;
  const int *chunk_slot;  // [nchunks]
  const int64_t *chunk_begin;  // [nchunks+1] into src
  const int *slot_chunk;  // [nslots+1] chunk range per slot
  const int64_t *src;     // contribution source indices into the scratch
  const int *src32;       // the same as 32-bit indices when the scratch is small enough, or null
  // runs (built when every source fits 32 bits): consecutive slots whose
  // contribution lists match term by term with sources one apart (the
  // columns of one node's dofs in a row), summed by one thread that reads a
  // single source index per contribution; slots with more than kRunMaxTerms
  // contributions stay with the chunks above (long_chunks, long_slots)
  int nruns;
  const int *run_slot;    // [nruns] first slot
  const int *run_meta;    // [nruns] length (bits 0-3) | contributions << 4
  const int *run_begin;   // [nruns] first source of the run's first slot in run_src
  const int *run_src;     // sources of each run's first slot
  int nlong_chunks, nlong_slots;
  const int *long_chunks; // chunks of the long slots
  const int *long_slots;  // the long slots
};
constexpr int kRunMaxLen = 6, kRunMaxTerms = 32;

// ---------------------------------------------------------------------------
// kernel launchers (xg_kernels.cu)
// ---------------------------------------------------------------------------
int launch_quad_update(const ContinuumView &v, cudaStream_t s);
int launch_quad_assemble(const ContinuumView &v, cudaStream_t s);
int launch_brick_update(const ContinuumView &v, cudaStream_t s);
int launch_brick_assemble(const ContinuumView &v, cudaStream_t s);
int launch_brick_geometry(const ContinuumView &v, double *geo, float2 *geo2, int *bad,
                          cudaStream_t s);
// recorders: kind 0 writes one row ([t] values), kind 1 updates an envelope
int launch_record(int kind, int n, const int *idx, const double *src, double t, int echo,
                  int first, double *out, cudaStream_t s);
// pairs: the scratch holds float pairs (hi, lo), 8 bytes an entry (the
// float-float brick tangent); needs the run map (GatherMap::run_slot).
int launch_gather(const GatherMap &g, const double *scratch, double *partial, double *out,
                  cudaStream_t s, bool pairs = false);
int gather_launch_count(const GatherMap &g, bool pairs = false);   // kernels launch_gather issues
int launch_j2_zero_state(const ContinuumView &v, cudaStream_t s);

// Block-Jacobi preconditioned CG (xg_pcg.cu)
struct PcgSystem {
  int n;
  const int *rowptr, *colidx;
  const double *vals;
  int nblk;
  const int *blk_start;   // [nblk+1] equation ranges of the diagonal blocks (<= 6)
  double *binv;           // inverted diagonal blocks, row major: [nblk*kb*kb], or [nblk*36]
                          // (padded to 6 x 6) when kb is 0
  // work vectors [n]
  double *r, *z, *p, *q;
  double *partials;       // [4*pcg_max_blocks() + 8] (3*... + 8 without the node-block copy)
  unsigned int *barrier;  // [2] grid barrier state
  int *flags;             // [4] status words
  double *scalars;        // [8]
  // optional node-block sliced ELL copy of the matrix (thread per node row:
  // the equations of one diagonal block against KB x KB blocks of the nodes
  // it couples to, one column index per block) for node rows of at most
  // nb_cap blocks; the rows of longer node rows in chunks of CSR entries, a
  // warp each; nb_vals null: every row is read from the CSR arrays warp per
  // row.  The block SpMV computes in float-float (each value and each entry
  // of p split into two single-precision numbers, xg_ff.h) on the
  // single-precision pipes; node rows with a value outside the split's range
  // stay in FP64.
  int kb;                 // block order: 2, 3 or 6 (the largest diagonal block), 0: no copy
  const long *nb_off;     // [ceil(nblk/32)+1] slice offsets, in blocks
  const int *nb_cols;     // [nb_off[last]] column node of each block
  const int *nb_len;      // [nblk] blocks of each node row
  const int *nb_pos;      // [nnz] slot of each CSR entry in nb_vals (-1: a long node row's)
  float2 *nb_vals;        // [nb_off[last]*kb*kb] (hi, lo), packed by pcg_factor_blocks
  unsigned char *blk_ff;  // [nblk] 1: the node row's values lie in the split's range
  float2 *p2;             // [nblk*(kb == 3 ? 4 : kb)] p split, node-major, padding zero
  int nb_cap;
  int nlong, nchunks;     // long rows, their chunks
  const int *chunk_row;   // [nchunks] row of each chunk
  const int *chunk_beg;   // [nchunks] first CSR entry of each chunk
  const int *long_chunk0; // [nlong+1] chunk range of each long row
  double *chunk_part;     // [nchunks] partial sums
};
// Factor the diagonal blocks (and pack the node-block values when present)
// after the matrix values changed.
int pcg_factor_blocks(const PcgSystem &S, cudaStream_t s);
// Host layout of the node-block copy of a CSR pattern whose diagonal blocks
// are blk_start's equation ranges (1..6 equations each): block order,
// slices, column nodes, each CSR entry's slot, and the chunks of the rows of
// node rows with more than cap blocks.  kb stays 0 (no copy) when a block
// is larger than 6 or the slots overflow 32-bit positions.
struct BlockEll {
  int kb = 0;
  std::vector<long> off;
  std::vector<int> cols, len, pos;
  std::vector<int> chunk_row, chunk_beg, long_chunk0;
};
int block_ell_layout(int n, const int *rowptr, const int *colidx, int nblk, const int *blk_start,
                     int cap, BlockEll &h);
// Device bytes of the copy (columns, values, positions, offsets, per-node
// arrays and p2).
size_t block_ell_bytes(const BlockEll &h, int nblk);
// Solve A x = b (device vectors).  x holds the initial guess (usually 0).
// Returns 0 when converged, XG_ESOLVE on breakdown, maxit or a barrier timeout.
// rows_per_block: the grid gets one block per that many rows (capped by
// co-residency); 0 takes the default of 64
int pcg_solve(const PcgSystem &S, const double *b, double *x, double rtol, int maxit,
              int *iters, double *relres, cudaStream_t s, int rows_per_block = 0);
int pcg_max_blocks();

// Skyline LDL' without pivoting on 32 x 32 tiles (xg_profile.cu)
struct ProfileSystem {
  int n, nt, W;            // equations, tile rows, envelope width in tiles
  const int *rowptr, *colidx;
  const double *vals;
  const int *ftile;        // [nt] first tile column of each tile row
  double *L;               // [nt*(W+1)*1024] factor tiles
  double *invD, *piv;      // [nt*32] reciprocal pivots, pivots
  const int4 *tasks;       // [ntasks] factor tasks (type, I, K, J) in dataflow order
  int ntasks;
  int *next_task;          // [1] task counter
  int *upd, *done;         // [nt*(W+1)] per tile: updates applied, factored
  double *sweep;           // [4*4*nt*32] values published by the sweeps (y, c, x, c')
  int *flags;              // [4]
  double min_diag_tol;
  // per tile row J, for the substitutions (row-major 32 x 32 each,
  // [nt*1024]): W_J = L_JJ^-T, F_J = L_JJ^-1 L_J,J-1, G_J = L_JJ^-T
  // L_J+1,J', E_J = L_JJ^-1 L_J,J-2, H_J = L_JJ^-T L_J+2,J',
  // Q_J = E_J - F_J F_J-1 and R_J = H_J - G_J G_J+1 (zero where a tile is
  // outside the envelope)
  double *Winv, *F, *G, *E, *H, *Q, *R;
  int *cpl;                // [nt] row J's coupling matrices written
  // right-hand sides whose forward sweep runs inside the factorisation
  // (fwd_nrhs 0: none), column r at fwd_x[r*fwd_ldx]
  int fwd_nrhs, fwd_ldx;
  const double *fwd_x;
};
int profile_plan(int n, const int *rowptr, const int *colidx, std::vector<int> &ftile, int &nt,
                 int &W);
void profile_tasks(int nt, int W, const std::vector<int> &ftile, std::vector<int> &tasks);
size_t profile_tile_doubles(int nt, int W);
int profile_tile_edge();
// Factor the CSR values into the tiles.  XG_ESOLVE on a failed pivot check
// (*bad_eq = the equation) or a dependency wait that timed out (*bad_eq = -1).
int profile_factor(const ProfileSystem &S, cudaStream_t s, int *bad_eq);
// Solve in place: x[r*ldx + i] holds right-hand side r on entry (ldx >=
// nt*32, entries past n zero), the solution on return; nrhs <= 4.
// backward_only: the factorisation ran the forward sweep of these
// right-hand sides (ProfileSystem::fwd_nrhs, the pipelined path only).
int profile_solve(const ProfileSystem &S, int nrhs, double *x, int ldx, cudaStream_t s,
                  bool backward_only = false);
// Whether the substitutions of this system run pipelined over co-resident
// blocks (the path whose forward sweep the factorisation can carry).
bool profile_pipelined(const ProfileSystem &S);

// The tiled envelope LDL' with its device buffers: planned once per pattern,
// factored once per tangent, then up to four right-hand sides per solve.
// Used by the device model (`system ProfileSPD`) and by the standalone linear
// system (xg_linsoe_*).
class ProfileSolver {
 public:
  ProfileSolver() = default;
  ProfileSolver(const ProfileSolver &) = delete;
  ProfileSolver &operator=(const ProfileSolver &) = delete;
  ~ProfileSolver();
  // Plan the envelope of the n-equation CSR pattern (host arrays, sorted
  // columns) and allocate its tiles; d_rowptr, d_colidx and d_vals are the
  // device copies the factorisation reads (the lower triangle).  XG_ENOMEM
  // (with the error text set) when the tiles would take more than half of
  // the free device memory.
  int setup(int n, const int *rowptr, const int *colidx, const int *d_rowptr,
            const int *d_colidx, const double *d_vals, cudaStream_t s);
  bool ready() const { return ready_; }
  // Factor the values now in d_vals.  XG_ESOLVE on a failed pivot check
  // (*bad_eq = the equation) or a dependency wait that timed out (*bad_eq =
  // -1).
  int factor(cudaStream_t s, int *bad_eq);
  // x[r] = A^-1 b[r] for r < nrhs (1..4; device vectors of n entries) with
  // the last factorisation.
  int solve(int nrhs, const double *const *b, double *const *x, cudaStream_t s);
  // Factor with the forward sweep of b[0..nrhs) running as tasks of the
  // factorisation (right behind its front); solve_backward then finishes
  // x[r] = A^-1 b[r].  Only for systems whose substitutions are pipelined
  // (can_fuse()).
  bool can_fuse() const { return ready_ && profile_pipelined(S_); }
  int factor_forward(int nrhs, const double *const *b, cudaStream_t s, int *bad_eq);
  int solve_backward(int nrhs, double *const *x, cudaStream_t s);
  const ProfileSystem &system() const { return S_; }

 private:
  template <class T>
  struct Buf {
    T *p = nullptr;
    int alloc(size_t count);
    ~Buf();
  };
  ProfileSystem S_{};
  int fwd_nrhs_ = 0;         // right-hand sides factor_forward swept
  bool ready_ = false;
  int ldx_ = 0;
  Buf<int> ftile_, flags_, tasks_, next_, upd_, done_, cpl_;
  Buf<double> L_, invD_, piv_, px_, Winv_, F_, G_, E_, H_, Q_, R_, sweep_;
};

// ProfileSPD for many small disconnected parts, one band per part
// (xg_band.cu)
struct BandSystem {
  int ncomp;
  const int *cstart;       // [ncomp+1] equation range of each part
  const int *bw;           // [ncomp] envelope width of each part
  const long *boff;        // [ncomp+1] band offset of each part
  double *band;            // [boff[ncomp]]
  const int *rowptr, *colidx;
  const double *vals;
  double *invD;            // [neq]
  int *flags;              // [4]
  double min_diag_tol;
  int bmax, nmax;          // widest band and largest part (launch shapes)
};
// Widths and offsets of the parts' bands; XG_EINVAL when a part couples to
// another or is wider than the kernel's staging.
int band_plan(int neq, const int *rowptr, const int *colidx, const std::vector<int> &cstart,
              std::vector<int> &bw, std::vector<long> &boff);
// Factor every part; with nrhs > 0 (at most 4) the right-hand sides x[r*ldx
// + eq] are carried through the forward substitution and the diagonal
// scaling on the way (band_solve(forward = false) completes them).
int band_factor(const BandSystem &S, cudaStream_t s, int *bad_eq, int nrhs = 0,
                double *x = nullptr, int ldx = 0);
// the same without the host read of the pivot flags (stream capture); the
// flags stay in S.flags
int band_factor_async(const BandSystem &S, cudaStream_t s, int nrhs, double *x, int ldx);
// x[r*ldx + i] right-hand side r in, solution out (equation numbering)
int band_solve(const BandSystem &S, int nrhs, double *x, int ldx, cudaStream_t s,
               bool forward = true);

// small device helpers (xg_kernels.cu)
int launch_axpy(int n, double a, const double *x, double *y, cudaStream_t s);
int launch_scatter_incr(int nu, const int *eqn, const double *dU, double f, double *U,
                        cudaStream_t s);
int launch_sub(int n, const double *a, const double *b, double *out, cudaStream_t s);
// the load factor of each of the eight load patterns
struct SpFactors { double f[8]; };
// U[idx[k]] = lam.f[pat[k]] * val[k] for the n imposed single-point constraints
int launch_enforce_sps(int n, const int *idx, const int *pat, const double *val,
                       const SpFactors &lam, double *U, cudaStream_t s);
// deterministic 2-norm squared of x (n) into *out (device), partials scratch
int launch_norm2(int n, const double *x, double *partials, double *out, cudaStream_t s);

}  // namespace xg

namespace xg {
// Sets the text returned by xg_last_error() (xg_model.cpp).
void record_error(const char *msg);
}  // namespace xg

namespace xg {
// Force-based frame element set (ForceBeamColumn2d/3d with fiber sections).
struct FrameView {
  int ne, nb, nip, ndf;       // nb: basic dofs 3 (2D) or 6 (3D)
  const double *U;            // [nn*ndf] trial displacements
  const int *conn;            // [ne*2] node indices
  const double *L, *R;        // [ne] length; [ne*9] local axes (2D: cos, sin)
  const int *sec;             // [ne] section row
  const int *sec_fstart;      // [nsec+1]
  const double *fy, *fz, *fA; // fiber geometry per section
  // per fiber: coordinates about the section centroid and the products of
  // the section sums, [6][nfib]: A, -y A, z A, y^2 A, z^2 A, -y z A
  const double *fyc, *fzc, *fk;
  int nfib;
  const int *fmat;            // fiber uniaxial row
  const double *ybar, *zbar, *GJ;   // [nsec]
  const double *fs0;          // [nsec*16] initial section flexibility
  const int *utype;           // [nuni]
  const double *uparam;       // [nuni*XG_UNI_NPARAM]
  const long *foff;           // [ne+1] first fiber record of each element
  const double *fh_c;         // committed fiber records [nrec*12]
  double *fh_t;               // trial fiber records
  double *st;                 // trial element state [ne*stride]
  int max_iters;
  double tol;
  double xi[10], wt[10];      // Lobatto locations and weights
  int *nfail;                 // elements whose compatibility iteration failed
  double *Ke, *Re;            // element tangent / force scratch
  unsigned long long *work;   // [2] fiber and section state determinations
  int pdelta2d;               // PDeltaCrdTransf2d geometric terms
};
int frame_state_stride(int nip);
// Concrete02 rows of the device parameter table: the per-material constants
// into slots 7-11
int launch_c02_constants(double *uparam, const int *utype, int n, cudaStream_t s);
int launch_fbc_update(const FrameView &v, cudaStream_t s, int warps = 4);
int launch_fbc_assemble(const FrameView &v, cudaStream_t s);
int launch_fbc_commit(const FrameView &v, double *st_c, double *fh_c, long nrec, cudaStream_t s);
int launch_fbc_revert(const FrameView &v, const double *st_c, long nrec, cudaStream_t s);
// Fill st_scratch (frame_state_stride records) with Se = 0 and kv = the
// initial element stiffness (ForceBeamColumn*::getInitialStiff), so that
// launch_fbc_assemble on a view whose st is st_scratch gives K0 per element.
int launch_fbc_kv0(const FrameView &v, double *st_scratch, cudaStream_t s);

// Transient step (xg_dynamic.cu)
struct DynView {
  int nu, neq, ndf;
  long nnz;
  const int *eqn;             // [nu] equation of each (node, dof)
  double *U, *V, *A;          // [nu] trial displacement, velocity, acceleration
  const double *Vc, *Ac;      // [nu] committed velocity, acceleration
  const double *mass;         // [nu] lumped mass
  const int *eq_ptr, *eq_dofs;  // (node, dof) list of each equation
  const double *meq;          // [neq] mass summed on each equation
  const double *meq_am;       // [neq] alphaM-weighted mass on each equation
  const double *am_node;      // [nn] alphaM per node or null
  const int *diag_pos;        // [neq] CSR position of each diagonal
  int gm_npts, gm_dof;        // UniformExcitation records
  double gm_dt;
  const double *gm;           // [records*gm_npts]
  const int *gm_rec;          // [nn] record of each node or null
};
int launch_newmark_predict(const DynView &d, double a1, double a2, double a3, double a4,
                           cudaStream_t s);
int launch_newmark_correct(const DynView &d, const double *dU, double c2, double c3,
                           cudaStream_t s);
// t_dev: the time read from device memory instead of t (captured steps)
int launch_dyn_unbalance(const DynView &d, const double *fext, const double *pint,
                         const double *k0vals, const int *rowptr, const int *colidx,
                         double bk0, double am, double t, double *veq, double *k0v, double *B,
                         cudaStream_t s, const double *t_dev = nullptr);
// captured Newmark step (a graph with a conditional loop over Newton iterations)
int launch_step_begin(double *t, double dt, int *stat, int *active, int ncomp, cudaStream_t s);
int launch_newton_check(int ncomp, const double *cnorm, double tol, int max_iter, int *active,
                        int *stat, cudaGraphConditionalHandle h, cudaStream_t s);
int launch_dyn_tangent(const DynView &d, double *vals, const double *k0vals, double c1,
                       double c2bk0, double c2, double c3, cudaStream_t s);
// x[b*len + i] *= scale ? scale[b] : s0
int launch_scale_blocks(int nblk, int len, const double *scale, double s0, double *x,
                        cudaStream_t s);
int launch_comp_norm2(int ncomp, const int *cstart, const double *x, double *out,
                      cudaStream_t s);
int launch_comp_mask(int neq, const int *comp_of, const int *active, double *B, cudaStream_t s);
// y = A x over the CSR pattern
int launch_spmv(int n, const int *rowptr, const int *colidx, const double *vals, const double *x,
                double *y, cudaStream_t s);

// Adjoint of a Newmark run of force-based frames (xg_adjoint.cu)
struct NewmarkCoef {
  double c2, c3;              // velocity / acceleration per displacement increment
  double a1, a2, a3, a4;      // predictor: V = a1 Vc + a2 Ac, A = a4 Ac + a3 Vc
};
// materials per element section the adjoint keeps apart (parameter adjoints
// are accumulated per element and material slot)
constexpr int kAdjSlots = 4;

struct AdjView {
  const double *st;           // converged element state of the step [ne*stride]
  const double *fh_prev;      // committed fiber records before the step [nrec*12]
  double *hbar;               // [nrec*12] record adjoint: after the step in, before it out
  double *theta;              // [ne*kAdjSlots*3] parameter adjoint per element and material slot
  double *scr;                // [ne*(6+nip*4)] pass A's z and section ebar
  const int *eqn;             // [nn*ndf]
  const double *mu;           // [neq] adjoint solution of the step
  const double *Vn;           // [nn*ndf] velocity after the step (betaK0 term)
  const double *bk0;          // [ne] betaK0 per element, or null
  double bk0_all;             // betaK0 when bk0 is null
  int use_k0;                 // betaK0 K0 damping present
  const int *elem_uni;        // [ne] the material of slot 0 (the betaK0 term's single material)
  const int *fslot;           // [section fibers] slot of each fiber's material in its section
};
int launch_adj_elem_a(const FrameView &v, const AdjView &a, cudaStream_t s);
int launch_adj_elem_b(const FrameView &v, const AdjView &a, cudaStream_t s);
int launch_adj_pdelta(const FrameView &v, const AdjView &a, cudaStream_t s);

// Direct differentiation (DDM) of a Newmark run along one direction in the
// materials' parameters, after each converged step (the element state in the
// FrameView is the step's converged one)
struct DdmView {
  const double *fh_prev;      // committed fiber records before the step [nrec*12]
  double *dh;                 // [nrec*12] record tangents: before the step in, after it out
  const double *dth;          // [num_uni*3] the direction's tangent of parameters 0-2
  double *q;                  // [ne*nip*4] section force tangents at fixed deformation
  double *z;                  // [ne*6] sum over sections of w L b' fs q
  const int *eqn;             // [nn*ndf]
  const double *dU;           // [neq] the step's displacement tangent (pass 2)
  const double *Vn;           // [nn*ndf] velocity after the step (betaK0 term)
  const double *bk0;          // [ne] betaK0 per element, or null
  double bk0_all;             // betaK0 when bk0 is null
  const int *elem_uni;        // [ne] the single material of a betaK0 element
};
int launch_ddm_init_records(const FrameView &v, const DdmView &d, cudaStream_t s);
int launch_ddm_pdelta(const FrameView &v, const int *eqn, const double *x, cudaStream_t s);
int launch_ddm_k0(const FrameView &v, const DdmView &d, cudaStream_t s);
int launch_ddm_k0_vec(int neq, const double *dU, const double *dV, const double *dA,
                      const NewmarkCoef &c, double *out, cudaStream_t s);
int launch_ddm_cond(const FrameView &v, const DdmView &d, cudaStream_t s);
int launch_ddm_commit(const FrameView &v, const DdmView &d, cudaStream_t s);
int launch_ddm_rhs(int neq, const double *dPc, const double *dU, const double *dV,
                   const double *dA, const double *meq, const double *meq_am,
                   const NewmarkCoef &c, double *rhs, cudaStream_t s);
int launch_ddm_update(int neq, const double *x, const NewmarkCoef &c, double *dU, double *dV,
                      double *dA, cudaStream_t s);
int launch_ddm_objective(int nterm, const int *dof, const double *w, const int *eqn,
                         const double *U, const double *dU, double *dJ, cudaStream_t s);
int launch_adj_init_records(const FrameView &v, const AdjView &a, cudaStream_t s);
int launch_adj_objective(int nterm, const int *dof, const double *w, const double *U, double *J,
                         cudaStream_t s);
int launch_adj_objective_grad(int nterm, const int *dof, const double *w, const int *eqn,
                              const double *U, double *Ubar, cudaStream_t s);
int launch_adj_rhs(int neq, const double *Ub, const double *Vb, const double *Ab,
                   const double *uA, double c2, double c3, double *rhs, cudaStream_t s);
int launch_adj_prev(int neq, const double *mu, const double *kmu, const double *meq,
                    const double *meq_am, const NewmarkCoef &c, double *Ub, double *Vb,
                    double *Ab, cudaStream_t s);
}  // namespace xg
