// xg_model.cpp -- host side of libxara_gpu.so: the model store, DOF
// numbering, sparsity pattern, gather maps, and the Newton-Raphson driver
// that keeps every vector of a step on the device.
//
// The integer pipeline (handler IDs, RCM order, equation numbers, CSR
// pattern) restates the reference's algorithm and is bit-exact against it:
//   PlainHandler::handle            analysis/handler/PlainHandler.cpp:60-200
//   AnalysisModel::getDOFGroupGraph analysis/model/AnalysisModel.cpp:356-392
//   RCM::number (no GPS)            graph/numberer/RCM.cpp:67-277
//   DOF_Numberer::numberDOF         analysis/numberer/DOF_Numberer.cpp:93-205
//   SparseGenColLinSOE::setSize     system_of_eqn/linearSOE/sparseGEN/SparseGenColLinSOE.cpp:161-261
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <memory>
#include <vector>

#include "xg_internal.h"

using namespace xg;

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(XG_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                       \
  } while (0)

#define RET(call)                                                                  \
  do {                                                                             \
    int r_ = (call);                                                               \
    if (r_ != 0) {                                                                 \
      if (g_err.empty()) fail(r_, "%s failed (%d)", #call, r_);                    \
      return r_;                                                                   \
    }                                                                              \
  } while (0)

template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  int alloc(size_t count) {
    free();
    n = count;
    if (count == 0) return 0;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
      p = nullptr;
      return fail(XG_ENOMEM, "cudaMalloc of %zu bytes failed", count * sizeof(T));
    }
    return 0;
  }
  int upload(const T *h, size_t count, cudaStream_t s) {
    RET(alloc(count));
    if (count) CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    return 0;
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { free(); }
};

struct HostGather {
  std::vector<int> slot_chunk, chunk_slot;
  std::vector<int64_t> chunk_begin;
  std::vector<int64_t> src;
  // runs (GatherMap): empty when a source does not fit 32 bits
  std::vector<int> run_slot, run_meta, run_begin, run_src, long_chunks, long_slots;
};

// Build chunked gather lists from (slot, src) pairs given in assembly order.
void build_gather(int nslots, const std::vector<int> &slot_of, const std::vector<int64_t> &src_of,
                  HostGather &g, int chunk = 32) {
  std::vector<int64_t> cnt(nslots + 1, 0);
  for (int s : slot_of) cnt[s + 1]++;
  std::vector<int64_t> ptr(nslots + 1, 0);
  for (int i = 0; i < nslots; i++) ptr[i + 1] = ptr[i] + cnt[i + 1];
  g.src.assign(ptr[nslots], 0);
  std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
  for (size_t k = 0; k < slot_of.size(); k++) g.src[fill[slot_of[k]]++] = src_of[k];
  g.slot_chunk.assign(nslots + 1, 0);
  g.chunk_slot.clear();
  g.chunk_begin.clear();
  for (int s = 0; s < nslots; s++) {
    g.slot_chunk[s] = (int)g.chunk_slot.size();
    int64_t b = ptr[s], e = ptr[s + 1];
    if (b == e) {
      g.chunk_slot.push_back(s);
      g.chunk_begin.push_back(b);
    }
    for (int64_t c = b; c < e; c += chunk) {
      g.chunk_slot.push_back(s);
      g.chunk_begin.push_back(c);
    }
  }
  g.slot_chunk[nslots] = (int)g.chunk_slot.size();
  g.chunk_begin.push_back(ptr[nslots]);
  // chunk c sums src[chunk_begin[c], chunk_begin[c+1]): the chunks of a slot
  // and of consecutive slots tile [0, total) (an empty slot has one empty
  // chunk starting where the next slot starts).

  // runs: slot s opens a run that slots s+1 .. s+len-1 continue while they
  // have the same number of contributions (at most kRunMaxTerms) and each
  // contribution's source is the run's first slot's plus the offset
  g.run_slot.clear(); g.run_meta.clear(); g.run_begin.clear(); g.run_src.clear();
  g.long_chunks.clear(); g.long_slots.clear();
  int64_t mx = 0;
  for (int64_t v : g.src) mx = std::max(mx, v);
  if (mx + kRunMaxLen >= INT32_MAX || (int64_t)g.src.size() >= INT32_MAX) return;
  for (int s0 = 0; s0 < nslots;) {
    const int64_t b = ptr[s0], n = ptr[s0 + 1] - b;
    if (n > kRunMaxTerms) {
      g.long_slots.push_back(s0);
      for (int c = g.slot_chunk[s0]; c < g.slot_chunk[s0 + 1]; c++) g.long_chunks.push_back(c);
      s0++;
      continue;
    }
    int len = 1;
    while (len < kRunMaxLen && s0 + len < nslots && ptr[s0 + len + 1] - ptr[s0 + len] == n) {
      const int64_t bl = ptr[s0 + len];
      bool same = true;
      for (int64_t q = 0; q < n && same; q++) same = g.src[bl + q] == g.src[b + q] + len;
      if (!same) break;
      len++;
    }
    g.run_slot.push_back(s0);
    g.run_meta.push_back(len | (int)n << 4);
    g.run_begin.push_back((int)g.run_src.size());
    for (int64_t q = 0; q < n; q++) g.run_src.push_back((int)g.src[b + q]);
    s0 += len;
  }
  // runs ordered by (length, contributions) inside windows of 4,096 runs (a
  // few hundred rows): a warp's threads then run the same loop, and the runs
  // that read neighbouring entries of one element row stay close enough in
  // time for the L2 to serve them (ordered over the whole map, the gather
  // read 3 times its bytes from DRAM)
  constexpr size_t kWindow = 4096;
  std::vector<int> ord(g.run_slot.size());
  for (size_t i = 0; i < ord.size(); i++) ord[i] = (int)i;
  auto by_shape = [&](int x, int y) {
    const int mx = g.run_meta[x], my = g.run_meta[y];
    return (mx & 15) != (my & 15) ? (mx & 15) < (my & 15) : (mx >> 4) < (my >> 4);
  };
  for (size_t w0 = 0; w0 < ord.size(); w0 += kWindow)
    std::stable_sort(ord.begin() + w0, ord.begin() + std::min(ord.size(), w0 + kWindow), by_shape);
  std::vector<int> rs(ord.size()), rm(ord.size()), rb(ord.size());
  for (size_t i = 0; i < ord.size(); i++) {
    rs[i] = g.run_slot[ord[i]];
    rm[i] = g.run_meta[ord[i]];
    rb[i] = g.run_begin[ord[i]];
  }
  g.run_slot.swap(rs);
  g.run_meta.swap(rm);
  g.run_begin.swap(rb);
}

}  // namespace

struct xg_model {
  // description (copied)
  int ndm = 0, ndf = 0, nn = 0, ne = 0, nen = 0, nip = 0, ned = 0, etype = 0;
  double thickness = 1.0;
  std::vector<int> node_tag, elem_tag, conn;   // conn: node indices [ne*nen]
  std::vector<double> crd;                     // [nn*ndm]
  std::vector<int> mat;
  std::vector<double> j2;
  int num_sp = 0, num_mp = 0, num_loads = 0, handler = 0;
  std::vector<int> sp_node, sp_dof, sp_pat, mp_r, mp_c, mp_dof, load_node, load_pat;
  // Transformation handler: the imposed single-point constraints (sp in a
  // load pattern) as (U index, pattern, value) on the device
  int num_isp = 0;
  DBuf<int> d_isp_idx, d_isp_pat;
  DBuf<double> d_isp_val;
  int enforce_sps(double t);
  std::vector<double> sp_val, load_val;

  // numbering
  int neq = 0, nnz = 0;
  std::vector<int> eqn;                        // [nn*ndf]
  std::vector<int> rowptr, colidx;
  std::vector<int> blk_start;

  // device
  cudaStream_t stream = nullptr;
  DBuf<int> d_conn, d_mat, d_eqn, d_rowptr, d_colidx, d_blk, d_nfail;
  DBuf<double> d_crd, d_j2, d_U, d_Uc;
  DBuf<double> d_epc, d_xic, d_ept, d_xit, d_sig, d_tan;
  DBuf<double> d_sig_c, d_tan_c;               // trial state at the last commit
  DBuf<double> d_Ke, d_Re, d_partial;
  DBuf<double> d_vals, d_resid;
  DBuf<int> d_gk_slot_chunk, d_gk_chunk_slot, d_gr_slot_chunk, d_gr_chunk_slot;
  DBuf<int64_t> d_gk_chunk_begin, d_gk_src, d_gr_chunk_begin, d_gr_src;
  DBuf<int> d_gk_src32, d_gr_src32;
  DBuf<int> d_gk_run[6], d_gr_run[6];   // run_slot run_meta run_begin run_src long_chunks long_slots
  GatherMap gk{}, gr{};
  // solver
  DBuf<double> d_binv, d_r, d_z, d_p, d_q, d_pcg_part, d_scalars;
  DBuf<unsigned int> d_barrier;
  DBuf<int> d_flags;
  // recorders (NodeRecorder / EnvelopeNodeRecorder): values gathered on the
  // device after every committed step of xg_analyze
  struct Recorder {
    int kind = 0, response = 0, echo = 0, ncol = 0, rows = 0, cap = 0, nvals = 0;
    double dT = 0.0, next = 0.0;
    bool first = true;
    DBuf<int> idx;
    DBuf<double> data;     // node: [cap][ncol]; envelope: [3][ncol]
  };
  std::vector<std::unique_ptr<Recorder>> recorders;
  int record_step();
  PcgSystem pcg{};
  bool blocks_factored = false;
  // node-block sliced ELL copy of the matrix for the PCG's SpMV, built at
  // the first PCG solve (skipped, keeping the CSR SpMV, when it would take
  // more than half of the free device memory)
  DBuf<long> d_nb_off;
  DBuf<int> d_nb_cols, d_nb_len, d_nb_pos;
  DBuf<float2> d_nb_vals, d_p2;
  DBuf<double> d_chunk_part;
  DBuf<unsigned char> d_blk_ff;
  DBuf<double> d_geo;   // bricks: per-point shape-function gradients and Jacobian determinant
  DBuf<float2> d_geo2;  // bricks: the gradients split into float pairs (float-float tangent)
  DBuf<int> d_chunk_row, d_chunk_beg, d_long_chunk0;
  bool blocks_tried = false;
  long long pcg_blocks = 0;   // node-pair blocks of the PCG's copy
  int ensure_pcg_blocks();
  int pcg_prepare();
  double rtol = 1e-12;
  int maxit = 20000;
  // `system ProfileSPD` on the device (xg_profile.cu)
  int system = XG_SYSTEM_PROFILE_SPD;
  ProfileSolver envelope;                      // one envelope (connected model)
  bool prof_ready = false, prof_factored = false;
  DBuf<int> d_pflags;
  DBuf<double> d_invD, d_px;
  int prof_ldx = 0;
  bool prof_band = false;                      // many small parts: one band each
  BandSystem bsys{};
  DBuf<int> d_bw;
  DBuf<long> d_boff;
  DBuf<double> d_band;
  int ensure_profile();
  int solve_profile(int nrhs, const double *const *b, double *const *x);
  // Newton vectors
  DBuf<double> d_fext, d_B, d_dU, d_phat, d_dUhat, d_x, d_b, d_norm, d_Fref;
  std::vector<int> ref_patterns;               // pattern id of each d_Fref row
  // transient (Newmark, Rayleigh, UniformExcitation)
  std::vector<double> node_mass;               // [nn*ndf]
  DBuf<double> d_V, d_A, d_Vc, d_Ac, d_mass, d_meq, d_meq_am, d_am_node, d_bk0_elem;
  DBuf<double> d_K0vals, d_veq, d_k0v, d_gm, d_cnorm;
  DBuf<int> d_eq_ptr, d_eq_dofs, d_diag_pos, d_gm_rec, d_cstart, d_comp_of, d_active;
  std::vector<int> comp_start;                 // equation ranges of disconnected parts
  bool k0_ready = false;
  DynView dview() {
    DynView v{};
    v.nu = nn * ndf; v.neq = neq; v.ndf = ndf; v.nnz = nnz;
    v.eqn = d_eqn.p; v.U = d_U.p; v.V = d_V.p; v.A = d_A.p; v.Vc = d_Vc.p; v.Ac = d_Ac.p;
    v.mass = d_mass.p; v.eq_ptr = d_eq_ptr.p; v.eq_dofs = d_eq_dofs.p; v.meq = d_meq.p;
    v.meq_am = d_meq_am.p; v.am_node = phase.alpha_m_node ? d_am_node.p : nullptr;
    v.diag_pos = d_diag_pos.p;
    v.gm_npts = phase.gm_npts; v.gm_dof = phase.gm_dof; v.gm_dt = phase.gm_dt;
    v.gm = d_gm.p; v.gm_rec = phase.gm_node_record ? d_gm_rec.p : nullptr;
    return v;
  }
  int upload_dynamics();
  int step_newmark(xg_step_stats *st);
  // adjoint of a Newmark run (xg_adjoint_forward / xg_adjoint_backward): the
  // committed state every K steps (U V A, fiber records, element state), the
  // K+1 states of the segment being swept, and the adjoint vectors
  struct AdjRun {
    bool have = false;
    int N = 0, K = 0, nterm = 0, nck = 0;
    size_t len = 0;                        // doubles in one saved state
    std::vector<double> ck_time, Jk;        // checkpoint times; the objective's terms
    std::vector<int> elem_uni, fslot, sec_slots;   // sec_slots: [nsec*kAdjSlots] materials
    DBuf<int> dof, d_elem_uni, d_fslot;
    DBuf<double> w, J, ck, seg, Ub, Vb, Ab, hbar, theta, scr, mu, rhs, tmp, kmu, mu2, rhs2;
    int pd_solves = 0;                     // solves of the P-Delta fixed point, last sweep
  } adj;
  long steps_since_reset = 0;
  size_t adj_off_fh() const { return 3 * (size_t)nn * ndf; }
  size_t adj_off_st() const { return adj_off_fh() + (size_t)fb_nrec * 12; }
  int adj_save(double *dst);
  int adj_load(const double *src, double t);
  int adjoint_forward(const xg_phase_desc *ph, int N, int K, const xg_objective_desc *obj,
                      double *J);
  int adjoint_backward(double scale, double *grad, int num_uni);
  int adj_pdelta_refine(const xg::FrameView &fv, const xg::AdjView &av);
  // direct differentiation (xg_ddm_forward): per direction the displacement,
  // velocity and acceleration tangents [nd*neq] and the record tangents
  // [nd*nrec*12]; the committed records before the running step
  struct DdmRun {
    bool have = false;
    int nd = 0, nterm = 0;
    std::vector<double> dJt;               // [nd][nterm] the objective's tangent term by term
    DBuf<int> dof, elem_uni;
    DBuf<double> w, J, dJd, dth, dU, dV, dA, dh, fh_prev, q, z, rhs, x, t0, t1;
  } ddm;
  int ddm_forward(const xg_phase_desc *ph, int N, int nd, const double *dtheta,
                  const xg_objective_desc *obj, double *J, double *dJ);
  int ddm_pdelta_refine(const xg::FrameView &fv);
  // analysis state
  xg_phase_desc phase{};
  bool have_phase = false;
  std::vector<double> gm;
  double time = 0.0, time_c = 0.0;
  double lambda_const[8] = {0};
  int pattern_const[8] = {0}, added[8] = {0};
  int dc_eq = -1;
  int last_solver_iters = 0;
  int phase_steps_done = 0;
  bool phase_closed = false;
  int last_nfail = 0;
  // online autotuner: candidates tried in turn on the first launches of an
  // analysis, each timed with CUDA events and normalised by its work (fiber
  // state determinations, PCG iterations); the cheapest is kept
  struct Tuner {
    bool on = false, done = true;
    std::vector<int> cand;
    std::vector<double> cost;
    std::vector<int> samples;
    int chosen = 0, reps = 3;
    void start(std::vector<int> c, int dflt) {
      cand = c; cost.assign(c.size(), 0.0); samples.assign(c.size(), 0);
      on = true; done = false; chosen = dflt;
    }
    int next() const {            // candidate index to try, or -1 when done
      for (size_t k = 0; k < cand.size(); k++)
        if (samples[k] < reps) return (int)k;
      return -1;
    }
    void record(int k, double c) {
      cost[k] += c;
      samples[k]++;
      if (next() < 0) {
        size_t best = 0;
        for (size_t j = 1; j < cand.size(); j++)
          if (cost[j] < cost[best]) best = j;
        chosen = cand[best];
        done = true;
      }
    }
  };
  Tuner tune_elem, tune_pcg;
  // a Newmark step of a many-part model as one CUDA graph: the predictor,
  // then a conditional loop whose body is one Newton iteration ending in a
  // device-side convergence check (xg_analysis_set_graph)
  struct StepGraph {
    bool want = false, built = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    DBuf<double> t;
    DBuf<int> stat;
    long launches = 0;
  } sg;
  void free_step_graph() {
    if (sg.exec) cudaGraphExecDestroy(sg.exec);
    if (sg.graph) cudaGraphDestroy(sg.graph);
    sg.exec = nullptr;
    sg.graph = nullptr;
    sg.built = false;
  }
  bool step_graph_usable() const;
  int build_step_graph();
  int step_newmark_graph(xg_step_stats *st);
  int fbc_warps = 4, pcg_rows = 64;
  cudaEvent_t tune_a = nullptr, tune_b = nullptr;
  // per-kernel CUDA-event timing on the model's stream (xg_profile_*)
  struct ProfSlot {
    const char *name;
    double ms;
    long launches;
    cudaEvent_t a, b;
    bool pending;
  };
  std::vector<ProfSlot> prof;
  bool prof_on = false;
  enum { P_UPDATE, P_ASSEMBLE, P_GATHER_K, P_GATHER_R, P_PCG_FACTOR, P_PCG, P_LDL_FACTOR,
         P_LDL_SOLVE, P_NSLOTS };
  void prof_init() {
    const char *names[P_NSLOTS] = {
        frames() ? "fbc_update" : etype == XG_ELE_QUAD ? "quad_update" : "brick_update",
        frames() ? "fbc_assemble" : etype == XG_ELE_QUAD ? "quad_assemble" : "brick_assemble",
        "gather_tangent", "gather_resid", "pcg_factor_blocks", "pcg", "ldl_factor", "ldl_solve"};
    for (int k = 0; k < P_NSLOTS; k++) {
      ProfSlot p{names[k], 0.0, 0, nullptr, nullptr, false};
      cudaEventCreate(&p.a);
      cudaEventCreate(&p.b);
      prof.push_back(p);
    }
  }
  void prof_begin(int k) {
    if (prof_on) cudaEventRecord(prof[k].a, stream);
  }
  void prof_end(int k, int launches) {
    if (!prof_on) return;
    cudaEventRecord(prof[k].b, stream);
    prof[k].launches += launches;
    prof[k].pending = true;
  }
  void prof_flush() {
    if (!prof_on) return;
    for (auto &p : prof)
      if (p.pending) {
        cudaEventSynchronize(p.b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        p.ms += ms;
        p.pending = false;
      }
  }

  ContinuumView view() {
    ContinuumView v{};
    v.ne = ne; v.nn = nn; v.nen = nen; v.nip = nip; v.ndf = ndf; v.ndm = ndm;
    v.conn = d_conn.p; v.crd = d_crd.p; v.U = d_U.p; v.mat = d_mat.p; v.j2 = d_j2.p;
    v.thickness = thickness;
    v.ep_c = d_epc.p; v.xi_c = d_xic.p; v.ep_t = d_ept.p; v.xi_t = d_xit.p;
    v.sig = d_sig.p; v.tan = d_tan.p; v.nfail = d_nfail.p;
    v.Ke = d_Ke.p; v.Re = d_Re.p;
    v.geo = d_geo.p;
    v.geo2 = d_geo2.p;
    return v;
  }
  bool frames() const { return etype == XG_ELE_FBC2D || etype == XG_ELE_FBC3D; }
  int nhist() const { return etype == XG_ELE_QUAD ? 4 : 6; }
  int nsig() const { return etype == XG_ELE_QUAD ? 3 : 6; }
  int ntan() const { return etype == XG_ELE_QUAD ? 6 : 9; }
  long npts() const { return (long)ne * nip; }
  // the element scratch holds float pairs (the float-float brick tangent)
  bool ke_pairs() const { return etype == XG_ELE_BRICK && d_geo2.p != nullptr; }
  int ke_size() const {
    if (frames()) return ned * ned;
    return ned * ned;
  }
  // force-based frames: section and material tables, element state
  int fb_nb = 0, fb_nip = 0, fb_max_iters = 10, geom_transf = 0;
  double fb_tol = 1e-12;
  std::vector<int> sec_fstart, fmat, utype;
  std::vector<double> fy, fz, fA, GJ, uparam;
  long fb_nrec = 0;
  DBuf<int> d_fconn, d_fsec, d_sec_fstart, d_fmat, d_utype;
  DBuf<long> d_foff;
  DBuf<double> d_fL, d_fR, d_fy, d_fz, d_fA, d_ybar, d_zbar, d_GJ, d_fs0, d_uparam;
  DBuf<double> d_fyc, d_fzc, d_fk;   // centred fiber coordinates, section-sum products
  DBuf<double> d_fh_c, d_fh_t, d_st, d_st_c;
  DBuf<unsigned long long> d_work;        // frame work counters
  long long point_updates = 0, elem_updates = 0;   // continuum work counters
  std::vector<double> fh_init;
  std::vector<double> crd_vecxz;
  double lob_xi[10] = {0}, lob_wt[10] = {0};
  FrameView fview() {
    FrameView v{};
    v.ne = ne; v.nb = fb_nb; v.nip = fb_nip; v.ndf = ndf;
    v.U = d_U.p; v.conn = d_fconn.p; v.L = d_fL.p; v.R = d_fR.p; v.sec = d_fsec.p;
    v.sec_fstart = d_sec_fstart.p; v.fy = d_fy.p; v.fz = d_fz.p; v.fA = d_fA.p;
    v.fyc = d_fyc.p; v.fzc = d_fzc.p; v.fk = d_fk.p; v.nfib = (int)fy.size();
    v.fmat = d_fmat.p; v.ybar = d_ybar.p; v.zbar = d_zbar.p; v.GJ = d_GJ.p; v.fs0 = d_fs0.p;
    v.utype = d_utype.p; v.uparam = d_uparam.p; v.foff = d_foff.p; v.fh_c = d_fh_c.p;
    v.fh_t = d_fh_t.p; v.st = d_st.p; v.max_iters = fb_max_iters; v.tol = fb_tol;
    for (int i = 0; i < 10; i++) { v.xi[i] = lob_xi[i]; v.wt[i] = lob_wt[i]; }
    v.nfail = d_nfail.p; v.Ke = d_Ke.p; v.Re = d_Re.p; v.work = d_work.p;
    v.pdelta2d = (fb_nb == 3 && geom_transf == 1) ? 1 : 0;
    return v;
  }
  int upload_frames();
  int commit_state();
  int revert_state();

  ~xg_model() {
    free_step_graph();
    for (auto &p : prof) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    if (tune_a) cudaEventDestroy(tune_a);
    if (tune_b) cudaEventDestroy(tune_b);
    if (stream) cudaStreamDestroy(stream);
  }

  int number();
  int build_maps(HostGather &gk_h, HostGather &gr_h);
  int upload(const HostGather &gk_h, const HostGather &gr_h);
  int element_state(bool compute);
  int solve(const double *b, double *x, int *iters);
  // two systems with the same tangent (DisplacementControl::update solves
  // the unbalance and the reference load with one factorisation)
  int solve2(const double *b1, double *x1, const double *b2, double *x2) {
    if (system == XG_SYSTEM_PROFILE_SPD) {
      const double *bs[2] = {b1, b2};
      double *xs[2] = {x1, x2};
      return solve_profile(2, bs, xs);
    }
    RET(solve(b1, x1, nullptr));
    return solve(b2, x2, nullptr);
  }
  int form_fext(double t);
  int step(xg_step_stats *st);
  int init_phase();
  double lambda_of(int p, double t) const {
    if (p < 0 || p >= 8 || !added[p]) return 0.0;
    return pattern_const[p] ? lambda_const[p] : t;
  }
};

// ---------------------------------------------------------------------------
// numbering and pattern
// ---------------------------------------------------------------------------
int xg_model::number() {
  // handler IDs: -2 free, -1 SP, -4 MP-constrained
  eqn.assign((size_t)nn * ndf, -2);
  auto index_of = [&](int tag) -> int {
    auto it = std::lower_bound(node_tag.begin(), node_tag.end(), tag);
    if (it == node_tag.end() || *it != tag) return -1;
    return (int)(it - node_tag.begin());
  };
  for (int s = 0; s < num_sp; s++) {
    int n = index_of(sp_node[s]);
    if (n < 0 || sp_dof[s] < 0 || sp_dof[s] >= ndf) return fail(XG_EINVAL, "bad sp %d", s);
    sp_node[s] = n;
    eqn[(size_t)n * ndf + sp_dof[s]] = -1;
  }
  for (int q = 0; q < num_mp; q++) {
    int c = index_of(mp_c[q]), r = index_of(mp_r[q]);
    if (c < 0 || r < 0 || mp_dof[q] < 0 || mp_dof[q] >= ndf) return fail(XG_EINVAL, "bad mp %d", q);
    mp_c[q] = c;
    mp_r[q] = r;
    if (eqn[(size_t)c * ndf + mp_dof[q]] == -2) eqn[(size_t)c * ndf + mp_dof[q]] = -4;
  }
  for (int i = 0; i < num_loads; i++) {
    int n = index_of(load_node[i]);
    if (n < 0) return fail(XG_EINVAL, "bad load node %d", load_node[i]);
    load_node[i] = n;
  }
  // node graph: vertices in tag order, edges between the nodes of an element
  std::vector<int64_t> deg(nn + 1, 0);
  for (int e = 0; e < ne; e++)
    for (int a = 0; a < nen; a++) deg[conn[(size_t)e * nen + a] + 1] += nen - 1;
  std::vector<int64_t> aptr(nn + 1, 0);
  for (int i = 0; i < nn; i++) aptr[i + 1] = aptr[i] + deg[i + 1];
  std::vector<int> araw(aptr[nn]);
  std::vector<int64_t> fill(aptr.begin(), aptr.end() - 1);
  for (int e = 0; e < ne; e++) {
    const int *c = &conn[(size_t)e * nen];
    for (int a = 0; a < nen; a++)
      for (int b = 0; b < nen; b++)
        if (a != b) araw[fill[c[a]]++] = c[b];
  }
  std::vector<int64_t> adjp(nn + 1, 0);
  std::vector<int> adj;
  adj.reserve(araw.size());
  for (int n = 0; n < nn; n++) {
    auto b = araw.begin() + aptr[n], en = araw.begin() + aptr[n + 1];
    std::sort(b, en);
    auto last = std::unique(b, en);
    for (auto it = b; it != last; ++it)
      if (*it != n) adj.push_back(*it);
    adjp[n + 1] = (int64_t)adj.size();
  }
  std::vector<int>().swap(araw);
  // reverse Cuthill-McKee from the first vertex (RCM(false))
  std::vector<int> mark(nn, -1), res(nn, 0);
  if (nn > 0) {
    int cur = nn - 1, next = cur - 1, iter = 0;
    res[cur] = 0;
    mark[0] = cur;
    while (next >= 0) {
      const int v = res[cur];
      for (int64_t k = adjp[v]; k < adjp[v + 1]; k++) {
        const int w = adj[k];
        if (mark[w] == -1) {
          mark[w] = next;
          res[next--] = w;
        }
      }
      cur--;
      if (cur == next && cur >= 0) {
        while (iter < nn && mark[iter] != -1) iter++;
        if (iter >= nn) break;
        const int w = iter++;
        next--;
        mark[w] = cur;
        res[cur] = w;
      }
    }
  }
  // equations in RCM order; diagonal blocks = the free dofs of one node
  int eq = 0;
  blk_start.clear();
  for (int i = 0; i < nn; i++) {
    const int n = res[i];
    const int before = eq;
    for (int j = 0; j < ndf; j++)
      if (eqn[(size_t)n * ndf + j] == -2) eqn[(size_t)n * ndf + j] = eq++;
    if (eq > before) blk_start.push_back(before);
  }
  blk_start.push_back(eq);
  neq = eq;
  for (int q = 0; q < num_mp; q++) {
    int &id = eqn[(size_t)mp_c[q] * ndf + mp_dof[q]];
    if (id == -4) id = eqn[(size_t)mp_r[q] * ndf + mp_dof[q]];
    if (id < 0) return fail(XG_EINVAL, "equalDOF on a constrained retained dof (mp %d)", q);
  }
  // pattern: row r = diagonal + equations sharing an element with r
  std::vector<int> owners(neq, -1);      // single owner node, or -2 when shared
  for (int n = 0; n < nn; n++)
    for (int j = 0; j < ndf; j++) {
      const int r = eqn[(size_t)n * ndf + j];
      if (r < 0) continue;
      if (owners[r] == -1) owners[r] = n;
      else if (owners[r] != n) owners[r] = -2;
    }
  auto node_cols = [&](int n, std::vector<int> &out) {
    out.clear();
    for (int j = 0; j < ndf; j++)
      if (eqn[(size_t)n * ndf + j] >= 0) out.push_back(eqn[(size_t)n * ndf + j]);
    for (int64_t k = adjp[n]; k < adjp[n + 1]; k++) {
      const int o = adj[k];
      for (int j = 0; j < ndf; j++)
        if (eqn[(size_t)o * ndf + j] >= 0) out.push_back(eqn[(size_t)o * ndf + j]);
    }
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
  };
  std::vector<std::vector<int>> shared_rows;
  std::vector<int> shared_index(neq, -1);
  for (int r = 0; r < neq; r++)
    if (owners[r] == -2) {
      shared_index[r] = (int)shared_rows.size();
      shared_rows.emplace_back();
    }
  std::vector<int> rowlen(neq, 0), tmp;
  for (int n = 0; n < nn; n++) {
    bool any = false;
    for (int j = 0; j < ndf; j++) any |= eqn[(size_t)n * ndf + j] >= 0;
    if (!any) continue;
    node_cols(n, tmp);
    for (int j = 0; j < ndf; j++) {
      const int r = eqn[(size_t)n * ndf + j];
      if (r < 0) continue;
      if (owners[r] >= 0) rowlen[r] = (int)tmp.size();
      else shared_rows[shared_index[r]].insert(shared_rows[shared_index[r]].end(), tmp.begin(),
                                                tmp.end());
    }
  }
  for (auto &row : shared_rows) {
    std::sort(row.begin(), row.end());
    row.erase(std::unique(row.begin(), row.end()), row.end());
  }
  for (int r = 0; r < neq; r++)
    if (owners[r] == -2) rowlen[r] = (int)shared_rows[shared_index[r]].size();
  rowptr.assign(neq + 1, 0);
  for (int r = 0; r < neq; r++) rowptr[r + 1] = rowptr[r] + rowlen[r];
  nnz = rowptr[neq];
  colidx.assign((size_t)nnz, 0);
  for (int n = 0; n < nn; n++) {
    bool need = false;
    for (int j = 0; j < ndf; j++) {
      const int r = eqn[(size_t)n * ndf + j];
      need |= r >= 0 && owners[r] >= 0;
    }
    if (!need) continue;
    node_cols(n, tmp);
    for (int j = 0; j < ndf; j++) {
      const int r = eqn[(size_t)n * ndf + j];
      if (r >= 0 && owners[r] >= 0) std::copy(tmp.begin(), tmp.end(), colidx.begin() + rowptr[r]);
    }
  }
  for (int r = 0; r < neq; r++)
    if (owners[r] == -2)
      std::copy(shared_rows[shared_index[r]].begin(), shared_rows[shared_index[r]].end(),
                colidx.begin() + rowptr[r]);
  return 0;
}

// Element -> CSR slot contributions, in assembly order (element tag order,
// then the element matrix in row-major order), as FE_Element::addKtToTang /
// SparseGenColLinSOE::addA accumulate them.
int xg_model::build_maps(HostGather &gk_h, HostGather &gr_h) {
  const int ks = ke_size();
  std::vector<int> slot_of;
  std::vector<int64_t> src_of;
  slot_of.reserve((size_t)ne * ned * ned);
  src_of.reserve((size_t)ne * ned * ned);
  std::vector<int> ids(ned);
  for (int e = 0; e < ne; e++) {
    for (int a = 0; a < nen; a++)
      for (int j = 0; j < ndf; j++) ids[a * ndf + j] = eqn[(size_t)conn[(size_t)e * nen + a] * ndf + j];
    for (int i = 0; i < ned; i++) {
      const int r = ids[i];
      if (r < 0) continue;
      const int *rb = &colidx[rowptr[r]], *re = &colidx[rowptr[r + 1]];
      for (int j = 0; j < ned; j++) {
        const int c = ids[j];
        if (c < 0) continue;
        const int *pos = std::lower_bound(rb, re, c);
        if (pos == re || *pos != c) return fail(XG_EINVAL, "pattern lookup failed");
        slot_of.push_back((int)(pos - colidx.data()));
        src_of.push_back((int64_t)e * ks + i * ned + j);
      }
    }
  }
  build_gather(nnz, slot_of, src_of, gk_h);
  slot_of.clear();
  src_of.clear();
  for (int e = 0; e < ne; e++)
    for (int a = 0; a < nen; a++)
      for (int j = 0; j < ndf; j++) {
        const int r = eqn[(size_t)conn[(size_t)e * nen + a] * ndf + j];
        if (r < 0) continue;
        slot_of.push_back(r);
        src_of.push_back((int64_t)e * ned + a * ndf + j);
      }
  build_gather(neq, slot_of, src_of, gr_h);
  return 0;
}

int xg_model::upload(const HostGather &gk_h, const HostGather &gr_h) {
  cudaStream_t s = stream;
  // SoA connectivity and coordinates
  std::vector<int> conn_soa((size_t)ne * nen);
  for (int e = 0; e < ne; e++)
    for (int a = 0; a < nen; a++) conn_soa[(size_t)a * ne + e] = conn[(size_t)e * nen + a];
  std::vector<double> crd_soa((size_t)nn * ndm);
  for (int n = 0; n < nn; n++)
    for (int k = 0; k < ndm; k++) crd_soa[(size_t)k * nn + n] = crd[(size_t)n * ndm + k];
  RET(d_conn.upload(conn_soa.data(), conn_soa.size(), s));
  RET(d_crd.upload(crd_soa.data(), crd_soa.size(), s));
  RET(d_mat.upload(mat.data(), mat.size(), s));
  RET(d_j2.upload(j2.data(), j2.size(), s));
  RET(d_eqn.upload(eqn.data(), eqn.size(), s));
  RET(d_rowptr.upload(rowptr.data(), rowptr.size(), s));
  RET(d_colidx.upload(colidx.data(), colidx.size(), s));
  RET(d_blk.upload(blk_start.data(), blk_start.size(), s));
  const size_t nu = (size_t)nn * ndf;
  RET(d_U.alloc(nu)); RET(d_Uc.alloc(nu));
  CK(cudaMemsetAsync(d_U.p, 0, nu * sizeof(double), s));
  CK(cudaMemsetAsync(d_Uc.p, 0, nu * sizeof(double), s));
  const long np = npts();
  RET(d_epc.alloc(np * nhist())); RET(d_ept.alloc(np * nhist()));
  RET(d_xic.alloc(np)); RET(d_xit.alloc(np));
  RET(d_sig.alloc(np * nsig())); RET(d_tan.alloc(np * ntan()));
  RET(d_sig_c.alloc(np * nsig())); RET(d_tan_c.alloc(np * ntan()));
  RET(d_nfail.alloc(1));
  CK(cudaMemsetAsync(d_nfail.p, 0, sizeof(int), s));
  RET(d_Ke.alloc((size_t)ne * ke_size()));
  RET(d_Re.alloc((size_t)ne * ned));
  RET(d_vals.alloc(nnz > 0 ? nnz : 1)); RET(d_resid.alloc(neq > 0 ? neq : 1));
  RET(d_gk_slot_chunk.upload(gk_h.slot_chunk.data(), gk_h.slot_chunk.size(), s));
  RET(d_gk_chunk_slot.upload(gk_h.chunk_slot.data(), gk_h.chunk_slot.size(), s));
  RET(d_gk_chunk_begin.upload(gk_h.chunk_begin.data(), gk_h.chunk_begin.size(), s));
  // the runs of a map, when it has them
  auto upload_runs = [&](const HostGather &h, DBuf<int> *d, GatherMap &g) -> int {
    if (h.run_slot.empty() && h.long_slots.empty()) return 0;
    const std::vector<int> *v[6] = {&h.run_slot, &h.run_meta, &h.run_begin, &h.run_src,
                                    &h.long_chunks, &h.long_slots};
    for (int k = 0; k < 6; k++) RET(d[k].upload(v[k]->data(), v[k]->size(), s));
    g.nruns = (int)h.run_slot.size();
    g.run_slot = d[0].p ? d[0].p : d[5].p;   // non-null marks a map with runs
    g.run_meta = d[1].p; g.run_begin = d[2].p; g.run_src = d[3].p;
    g.nlong_chunks = (int)h.long_chunks.size(); g.long_chunks = d[4].p;
    g.nlong_slots = (int)h.long_slots.size(); g.long_slots = d[5].p;
    return 0;
  };
  // 32-bit source indices when every index fits (the usual case)
  auto upload_src = [&](const std::vector<int64_t> &src, DBuf<int64_t> &d64, DBuf<int> &d32) {
    int64_t mx = 0;
    for (int64_t v : src) mx = std::max(mx, v);
    if (mx < INT32_MAX) {
      std::vector<int> s32(src.begin(), src.end());
      return d32.upload(s32.data(), s32.size(), s);
    }
    return d64.upload(src.data(), src.size(), s);
  };
  RET(upload_src(gk_h.src, d_gk_src, d_gk_src32));
  RET(d_gr_slot_chunk.upload(gr_h.slot_chunk.data(), gr_h.slot_chunk.size(), s));
  RET(d_gr_chunk_slot.upload(gr_h.chunk_slot.data(), gr_h.chunk_slot.size(), s));
  RET(d_gr_chunk_begin.upload(gr_h.chunk_begin.data(), gr_h.chunk_begin.size(), s));
  RET(upload_src(gr_h.src, d_gr_src, d_gr_src32));
  gk.nslots = nnz; gk.nchunks = (int)gk_h.chunk_slot.size();
  gk.chunk_slot = d_gk_chunk_slot.p; gk.chunk_begin = d_gk_chunk_begin.p;
  gk.slot_chunk = d_gk_slot_chunk.p; gk.src = d_gk_src.p; gk.src32 = d_gk_src32.p;
  RET(upload_runs(gk_h, d_gk_run, gk));
  RET(upload_runs(gr_h, d_gr_run, gr));
  gr.nslots = neq; gr.nchunks = (int)gr_h.chunk_slot.size();
  gr.chunk_slot = d_gr_chunk_slot.p; gr.chunk_begin = d_gr_chunk_begin.p;
  gr.slot_chunk = d_gr_slot_chunk.p; gr.src = d_gr_src.p; gr.src32 = d_gr_src32.p;
  RET(d_partial.alloc(std::max(gk.nchunks, gr.nchunks) + 1));
  // solver
  const int nblk = (int)blk_start.size() - 1;
  RET(d_binv.alloc((size_t)std::max(nblk, 1) * 36));
  const size_t nv = neq > 0 ? neq : 1;
  RET(d_r.alloc(nv)); RET(d_z.alloc(nv)); RET(d_p.alloc(nv)); RET(d_q.alloc(nv));
  RET(d_pcg_part.alloc(4 * (size_t)pcg_max_blocks() + 8));
  RET(d_scalars.alloc(8));
  RET(d_barrier.alloc(2));
  RET(d_flags.alloc(4));
  pcg.n = neq; pcg.rowptr = d_rowptr.p; pcg.colidx = d_colidx.p; pcg.vals = d_vals.p;
  pcg.nblk = nblk; pcg.blk_start = d_blk.p; pcg.binv = d_binv.p;
  pcg.r = d_r.p; pcg.z = d_z.p; pcg.p = d_p.p; pcg.q = d_q.p;
  pcg.partials = d_pcg_part.p; pcg.barrier = d_barrier.p; pcg.flags = d_flags.p;
  pcg.scalars = d_scalars.p;
  RET(d_fext.alloc(nv)); RET(d_B.alloc(nv)); RET(d_dU.alloc(nv)); RET(d_phat.alloc(nv));
  RET(d_dUhat.alloc(nv)); RET(d_x.alloc(nv)); RET(d_b.alloc(nv)); RET(d_norm.alloc(1));
  // reference load vector of every pattern that has nodal loads
  std::vector<int> pats;
  for (int i = 0; i < num_loads; i++)
    if (std::find(pats.begin(), pats.end(), load_pat[i]) == pats.end()) pats.push_back(load_pat[i]);
  ref_patterns = pats;
  std::vector<double> F(pats.size() * nv, 0.0);
  for (size_t k = 0; k < pats.size(); k++)
    for (int i = 0; i < num_loads; i++) {
      if (load_pat[i] != pats[k]) continue;
      for (int j = 0; j < ndf; j++) {
        const int r = eqn[(size_t)load_node[i] * ndf + j];
        if (r >= 0) F[k * nv + r] += load_val[(size_t)i * ndf + j];
      }
    }
  if (!F.empty()) RET(d_Fref.upload(F.data(), F.size(), s));
  if (handler == XG_HANDLER_TRANSFORMATION) {
    // the imposed values: U index (sp_node holds node indices by now),
    // pattern and reference value of every sp inside a load pattern
    std::vector<int> idx, pat;
    std::vector<double> val;
    for (int k = 0; k < num_sp; k++)
      if (sp_pat[k] >= 0) {
        idx.push_back(sp_node[k] * ndf + sp_dof[k]);
        pat.push_back(sp_pat[k]);
        val.push_back(sp_val[k]);
      }
    num_isp = (int)idx.size();
    if (num_isp) {
      RET(d_isp_idx.upload(idx.data(), idx.size(), s));
      RET(d_isp_pat.upload(pat.data(), pat.size(), s));
      RET(d_isp_val.upload(val.data(), val.size(), s));
    }
  }
  RET(upload_dynamics());
  if (frames()) {
    RET(upload_frames());
  } else {
    if (etype == XG_ELE_BRICK) {
      RET(d_geo.alloc((size_t)25 * np));
      // the float-float tangent writes float pairs that only the run gather
      // reads: without a run map (a scratch past 32-bit indices) the FP64 one
      if (gk.run_slot && gk.src32) RET(d_geo2.alloc((size_t)24 * np));
      CK(cudaMemsetAsync(d_nfail.p, 0, sizeof(int), s));
      RET(launch_brick_geometry(view(), d_geo.p, d_geo2.p, d_nfail.p, s));
      int bad = 0;
      CK(cudaMemcpyAsync(&bad, d_nfail.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      CK(cudaMemsetAsync(d_nfail.p, 0, sizeof(int), s));
      // a gradient outside the float pairs' range: the tangent in FP64
      if (bad) d_geo2.free();
    }
    // zero-strain material state
    RET(launch_j2_zero_state(view(), s));
    CK(cudaMemcpyAsync(d_sig_c.p, d_sig.p, np * nsig() * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_tan_c.p, d_tan.p, np * ntan() * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  CK(cudaStreamSynchronize(s));
  return 0;
}

namespace {
// LobattoBeamIntegration::getSectionLocations / getSectionWeights
// (quadrature/Frame/LobattoBeamIntegration.cpp:110-320): the reference's
// truncated constants, mapped to [0, 1], weights halved.
void lobatto_points(int n, double *xi, double *wt) {
  static const double x3[3] = {-1.0, 0.0, 1.0};
  static const double w3[3] = {0.333333333333333, 1.333333333333333, 0.333333333333333};
  static const double x4[4] = {-1.0, -0.44721360, 0.44721360, 1.0};
  static const double w4[4] = {0.166666666666667, 0.833333333333333, 0.833333333333333,
                               0.166666666666667};
  static const double x5[5] = {-1.0, -0.65465367, 0.0, 0.65465367, 1.0};
  static const double w5[5] = {0.1, 0.5444444444, 0.7111111111, 0.5444444444, 0.1};
  const double *x = n == 3 ? x3 : n == 4 ? x4 : x5;
  const double *w = n == 3 ? w3 : n == 4 ? w4 : w5;
  for (int i = 0; i < n; i++) {
    xi[i] = 0.5 * (x[i] + 1.0);
    wt[i] = 0.5 * w[i];
  }
}

// Initial tangent of a uniaxial row (Steel02 E0; Concrete02 and Concrete01
// 2 fc / epsc0 after the constructors' sign normalisation, Concrete02.cpp:
// 97-111, Concrete01.cpp:89-112).
double uniaxial_initial_tangent(int type, const double *q) {
  if (type == XG_UNI_STEEL02 || type == XG_UNI_STEEL01) return q[1];
  if (type == XG_UNI_CONCRETE02 || type == XG_UNI_CONCRETE01) {
    const double fc = q[0] > 0 ? -q[0] : q[0], e0 = q[1] > 0 ? -q[1] : q[1];
    return 2.0 * fc / e0;
  }
  return q[0];
}

// Committed record of a fresh material (Steel02::revertToStart, Steel02.cpp:
// 70-95; Concrete02 constructor, Concrete02.cpp:97-111).
void uniaxial_initial_record(int type, const double *q, double *h) {
  for (int c = 0; c < 12; c++) h[c] = 0.0;
  if (type == XG_UNI_STEEL02) {
    h[1] = q[0] / q[1];
    h[0] = -h[1];
    h[8] = q[1];
    if (q[10] != 0.0) { h[10] = q[10] / q[1]; h[9] = q[10]; }
  } else if (type == XG_UNI_STEEL01) {
    // Steel01::revertToStart (Steel01.cpp:285-310): shifts 1, tangent E0
    h[2] = 1.0;
    h[3] = 1.0;
    h[8] = q[1];
  } else if (type == XG_UNI_CONCRETE01) {
    // Concrete01::revertToStart (Concrete01.cpp:435-457): unloading slope
    // and tangent Ec0
    h[2] = uniaxial_initial_tangent(type, q);
    h[8] = h[2];
  } else {
    h[8] = uniaxial_initial_tangent(type, q);
  }
}

// small dense inverse (Gauss-Jordan, partial pivoting)
void host_inverse(int n, const double *A, double *Ai) {
  double M[6][12];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < 2 * n; j++) M[i][j] = j < n ? A[i * n + j] : (j - n == i ? 1.0 : 0.0);
  for (int c = 0; c < n; c++) {
    int piv = c;
    for (int i = c + 1; i < n; i++)
      if (std::fabs(M[i][c]) > std::fabs(M[piv][c])) piv = i;
    if (piv != c)
      for (int j = 0; j < 2 * n; j++) std::swap(M[c][j], M[piv][j]);
    const double inv = 1.0 / M[c][c];
    for (int j = 0; j < 2 * n; j++) M[c][j] *= inv;
    for (int i = 0; i < n; i++) {
      if (i == c) continue;
      const double f = M[i][c];
      for (int j = 0; j < 2 * n; j++) M[i][j] -= f * M[c][j];
    }
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) Ai[i * n + j] = M[i][n + j];
}
}  // namespace

// Frame element set: geometry (LinearCrdTransf2d::computeElemtLengthAndOrient,
// coordTransformation/LinearCrdTransf2d.cpp:175-220; FrameTransform::Orient,
// coordTransformation/FrameTransform.h:105-129), section centroids
// (FiberSection2d::addFiber, material/section/FiberSection2d.cpp:148-153),
// initial section flexibilities, fresh fiber records, zero element state,
// then the update Domain::addElement performs (domain/domain/Domain.cpp:390-392).
int xg_model::upload_frames() {
  cudaStream_t s = stream;
  lobatto_points(fb_nip, lob_xi, lob_wt);
  const int nsec = (int)sec_fstart.size() - 1;
  std::vector<double> Lh(ne), Rh((size_t)ne * 9, 0.0);
  for (int e = 0; e < ne; e++) {
    const int a = conn[2 * (size_t)e], b = conn[2 * (size_t)e + 1];
    double dx[3] = {0, 0, 0};
    for (int k = 0; k < ndm; k++) dx[k] = crd[(size_t)b * ndm + k] - crd[(size_t)a * ndm + k];
    const double L = std::sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
    if (L == 0.0) return fail(XG_EINVAL, "element %d has zero length", e);
    Lh[e] = L;
    double *R = &Rh[9 * (size_t)e];
    if (ndm == 2) {
      R[0] = dx[0] / L;
      R[1] = dx[1] / L;
    } else {
      const double *vz = &crd_vecxz[3 * (size_t)e];
      const double e1[3] = {dx[0] / L, dx[1] / L, dx[2] / L};
      double e2[3] = {vz[1] * e1[2] - vz[2] * e1[1], vz[2] * e1[0] - vz[0] * e1[2],
                      vz[0] * e1[1] - vz[1] * e1[0]};
      const double yn = std::sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
      if (yn == 0.0) return fail(XG_EINVAL, "element %d: vecxz parallel to the axis", e);
      for (int k = 0; k < 3; k++) e2[k] /= yn;
      const double e3[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                            e1[0] * e2[1] - e1[1] * e2[0]};
      for (int k = 0; k < 3; k++) {
        R[3 * k + 0] = e1[k];
        R[3 * k + 1] = e2[k];
        R[3 * k + 2] = e3[k];
      }
    }
  }
  const int order = fb_nb == 3 ? 2 : 4;
  std::vector<double> ybar(nsec), zbar(nsec), fs0((size_t)nsec * 16, 0.0);
  for (int sc = 0; sc < nsec; sc++) {
    double A = 0, Qz = 0, Qy = 0;
    double k[16] = {0};
    for (int f = sec_fstart[sc]; f < sec_fstart[sc + 1]; f++) {
      A += fA[f];
      Qz += fy[f] * fA[f];
      Qy += fz[f] * fA[f];
    }
    ybar[sc] = Qz / A;
    zbar[sc] = Qy / A;
    for (int f = sec_fstart[sc]; f < sec_fstart[sc + 1]; f++) {
      const int u = fmat[f];
      const double EA = uniaxial_initial_tangent(utype[u], &uparam[(size_t)u * XG_UNI_NPARAM]) * fA[f];
      const double y = fy[f] - ybar[sc], z = fz[f] - zbar[sc];
      if (order == 2) {
        const double ks1 = EA * -y;
        k[0] += EA; k[1] += ks1; k[3] += ks1 * -y;
      } else {
        k[0] += EA; k[1] += -y * EA; k[2] += z * EA;
        k[5] += y * y * EA; k[10] += z * z * EA; k[6] += -y * z * EA;
      }
    }
    if (order == 2) k[2] = k[1];
    else { k[4] = k[1]; k[8] = k[2]; k[9] = k[6]; k[15] = GJ[sc]; }
    host_inverse(order, k, &fs0[(size_t)sc * 16]);
  }
  std::vector<long> foff(ne + 1, 0);
  for (int e = 0; e < ne; e++) {
    const int sc = mat[e];
    foff[e + 1] = foff[e] + (long)fb_nip * (sec_fstart[sc + 1] - sec_fstart[sc]);
  }
  fb_nrec = foff[ne];
  fh_init.assign((size_t)fb_nrec * 12, 0.0);
  for (int e = 0; e < ne; e++) {
    const int sc = mat[e], nf = sec_fstart[sc + 1] - sec_fstart[sc];
    for (int ip = 0; ip < fb_nip; ip++)
      for (int f = 0; f < nf; f++) {
        const int u = fmat[sec_fstart[sc] + f];
        uniaxial_initial_record(utype[u], &uparam[(size_t)u * XG_UNI_NPARAM],
                                &fh_init[((size_t)foff[e] + (size_t)ip * nf + f) * 12]);
      }
  }
  RET(d_fconn.upload(conn.data(), conn.size(), s));
  RET(d_fsec.upload(mat.data(), mat.size(), s));
  RET(d_fL.upload(Lh.data(), Lh.size(), s));
  RET(d_fR.upload(Rh.data(), Rh.size(), s));
  RET(d_sec_fstart.upload(sec_fstart.data(), sec_fstart.size(), s));
  RET(d_fy.upload(fy.data(), fy.size(), s));
  RET(d_fz.upload(fz.data(), fz.size(), s));
  RET(d_fA.upload(fA.data(), fA.size(), s));
  RET(d_fmat.upload(fmat.data(), fmat.size(), s));
  RET(d_ybar.upload(ybar.data(), ybar.size(), s));
  RET(d_zbar.upload(zbar.data(), zbar.size(), s));
  {
    // the fibers' centred coordinates and the products the section sums
    // take (the tangent and the stress times each of them)
    const size_t nf = fy.size();
    std::vector<double> yc(nf), zc(nf), fk(6 * nf);
    for (int sc = 0; sc < nsec; sc++)
      for (int f = sec_fstart[sc]; f < sec_fstart[sc + 1]; f++) {
        const double y = fy[f] - ybar[sc], z = fz[f] - zbar[sc], A = fA[f];
        yc[f] = y;
        zc[f] = z;
        fk[f] = A;
        fk[nf + f] = -y * A;
        fk[2 * nf + f] = z * A;
        fk[3 * nf + f] = y * y * A;
        fk[4 * nf + f] = z * z * A;
        fk[5 * nf + f] = -y * z * A;
      }
    RET(d_fyc.upload(yc.data(), nf, s));
    RET(d_fzc.upload(zc.data(), nf, s));
    RET(d_fk.upload(fk.data(), fk.size(), s));
  }
  RET(d_GJ.upload(GJ.data(), GJ.size(), s));
  RET(d_fs0.upload(fs0.data(), fs0.size(), s));
  RET(d_utype.upload(utype.data(), utype.size(), s));
  // device parameter table: Steel02 rows carry Fy/E0 in slot 11, Concrete02
  // rows their per-material constants in slots 7-11
  std::vector<double> up_dev(uparam);
  for (size_t u = 0; u < utype.size(); u++)
    if (utype[u] == XG_UNI_STEEL02)
      up_dev[u * XG_UNI_NPARAM + 11] = up_dev[u * XG_UNI_NPARAM] / up_dev[u * XG_UNI_NPARAM + 1];
  RET(d_uparam.upload(up_dev.data(), up_dev.size(), s));
  RET(launch_c02_constants(d_uparam.p, d_utype.p, (int)utype.size(), s));
  RET(d_foff.upload(foff.data(), foff.size(), s));
  RET(d_work.alloc(2));
  CK(cudaMemsetAsync(d_work.p, 0, 2 * sizeof(unsigned long long), s));
  RET(d_fh_c.upload(fh_init.data(), fh_init.size(), s));
  RET(d_fh_t.upload(fh_init.data(), fh_init.size(), s));
  const size_t nst = (size_t)ne * frame_state_stride(fb_nip);
  RET(d_st.alloc(nst > 0 ? nst : 1));
  RET(d_st_c.alloc(nst > 0 ? nst : 1));
  CK(cudaMemsetAsync(d_st.p, 0, (nst > 0 ? nst : 1) * sizeof(double), s));
  CK(cudaMemsetAsync(d_st_c.p, 0, (nst > 0 ? nst : 1) * sizeof(double), s));
  // the update Domain::addElement performs, at zero displacement
  RET(element_state(true));
  int nf = 0;
  CK(cudaMemcpyAsync(&nf, d_nfail.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (nf) return fail(XG_EELEMENT, "%d elements failed their initial state determination", nf);
  return 0;
}

// Domain::update (when compute) and the element K / P assembled into the
// CSR values and the resisting force.
// Per-equation (node, dof) lists, masses and diagonal positions, zero
// velocity and acceleration, and the disconnected parts of the model (each
// a contiguous equation range after RCM) for per-part convergence.
int xg_model::upload_dynamics() {
  cudaStream_t s = stream;
  const int nu = nn * ndf;
  std::vector<int> cnt(neq + 1, 0), ptr(neq + 1, 0), dofs(std::max(nu, 1), 0);
  for (int a = 0; a < nu; a++)
    if (eqn[a] >= 0) cnt[eqn[a]]++;
  for (int e = 0; e < neq; e++) ptr[e + 1] = ptr[e] + cnt[e];
  std::vector<int> fillp(ptr.begin(), ptr.end() - 1);
  std::vector<double> meq(std::max(neq, 1), 0.0);
  for (int a = 0; a < nu; a++) {
    const int e = eqn[a];
    if (e < 0) continue;
    dofs[fillp[e]++] = a;
    meq[e] += node_mass[a];
  }
  std::vector<int> dpos(std::max(neq, 1), 0);
  for (int e = 0; e < neq; e++) {
    const int *b = colidx.data() + rowptr[e], *en = colidx.data() + rowptr[e + 1];
    dpos[e] = (int)(std::lower_bound(b, en, e) - colidx.data());
  }
  RET(d_eq_ptr.upload(ptr.data(), ptr.size(), s));
  RET(d_eq_dofs.upload(dofs.data(), dofs.size(), s));
  RET(d_meq.upload(meq.data(), meq.size(), s));
  RET(d_diag_pos.upload(dpos.data(), dpos.size(), s));
  RET(d_mass.upload(node_mass.data(), std::max<size_t>(node_mass.size(), 1), s));
  for (auto *b : {&d_V, &d_A, &d_Vc, &d_Ac}) {
    RET(b->alloc(std::max(nu, 1)));
    CK(cudaMemsetAsync(b->p, 0, std::max(nu, 1) * sizeof(double), s));
  }
  RET(d_veq.alloc(std::max(neq, 1)));
  RET(d_k0v.alloc(std::max(neq, 1)));
  // disconnected parts: union of the nodes of every element and equalDOF pair
  std::vector<int> parent(nn);
  for (int i = 0; i < nn; i++) parent[i] = i;
  auto find = [&](int x) {
    while (parent[x] != x) x = parent[x] = parent[parent[x]];
    return x;
  };
  for (int e = 0; e < ne; e++)
    for (int a = 1; a < nen; a++) {
      const int x = find(conn[(size_t)e * nen]), y = find(conn[(size_t)e * nen + a]);
      if (x != y) parent[std::max(x, y)] = std::min(x, y);
    }
  for (size_t q = 0; q < mp_c.size(); q++) {
    const int x = find(mp_c[q]), y = find(mp_r[q]);
    if (x != y) parent[std::max(x, y)] = std::min(x, y);
  }
  std::vector<int> lo(nn, INT32_MAX), hi(nn, -1), count(nn, 0);
  for (int a = 0; a < nu; a++) {
    const int e = eqn[a];
    if (e < 0) continue;
    const int r = find(a / ndf);
    lo[r] = std::min(lo[r], e);
    hi[r] = std::max(hi[r], e);
  }
  for (int e = 0; e < neq; e++) count[find(dofs[ptr[e]] / ndf)]++;
  std::vector<std::pair<int, int>> ranges;
  bool contiguous = true;
  for (int r = 0; r < nn; r++) {
    if (hi[r] < 0) continue;
    if (hi[r] - lo[r] + 1 != count[r]) contiguous = false;
    ranges.push_back({lo[r], hi[r] + 1});
  }
  std::sort(ranges.begin(), ranges.end());
  comp_start.assign(1, 0);
  if (contiguous) {
    for (auto &rg : ranges) comp_start.push_back(rg.second);
  } else {
    comp_start.push_back(neq);
  }
  const int ncomp = (int)comp_start.size() - 1;
  std::vector<int> comp_of(std::max(neq, 1), 0);
  for (int c = 0; c < ncomp; c++)
    for (int e = comp_start[c]; e < comp_start[c + 1]; e++) comp_of[e] = c;
  RET(d_cstart.upload(comp_start.data(), comp_start.size(), s));
  RET(d_comp_of.upload(comp_of.data(), comp_of.size(), s));
  RET(d_active.alloc(std::max(ncomp, 1)));
  RET(d_cnorm.alloc(std::max(ncomp, 1)));
  return 0;
}

// One transient step: Newmark::newStep, NewtonRaphson::solveCurrentStep with
// the effective tangent and the dynamic unbalance, then commit.  Each
// disconnected part of the model carries its own convergence test: a part
// whose displacement increment (or unbalance) norm has passed stops
// iterating -- its right-hand side is zeroed, so its state does not move --
// while the others go on, exactly as if every part ran alone.
// The captured step applies to Newmark runs of models in several parts with
// the per-part band LDL', constant external loads, and no per-kernel timing
// or autotuning in progress (those read the device between launches).
bool xg_model::step_graph_usable() const {
  if (!sg.want || phase.integrator != XG_INT_NEWMARK || system != XG_SYSTEM_PROFILE_SPD) return false;
  if (!prof_ready || !prof_band || prof_on) return false;
  if ((tune_elem.on && !tune_elem.done) || (tune_pcg.on && !tune_pcg.done)) return false;
  for (int p : ref_patterns)
    if (p >= 0 && p < 8 && added[p] && !pattern_const[p]) return false;
  return true;
}

int xg_model::build_step_graph() {
  free_step_graph();
  cudaStream_t s = stream;
  const int ncomp = (int)comp_start.size() - 1;
  const double dt = phase.dt, gam = phase.gamma, bet = phase.beta;
  const double c1 = 1.0, c2 = gam / (bet * dt), c3 = 1.0 / (bet * dt * dt);
  const double a1 = 1.0 - gam / bet, a2 = dt * (1.0 - 0.5 * gam / bet);
  const double a3 = -1.0 / (bet * dt), a4 = 1.0 - 0.5 / bet;
  DynView dv = dview();
  RET(sg.t.alloc(1));
  RET(sg.stat.alloc(4));
  RET(form_fext(time));                  // constant over the phase
  CK(cudaStreamSynchronize(s));
  cudaGraph_t parent = nullptr, pre = nullptr;
  CK(cudaGraphCreate(&parent, 0));
  CK(cudaGraphCreate(&pre, 0));
  auto give_up = [&](int code, const char *what) {
    cudaGraph_t dummy = nullptr;
    cudaStreamEndCapture(s, &dummy);
    cudaGraphDestroy(pre);
    cudaGraphDestroy(parent);
    return fail(code, "step graph: %s", what);
  };
  // Newmark::newStep and the first unbalance
  CK(cudaStreamBeginCaptureToGraph(s, pre, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  int r = launch_step_begin(sg.t.p, dt, sg.stat.p, d_active.p, ncomp, s);
  if (!r) r = launch_newmark_predict(dv, a1, a2, a3, a4, s);
  if (!r) r = element_state(true);
  if (!r) r = launch_dyn_unbalance(dv, d_fext.p, d_resid.p, d_K0vals.p, d_rowptr.p, d_colidx.p,
                                   k0_ready ? 1.0 : 0.0, phase.alpha_m, 0.0, d_veq.p, d_k0v.p,
                                   d_B.p, s, sg.t.p);
  if (r) return give_up(r, "capture of the predictor failed");
  cudaGraph_t got = nullptr;
  CK(cudaStreamEndCapture(s, &got));
  // the Newton loop: a conditional while node, one iteration per pass
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, parent, 1, cudaGraphCondAssignDefault));
  cudaGraphNode_t npre, ncond;
  CK(cudaGraphAddChildGraphNode(&npre, parent, nullptr, 0, pre));
  cudaGraphDestroy(pre);
  pre = nullptr;
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  CK(cudaGraphAddNode(&ncond, parent, &npre, nullptr, 1, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  r = launch_dyn_tangent(dv, d_vals.p, d_K0vals.p, c1, k0_ready ? c2 : 0.0, c2, c3, s);
  if (!r && cudaMemcpyAsync(d_px.p, d_B.p, (size_t)neq * sizeof(double), cudaMemcpyDeviceToDevice,
                            s) != cudaSuccess)
    r = XG_ECUDA;
  if (!r) r = band_factor_async(bsys, s, 1, d_px.p, prof_ldx);
  if (!r) r = band_solve(bsys, 1, d_px.p, prof_ldx, s, false);
  if (!r && cudaMemcpyAsync(d_dU.p, d_px.p, (size_t)neq * sizeof(double), cudaMemcpyDeviceToDevice,
                            s) != cudaSuccess)
    r = XG_ECUDA;
  if (!r) r = launch_newmark_correct(dv, d_dU.p, c2, c3, s);
  if (!r) r = element_state(true);
  if (!r) r = launch_dyn_unbalance(dv, d_fext.p, d_resid.p, d_K0vals.p, d_rowptr.p, d_colidx.p,
                                   k0_ready ? 1.0 : 0.0, phase.alpha_m, 0.0, d_veq.p, d_k0v.p,
                                   d_B.p, s, sg.t.p);
  if (!r) r = launch_comp_norm2(ncomp, d_cstart.p,
                                phase.test == XG_TEST_NORM_DISP_INCR ? d_dU.p : d_B.p, d_cnorm.p, s);
  if (!r) r = launch_newton_check(ncomp, d_cnorm.p, phase.tol, phase.max_iter, d_active.p,
                                  sg.stat.p, h, s);
  if (!r && ncomp > 1) r = launch_comp_mask(neq, d_comp_of.p, d_active.p, d_B.p, s);
  if (r) return give_up(r, "capture of the Newton iteration failed");
  CK(cudaStreamEndCapture(s, &got));
  CK(cudaGraphInstantiate(&sg.exec, parent, 0));
  sg.graph = parent;
  sg.built = true;
  // the graph's kernels per step: 5 before the loop (plus the element
  // state's), 12 per Newton iteration
  return 0;
}

// One Newmark step as a graph launch; the host reads the iteration count,
// the status and the pivot flags once, then commits (or reverts).
int xg_model::step_newmark_graph(xg_step_stats *st) {
  cudaStream_t s = stream;
  if (!sg.built) RET(build_step_graph());
  CK(cudaMemcpyAsync(sg.t.p, &time, sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaGraphLaunch(sg.exec, s));
  sg.launches++;
  int hstat[4] = {0, 0, 0, 0}, hflags[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(hstat, sg.stat.p, sizeof hstat, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(hflags, bsys.flags, sizeof hflags, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  blocks_factored = false;
  prof_factored = false;
  const int ncomp = (int)comp_start.size() - 1;
  if (st) {
    st->newton_iters = hstat[0];
    st->solver_iters = 0;
    st->elem_iters = 0;
    st->status = hstat[1] == 1 ? 0 : XG_ENOCONV;
  }
  if (hflags[0] == 3)
    return fail(XG_ESOLVE, "ProfileSPD: pivot %d fails the check (aii == 0, |aii| <= 1e-12, or "
                "a first pivot <= 0)", hflags[1]);
  if (hstat[1] != 1)
    return fail(XG_ENOCONV, "Newton did not converge in %d iterations (%d of %d parts)",
                hstat[0], hstat[2], ncomp);
  time += phase.dt;
  RET(commit_state());
  CK(cudaMemcpyAsync(d_Vc.p, d_V.p, (size_t)nn * ndf * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(d_Ac.p, d_A.p, (size_t)nn * ndf * sizeof(double), cudaMemcpyDeviceToDevice, s));
  time_c = time;
  return 0;
}

int xg_model::step_newmark(xg_step_stats *st) {
  if (step_graph_usable()) return step_newmark_graph(st);
  cudaStream_t s = stream;
  last_solver_iters = 0;
  const double t_commit = time;
  const double dt = phase.dt, gam = phase.gamma, bet = phase.beta;
  const double c1 = 1.0, c2 = gam / (bet * dt), c3 = 1.0 / (bet * dt * dt);
  const double a1 = 1.0 - gam / bet, a2 = dt * (1.0 - 0.5 * gam / bet);
  const double a3 = -1.0 / (bet * dt), a4 = 1.0 - 0.5 / bet;
  const double am = phase.alpha_m;
  DynView dv = dview();
  const int ncomp = (int)comp_start.size() - 1;
  std::vector<int> active(std::max(ncomp, 1), 1), iters(std::max(ncomp, 1), 0);
  std::vector<double> cn(std::max(ncomp, 1));
  CK(cudaMemcpyAsync(d_active.p, active.data(), ncomp * sizeof(int), cudaMemcpyHostToDevice, s));
  RET(launch_newmark_predict(dv, a1, a2, a3, a4, s));
  time += dt;
  RET(element_state(true));          // Domain::update in updateDomain
  int it = 0, nactive = ncomp;
  bool ok = false;
  while (true) {
    RET(form_fext(time));
    RET(launch_dyn_unbalance(dv, d_fext.p, d_resid.p, d_K0vals.p, d_rowptr.p, d_colidx.p,
                             k0_ready ? 1.0 : 0.0, am, time, d_veq.p, d_k0v.p, d_B.p, s));
    if (it > 0) {
      RET(launch_comp_norm2(ncomp, d_cstart.p,
                            phase.test == XG_TEST_NORM_DISP_INCR ? d_dU.p : d_B.p, d_cnorm.p, s));
      CK(cudaMemcpyAsync(cn.data(), d_cnorm.p, ncomp * sizeof(double), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      for (int c = 0; c < ncomp; c++)
        if (active[c] && std::sqrt(cn[c]) <= phase.tol) {
          active[c] = 0;
          iters[c] = it;
          nactive--;
        }
      if (nactive == 0) { ok = true; break; }
      if (it >= phase.max_iter) break;
      CK(cudaMemcpyAsync(d_active.p, active.data(), ncomp * sizeof(int), cudaMemcpyHostToDevice,
                         s));
      if (ncomp > 1) RET(launch_comp_mask(neq, d_comp_of.p, d_active.p, d_B.p, s));
    }
    RET(launch_dyn_tangent(dv, d_vals.p, d_K0vals.p, c1, k0_ready ? c2 : 0.0, c2, c3, s));
    blocks_factored = false;
    prof_factored = false;
    RET(solve(d_B.p, d_dU.p, nullptr));
    RET(launch_newmark_correct(dv, d_dU.p, c2, c3, s));
    RET(element_state(true));
    it++;
  }
  if (st) {
    st->newton_iters = it;
    st->solver_iters = last_solver_iters;
    st->elem_iters = 0;
    st->status = ok ? 0 : XG_ENOCONV;
  }
  if (!ok) {
    time = t_commit;
    return fail(XG_ENOCONV, "Newton did not converge in %d iterations (%d of %d parts)", it,
                nactive, ncomp);
  }
  RET(commit_state());
  CK(cudaMemcpyAsync(d_Vc.p, d_V.p, (size_t)nn * ndf * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(d_Ac.p, d_A.p, (size_t)nn * ndf * sizeof(double), cudaMemcpyDeviceToDevice, s));
  time_c = time;
  return 0;
}

int xg_model::element_state(bool compute) {
  ContinuumView v = view();
  cudaStream_t s = stream;
  if (frames()) {
    FrameView fv = fview();
    if (compute) {
      CK(cudaMemsetAsync(d_nfail.p, 0, sizeof(int), s));
      prof_begin(P_UPDATE);
      elem_updates += ne;
      const int k = (tune_elem.on && !tune_elem.done) ? tune_elem.next() : -1;
      if (k >= 0) {
        unsigned long long w0 = 0, w1 = 0;
        CK(cudaMemcpyAsync(&w0, d_work.p, sizeof w0, cudaMemcpyDeviceToHost, s));
        CK(cudaEventRecord(tune_a, s));
        RET(launch_fbc_update(fv, s, tune_elem.cand[k]));
        CK(cudaEventRecord(tune_b, s));
        CK(cudaMemcpyAsync(&w1, d_work.p, sizeof w1, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, tune_a, tune_b));
        if (w1 > w0) tune_elem.record(k, ms / ((double)(w1 - w0) * 1e-6));
        if (tune_elem.done) fbc_warps = tune_elem.chosen;
      } else {
        RET(launch_fbc_update(fv, s, fbc_warps));
      }
      prof_end(P_UPDATE, 1);
    }
    prof_begin(P_ASSEMBLE);
    RET(launch_fbc_assemble(fv, s));
    prof_end(P_ASSEMBLE, 1);
  } else {
    if (compute) {
      CK(cudaMemsetAsync(d_nfail.p, 0, sizeof(int), s));
      prof_begin(P_UPDATE);
      point_updates += (long long)npts();
      elem_updates += ne;
      RET(etype == XG_ELE_QUAD ? launch_quad_update(v, s) : launch_brick_update(v, s));
      prof_end(P_UPDATE, 1);
    }
    prof_begin(P_ASSEMBLE);
    RET(etype == XG_ELE_QUAD ? launch_quad_assemble(v, s) : launch_brick_assemble(v, s));
    prof_end(P_ASSEMBLE, 1);
  }
  prof_begin(P_GATHER_K);
  RET(launch_gather(gk, d_Ke.p, d_partial.p, d_vals.p, s, ke_pairs()));
  prof_end(P_GATHER_K, gather_launch_count(gk, ke_pairs()));
  prof_begin(P_GATHER_R);
  RET(launch_gather(gr, d_Re.p, d_partial.p, d_resid.p, s));
  prof_end(P_GATHER_R, gather_launch_count(gr));
  prof_flush();
  blocks_factored = false;
  prof_factored = false;
  return 0;
}

// Envelope plan and tile storage of the device LDL' (once per model).
int xg_model::ensure_profile() {
  if (prof_ready) return 0;
  const int ncomp = (int)comp_start.size() - 1;
  if (ncomp > 1) {
    // disconnected parts: each part's LDL' in its own band, all in one launch
    std::vector<int> bw;
    std::vector<long> boff;
    if (band_plan(neq, rowptr.data(), colidx.data(), comp_start, bw, boff) == 0) {
      size_t free_b = 0, total_b = 0;
      CK(cudaMemGetInfo(&free_b, &total_b));
      if ((size_t)boff[ncomp] * sizeof(double) < free_b / 2) {
        RET(d_bw.upload(bw.data(), bw.size(), stream));
        RET(d_boff.upload(boff.data(), boff.size(), stream));
        RET(d_band.alloc(std::max<long>(boff[ncomp], 1)));
        RET(d_invD.alloc(std::max(neq, 1)));
        RET(d_pflags.alloc(4));
        prof_ldx = std::max(neq, 1);
        RET(d_px.alloc((size_t)prof_ldx * 4));
        bsys.ncomp = ncomp; bsys.cstart = d_cstart.p; bsys.bw = d_bw.p; bsys.boff = d_boff.p;
        bsys.band = d_band.p; bsys.rowptr = d_rowptr.p; bsys.colidx = d_colidx.p;
        bsys.vals = d_vals.p; bsys.invD = d_invD.p; bsys.flags = d_pflags.p;
        bsys.min_diag_tol = 1.0e-12;   // ProfileSPDLinDirectSolver.h:49 default
        bsys.bmax = *std::max_element(bw.begin(), bw.end());
        bsys.nmax = 0;
        for (int c = 0; c < ncomp; c++)
          bsys.nmax = std::max(bsys.nmax, comp_start[c + 1] - comp_start[c]);
        prof_band = true;
        prof_ready = true;
        return 0;
      }
    }
  }
  {
    const int r = envelope.setup(neq, rowptr.data(), colidx.data(), d_rowptr.p, d_colidx.p,
                                 d_vals.p, stream);
    if (r) return r;   // envelope.setup set the error text
  }
  prof_ready = true;
  return 0;
}

// Factor once per tangent, then solve nrhs systems sharing the factors.
int xg_model::solve_profile(int nrhs, const double *const *b, double *const *x) {
  RET(ensure_profile());
  if (prof_band) {
    // the band factorisation carries the right-hand sides through the
    // forward substitution
    for (int r = 0; r < nrhs; r++)
      CK(cudaMemcpyAsync(d_px.p + (size_t)r * prof_ldx, b[r], (size_t)neq * sizeof(double),
                         cudaMemcpyDeviceToDevice, stream));
    const bool fused = !prof_factored;
    if (fused) {
      prof_begin(P_LDL_FACTOR);
      int bad = -1;
      const int r = band_factor(bsys, stream, &bad, nrhs, d_px.p, prof_ldx);
      prof_end(P_LDL_FACTOR, 1);
      if (r) {
        if (bad >= 0) return fail(XG_ESOLVE, "ProfileSPD: pivot %d fails the check (aii == 0, "
                                  "|aii| <= 1e-12, or a first pivot <= 0)", bad);
        return fail(r, "ProfileSPD: band factorisation failed");
      }
      prof_factored = true;
    }
    prof_begin(P_LDL_SOLVE);
    RET(band_solve(bsys, nrhs, d_px.p, prof_ldx, stream, !fused));
    prof_end(P_LDL_SOLVE, fused ? 1 : 2);
    for (int r = 0; r < nrhs; r++)
      CK(cudaMemcpyAsync(x[r], d_px.p + (size_t)r * prof_ldx, (size_t)neq * sizeof(double),
                         cudaMemcpyDeviceToDevice, stream));
    prof_flush();
    return 0;
  }
  if (!prof_factored && envelope.can_fuse()) {
    // the tangent is new and its right-hand sides are known: the forward
    // sweep runs inside the factorisation, then the backward sweep
    prof_begin(P_LDL_FACTOR);
    int bad = -1;
    const int r = envelope.factor_forward(nrhs, b, stream, &bad);
    prof_end(P_LDL_FACTOR, 2);
    if (r) {
      if (bad >= 0) return fail(XG_ESOLVE, "ProfileSPD: pivot %d fails the check (aii == 0, "
                                "|aii| <= 1e-12, or a first pivot <= 0)", bad);
      return fail(XG_ESOLVE, "ProfileSPD: factorisation barrier timed out");
    }
    prof_factored = true;
    prof_begin(P_LDL_SOLVE);
    RET(envelope.solve_backward(nrhs, x, stream));
    prof_end(P_LDL_SOLVE, 1);
    prof_flush();
    return 0;
  }
  if (!prof_factored) {
    prof_begin(P_LDL_FACTOR);
    int bad = -1;
    const int r = envelope.factor(stream, &bad);
    prof_end(P_LDL_FACTOR, 2);
    if (r) {
      if (bad >= 0) return fail(XG_ESOLVE, "ProfileSPD: pivot %d fails the check (aii == 0, "
                                "|aii| <= 1e-12, or a first pivot <= 0)", bad);
      return fail(XG_ESOLVE, "ProfileSPD: factorisation barrier timed out");
    }
    prof_factored = true;
  }
  prof_begin(P_LDL_SOLVE);
  RET(envelope.solve(nrhs, b, x, stream));
  prof_end(P_LDL_SOLVE, 1);
  prof_flush();
  return 0;
}

// Recorder::record (NodeRecorder.cpp:180-210): at the committed time, when
// dT is zero or the time has reached the next stamp less dT * 1e-6.
int xg_model::record_step() {
  for (auto &rp : recorders) {
    Recorder &r = *rp;
    if (!(r.dT == 0.0 || time_c - r.next >= -r.dT * 1e-6)) continue;
    if (r.dT != 0.0) r.next = time_c + r.dT;
    const double *src = r.response == 0 ? d_Uc.p : r.response == 1 ? d_Vc.p : d_Ac.p;
    if (r.kind == 0) {
      if (r.rows == r.cap) {
        // grow by doubling (a device copy; no host round trip per step)
        const int cap = std::max(2 * r.cap, 64);
        DBuf<double> nd;
        RET(nd.alloc((size_t)cap * r.ncol));
        if (r.rows) CK(cudaMemcpyAsync(nd.p, r.data.p, (size_t)r.rows * r.ncol * sizeof(double),
                                       cudaMemcpyDeviceToDevice, stream));
        CK(cudaStreamSynchronize(stream));
        std::swap(r.data.p, nd.p);
        std::swap(r.data.n, nd.n);
        r.cap = cap;
      }
      RET(launch_record(0, r.nvals, r.idx.p, src, time_c, r.echo, 0,
                        r.data.p + (size_t)r.rows * r.ncol, stream));
      r.rows++;
    } else {
      RET(launch_record(1, r.nvals, r.idx.p, src, time_c, r.echo, r.first ? 1 : 0, r.data.p,
                        stream));
      r.first = false;
      r.rows = 3;
    }
  }
  return 0;
}

int xg_model::ensure_pcg_blocks() {
  if (blocks_tried || neq == 0) return 0;
  blocks_tried = true;
  constexpr int kCap = 96;   // node rows with more blocks go in chunks of CSR entries
  BlockEll h;
  const int nblk = (int)blk_start.size() - 1;
  if (!block_ell_layout(neq, rowptr.data(), colidx.data(), nblk, blk_start.data(), kCap, h))
    return 0;
  size_t freeb = 0, totalb = 0;
  CK(cudaMemGetInfo(&freeb, &totalb));
  if (block_ell_bytes(h, nblk) > freeb / 2) return 0;
  const int ks = h.kb == 3 ? 4 : h.kb;
  RET(d_nb_off.upload(h.off.data(), h.off.size(), stream));
  RET(d_nb_cols.upload(h.cols.data(), h.cols.size(), stream));
  RET(d_nb_len.upload(h.len.data(), h.len.size(), stream));
  RET(d_nb_pos.upload(h.pos.data(), h.pos.size(), stream));
  RET(d_nb_vals.alloc(std::max<size_t>((size_t)h.off.back() * h.kb * h.kb, 1)));
  CK(cudaMemsetAsync(d_nb_vals.p, 0, d_nb_vals.n * sizeof(float2), stream));
  RET(d_p2.alloc((size_t)nblk * ks));
  CK(cudaMemsetAsync(d_p2.p, 0, d_p2.n * sizeof(float2), stream));
  RET(d_blk_ff.alloc(nblk));
  const int nch = (int)h.chunk_row.size();
  RET(d_chunk_row.upload(h.chunk_row.data(), h.chunk_row.size(), stream));
  RET(d_chunk_beg.upload(h.chunk_beg.data(), h.chunk_beg.size(), stream));
  RET(d_long_chunk0.upload(h.long_chunk0.data(), h.long_chunk0.size(), stream));
  RET(d_chunk_part.alloc(std::max(nch, 1)));
  pcg.kb = h.kb;
  pcg_blocks = 0;
  for (int i = 0; i < nblk; i++)
    if (h.len[i] <= kCap) pcg_blocks += h.len[i];
  pcg.nb_off = d_nb_off.p;
  pcg.nb_cols = d_nb_cols.p;
  pcg.nb_len = d_nb_len.p;
  pcg.nb_pos = d_nb_pos.p;
  pcg.nb_vals = d_nb_vals.p;
  pcg.blk_ff = d_blk_ff.p;
  pcg.p2 = d_p2.p;
  pcg.nb_cap = kCap;
  pcg.nlong = (int)h.long_chunk0.size() - 1;
  pcg.nchunks = nch;
  pcg.chunk_row = d_chunk_row.p;
  pcg.chunk_beg = d_chunk_beg.p;
  pcg.long_chunk0 = d_long_chunk0.p;
  pcg.chunk_part = d_chunk_part.p;
  return 0;
}

// Before a PCG solve on new matrix values: the diagonal blocks' inverses and
// the node-block values.
int xg_model::pcg_prepare() {
  RET(ensure_pcg_blocks());
  RET(pcg_factor_blocks(pcg, stream));
  blocks_factored = true;
  return 0;
}

int xg_model::solve(const double *b, double *x, int *iters) {
  if (system == XG_SYSTEM_PROFILE_SPD) {
    if (iters) *iters = 0;
    return solve_profile(1, &b, &x);
  }
  if (!blocks_factored) {
    prof_begin(P_PCG_FACTOR);
    RET(pcg_prepare());
    prof_end(P_PCG_FACTOR, 1);
  }
  CK(cudaMemsetAsync(x, 0, (neq > 0 ? neq : 1) * sizeof(double), stream));
  double relres = 0.0;
  int it = 0;
  prof_begin(P_PCG);
  const int k = (tune_pcg.on && !tune_pcg.done) ? tune_pcg.next() : -1;
  if (k >= 0) CK(cudaEventRecord(tune_a, stream));
  int r = pcg_solve(pcg, b, x, rtol, maxit, &it, &relres, stream,
                    k >= 0 ? tune_pcg.cand[k] : pcg_rows);
  if (k >= 0) {
    CK(cudaEventRecord(tune_b, stream));
    CK(cudaEventSynchronize(tune_b));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, tune_a, tune_b));
    if (it > 0) tune_pcg.record(k, ms / it);
    if (tune_pcg.done) pcg_rows = tune_pcg.chosen;
  }
  prof_end(P_PCG, 1);
  prof_flush();
  last_solver_iters += it;
  if (iters) *iters = it;
  if (r != 0)
    return fail(XG_ESOLVE, "PCG did not converge: %d iterations, relative residual %.3e", it,
                relres);
  return 0;
}

int xg_model::form_fext(double t) {
  CK(cudaMemsetAsync(d_fext.p, 0, (neq > 0 ? neq : 1) * sizeof(double), stream));
  for (size_t k = 0; k < ref_patterns.size(); k++) {
    const double lam = lambda_of(ref_patterns[k], t);
    if (lam != 0.0) RET(launch_axpy(neq, lam, d_Fref.p + k * (size_t)(neq > 0 ? neq : 1), d_fext.p, stream));
  }
  return 0;
}

// Phase set-up: DisplacementControl::domainChanged (phat, :372-392).
int xg_model::init_phase() {
  if (phase.pattern >= 0 && phase.pattern < 8) added[phase.pattern] = 1;
  dc_eq = -1;
  if (phase.integrator == XG_INT_DISP_CONTROL) {
    auto it = std::lower_bound(node_tag.begin(), node_tag.end(), phase.dc_node);
    if (it == node_tag.end() || *it != phase.dc_node) return fail(XG_EINVAL, "bad control node");
    const int n = (int)(it - node_tag.begin());
    if (phase.dc_dof < 0 || phase.dc_dof >= ndf) return fail(XG_EINVAL, "bad control dof");
    dc_eq = eqn[(size_t)n * ndf + phase.dc_dof];
    if (dc_eq < 0) return fail(XG_EINVAL, "control dof is constrained");
    RET(form_fext(time + 1.0));
    RET(element_state(false));
    RET(launch_sub(neq, d_fext.p, d_resid.p, d_phat.p, stream));
  } else if (phase.integrator == XG_INT_NEWMARK) {
    if (phase.dt <= 0.0 || phase.beta == 0.0)
      return fail(XG_EINVAL, "Newmark needs dt > 0 and beta != 0");
    if (phase.beta_k != 0.0 || phase.beta_k_comm != 0.0)
      return fail(XG_EINVAL, "Rayleigh betaK and betaKc are not supported (use betaK0)");
    const bool any_bk0 = phase.beta_k_init != 0.0 || phase.beta_k_init_elem != nullptr;
    if (any_bk0 && !frames())
      return fail(XG_EINVAL, "Rayleigh betaK0 needs force-based frame elements");
    {
      // alphaM-weighted mass on each equation
      std::vector<double> meq_am(std::max(neq, 1), 0.0), amn;
      if (phase.alpha_m_node) amn.assign(phase.alpha_m_node, phase.alpha_m_node + nn);
      for (int a = 0; a < nn * ndf; a++) {
        const int e = eqn[a];
        if (e < 0) continue;
        meq_am[e] += (phase.alpha_m_node ? amn[a / ndf] : phase.alpha_m) * node_mass[a];
      }
      RET(d_meq_am.upload(meq_am.data(), meq_am.size(), stream));
      if (phase.alpha_m_node) RET(d_am_node.upload(amn.data(), amn.size(), stream));
    }
    if (phase.gm_npts > 0) {
      const int nrec = std::max(phase.gm_count, 1);
      if (!phase.gm_accel || phase.gm_dt <= 0.0 || phase.gm_dof < 0 || phase.gm_dof >= ndf)
        return fail(XG_EINVAL, "bad ground motion");
      RET(d_gm.upload(phase.gm_accel, (size_t)nrec * phase.gm_npts, stream));
      if (phase.gm_node_record) {
        for (int i = 0; i < nn; i++)
          if (phase.gm_node_record[i] < 0 || phase.gm_node_record[i] >= nrec)
            return fail(XG_EINVAL, "ground-motion record of node %d out of range", i);
        RET(d_gm_rec.upload(phase.gm_node_record, nn, stream));
      }
    }
    k0_ready = false;
    if (any_bk0) {
      // betaK0 K0: K0 per element (records with Se = 0, kv = kv0), scaled
      // by the element's betaK0, gathered into CSR values
      DBuf<double> st0;
      RET(st0.alloc((size_t)ne * frame_state_stride(fb_nip)));
      RET(launch_fbc_kv0(fview(), st0.p, stream));
      FrameView fv = fview();
      fv.st = st0.p;
      RET(launch_fbc_assemble(fv, stream));
      if (phase.beta_k_init_elem) RET(d_bk0_elem.upload(phase.beta_k_init_elem, ne, stream));
      RET(launch_scale_blocks(ne, ke_size(), phase.beta_k_init_elem ? d_bk0_elem.p : nullptr,
                              phase.beta_k_init, d_Ke.p, stream));
      RET(d_K0vals.alloc(nnz > 0 ? nnz : 1));
      RET(launch_gather(gk, d_Ke.p, d_partial.p, d_K0vals.p, stream));
      CK(cudaStreamSynchronize(stream));
      k0_ready = true;
    }
  } else if (phase.integrator != XG_INT_LOAD_CONTROL) {
    return fail(XG_EINVAL, "integrator %d not supported", phase.integrator);
  }
  return 0;
}

static int read_scalar(const double *d, double *h, cudaStream_t s) {
  if (cudaMemcpyAsync(h, d, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return XG_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return XG_ECUDA;
  return 0;
}

// One step: integrator newStep, NewtonRaphson::solveCurrentStep, commit
// (runtime/runtime/BasicAnalysisBuilder.cpp:337-420).
int xg_model::step(xg_step_stats *st) {
  steps_since_reset++;
  if (phase.integrator == XG_INT_NEWMARK) return step_newmark(st);
  cudaStream_t s = stream;
  last_solver_iters = 0;
  const int nu = nn * ndf;
  const double t_commit = time;
  const bool transformation = handler == XG_HANDLER_TRANSFORMATION;
  if (phase.integrator == XG_INT_LOAD_CONTROL) {
    // LoadControl::newStep (Static/LoadControl.cpp:70-100):
    // applyLoadDomain; PlainHandler updates no element before
    // formUnbalance, the Transformation handler enforces the sp values and
    // updates every element
    time += phase.d_lambda;
    if (transformation) RET(enforce_sps(time));
    RET(element_state(transformation));
  } else {
    // DisplacementControl::newStep (Static/DisplacementControl.cpp:121-200)
    RET(element_state(false));
    RET(solve(d_phat.p, d_dUhat.p, nullptr));
    double dUahat;
    RET(read_scalar(d_dUhat.p + dc_eq, &dUahat, s));
    if (dUahat == 0.0) return fail(XG_ESOLVE, "zero reference displacement at the control dof");
    const double dlambda = phase.dc_incr / dUahat;
    time += dlambda;
    RET(launch_scatter_incr(nu, d_eqn.p, d_dUhat.p, dlambda, d_U.p, s));
    if (transformation) RET(enforce_sps(time));   // applyLoadDomain(currentLambda)
    RET(element_state(true));
  }
  RET(form_fext(time));
  RET(launch_sub(neq, d_fext.p, d_resid.p, d_B.p, s));
  int it = 0;
  bool ok = false;
  while (true) {
    if (phase.integrator != XG_INT_DISP_CONTROL) RET(solve(d_B.p, d_dU.p, nullptr));
    if (phase.integrator == XG_INT_DISP_CONTROL) {
      // DisplacementControl::update (:202-250)
      RET(solve2(d_B.p, d_dU.p, d_phat.p, d_dUhat.p));
      double dUahat, dUabar;
      RET(read_scalar(d_dUhat.p + dc_eq, &dUahat, s));
      RET(read_scalar(d_dU.p + dc_eq, &dUabar, s));
      if (dUahat == 0.0) return fail(XG_ESOLVE, "zero reference displacement at the control dof");
      const double dLambda = -dUabar / dUahat;
      RET(launch_axpy(neq, dLambda, d_dUhat.p, d_dU.p, s));
      time += dLambda;
    }
    RET(launch_scatter_incr(nu, d_eqn.p, d_dU.p, 1.0, d_U.p, s));
    if (transformation && phase.integrator == XG_INT_DISP_CONTROL) RET(enforce_sps(time));
    RET(element_state(true));
    RET(form_fext(time));
    RET(launch_sub(neq, d_fext.p, d_resid.p, d_B.p, s));
    it++;
    RET(launch_norm2(neq, phase.test == XG_TEST_NORM_DISP_INCR ? d_dU.p : d_B.p, d_partial.p,
                     d_norm.p, s));
    double n2;
    RET(read_scalar(d_norm.p, &n2, s));
    if (std::sqrt(n2) <= phase.tol) { ok = true; break; }
    if (it >= phase.max_iter) break;
  }
  if (st) {
    st->newton_iters = it;
    st->solver_iters = last_solver_iters;
    st->elem_iters = 0;
    st->status = ok ? 0 : XG_ENOCONV;
  }
  if (!ok) {
    time = t_commit;
    return fail(XG_ENOCONV, "Newton did not converge in %d iterations", it);
  }
  // commit (Domain::commit -> element and material commitState)
  RET(commit_state());
  time_c = time;
  return 0;
}

// TransformationConstraintHandler::applyLoad -> enforceSPs
// (analysis/handler/TransformationConstraintHandler.cpp:456-480): every
// imposed sp sets its dof's trial displacement to its pattern's load
// factor at time t times its value; the caller then updates every element
// (FE_Element::updateElement there).
int xg_model::enforce_sps(double t) {
  if (num_isp == 0) return 0;
  SpFactors lam{};
  for (int p = 0; p < 8; p++) lam.f[p] = lambda_of(p, t);
  return launch_enforce_sps(num_isp, d_isp_idx.p, d_isp_pat.p, d_isp_val.p, lam, d_U.p, stream);
}

int xg_model::commit_state() {
  cudaStream_t s = stream;
  const size_t nu = (size_t)nn * ndf;
  if (frames()) {
    RET(launch_fbc_commit(fview(), d_st_c.p, d_fh_c.p, fb_nrec * 12, s));
  } else {
    const long np = npts();
    CK(cudaMemcpyAsync(d_epc.p, d_ept.p, np * nhist() * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_xic.p, d_xit.p, np * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_sig_c.p, d_sig.p, np * nsig() * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_tan_c.p, d_tan.p, np * ntan() * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  CK(cudaMemcpyAsync(d_Uc.p, d_U.p, nu * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return 0;
}

int xg_model::revert_state() {
  cudaStream_t s = stream;
  if (frames()) {
    RET(launch_fbc_revert(fview(), d_st_c.p, fb_nrec * 12, s));
  } else {
    const long np = npts();
    CK(cudaMemcpyAsync(d_ept.p, d_epc.p, np * nhist() * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_xit.p, d_xic.p, np * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_sig.p, d_sig_c.p, np * nsig() * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_tan.p, d_tan_c.p, np * ntan() * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  CK(cudaMemcpyAsync(d_U.p, d_Uc.p, (size_t)nn * ndf * sizeof(double), cudaMemcpyDeviceToDevice, s));
  // Newmark::revertToLastStep
  CK(cudaMemcpyAsync(d_V.p, d_Vc.p, (size_t)nn * ndf * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(d_A.p, d_Ac.p, (size_t)nn * ndf * sizeof(double), cudaMemcpyDeviceToDevice, s));
  // Domain::revertToLastCommit ends with Domain::update at the committed
  // displacements (domain/domain/Domain.cpp:1925-1949)
  return element_state(true);
}

// ---------------------------------------------------------------------------
// adjoint of a Newmark run
// ---------------------------------------------------------------------------
// committed state -> dst: U V A [nn*ndf each], fiber records, element state
int xg_model::adj_save(double *dst) {
  cudaStream_t s = stream;
  const size_t nu = (size_t)nn * ndf, nst = (size_t)ne * frame_state_stride(fb_nip);
  CK(cudaMemcpyAsync(dst, d_Uc.p, nu * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(dst + nu, d_Vc.p, nu * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(dst + 2 * nu, d_Ac.p, nu * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(dst + adj_off_fh(), d_fh_c.p, (size_t)fb_nrec * 12 * sizeof(double),
                     cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(dst + adj_off_st(), d_st_c.p, nst * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return 0;
}

// a saved state becomes the committed and the trial state (as right after
// the commit that produced it)
int xg_model::adj_load(const double *src, double t) {
  cudaStream_t s = stream;
  const size_t nu = (size_t)nn * ndf, nst = (size_t)ne * frame_state_stride(fb_nip);
  const size_t nrec = (size_t)fb_nrec * 12;
  for (double *d : {d_U.p, d_Uc.p})
    CK(cudaMemcpyAsync(d, src, nu * sizeof(double), cudaMemcpyDeviceToDevice, s));
  for (double *d : {d_V.p, d_Vc.p})
    CK(cudaMemcpyAsync(d, src + nu, nu * sizeof(double), cudaMemcpyDeviceToDevice, s));
  for (double *d : {d_A.p, d_Ac.p})
    CK(cudaMemcpyAsync(d, src + 2 * nu, nu * sizeof(double), cudaMemcpyDeviceToDevice, s));
  for (double *d : {d_fh_c.p, d_fh_t.p})
    CK(cudaMemcpyAsync(d, src + adj_off_fh(), nrec * sizeof(double), cudaMemcpyDeviceToDevice, s));
  for (double *d : {d_st.p, d_st_c.p})
    CK(cudaMemcpyAsync(d, src + adj_off_st(), nst * sizeof(double), cudaMemcpyDeviceToDevice, s));
  time = time_c = t;
  blocks_factored = false;
  prof_factored = false;
  return 0;
}

// Newmark run of num_steps from the initial state with the objective
// J = sum over steps n and terms k of w_k U_n[dof_k]^2, keeping the
// committed state every K steps for the reverse sweep.
int xg_model::adjoint_forward(const xg_phase_desc *ph, int N, int K, const xg_objective_desc *obj,
                              double *J) {
  adj.have = false;
  if (!frames()) return fail(XG_EINVAL, "the adjoint covers force-based frame models");
  if (!ph || ph->integrator != XG_INT_NEWMARK)
    return fail(XG_EINVAL, "the adjoint covers Newmark runs");
  if (N < 1 || K < 1 || !obj || obj->num_terms < 0 || (obj->num_terms > 0 &&
      (!obj->node || !obj->dof || !obj->weight)))
    return fail(XG_EINVAL, "bad adjoint run settings");
  if (steps_since_reset != 0 || have_phase)
    return fail(XG_ESTATE, "the adjoint runs from the model's initial state (xg_reset first)");
  // fiber materials: Steel02 without initial stress, Concrete02 or elastic,
  // at most kAdjSlots of them per section (slots in order of first fiber)
  const int nsec = (int)sec_fstart.size() - 1;
  adj.fslot.assign(std::max(sec_fstart.back(), 1), 0);
  adj.sec_slots.assign((size_t)std::max(nsec, 1) * kAdjSlots, -1);
  std::vector<char> sec_single(std::max(nsec, 1), 1);   // one Steel02 / elastic material
  for (int sc = 0; sc < nsec; sc++) {
    int *sl = adj.sec_slots.data() + (size_t)sc * kAdjSlots;
    for (int f = sec_fstart[sc]; f < sec_fstart[sc + 1]; f++) {
      const int u = fmat[f];
      int m = 0;
      while (m < kAdjSlots && sl[m] >= 0 && sl[m] != u) m++;
      if (m == kAdjSlots)
        return fail(XG_EINVAL, "the adjoint keeps at most %d materials per section (section %d)",
                    kAdjSlots, sc);
      sl[m] = u;
      adj.fslot[f] = m;
      if (utype[u] == XG_UNI_STEEL02) {
        if (uparam[(size_t)u * XG_UNI_NPARAM + 10] != 0.0)
          return fail(XG_EINVAL, "the adjoint does not cover Steel02 with an initial stress");
      } else if (utype[u] == XG_UNI_CONCRETE02 || utype[u] == XG_UNI_CONCRETE01) {
        sec_single[sc] = 0;
      } else if (utype[u] != XG_UNI_ELASTIC && utype[u] != XG_UNI_STEEL01) {
        return fail(XG_EINVAL, "the adjoint covers Steel02, Steel01, Concrete02, Concrete01 and "
                    "elastic fibers");
      }
      if (m > 0) sec_single[sc] = 0;
    }
  }
  adj.elem_uni.assign(ne, 0);
  for (int e = 0; e < ne; e++) adj.elem_uni[e] = std::max(adj.sec_slots[(size_t)mat[e] * kAdjSlots], 0);
  std::vector<int> dofs(obj->num_terms);
  for (int k = 0; k < obj->num_terms; k++) {
    auto it = std::lower_bound(node_tag.begin(), node_tag.end(), obj->node[k]);
    if (it == node_tag.end() || *it != obj->node[k] || obj->dof[k] < 0 || obj->dof[k] >= ndf)
      return fail(XG_EINVAL, "objective term %d: bad node or dof", k);
    dofs[k] = (int)(it - node_tag.begin()) * ndf + obj->dof[k];
  }
  for (int e = 0; e < ne; e++) {
    const double bk = ph->beta_k_init_elem ? ph->beta_k_init_elem[e] : ph->beta_k_init;
    if (bk != 0.0 && !sec_single[mat[e]])
      return fail(XG_EINVAL, "betaK0 damping in the adjoint needs one Steel02, Steel01 or "
                  "elastic material per element (element %d)", e);
  }
  RET(xg_analysis_set_phase(this, ph));
  cudaStream_t s = stream;
  adj.N = N;
  adj.K = K;
  adj.nterm = obj->num_terms;
  adj.nck = (N + K - 1) / K;
  adj.len = adj_off_st() + (size_t)ne * frame_state_stride(fb_nip);
  const size_t segslots = (size_t)std::min(K, N) + 1;
  size_t free_b = 0, total_b = 0;
  CK(cudaMemGetInfo(&free_b, &total_b));
  const size_t need = ((size_t)adj.nck + 1 + segslots) * adj.len * sizeof(double);
  if (need > free_b / 10 * 8)
    return fail(XG_ENOMEM, "adjoint checkpoints need %.1f GB (fewer steps per checkpoint "
                "lower it)", need * 1e-9);
  RET(adj.ck.alloc(((size_t)adj.nck + 1) * adj.len));
  RET(adj.seg.alloc(segslots * adj.len));
  RET(adj.dof.upload(dofs.data(), std::max<size_t>(dofs.size(), 1), s));
  std::vector<double> wv(obj->weight, obj->weight + obj->num_terms);
  wv.resize(std::max<size_t>(wv.size(), 1));
  RET(adj.w.upload(wv.data(), wv.size(), s));
  RET(adj.d_elem_uni.upload(adj.elem_uni.data(), std::max<size_t>(adj.elem_uni.size(), 1), s));
  RET(adj.d_fslot.upload(adj.fslot.data(), adj.fslot.size(), s));
  RET(adj.J.alloc(std::max(adj.nterm, 1)));
  CK(cudaMemsetAsync(adj.J.p, 0, std::max(adj.nterm, 1) * sizeof(double), s));
  adj.ck_time.assign(adj.nck + 1, 0.0);
  RET(adj_save(adj.ck.p));
  adj.ck_time[0] = time_c;
  for (int n = 1; n <= N; n++) {
    RET(step(nullptr));
    phase_steps_done++;
    RET(launch_adj_objective(adj.nterm, adj.dof.p, adj.w.p, d_Uc.p, adj.J.p, s));
    if (n % K == 0 && n < N) {
      RET(adj_save(adj.ck.p + (size_t)(n / K) * adj.len));
      adj.ck_time[n / K] = time_c;
    }
  }
  RET(adj_save(adj.ck.p + (size_t)adj.nck * adj.len));
  adj.ck_time[adj.nck] = time_c;
  adj.Jk.assign(std::max(adj.nterm, 1), 0.0);
  CK(cudaMemcpyAsync(adj.Jk.data(), adj.J.p, adj.Jk.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  double Jh = 0.0;
  for (int k = 0; k < adj.nterm; k++) Jh += adj.Jk[k];
  if (J) *J = Jh;
  adj.have = true;
  return 0;
}

// The 2D P-Delta step's adjoint equation J' mu = rhs, J' = K + C' with K the
// factored symmetric tangent and C' the per-element terms of k_adj_pdelta:
// mu <- K^-1 (rhs - C' mu) from the first solve's mu until a solve changes
// mu by no more than the solver's accuracy.  The iteration contracts as the
// forward step's Newton iteration on the same tangent does.
int xg_model::adj_pdelta_refine(const xg::FrameView &fv, const xg::AdjView &av) {
  cudaStream_t s = stream;
  constexpr int kMaxSolves = 100;
  const double tol = system == XG_SYSTEM_PROFILE_SPD ? 1e-14 : std::max(1e-14, 10.0 * rtol);
  for (int k = 0; k < kMaxSolves; k++) {
    RET(launch_adj_pdelta(fv, av, s));
    RET(launch_gather(gr, d_Re.p, d_partial.p, adj.tmp.p, s));
    RET(launch_sub(neq, adj.rhs.p, adj.tmp.p, adj.rhs2.p, s));
    RET(solve(adj.rhs2.p, adj.mu2.p, nullptr));
    adj.pd_solves++;
    RET(launch_sub(neq, adj.mu2.p, adj.mu.p, adj.tmp.p, s));
    double dn = 0.0, mn = 0.0;
    RET(launch_norm2(neq, adj.tmp.p, d_partial.p, d_norm.p, s));
    RET(read_scalar(d_norm.p, &dn, s));
    RET(launch_norm2(neq, adj.mu2.p, d_partial.p, d_norm.p, s));
    RET(read_scalar(d_norm.p, &mn, s));
    CK(cudaMemcpyAsync(adj.mu.p, adj.mu2.p, (size_t)neq * sizeof(double),
                       cudaMemcpyDeviceToDevice, s));
    if (std::sqrt(dn) <= tol * std::sqrt(mn)) return 0;
  }
  return fail(XG_ENOCONV, "adjoint: the P-Delta terms' fixed-point iteration did not converge "
              "in %d solves", kMaxSolves);
}

// Reverse sweep: segment by segment from the last, the segment's steps are
// run again from its checkpoint (the kernels are deterministic, so the
// states repeat bit for bit) and swept backwards.  grad[u*3+k] = scale *
// dJ/d uni_param[u][k], k = 0..2.  The model ends at the run's last state.
int xg_model::adjoint_backward(double scale, double *grad, int num_uni) {
  if (!adj.have) return fail(XG_ESTATE, "no adjoint run (xg_adjoint_forward first)");
  adj.pd_solves = 0;
  if (!grad || num_uni != (int)utype.size()) return fail(XG_EINVAL, "bad gradient buffer");
  cudaStream_t s = stream;
  const size_t nu = (size_t)nn * ndf, nrec = (size_t)fb_nrec * 12;
  const size_t ne1 = std::max(neq, 1);
  for (auto *b : {&adj.Ub, &adj.Vb, &adj.Ab, &adj.mu, &adj.rhs, &adj.tmp, &adj.kmu, &adj.mu2,
                  &adj.rhs2}) {
    RET(b->alloc(ne1));
    CK(cudaMemsetAsync(b->p, 0, ne1 * sizeof(double), s));
  }
  RET(adj.hbar.alloc(std::max<size_t>(nrec, 1)));
  CK(cudaMemsetAsync(adj.hbar.p, 0, std::max<size_t>(nrec, 1) * sizeof(double), s));
  const size_t nth = std::max<size_t>((size_t)ne * kAdjSlots * 3, 1);
  RET(adj.theta.alloc(nth));
  CK(cudaMemsetAsync(adj.theta.p, 0, nth * sizeof(double), s));
  RET(adj.scr.alloc(std::max<size_t>((size_t)ne * (6 + fb_nip * 4), 1)));
  const double dt = phase.dt, gam = phase.gamma, bet = phase.beta;
  NewmarkCoef c{};
  c.c2 = gam / (bet * dt);
  c.c3 = 1.0 / (bet * dt * dt);
  c.a1 = 1.0 - gam / bet;
  c.a2 = dt * (1.0 - 0.5 * gam / bet);
  c.a3 = -1.0 / (bet * dt);
  c.a4 = 1.0 - 0.5 / bet;
  AdjView av{};
  av.hbar = adj.hbar.p;
  av.theta = adj.theta.p;
  av.scr = adj.scr.p;
  av.eqn = d_eqn.p;
  av.mu = adj.mu.p;
  av.bk0 = phase.beta_k_init_elem ? d_bk0_elem.p : nullptr;
  av.bk0_all = phase.beta_k_init;
  av.use_k0 = k0_ready ? 1 : 0;
  av.elem_uni = adj.d_elem_uni.p;
  av.fslot = adj.d_fslot.p;
  const int N = adj.N, K = adj.K;
  // the objective's last term
  RET(launch_adj_objective_grad(adj.nterm, adj.dof.p, adj.w.p, d_eqn.p,
                                adj.ck.p + (size_t)adj.nck * adj.len, adj.Ub.p, s));
  const size_t nst = (size_t)ne * frame_state_stride(fb_nip);
  for (int sg = adj.nck - 1; sg >= 0; sg--) {
    const int n0 = sg * K, n1 = std::min(N, n0 + K);
    const double *ckp = adj.ck.p + (size_t)sg * adj.len;
    RET(adj_load(ckp, adj.ck_time[sg]));
    CK(cudaMemcpyAsync(adj.seg.p, ckp, adj.len * sizeof(double), cudaMemcpyDeviceToDevice, s));
    for (int n = n0 + 1; n <= n1; n++) {
      RET(step_newmark(nullptr));
      RET(adj_save(adj.seg.p + (size_t)(n - n0) * adj.len));
    }
    for (int n = n1; n > n0; n--) {
      const double *Sj = adj.seg.p + (size_t)(n - n0) * adj.len;
      const double *Sp = Sj - adj.len;
      // effective tangent at the step's converged state (the committed
      // element state after it), as the forward step forms it
      CK(cudaMemcpyAsync(d_st.p, Sj + adj_off_st(), nst * sizeof(double),
                         cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(d_U.p, Sj, nu * sizeof(double), cudaMemcpyDeviceToDevice, s));
      FrameView fv = fview();
      RET(launch_fbc_assemble(fv, s));
      RET(launch_gather(gk, d_Ke.p, d_partial.p, d_vals.p, s));
      RET(launch_dyn_tangent(dview(), d_vals.p, d_K0vals.p, 1.0, k0_ready ? c.c2 : 0.0, c.c2,
                             c.c3, s));
      blocks_factored = false;
      prof_factored = false;
      av.st = Sj + adj_off_st();
      av.fh_prev = Sp + adj_off_fh();
      av.Vn = Sj + nu;
      RET(launch_adj_elem_a(fv, av, s));
      RET(launch_gather(gr, d_Re.p, d_partial.p, adj.tmp.p, s));
      RET(launch_adj_rhs(neq, adj.Ub.p, adj.Vb.p, adj.Ab.p, adj.tmp.p, c.c2, c.c3, adj.rhs.p, s));
      RET(solve(adj.rhs.p, adj.mu.p, nullptr));
      if (fv.pdelta2d) RET(adj_pdelta_refine(fv, av));
      RET(launch_adj_elem_b(fv, av, s));
      if (k0_ready) RET(launch_spmv(neq, d_rowptr.p, d_colidx.p, d_K0vals.p, adj.mu.p, adj.kmu.p, s));
      RET(launch_adj_prev(neq, adj.mu.p, k0_ready ? adj.kmu.p : nullptr, d_meq.p, d_meq_am.p, c,
                          adj.Ub.p, adj.Vb.p, adj.Ab.p, s));
      if (n - 1 >= 1)
        RET(launch_adj_objective_grad(adj.nterm, adj.dof.p, adj.w.p, d_eqn.p, Sp, adj.Ub.p, s));
    }
  }
  // the fresh records' parameters
  RET(launch_adj_init_records(fview(), av, s));
  std::vector<double> th((size_t)ne * kAdjSlots * 3);
  if (ne) CK(cudaMemcpyAsync(th.data(), adj.theta.p, th.size() * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int k = 0; k < num_uni * 3; k++) grad[k] = 0.0;
  for (int e = 0; e < ne; e++)
    for (int m = 0; m < kAdjSlots; m++) {
      const int u = adj.sec_slots[(size_t)mat[e] * kAdjSlots + m];
      if (u < 0) continue;
      for (int k = 0; k < 3; k++)
        grad[(size_t)u * 3 + k] += scale * th[((size_t)e * kAdjSlots + m) * 3 + k];
    }
  RET(adj_load(adj.ck.p + (size_t)adj.nck * adj.len, adj.ck_time[adj.nck]));
  return element_state(true);
}

// The 2D P-Delta step's tangent equation (K + C) x = rhs, K the factored
// symmetric tangent and C the per-element terms of k_ddm_pdelta:
// x <- K^-1 (rhs - C x) from the first solve's x until a solve changes x by
// no more than the solver's accuracy (as adj_pdelta_refine does for the
// transposed equation).
int xg_model::ddm_pdelta_refine(const xg::FrameView &fv) {
  cudaStream_t s = stream;
  constexpr int kMaxSolves = 100;
  const double tol = system == XG_SYSTEM_PROFILE_SPD ? 1e-14 : std::max(1e-14, 10.0 * rtol);
  for (int k = 0; k < kMaxSolves; k++) {
    RET(launch_ddm_pdelta(fv, d_eqn.p, ddm.x.p, s));
    RET(launch_gather(gr, d_Re.p, d_partial.p, ddm.t0.p, s));
    RET(launch_sub(neq, ddm.rhs.p, ddm.t0.p, ddm.t1.p, s));
    RET(solve(ddm.t1.p, ddm.t0.p, nullptr));
    RET(launch_sub(neq, ddm.t0.p, ddm.x.p, ddm.t1.p, s));
    double dn = 0.0, xn = 0.0;
    RET(launch_norm2(neq, ddm.t1.p, d_partial.p, d_norm.p, s));
    RET(read_scalar(d_norm.p, &dn, s));
    RET(launch_norm2(neq, ddm.t0.p, d_partial.p, d_norm.p, s));
    RET(read_scalar(d_norm.p, &xn, s));
    CK(cudaMemcpyAsync(ddm.x.p, ddm.t0.p, (size_t)neq * sizeof(double), cudaMemcpyDeviceToDevice,
                       s));
    if (std::sqrt(dn) <= tol * std::sqrt(xn)) return 0;
  }
  return fail(XG_ENOCONV, "DDM: the P-Delta terms' fixed-point iteration did not converge in %d "
              "solves", kMaxSolves);
}

// Newmark (or LoadControl) run of num_steps from the initial state with the
// direct differentiation after every converged step
// (Newmark::computeSensitivities, Newmark.cpp:904-959, one direction per
// parameter combination):
//   K_eff dU = -dP|_U + M (c3 dU' - a3 dV' - a4 dA') + alphaM M (c2 dU' - a1 dV' - a2 dA')
// with K_eff formed again at the converged state (the reference solves with
// the last Newton iteration's factors), then the record tangents committed.
// J as xg_adjoint_forward; dJ[k] = dJ/dtheta along direction k.
int xg_model::ddm_forward(const xg_phase_desc *ph, int N, int nd, const double *dtheta,
                          const xg_objective_desc *obj, double *J, double *dJ) {
  ddm.have = false;
  if (!frames()) return fail(XG_EINVAL, "the DDM covers force-based frame models");
  if (!ph || (ph->integrator != XG_INT_NEWMARK && ph->integrator != XG_INT_LOAD_CONTROL))
    return fail(XG_EINVAL, "the DDM covers Newmark and LoadControl runs");
  const bool dyn = ph->integrator == XG_INT_NEWMARK;
  if (N < 1 || nd < 1 || !dtheta || !obj || obj->num_terms < 0 ||
      (obj->num_terms > 0 && (!obj->node || !obj->dof || !obj->weight)))
    return fail(XG_EINVAL, "bad DDM run settings");
  if (steps_since_reset != 0 || have_phase)
    return fail(XG_ESTATE, "the DDM runs from the model's initial state (xg_reset first)");
  for (size_t u = 0; u < utype.size(); u++) {
    if (utype[u] != XG_UNI_STEEL02 && utype[u] != XG_UNI_STEEL01 &&
        utype[u] != XG_UNI_CONCRETE02 && utype[u] != XG_UNI_CONCRETE01 &&
        utype[u] != XG_UNI_ELASTIC)
      return fail(XG_EINVAL, "the DDM covers Steel02, Steel01, Concrete02, Concrete01 and "
                  "elastic fibers (material %d)", (int)u);
    if (utype[u] == XG_UNI_STEEL02 && uparam[u * XG_UNI_NPARAM + 10] != 0.0)
      return fail(XG_EINVAL, "the DDM does not cover Steel02 with an initial stress");
  }
  // betaK0 damping on elements with a single Steel02, Steel01 or elastic
  // material, in which K0 is linear in E
  std::vector<int> elem_uni(std::max(ne, 1), 0);
  for (int e = 0; e < ne; e++) {
    const int sc = mat[e];
    const int u0 = fmat[sec_fstart[sc]];
    elem_uni[e] = u0;
    const double bk = ph->beta_k_init_elem ? ph->beta_k_init_elem[e] : ph->beta_k_init;
    if (bk == 0.0) continue;
    bool single = utype[u0] == XG_UNI_STEEL02 || utype[u0] == XG_UNI_STEEL01 ||
                  utype[u0] == XG_UNI_ELASTIC;
    for (int f = sec_fstart[sc]; f < sec_fstart[sc + 1]; f++) single = single && fmat[f] == u0;
    if (!single)
      return fail(XG_EINVAL, "betaK0 damping in the DDM needs one Steel02, Steel01 or elastic "
                  "material per element (element %d)", e);
  }
  std::vector<int> dofs(obj->num_terms);
  for (int k = 0; k < obj->num_terms; k++) {
    auto it = std::lower_bound(node_tag.begin(), node_tag.end(), obj->node[k]);
    if (it == node_tag.end() || *it != obj->node[k] || obj->dof[k] < 0 || obj->dof[k] >= ndf)
      return fail(XG_EINVAL, "objective term %d: bad node or dof", k);
    dofs[k] = (int)(it - node_tag.begin()) * ndf + obj->dof[k];
  }
  RET(xg_analysis_set_phase(this, ph));
  cudaStream_t s = stream;
  const size_t ne1 = std::max(neq, 1), nrec = std::max<size_t>((size_t)fb_nrec * 12, 1);
  const size_t nuni3 = utype.size() * 3;
  ddm.nd = nd;
  ddm.nterm = obj->num_terms;
  {
    // per direction: U, V, A tangents and the record tangents
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t need = (size_t)nd * (3 * ne1 + nrec + nuni3) * sizeof(double);
    if (need > free_b / 10 * 8)
      return fail(XG_ENOMEM, "the DDM's %d directions need %.1f GB (fewer directions per run "
                  "lower it)", nd, need * 1e-9);
  }
  for (auto *b : {&ddm.dU, &ddm.dV, &ddm.dA}) {
    RET(b->alloc((size_t)nd * ne1));
    CK(cudaMemsetAsync(b->p, 0, (size_t)nd * ne1 * sizeof(double), s));
  }
  RET(ddm.dh.alloc((size_t)nd * nrec));
  RET(ddm.dth.upload(dtheta, (size_t)nd * nuni3, s));
  for (int k = 0; k < nd; k++) {             // the fresh records' tangents
    DdmView dv{};
    dv.dh = ddm.dh.p + (size_t)k * nrec;
    dv.dth = ddm.dth.p + (size_t)k * nuni3;
    RET(launch_ddm_init_records(fview(), dv, s));
  }
  RET(ddm.fh_prev.alloc(nrec));
  RET(ddm.q.alloc(std::max<size_t>((size_t)ne * fb_nip * 4, 1)));
  RET(ddm.z.alloc(std::max<size_t>((size_t)ne * 6, 1)));
  RET(ddm.rhs.alloc(ne1));
  RET(ddm.x.alloc(ne1));
  RET(ddm.t0.alloc(ne1));
  RET(ddm.t1.alloc(ne1));
  RET(ddm.elem_uni.upload(elem_uni.data(), elem_uni.size(), s));
  RET(ddm.dof.upload(dofs.data(), std::max<size_t>(dofs.size(), 1), s));
  std::vector<double> wv(obj->weight, obj->weight + obj->num_terms);
  wv.resize(std::max<size_t>(wv.size(), 1));
  RET(ddm.w.upload(wv.data(), wv.size(), s));
  RET(ddm.J.alloc(std::max(ddm.nterm, 1)));
  CK(cudaMemsetAsync(ddm.J.p, 0, std::max(ddm.nterm, 1) * sizeof(double), s));
  const size_t nt1 = std::max(ddm.nterm, 1);
  RET(ddm.dJd.alloc((size_t)nd * nt1));
  CK(cudaMemsetAsync(ddm.dJd.p, 0, (size_t)nd * nt1 * sizeof(double), s));
  // Newmark's relations; a LoadControl step has no inertia and no velocity
  // (LoadControl::computeSensitivities: K dU = -dP at fixed U), all zero
  NewmarkCoef c{};
  if (dyn) {
    const double dt = phase.dt, gam = phase.gamma, bet = phase.beta;
    c.c2 = gam / (bet * dt);
    c.c3 = 1.0 / (bet * dt * dt);
    c.a1 = 1.0 - gam / bet;
    c.a2 = dt * (1.0 - 0.5 * gam / bet);
    c.a3 = -1.0 / (bet * dt);
    c.a4 = 1.0 - 0.5 / bet;
  }
  for (int n = 1; n <= N; n++) {
    CK(cudaMemcpyAsync(ddm.fh_prev.p, d_fh_c.p, (size_t)fb_nrec * 12 * sizeof(double),
                       cudaMemcpyDeviceToDevice, s));
    RET(step(nullptr));
    phase_steps_done++;
    RET(launch_adj_objective(ddm.nterm, ddm.dof.p, ddm.w.p, d_Uc.p, ddm.J.p, s));
    // the effective tangent at the converged state
    FrameView fv = fview();
    RET(launch_fbc_assemble(fv, s));
    RET(launch_gather(gk, d_Ke.p, d_partial.p, d_vals.p, s));
    if (dyn)
      RET(launch_dyn_tangent(dview(), d_vals.p, d_K0vals.p, 1.0, k0_ready ? c.c2 : 0.0, c.c2,
                             c.c3, s));
    blocks_factored = false;
    prof_factored = false;
    for (int k = 0; k < nd; k++) {
      DdmView dv{};
      dv.fh_prev = ddm.fh_prev.p;
      dv.dh = ddm.dh.p + (size_t)k * nrec;
      dv.dth = ddm.dth.p + (size_t)k * nuni3;
      dv.q = ddm.q.p;
      dv.z = ddm.z.p;
      dv.eqn = d_eqn.p;
      dv.Vn = d_Vc.p;
      dv.bk0 = phase.beta_k_init_elem ? d_bk0_elem.p : nullptr;
      dv.bk0_all = phase.beta_k_init;
      dv.elem_uni = ddm.elem_uni.p;
      double *dUk = ddm.dU.p + (size_t)k * ne1, *dVk = ddm.dV.p + (size_t)k * ne1,
             *dAk = ddm.dA.p + (size_t)k * ne1;
      RET(launch_ddm_cond(fv, dv, s));
      if (dyn && k0_ready) RET(launch_ddm_k0(fv, dv, s));
      RET(launch_gather(gr, d_Re.p, d_partial.p, ddm.x.p, s));
      RET(launch_ddm_rhs(neq, ddm.x.p, dUk, dVk, dAk, dyn ? d_meq.p : nullptr,
                         dyn ? d_meq_am.p : nullptr, c, ddm.rhs.p, s));
      if (dyn && k0_ready) {
        // + betaK0 K0 (c2 dU' - a1 dV' - a2 dA')
        RET(launch_ddm_k0_vec(neq, dUk, dVk, dAk, c, ddm.t0.p, s));
        RET(launch_spmv(neq, d_rowptr.p, d_colidx.p, d_K0vals.p, ddm.t0.p, ddm.t1.p, s));
        RET(launch_axpy(neq, 1.0, ddm.t1.p, ddm.rhs.p, s));
      }
      RET(solve(ddm.rhs.p, ddm.x.p, nullptr));
      if (fv.pdelta2d) RET(ddm_pdelta_refine(fv));
      RET(launch_ddm_update(neq, ddm.x.p, c, dUk, dVk, dAk, s));
      dv.dU = dUk;
      RET(launch_ddm_commit(fv, dv, s));
      RET(launch_ddm_objective(ddm.nterm, ddm.dof.p, ddm.w.p, d_eqn.p, d_Uc.p, dUk,
                               ddm.dJd.p + (size_t)k * nt1, s));
    }
  }
  std::vector<double> Jk(nt1);
  ddm.dJt.assign((size_t)nd * nt1, 0.0);
  CK(cudaMemcpyAsync(Jk.data(), ddm.J.p, Jk.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(ddm.dJt.data(), ddm.dJd.p, ddm.dJt.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  double Jh = 0.0;
  for (int k = 0; k < ddm.nterm; k++) Jh += Jk[k];
  if (J) *J = Jh;
  if (dJ)
    for (int k = 0; k < nd; k++) {
      double t = 0.0;
      for (int j = 0; j < ddm.nterm; j++) t += ddm.dJt[(size_t)k * nt1 + j];
      dJ[k] = t;
    }
  ddm.have = true;
  return 0;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char *xg_last_error(void) { return g_err.c_str(); }
int xg_version(void) { return 1; }

static int plan_model(const xg_model_desc *d, xg_model **out);

int xg_model_create(const xg_model_desc *d, xg_model **out) {
  g_err.clear();
  if (!d || !out) return fail(XG_EINVAL, "null argument");
  *out = nullptr;
  xg_model *m = nullptr;
  int r = plan_model(d, &m);
  if (r) return r;
  HostGather gk_h, gr_h;
  r = m->build_maps(gk_h, gr_h);
  if (r) { delete m; return r; }
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete m;
    return fail(XG_ECUDA, "no CUDA device");
  }
  m->prof_init();
  r = m->upload(gk_h, gr_h);
  if (r) { delete m; return r; }
  *out = m;
  return 0;
}

int xg_model_plan(const xg_model_desc *d, int *eqn, int *rowptr, int *colidx, int *num_eqn,
                  int *nnz) {
  g_err.clear();
  if (!d) return fail(XG_EINVAL, "null argument");
  xg_model *m = nullptr;
  int r = plan_model(d, &m);
  if (r) return r;
  if (num_eqn) *num_eqn = m->neq;
  if (nnz) *nnz = m->nnz;
  if (eqn) std::copy(m->eqn.begin(), m->eqn.end(), eqn);
  if (rowptr) std::copy(m->rowptr.begin(), m->rowptr.end(), rowptr);
  if (colidx) std::copy(m->colidx.begin(), m->colidx.end(), colidx);
  delete m;
  return 0;
}

// Host part of model creation: validate and copy the description, number
// the DOFs and build the pattern.  No device work.
static int plan_model(const xg_model_desc *d, xg_model **out) {
  const bool fr = d->elem_type == XG_ELE_FBC2D || d->elem_type == XG_ELE_FBC3D;
  if (d->elem_type != XG_ELE_QUAD && d->elem_type != XG_ELE_BRICK && !fr)
    return fail(XG_EINVAL, "element type %d not supported", d->elem_type);
  if (d->elem_type == XG_ELE_FBC2D && (d->ndm != 2 || d->ndf != 3))
    return fail(XG_EINVAL, "forceBeamColumn 2D needs ndm 2, ndf 3");
  if (d->elem_type == XG_ELE_FBC3D && (d->ndm != 3 || d->ndf != 6))
    return fail(XG_EINVAL, "forceBeamColumn 3D needs ndm 3, ndf 6");
  if (fr && (d->fbc_num_ip < 3 || d->fbc_num_ip > 5))
    return fail(XG_EINVAL, "forceBeamColumn needs 3..5 Lobatto points");
  if (fr && d->geom_transf != 0 && d->geom_transf != 1)
    return fail(XG_EINVAL, "geomTransf %d not supported (0 Linear, 1 PDelta)", d->geom_transf);
  if (fr && (d->num_sec <= 0 || !d->sec_fiber_start || !d->fib_y || !d->fib_area ||
             !d->fib_mat || d->num_uni <= 0 || !d->uni_type || !d->uni_param))
    return fail(XG_EINVAL, "forceBeamColumn needs fiber sections and uniaxial materials");
  if (d->elem_type == XG_ELE_FBC3D && (!d->fib_z || !d->sec_GJ || !d->elem_vecxz))
    return fail(XG_EINVAL, "3D fiber sections need z, GJ and vecxz");
  if (d->elem_type == XG_ELE_QUAD && (d->ndm != 2 || d->ndf != 2))
    return fail(XG_EINVAL, "quad needs ndm 2, ndf 2");
  if (d->elem_type == XG_ELE_BRICK && (d->ndm != 3 || d->ndf != 3))
    return fail(XG_EINVAL, "stdBrick needs ndm 3, ndf 3");
  if (d->num_nodes <= 0 || d->num_elems < 0 || !d->node_tag || !d->node_crd)
    return fail(XG_EINVAL, "empty model");
  if (d->num_elems > 0 && (!d->elem_tag || !d->elem_conn || !d->elem_mat || (!fr && !d->j2_param)))
    return fail(XG_EINVAL, "missing element arrays");
  if (d->handler != XG_HANDLER_PLAIN && d->handler != XG_HANDLER_TRANSFORMATION)
    return fail(XG_EINVAL, "constraint handler %d not supported", d->handler);
  if (d->handler == XG_HANDLER_TRANSFORMATION && d->num_mp > 0)
    return fail(XG_EINVAL, "the Transformation handler is supported with single-point "
                "constraints only (no equalDOF)");
  for (int i = 0; i < d->num_sp; i++) {
    if (!d->sp_pattern || d->sp_pattern[i] < 0) continue;
    if (d->handler != XG_HANDLER_TRANSFORMATION)
      return fail(XG_EINVAL, "imposed sp values need the Transformation handler");
    if (d->sp_pattern[i] >= 8) return fail(XG_EINVAL, "sp pattern must be in [0, 8)");
  }
  auto *m = new xg_model();
  m->ndm = d->ndm; m->ndf = d->ndf; m->nn = d->num_nodes; m->ne = d->num_elems;
  m->etype = d->elem_type;
  m->nen = fr ? 2 : (d->elem_type == XG_ELE_QUAD ? 4 : 8);
  m->nip = fr ? 0 : m->nen;
  m->ned = m->nen * m->ndf;
  m->thickness = d->thickness;
  m->node_tag.assign(d->node_tag, d->node_tag + m->nn);
  if (d->node_mass) m->node_mass.assign(d->node_mass, d->node_mass + (size_t)m->nn * d->ndf);
  else m->node_mass.assign((size_t)m->nn * d->ndf, 0.0);
  for (int i = 1; i < m->nn; i++)
    if (m->node_tag[i] <= m->node_tag[i - 1]) {
      delete m;
      return fail(XG_EINVAL, "node tags must be strictly ascending");
    }
  m->crd.assign(d->node_crd, d->node_crd + (size_t)m->nn * m->ndm);
  m->elem_tag.assign(d->elem_tag, d->elem_tag + m->ne);
  for (int i = 1; i < m->ne; i++)
    if (m->elem_tag[i] <= m->elem_tag[i - 1]) {
      delete m;
      return fail(XG_EINVAL, "element tags must be strictly ascending");
    }
  m->conn.resize((size_t)m->ne * m->nen);
  for (size_t k = 0; k < m->conn.size(); k++) {
    auto it = std::lower_bound(m->node_tag.begin(), m->node_tag.end(), d->elem_conn[k]);
    if (it == m->node_tag.end() || *it != d->elem_conn[k]) {
      const size_t bad_elem = k / m->nen;
      delete m;
      return fail(XG_EINVAL, "element %zu refers to a missing node", bad_elem);
    }
    m->conn[k] = (int)(it - m->node_tag.begin());
  }
  m->mat.assign(d->elem_mat, d->elem_mat + m->ne);
  if (!fr) {
    m->j2.assign(d->j2_param, d->j2_param + (size_t)d->num_j2 * XG_J2_NPARAM);
    for (int e = 0; e < m->ne; e++)
      if (m->mat[e] < 0 || m->mat[e] >= d->num_j2) {
        delete m;
        return fail(XG_EINVAL, "element %d: J2 row out of range", e);
      }
  } else {
    const int nsec = d->num_sec, nuni = d->num_uni;
    m->fb_nb = d->elem_type == XG_ELE_FBC2D ? 3 : 6;
    m->geom_transf = d->geom_transf;
    m->fb_nip = d->fbc_num_ip;
    m->fb_max_iters = d->fbc_max_iters > 0 ? d->fbc_max_iters : 10;
    m->fb_tol = d->fbc_tol > 0 ? d->fbc_tol : 1e-12;
    m->sec_fstart.assign(d->sec_fiber_start, d->sec_fiber_start + nsec + 1);
    const int nfib = m->sec_fstart[nsec];
    for (int s2 = 0; s2 < nsec; s2++)
      if (m->sec_fstart[s2 + 1] <= m->sec_fstart[s2]) {
        delete m;
        return fail(XG_EINVAL, "section %d has no fibers", s2);
      }
    m->fy.assign(d->fib_y, d->fib_y + nfib);
    m->fA.assign(d->fib_area, d->fib_area + nfib);
    m->fmat.assign(d->fib_mat, d->fib_mat + nfib);
    if (d->fib_z) m->fz.assign(d->fib_z, d->fib_z + nfib);
    else m->fz.assign(nfib, 0.0);
    if (d->sec_GJ) m->GJ.assign(d->sec_GJ, d->sec_GJ + nsec);
    else m->GJ.assign(nsec, 0.0);
    m->utype.assign(d->uni_type, d->uni_type + nuni);
    m->uparam.assign(d->uni_param, d->uni_param + (size_t)nuni * XG_UNI_NPARAM);
    for (int k = 0; k < nfib; k++)
      if (m->fmat[k] < 0 || m->fmat[k] >= nuni) {
        delete m;
        return fail(XG_EINVAL, "fiber %d: uniaxial row out of range", k);
      }
    for (int u = 0; u < nuni; u++)
      if (m->utype[u] != XG_UNI_STEEL02 && m->utype[u] != XG_UNI_CONCRETE02 &&
          m->utype[u] != XG_UNI_ELASTIC && m->utype[u] != XG_UNI_STEEL01 &&
          m->utype[u] != XG_UNI_CONCRETE01) {
        delete m;
        return fail(XG_EINVAL, "uniaxial row %d: unknown type %d", u, m->utype[u]);
      }
    for (int e = 0; e < m->ne; e++)
      if (m->mat[e] < 0 || m->mat[e] >= nsec) {
        delete m;
        return fail(XG_EINVAL, "element %d: section row out of range", e);
      }
    if (d->elem_vecxz) m->crd_vecxz.assign(d->elem_vecxz, d->elem_vecxz + (size_t)m->ne * 3);
  }
  m->num_sp = d->num_sp; m->num_mp = d->num_mp; m->num_loads = d->num_loads;
  m->handler = d->handler;
  if (m->num_sp) {
    m->sp_node.assign(d->sp_node, d->sp_node + m->num_sp);
    m->sp_dof.assign(d->sp_dof, d->sp_dof + m->num_sp);
    if (d->sp_pattern) m->sp_pat.assign(d->sp_pattern, d->sp_pattern + m->num_sp);
    else m->sp_pat.assign(m->num_sp, -1);
    if (d->sp_value) m->sp_val.assign(d->sp_value, d->sp_value + m->num_sp);
    else m->sp_val.assign(m->num_sp, 0.0);
  }
  if (m->num_mp) {
    m->mp_r.assign(d->mp_retained, d->mp_retained + m->num_mp);
    m->mp_c.assign(d->mp_constrained, d->mp_constrained + m->num_mp);
    m->mp_dof.assign(d->mp_dof, d->mp_dof + m->num_mp);
  }
  if (m->num_loads) {
    m->load_node.assign(d->load_node, d->load_node + m->num_loads);
    m->load_pat.assign(d->load_pattern, d->load_pattern + m->num_loads);
    m->load_val.assign(d->load_value, d->load_value + (size_t)m->num_loads * m->ndf);
    for (int p : m->load_pat)
      if (p < 0 || p >= 8) {
        delete m;
        return fail(XG_EINVAL, "load pattern must be in [0, 8)");
      }
  }
  int r = m->number();
  if (r) { delete m; return r; }
  *out = m;
  return 0;
}

int xg_model_destroy(xg_model *m) {
  delete m;
  return 0;
}

int xg_model_sizes(const xg_model *m, int *num_eqn, int *nnz) {
  if (!m) return fail(XG_EINVAL, "null model");
  if (num_eqn) *num_eqn = m->neq;
  if (nnz) *nnz = m->nnz;
  return 0;
}

int xg_model_numbering(const xg_model *m, int *eqn) {
  if (!m || !eqn) return fail(XG_EINVAL, "null argument");
  std::copy(m->eqn.begin(), m->eqn.end(), eqn);
  return 0;
}

int xg_model_pattern(const xg_model *m, int *rowptr, int *colidx) {
  if (!m || !rowptr || !colidx) return fail(XG_EINVAL, "null argument");
  std::copy(m->rowptr.begin(), m->rowptr.end(), rowptr);
  std::copy(m->colidx.begin(), m->colidx.end(), colidx);
  return 0;
}

int xg_elemset_set_trial_disp(xg_model *m, const double *u) {
  if (!m || !u) return fail(XG_EINVAL, "null argument");
  CK(cudaMemcpyAsync(m->d_U.p, u, (size_t)m->nn * m->ndf * sizeof(double), cudaMemcpyHostToDevice,
                     m->stream));
  CK(cudaStreamSynchronize(m->stream));
  return 0;
}

int xg_elemset_set_trial_disp_device(xg_model *m, const double *u_dev) {
  if (!m || !u_dev) return fail(XG_EINVAL, "null argument");
  CK(cudaMemcpyAsync(m->d_U.p, u_dev, (size_t)m->nn * m->ndf * sizeof(double),
                     cudaMemcpyDeviceToDevice, m->stream));
  return 0;
}

int xg_elemset_update(xg_model *m, double *csr_vals, double *resid) {
  if (!m) return fail(XG_EINVAL, "null model");
  RET(m->element_state(true));
  if (csr_vals)
    CK(cudaMemcpyAsync(csr_vals, m->d_vals.p, (size_t)m->nnz * sizeof(double),
                       cudaMemcpyDeviceToHost, m->stream));
  if (resid)
    CK(cudaMemcpyAsync(resid, m->d_resid.p, (size_t)m->neq * sizeof(double),
                       cudaMemcpyDeviceToHost, m->stream));
  CK(cudaMemcpyAsync(&m->last_nfail, m->d_nfail.p, sizeof(int), cudaMemcpyDeviceToHost,
                     m->stream));
  CK(cudaStreamSynchronize(m->stream));
  // Brick::update and J2PlaneStrain::setTrialStrain discard the return-map
  // status (Brick.cpp:839, J2PlaneStrain.cpp:133); the count is kept for
  // xg_profile_get ("return_map_cap_hits") only.
  return 0;
}

int xg_elemset_element_matrices(const xg_model *m, double *K, double *P) {
  if (!m) return fail(XG_EINVAL, "null model");
  const int ned = m->ned;
  const size_t nk = (size_t)m->ne * m->ke_size();
  if (K) {
    std::vector<double> ke(nk);
    CK(cudaMemcpyAsync(ke.data(), m->d_Ke.p, nk * sizeof(double), cudaMemcpyDeviceToHost,
                       m->stream));
    CK(cudaStreamSynchronize(m->stream));
    for (int e = 0; e < m->ne; e++) {
      double *out = K + (size_t)e * ned * ned;
      const double *in = ke.data() + (size_t)e * m->ke_size();
      if (!m->ke_pairs()) {
        std::copy(in, in + (size_t)ned * ned, out);
        continue;
      }
      // float pairs (hi, lo), 8 bytes an entry
      const float *pr = reinterpret_cast<const float *>(in);
      for (int k = 0; k < ned * ned; k++) out[k] = (double)pr[2 * k] + (double)pr[2 * k + 1];
    }
  }
  if (P) {
    CK(cudaMemcpyAsync(P, m->d_Re.p, (size_t)m->ne * ned * sizeof(double),
                       cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
  }
  return 0;
}

int xg_profile_enable(xg_model *m, int enable) {
  if (!m) return fail(XG_EINVAL, "null model");
  m->prof_on = enable != 0;
  for (auto &p : m->prof) { p.ms = 0.0; p.launches = 0; }
  m->point_updates = m->elem_updates = 0;
  if (m->d_work.p) CK(cudaMemsetAsync(m->d_work.p, 0, 2 * sizeof(unsigned long long), m->stream));
  return 0;
}

int xg_analysis_autotune(xg_model *m, int what) {
  if (!m) return fail(XG_EINVAL, "null model");
  if (!m->tune_a) {
    CK(cudaEventCreate(&m->tune_a));
    CK(cudaEventCreate(&m->tune_b));
  }
  if ((what & XG_TUNE_ELEMENT) && m->frames()) m->tune_elem.start({1, 2, 4, 8}, m->fbc_warps);
  if (what & XG_TUNE_PCG) m->tune_pcg.start({32, 64, 128, 256}, m->pcg_rows);
  return 0;
}

int xg_autotune_result(const xg_model *m, int *elem_warps, int *pcg_rows_per_block,
                       int *pending) {
  if (!m) return fail(XG_EINVAL, "null model");
  if (elem_warps) *elem_warps = m->fbc_warps;
  if (pcg_rows_per_block) *pcg_rows_per_block = m->pcg_rows;
  if (pending) *pending = (m->tune_elem.on && !m->tune_elem.done) + (m->tune_pcg.on && !m->tune_pcg.done);
  return 0;
}

int xg_model_stream(const xg_model *m, void **stream) {
  if (!m || !stream) return fail(XG_EINVAL, "null argument");
  *stream = (void *)m->stream;
  return 0;
}

int xg_model_pcg_layout(const xg_model *m, int *block_order, long long *blocks,
                        long long *chunked_rows) {
  if (!m || !block_order || !blocks || !chunked_rows) return fail(XG_EINVAL, "null argument");
  *block_order = m->pcg.nb_vals ? m->pcg.kb : 0;
  *blocks = m->pcg_blocks;
  *chunked_rows = m->pcg.nb_vals ? m->pcg.nlong : 0;
  return 0;
}

int xg_profile_counters(xg_model *m, long long *point_updates, long long *section_updates,
                        long long *element_updates) {
  if (!m) return fail(XG_EINVAL, "null model");
  long long pu = m->point_updates, su = 0;
  if (m->frames() && m->d_work.p) {
    unsigned long long w[2] = {0, 0};
    CK(cudaMemcpyAsync(w, m->d_work.p, sizeof w, cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    pu = (long long)w[0];
    su = (long long)w[1];
  }
  if (point_updates) *point_updates = pu;
  if (section_updates) *section_updates = su;
  if (element_updates) *element_updates = m->elem_updates;
  return 0;
}

int xg_profile_get(const xg_model *m, int k, char *name, int cap, double *ms, long *launches) {
  if (!m) return fail(XG_EINVAL, "null model");
  if (k == (int)m->prof.size()) {
    if (name && cap > 0) snprintf(name, cap, "%s", "return_map_cap_hits");
    if (ms) *ms = 0.0;
    if (launches) *launches = m->last_nfail;
    return 0;
  }
  if (k < 0 || k > (int)m->prof.size()) return fail(XG_EINVAL, "no profile slot %d", k);
  if (name && cap > 0) snprintf(name, cap, "%s", m->prof[k].name);
  if (ms) *ms = m->prof[k].ms;
  if (launches) *launches = m->prof[k].launches;
  return 0;
}

int xg_elemset_commit(xg_model *m) {
  if (!m) return fail(XG_EINVAL, "null model");
  RET(m->commit_state());
  CK(cudaStreamSynchronize(m->stream));
  m->time_c = m->time;
  return 0;
}

// revertToLastCommit: the trial state returns to the state at the last commit
int xg_elemset_revert(xg_model *m) {
  if (!m) return fail(XG_EINVAL, "null model");
  RET(m->revert_state());
  CK(cudaStreamSynchronize(m->stream));
  m->time = m->time_c;
  return 0;
}

int xg_elemset_revert_to_start(xg_model *m) { return xg_reset(m); }

int xg_elemset_get_history(const xg_model *m, int which, double *out, long cap) {
  if (!m || !out) return fail(XG_EINVAL, "null argument");
  if (m->frames() && (which == 1 || which == 2)) {
    // committed fiber records [nrec*12] or committed element states
    const long need = which == 1 ? m->fb_nrec * 12 : (long)m->ne * frame_state_stride(m->fb_nip);
    if (cap < need) return fail(XG_EINVAL, "history needs %ld doubles", need);
    CK(cudaMemcpyAsync(out, which == 1 ? m->d_fh_c.p : m->d_st_c.p, need * sizeof(double),
                       cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    return (int)std::min<long>(need, 0x7fffffff);
  }
  if (which != 0 || m->frames())
    return fail(XG_EINVAL, "history kind %d not held by this model", which);
  const long np = m->npts(), nh = m->nhist();
  const long need = np * (nh + 1);
  if (cap < need) return fail(XG_EINVAL, "history needs %ld doubles", need);
  CK(cudaMemcpyAsync(out, m->d_epc.p, np * nh * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  CK(cudaMemcpyAsync(out + np * nh, m->d_xic.p, np * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  CK(cudaStreamSynchronize(m->stream));
  return (int)std::min<long>(need, 0x7fffffff);
}

int xg_elemset_set_history(xg_model *m, int which, const double *in, long n) {
  if (!m || !in) return fail(XG_EINVAL, "null argument");
  if (which != 0) return fail(XG_EINVAL, "history kind %d not held by this model", which);
  const long np = m->npts(), nh = m->nhist();
  if (n != np * (nh + 1)) return fail(XG_EINVAL, "history needs %ld doubles", np * (nh + 1));
  CK(cudaMemcpyAsync(m->d_epc.p, in, np * nh * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  CK(cudaMemcpyAsync(m->d_xic.p, in + np * nh, np * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  CK(cudaStreamSynchronize(m->stream));
  return 0;
}

int xg_soe_solve(xg_model *m, const double *b, double *x, double rtol, int maxit, int *iters,
                 double *relres) {
  if (!m || !b || !x) return fail(XG_EINVAL, "null argument");
  CK(cudaMemcpyAsync(m->d_b.p, b, (size_t)m->neq * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  if (m->system == XG_SYSTEM_PROFILE_SPD) {
    const double *bs[1] = {m->d_b.p};
    double *xs[1] = {m->d_x.p};
    RET(m->solve_profile(1, bs, xs));
    CK(cudaMemcpyAsync(x, m->d_x.p, (size_t)m->neq * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    if (iters) *iters = 0;
    if (relres) *relres = 0.0;
    return 0;
  }
  if (!m->blocks_factored) RET(m->pcg_prepare());
  CK(cudaMemsetAsync(m->d_x.p, 0, (size_t)std::max(m->neq, 1) * sizeof(double), m->stream));
  int it = 0;
  double rr = 0.0;
  int r = pcg_solve(m->pcg, m->d_b.p, m->d_x.p, rtol, maxit, &it, &rr, m->stream);
  if (iters) *iters = it;
  if (relres) *relres = rr;
  CK(cudaMemcpyAsync(x, m->d_x.p, (size_t)m->neq * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  CK(cudaStreamSynchronize(m->stream));
  if (r) return fail(XG_ESOLVE, "PCG: %d iterations, relative residual %.3e", it, rr);
  return 0;
}

int xg_soe_solve_device(xg_model *m, const double *b_dev, double *x_dev, double rtol, int maxit,
                        int *iters, double *relres) {
  if (!m || !b_dev || !x_dev) return fail(XG_EINVAL, "null argument");
  if (m->system == XG_SYSTEM_PROFILE_SPD) {
    RET(m->solve_profile(1, &b_dev, &x_dev));
    CK(cudaStreamSynchronize(m->stream));
    if (iters) *iters = 0;
    if (relres) *relres = 0.0;
    return 0;
  }
  if (!m->blocks_factored) RET(m->pcg_prepare());
  CK(cudaMemsetAsync(x_dev, 0, (size_t)std::max(m->neq, 1) * sizeof(double), m->stream));
  int it = 0;
  double rr = 0.0;
  const int r = pcg_solve(m->pcg, b_dev, x_dev, rtol, maxit, &it, &rr, m->stream);
  if (iters) *iters = it;
  if (relres) *relres = rr;
  if (r) return fail(XG_ESOLVE, "PCG: %d iterations, relative residual %.3e", it, rr);
  return 0;
}

int xg_analysis_set_phase(xg_model *m, const xg_phase_desc *ph) {
  if (!m || !ph) return fail(XG_EINVAL, "null argument");
  // `loadConst -time 0.0` after a finished phase that asks for it
  if (m->have_phase && m->phase.load_const && m->phase_steps_done >= m->phase.num_steps &&
      !m->phase_closed) {
    m->phase_closed = true;
    for (int p = 0; p < 8; p++)
      if (m->added[p] && !m->pattern_const[p]) {
        m->pattern_const[p] = 1;
        m->lambda_const[p] = m->time;
      }
    m->time = m->time_c = 0.0;
  }
  m->phase = *ph;
  m->have_phase = true;
  m->phase_steps_done = 0;
  m->phase_closed = false;
  m->free_step_graph();
  return m->init_phase();
}

// loadConst -time t (domain/domain/Domain.cpp setLoadConstant + setCurrentTime):
// every pattern applied so far keeps its current factor, the time becomes t
int xg_analysis_load_const(xg_model *m, double time) {
  if (!m) return fail(XG_EINVAL, "null model");
  for (int p = 0; p < 8; p++)
    if (m->added[p] && !m->pattern_const[p]) {
      m->pattern_const[p] = 1;
      m->lambda_const[p] = m->time;
    }
  m->time = m->time_c = time;
  m->phase_closed = true;
  return 0;
}

int xg_analysis_set_system(xg_model *m, int system) {
  if (!m) return fail(XG_EINVAL, "null model");
  if (system != XG_SYSTEM_BJPCG && system != XG_SYSTEM_PROFILE_SPD)
    return fail(XG_EINVAL, "unknown system %d", system);
  m->system = system;
  m->free_step_graph();
  if (system == XG_SYSTEM_PROFILE_SPD) RET(m->ensure_profile());
  return 0;
}

int xg_analysis_set_solver(xg_model *m, double rtol, int maxit) {
  if (!m || rtol <= 0.0 || maxit <= 0) return fail(XG_EINVAL, "bad solver settings");
  m->rtol = rtol;
  m->maxit = maxit;
  return 0;
}

int xg_analyze(xg_model *m, int num_steps, xg_step_stats *stats) {
  if (!m) return fail(XG_EINVAL, "null model");
  if (!m->have_phase) return fail(XG_ESTATE, "no analysis phase set");
  g_err.clear();
  for (int i = 0; i < num_steps; i++) {
    int r = m->step(stats ? &stats[i] : nullptr);
    if (r) {
      // BasicAnalysisBuilder::analyzeStatic: revert to the last commit
      std::string keep = g_err;
      xg_elemset_revert(m);
      g_err = keep;
      return r;
    }
    m->phase_steps_done++;
    RET(m->record_step());
  }
  return 0;
}

int xg_get_disp(const xg_model *m, double *u, double *lambda) {
  if (!m) return fail(XG_EINVAL, "null model");
  if (u) {
    CK(cudaMemcpyAsync(u, m->d_Uc.p, (size_t)m->nn * m->ndf * sizeof(double),
                       cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
  }
  if (lambda) *lambda = m->time_c;
  return 0;
}

int xg_get_response(const xg_model *m, int response, double *out) {
  if (!m || !out || response < XG_REC_DISP || response > XG_REC_ACCEL)
    return fail(XG_EINVAL, "bad argument");
  const double *src = response == XG_REC_DISP ? m->d_Uc.p
                      : response == XG_REC_VEL ? m->d_Vc.p : m->d_Ac.p;
  CK(cudaMemcpyAsync(out, src, (size_t)m->nn * m->ndf * sizeof(double), cudaMemcpyDeviceToHost,
                     m->stream));
  CK(cudaStreamSynchronize(m->stream));
  return 0;
}

int xg_recorder_add(xg_model *m, int kind, int response, const int *node_tags, int num_nodes,
                    const int *dofs, int num_dofs, int echo_time, double dT, int *id) {
  if (!m || !id || num_nodes < 0 || num_dofs < 0 || (num_nodes && !node_tags) ||
      (num_dofs && !dofs) || (kind != XG_REC_NODE && kind != XG_REC_ENVELOPE) ||
      response < XG_REC_DISP || response > XG_REC_ACCEL || dT < 0.0)
    return fail(XG_EINVAL, "bad recorder settings");
  std::vector<int> idx;
  for (int i = 0; i < num_nodes; i++) {
    auto it = std::lower_bound(m->node_tag.begin(), m->node_tag.end(), node_tags[i]);
    if (it == m->node_tag.end() || *it != node_tags[i])
      return fail(XG_EINVAL, "recorder: no node %d", node_tags[i]);
    const int n = (int)(it - m->node_tag.begin());
    for (int j = 0; j < num_dofs; j++) {
      if (dofs[j] < 0) return fail(XG_EINVAL, "recorder: bad dof %d", dofs[j]);
      // a dof the node does not have records 0 (NodeRecorder.cpp:258-262)
      idx.push_back(dofs[j] < m->ndf ? n * m->ndf + dofs[j] : -1);
    }
  }
  auto r = std::make_unique<xg_model::Recorder>();
  r->kind = kind;
  r->response = response;
  r->echo = echo_time ? 1 : 0;
  r->dT = dT;
  r->nvals = (int)idx.size();
  RET(r->idx.upload(idx.data(), idx.size(), m->stream));
  if (kind == XG_REC_NODE) {
    r->ncol = r->echo + r->nvals;
  } else {
    r->ncol = (r->echo ? 2 : 1) * r->nvals;
    RET(r->data.alloc(std::max<size_t>((size_t)3 * r->ncol, 1)));
    CK(cudaMemsetAsync(r->data.p, 0, std::max<size_t>((size_t)3 * r->ncol, 1) * sizeof(double),
                       m->stream));
  }
  CK(cudaStreamSynchronize(m->stream));
  m->recorders.push_back(std::move(r));
  *id = (int)m->recorders.size() - 1;
  return 0;
}

int xg_recorder_size(const xg_model *m, int id, int *rows, int *cols) {
  if (!m || id < 0 || id >= (int)m->recorders.size()) return fail(XG_EINVAL, "no recorder %d", id);
  const auto &r = *m->recorders[id];
  if (rows) *rows = r.rows;
  if (cols) *cols = r.ncol;
  return 0;
}

int xg_recorder_read(const xg_model *m, int id, double *out, int max_rows) {
  if (!m || id < 0 || id >= (int)m->recorders.size() || (!out && max_rows > 0))
    return fail(XG_EINVAL, "bad recorder read");
  const auto &r = *m->recorders[id];
  const int n = std::min(max_rows, r.rows);
  if (n > 0 && r.ncol > 0) {
    CK(cudaMemcpyAsync(out, r.data.p, (size_t)n * r.ncol * sizeof(double),
                       cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
  }
  return n;
}

// DataFileStream::write (handler/DataFileStream.cpp:463-483): the values of
// a row separated by blanks, a newline after the last, printed as a C++
// stream with setprecision(precision) prints them (%g).
int xg_recorder_write(const xg_model *m, int id, const char *path, int precision) {
  if (!m || !path || precision < 1 || precision > 17 || id < 0 ||
      id >= (int)m->recorders.size())
    return fail(XG_EINVAL, "bad recorder write");
  const auto &r = *m->recorders[id];
  std::vector<double> h((size_t)r.rows * r.ncol);
  if (!h.empty()) RET(xg_recorder_read(m, id, h.data(), r.rows) < 0 ? XG_ECUDA : 0);
  FILE *f = fopen(path, "w");
  if (!f) return fail(XG_EINVAL, "recorder: cannot open %s", path);
  for (int i = 0; i < r.rows; i++) {
    for (int j = 0; j < r.ncol; j++)
      fprintf(f, j + 1 < r.ncol ? "%.*g " : "%.*g\n", precision, h[(size_t)i * r.ncol + j]);
  }
  fclose(f);
  return 0;
}

int xg_reset(xg_model *m) {
  if (!m) return fail(XG_EINVAL, "null model");
  cudaStream_t s = m->stream;
  const size_t nu = (size_t)m->nn * m->ndf;
  CK(cudaMemsetAsync(m->d_U.p, 0, nu * sizeof(double), s));
  CK(cudaMemsetAsync(m->d_Uc.p, 0, nu * sizeof(double), s));
  for (auto *b : {&m->d_V, &m->d_A, &m->d_Vc, &m->d_Ac})
    CK(cudaMemsetAsync(b->p, 0, std::max<size_t>(nu, 1) * sizeof(double), s));
  if (m->frames()) {
    RET(m->upload_frames());
  } else {
    RET(launch_j2_zero_state(m->view(), s));
    const long np = m->npts();
    CK(cudaMemcpyAsync(m->d_sig_c.p, m->d_sig.p, np * m->nsig() * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(m->d_tan_c.p, m->d_tan.p, np * m->ntan() * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  CK(cudaStreamSynchronize(s));
  m->time = m->time_c = 0.0;
  for (int p = 0; p < 8; p++) {
    m->pattern_const[p] = 0;
    m->added[p] = 0;
    m->lambda_const[p] = 0.0;
  }
  m->have_phase = false;
  m->steps_since_reset = 0;
  m->adj.have = false;
  m->free_step_graph();
  return 0;
}

int xg_analysis_set_graph(xg_model *m, int enable) {
  if (!m) return fail(XG_EINVAL, "null model");
  m->sg.want = enable != 0;
  m->free_step_graph();
  return 0;
}

int xg_analysis_graph_steps(const xg_model *m, long *steps) {
  if (!m || !steps) return fail(XG_EINVAL, "null argument");
  *steps = m->sg.launches;
  return 0;
}

int xg_model_set_uniaxial_params(xg_model *m, const double *uni_param, int num_uni) {
  if (!m || !uni_param) return fail(XG_EINVAL, "null argument");
  if (!m->frames()) return fail(XG_EINVAL, "the model has no uniaxial materials");
  if (num_uni != (int)m->utype.size())
    return fail(XG_EINVAL, "%d materials given, the model has %zu", num_uni, m->utype.size());
  m->uparam.assign(uni_param, uni_param + (size_t)num_uni * XG_UNI_NPARAM);
  return xg_reset(m);
}

int xg_adjoint_forward(xg_model *m, const xg_phase_desc *ph, int num_steps, int ckpt_every,
                       const xg_objective_desc *obj, double *J) {
  if (!m) return fail(XG_EINVAL, "null model");
  g_err.clear();
  const int r = m->adjoint_forward(ph, num_steps, ckpt_every, obj, J);
  if (r) m->adj.have = false;
  return r;
}

int xg_adjoint_objective_terms(const xg_model *m, double *Jk, int num_terms) {
  if (!m || !Jk) return fail(XG_EINVAL, "null argument");
  if (!m->adj.have) return fail(XG_ESTATE, "no adjoint run (xg_adjoint_forward first)");
  if (num_terms != m->adj.nterm) return fail(XG_EINVAL, "the run has %d terms", m->adj.nterm);
  for (int k = 0; k < num_terms; k++) Jk[k] = m->adj.Jk[k];
  return 0;
}

int xg_adjoint_backward(xg_model *m, double scale, double *grad, int num_uni) {
  if (!m) return fail(XG_EINVAL, "null model");
  g_err.clear();
  return m->adjoint_backward(scale, grad, num_uni);
}

int xg_ddm_forward(xg_model *m, const xg_phase_desc *ph, int num_steps, int num_dir,
                   const double *dtheta, const xg_objective_desc *obj, double *J, double *dJ) {
  g_err.clear();
  if (!m) return fail(XG_EINVAL, "null model");
  return m->ddm_forward(ph, num_steps, num_dir, dtheta, obj, J, dJ);
}

int xg_ddm_objective_terms(const xg_model *m, int dir, double *dJk, int num_terms) {
  g_err.clear();
  if (!m || !dJk) return fail(XG_EINVAL, "null argument");
  if (!m->ddm.have) return fail(XG_ESTATE, "no DDM run (xg_ddm_forward first)");
  if (dir < 0 || dir >= m->ddm.nd) return fail(XG_EINVAL, "bad direction %d", dir);
  if (num_terms != m->ddm.nterm) return fail(XG_EINVAL, "the run has %d terms", m->ddm.nterm);
  const size_t nt1 = std::max(m->ddm.nterm, 1);
  for (int j = 0; j < num_terms; j++) dJk[j] = m->ddm.dJt[(size_t)dir * nt1 + j];
  return 0;
}

int xg_ddm_disp_sensitivity(const xg_model *m, int dir, double *out) {
  g_err.clear();
  if (!m || !out) return fail(XG_EINVAL, "null argument");
  if (!m->ddm.have) return fail(XG_ESTATE, "no DDM run (xg_ddm_forward first)");
  if (dir < 0 || dir >= m->ddm.nd) return fail(XG_EINVAL, "bad direction %d", dir);
  std::vector<double> x(std::max(m->neq, 1));
  const size_t ne1 = std::max(m->neq, 1);
  if (cudaMemcpyAsync(x.data(), m->ddm.dU.p + (size_t)dir * ne1, ne1 * sizeof(double),
                      cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
      cudaStreamSynchronize(m->stream) != cudaSuccess)
    return fail(XG_ECUDA, "copy failed");
  for (size_t a = 0; a < m->eqn.size(); a++) out[a] = m->eqn[a] >= 0 ? x[m->eqn[a]] : 0.0;
  return 0;
}

}  // extern "C"

namespace xg {
// Sets the text xg_last_error() returns (used by entry points defined in
// other translation units).
void record_error(const char *msg) { g_err = msg ? msg : ""; }
}  // namespace xg
