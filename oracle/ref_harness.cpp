// ref_harness.cpp -- test infrastructure, never part of the product.
//
// Builds a model with the reference's own C++ classes (compiled unchanged
// from its SRC/ tree by build_ref.py) from the flat xg_model_desc used by
// libxara_gpu.so, runs the reference's analysis loop and records, for every
// linear solve, the assembled right-hand side, the tangent values on the
// SparseGenColLinSOE pattern, the solution and the nodal trial
// displacements at that moment.  Model construction follows the reference's
// C++ unit-test pattern (tests/Other/UnitTests/Example1/main.cpp); the
// analysis objects are wired as BasicAnalysisBuilder::setLinks does
// (runtime/runtime/BasicAnalysisBuilder.cpp:134-180) and each step runs as in
// BasicAnalysisBuilder::analyzeStatic / analyzeTransient (:337-520).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <array>

#include <OPS_Globals.h>
#include <StandardStream.h>
#include <DummyStream.h>

#include <Domain.h>
#include <Node.h>
#include <SP_Constraint.h>
#include <MP_Constraint.h>
#include <LoadPattern.h>
#include <LinearSeries.h>
#include <NodalLoad.h>

#include <FourNodeQuad.h>
#include <Brick.h>
#include <J2PlaneStrain.h>
#include <J2ThreeDimensional.h>
#include <Steel01.h>
#include <Steel02.h>
#include <Concrete01.h>
#include <Concrete02.h>
#include <ElasticMaterial.h>
#include <FiberSection2d.h>
#include <FiberSection3d.h>
#include <ForceBeamColumn2d.h>
#include <ForceBeamColumn3d.h>
#include <LobattoBeamIntegration.h>
#include <LinearCrdTransf2d.h>
#include <PDeltaCrdTransf2d.h>
#include <BasicFrameTransf.h>
#include <Vector3D.h>
#include <FrameTransform.h>
#include <LinearFrameTransf.hpp>
#include <PDeltaFrameTransf3d.hpp>

#include <AnalysisModel.h>
#include <PlainHandler.h>
#include <TransformationConstraintHandler.h>
#include <DOF_Numberer.h>
#include <RCM.h>
#include <LoadControl.h>
#include <DisplacementControl.h>
#include <Newmark.h>
#include <Parameter.h>
#include <TransientIntegrator.h>
#include <UniformExcitation.h>
#include <GroundMotion.h>
#include <PathSeries.h>
#include <NewtonRaphson.h>
#include <CTestNormDispIncr.h>
#include <CTestNormUnbalance.h>
#include <LinearSOE.h>
#include <ProfileSPDLinSOE.h>
#include <ProfileSPDLinDirectSolver.h>
#include <SparseGenColLinSOE.h>
#include <SparseGenColLinSolver.h>
#include <Graph.h>
#include <DOF_Group.h>
#include <DataFileStream.h>
#include <NodeRecorder.h>
#include <EnvelopeNodeRecorder.h>
#include <NodeData.h>
#include <Vector.h>
#include <Matrix.h>
#include <ID.h>

#include "../include/xara_gpu.h"

// Globals that the reference's Tcl runtime normally defines
// (SRC/logging/logging.cpp needs tcl.h, so they are defined here).
static StandardStream ref_sserr;
static DummyStream ref_ssnul;
OPS_Stream *opserrPtr = &ref_ssnul;
OPS_Stream *opsdbgPtr = &ref_ssnul;
OPS_Stream *opslogPtr = &ref_ssnul;
OPS_Stream *opswrnPtr = &ref_ssnul;
OPS_Stream *opsmrdPtr = &ref_ssnul;

namespace {

using clk = std::chrono::steady_clock;

// SparseGenColLinSOE with its CSC storage readable by the harness.
class NoSolve : public SparseGenColLinSolver {
 public:
  NoSolve() : SparseGenColLinSolver(0) {}
  int solve() override { return 0; }
  int setSize() override { return 0; }
  int sendSelf(int, Channel &) override { return 0; }
  int recvSelf(int, Channel &, FEM_ObjectBroker &) override { return 0; }
};

class GenAccess : public SparseGenColLinSOE {
 public:
  explicit GenAccess(SparseGenColLinSolver &s) : SparseGenColLinSOE(s) {}
  int n() const { return size; }
  int nz() const { return nnz; }
  const double *a() const { return A; }
  const int *rows() const { return rowA; }
  const int *colStart() const { return colStartA; }
};

// The reference's own profile storage (ProfileSPDLinSOE.h: A, iDiagLoc), for
// comparing a device system's assembly with it.
class ProfAccess : public ProfileSPDLinSOE {
 public:
  explicit ProfAccess(ProfileSPDLinSolver &s) : ProfileSPDLinSOE(s) {}
  const double *a() const { return A; }
  const int *diagLoc() const { return iDiagLoc; }
  int psize() const { return profileSize; }
  bool factored() const { return isAfactored; }
};

struct Capture {
  int profile = 0;    // also keep ProfileSPDLinSOE's A at every captured solve
  std::vector<double> P, lastP;
  int enabled = 0;
  int cap = 0;
  int count = 0;
  int step = 0;       // global step index
  int iter = 0;       // solve index within the step
  std::vector<int> stepOf, iterOf;
  std::vector<double> B, A, X, U, lam;
};

struct Harness;

// LinearSOE that forwards every call to a ProfileSPDLinSOE (the reference
// default system, BasicAnalysisBuilder.cpp:820) for solving and to a
// SparseGenColLinSOE for the pattern and the tangent values.
class CaptureSOE : public LinearSOE {
 public:
  CaptureSOE(Harness *h)
      : LinearSOE(0), h_(h), gen_(nosolve_),
        prof_(*(new ProfileSPDLinDirectSolver())) {}
  int setLinks(AnalysisModel &m) override {
    LinearSOE::setLinks(m);
    gen_.setLinks(m);
    prof_.setLinks(m);
    if (obs) obs->setLinks(m);
    return 0;
  }
  int setSize(Graph &g) override {
    int r = gen_.setSize(g);
    if (r < 0) return r;
    if (obs && obs->setSize(g) < 0) return -1;
    return prof_.setSize(g);
  }
  int getNumEqn() const override { return prof_.getNumEqn(); }
  int addA(const Matrix &m, const ID &id, double f) override {
    gen_.addA(m, id, f);
    if (obs && obs->addA(m, id, f) < 0) obs_errors++;
    return prof_.addA(m, id, f);
  }
  int addB(const Vector &v, const ID &id, double f) override {
    gen_.addB(v, id, f);
    if (obs && obs->addB(v, id, f) < 0) obs_errors++;
    return prof_.addB(v, id, f);
  }
  int setB(const Vector &v, double f) override {
    gen_.setB(v, f);
    if (obs && obs->setB(v, f) < 0) obs_errors++;
    return prof_.setB(v, f);
  }
  void zeroA() override {
    gen_.zeroA();
    prof_.zeroA();
    if (obs) obs->zeroA();
  }
  void zeroB() override {
    gen_.zeroB();
    prof_.zeroB();
    if (obs) obs->zeroB();
  }
  const Vector &getX() override { return prof_.getX(); }
  const Vector &getB() override { return prof_.getB(); }
  double normRHS() override { return prof_.normRHS(); }
  void setX(int loc, double v) override { prof_.setX(loc, v); }
  void setX(const Vector &x) override { prof_.setX(x); }
  int solve() override;
  int sendSelf(int, Channel &) override { return 0; }
  int recvSelf(int, Channel &, FEM_ObjectBroker &) override { return 0; }

  GenAccess &gen() { return gen_; }
  const ProfAccess &profile() const { return prof_; }
  double solveSeconds = 0.0;
  // A second LinearSOE fed the same calls (a system under test), and a
  // callback run before every solve, while both hold the same A and B.
  LinearSOE *obs = nullptr;
  void (*on_solve)(void *) = nullptr;
  void *on_solve_ctx = nullptr;
  int obs_errors = 0;

 private:
  Harness *h_;
  NoSolve nosolve_;
  GenAccess gen_;
  ProfAccess prof_;
};

struct Harness {
  xg_model_desc d{};
  Domain *domain = nullptr;
  std::vector<Node *> nodes;
  AnalysisModel *model = nullptr;
  ConstraintHandler *handler = nullptr;
  DOF_Numberer *numberer = nullptr;
  CaptureSOE *soe = nullptr;
  Capture cap;
  int numbered = 0;
  int totalSteps = 0;
  double elemSeconds = 0.0, stepSeconds = 0.0;
  std::vector<LoadPattern *> patterns;
  LinearSOE *observer = nullptr;
  void (*on_solve)(void *) = nullptr;
  void *on_solve_ctx = nullptr;
  // DDM sensitivity (the reference's computeGradients): parameters added to
  // the Domain, and the objective J = sum over steps and terms of
  // w_k u(node_k, dof_k)^2 with its gradient accumulated after every step
  struct Ddm {
    int active = 0;
    std::vector<int> node_index, dof;
    std::vector<double> w, grad;
    double J = 0.0;
  } ddm;

  void snapshotU(double *out) {
    int ndf = d.ndf;
    for (size_t i = 0; i < nodes.size(); i++) {
      const Vector &u = nodes[i]->getTrialDisp();
      for (int j = 0; j < ndf; j++) out[i * ndf + j] = u(j);
    }
  }
};

int CaptureSOE::solve() {
  Capture &c = h_->cap;
  if (c.enabled && c.count < c.cap) {
    int n = gen_.n(), nz = gen_.nz();
    int nu = h_->d.num_nodes * h_->d.ndf;
    c.stepOf.push_back(c.step);
    c.iterOf.push_back(c.iter);
    c.lam.push_back(h_->domain->getCurrentTime());
    const Vector &b = prof_.getB();
    for (int i = 0; i < n; i++) c.B.push_back(b(i));
    c.A.insert(c.A.end(), gen_.a(), gen_.a() + nz);
    if (c.profile) {
      // ProfileSPDLinDirectSolver factors A in place: a second solve with
      // the same matrix finds the factor there, so keep the assembled A
      // from the last solve that had not factored it yet
      if (!prof_.factored()) c.lastP.assign(prof_.a(), prof_.a() + prof_.psize());
      c.P.insert(c.P.end(), c.lastP.begin(), c.lastP.end());
    }
    size_t off = c.U.size();
    c.U.resize(off + nu);
    h_->snapshotU(&c.U[off]);
  }
  if (on_solve) on_solve(on_solve_ctx);
  auto t0 = clk::now();
  int r = prof_.solve();
  solveSeconds += std::chrono::duration<double>(clk::now() - t0).count();
  if (c.enabled && c.count < c.cap) {
    const Vector &x = prof_.getX();
    for (int i = 0; i < gen_.n(); i++) c.X.push_back(x(i));
    c.count++;
  }
  c.iter++;
  return r;
}

UniaxialMaterial *make_uniaxial(int type, const double *q, int tag) {
  switch (type) {
    case XG_UNI_STEEL02:
      return new Steel02(tag, q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], q[9], q[10]);
    case XG_UNI_CONCRETE02:
      return new Concrete02(tag, q[0], q[1], q[2], q[3], q[4], q[5], q[6]);
    case XG_UNI_STEEL01:
      return new Steel01(tag, q[0], q[1], q[2], q[3], q[4], q[5], q[6]);
    case XG_UNI_CONCRETE01:
      return new Concrete01(tag, q[0], q[1], q[2], q[3]);
    case XG_UNI_ELASTIC:
      return new ElasticMaterial(tag, q[0]);
  }
  return nullptr;
}

// `section Fiber` with fibers (y[, z], A, material) and, in 3D, elastic torsion GJ.
SectionForceDeformation *make_section(const xg_model_desc &d, int s, int tag) {
  const int f0 = d.sec_fiber_start[s], f1 = d.sec_fiber_start[s + 1];
  std::vector<UniaxialMaterial *> protos(d.num_uni, nullptr);
  for (int u = 0; u < d.num_uni; u++)
    protos[u] = make_uniaxial(d.uni_type[u], d.uni_param + (size_t)u * XG_UNI_NPARAM, u + 1);
  SectionForceDeformation *sec = nullptr;
  if (d.ndm == 2) {
    FiberSection2d *fs = new FiberSection2d(tag, f1 - f0);
    for (int k = f0; k < f1; k++) fs->addFiber(*protos[d.fib_mat[k]], d.fib_area[k], d.fib_y[k]);
    sec = fs;
  } else {
    ElasticMaterial torsion(0, d.sec_GJ[s]);
    FiberSection3d *fs = new FiberSection3d(tag, f1 - f0, torsion);
    for (int k = f0; k < f1; k++)
      fs->addFiber(*protos[d.fib_mat[k]], d.fib_area[k], d.fib_y[k], d.fib_z[k]);
    sec = fs;
  }
  for (auto *p : protos) delete p;
  return sec;
}

int nen_of(int type) {
  switch (type) {
    case XG_ELE_QUAD: return 4;
    case XG_ELE_BRICK: return 8;
    default: return 2;
  }
}

}  // namespace

extern "C" {

int xref_version(void) { return 1; }

// Build the reference Domain for a model description.
void *xref_create(const xg_model_desc *desc) {
  Harness *h = new Harness();
  h->d = *desc;
  const xg_model_desc &d = *desc;
  h->domain = new Domain();
  Domain *dom = h->domain;
  for (int i = 0; i < d.num_nodes; i++) {
    const double *x = d.node_crd + (size_t)i * d.ndm;
    Node *n = nullptr;
    if (d.ndm == 2)
      n = new Node(d.node_tag[i], d.ndf, x[0], x[1]);
    else
      n = new Node(d.node_tag[i], d.ndf, x[0], x[1], x[2]);
    if (d.node_mass) {
      Matrix M(d.ndf, d.ndf);
      for (int j = 0; j < d.ndf; j++) M(j, j) = d.node_mass[(size_t)i * d.ndf + j];
      n->setMass(M);
    }
    dom->addNode(n);
    h->nodes.push_back(n);
  }
  int nen = nen_of(d.elem_type);
  for (int e = 0; e < d.num_elems; e++) {
    const int *c = d.elem_conn + (size_t)e * nen;
    Element *ele = nullptr;
    if (d.elem_type == XG_ELE_FBC2D || d.elem_type == XG_ELE_FBC3D) {
      const int nip = d.fbc_num_ip;
      SectionForceDeformation *proto = make_section(d, d.elem_mat[e], 1);
      std::vector<SectionForceDeformation *> secs(nip, proto);
      LobattoBeamIntegration lobatto;
      if (d.elem_type == XG_ELE_FBC2D) {
        CrdTransf *tr = d.geom_transf ? (CrdTransf *)new PDeltaCrdTransf2d(1)
                                      : (CrdTransf *)new LinearCrdTransf2d(1);
        ele = new ForceBeamColumn2d(d.elem_tag[e], c[0], c[1], nip, secs.data(), lobatto, *tr,
                                    0.0, d.fbc_max_iters, d.fbc_tol);
        delete tr;
      } else {
        const double *vz = d.elem_vecxz + 3 * (size_t)e;
        Vector3D vecxz{vz[0], vz[1], vz[2]};
        FrameTransform<2, 6> *t = d.geom_transf
                                      ? (FrameTransform<2, 6> *)new PDeltaFrameTransf<2, 6>(1, vecxz)
                                      : (FrameTransform<2, 6> *)new LinearFrameTransf<2, 6>(1, vecxz);
        BasicFrameTransf3d tr(t);
        ele = new ForceBeamColumn3d(d.elem_tag[e], c[0], c[1], nip, secs.data(), lobatto, tr,
                                    0.0, d.fbc_max_iters, d.fbc_tol);
      }
      delete proto;
      dom->addElement(ele);
      continue;
    }
    const double *p = d.j2_param + (size_t)d.elem_mat[e] * XG_J2_NPARAM;
    if (d.elem_type == XG_ELE_QUAD) {
      J2PlaneStrain mat(1, p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7]);
      std::array<int, 4> nd{c[0], c[1], c[2], c[3]};
      ele = new FourNodeQuad(d.elem_tag[e], nd, mat, d.thickness, 0.0, 0.0, 0.0, 0.0);
    } else if (d.elem_type == XG_ELE_BRICK) {
      J2ThreeDimensional mat(1, p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7]);
      ele = new Brick(d.elem_tag[e], c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], mat);
    } else {
      fprintf(stderr, "xref_create: element type %d not supported by the harness\n", d.elem_type);
      return nullptr;
    }
    dom->addElement(ele);
  }
  // constraints: homogeneous fixes in the domain, imposed values in patterns
  int maxPat = -1;
  for (int i = 0; i < d.num_sp; i++) maxPat = std::max(maxPat, d.sp_pattern[i]);
  for (int i = 0; i < d.num_loads; i++) maxPat = std::max(maxPat, d.load_pattern[i]);
  for (int p = 0; p <= maxPat; p++) h->patterns.push_back(nullptr);
  for (int i = 0; i < d.num_sp; i++) {
    if (d.sp_pattern[i] < 0) {
      SP_Constraint *sp = new SP_Constraint(d.sp_node[i], d.sp_dof[i], 0.0, true);
      dom->addSP_Constraint(sp);
    }
  }
  // equalDOF: MP_Constraint with an identity 1x1 constraint matrix
  for (int i = 0; i < d.num_mp; i++) {
    Matrix Ccr(1, 1);
    Ccr(0, 0) = 1.0;
    ID cdof(1), rdof(1);
    cdof(0) = d.mp_dof[i];
    rdof(0) = d.mp_dof[i];
    MP_Constraint *mp = new MP_Constraint(d.mp_retained[i], d.mp_constrained[i], Ccr, cdof, rdof);
    dom->addMP_Constraint(mp);
  }
  return h;
}

void xref_destroy(void *hp) {
  Harness *h = (Harness *)hp;
  if (!h) return;
  // The reference Domain owns a large object graph whose destructors reach
  // code the harness does not link; the process exits soon after, so the
  // objects are left to it.
  delete h;
}

// `recorder Node|EnvelopeNode -file path [-time] [-dT dT] [-precision p]
// -node tags... -dof dofs... disp|vel|accel` on the reference's domain
// (runtime/commands/domain/recorder.cpp: a DataFileStream, NodeData
// DisplTrial / VelocTrial / AccelTrial, relDeltaTTol 1e-5); dofs 0-based.
// The Domain's commit records; xref_close_recorders deletes them (the
// envelope writes its three rows then) and closes the files.
extern "C" int xref_add_node_recorder(void *hp, const char *path, int envelope, int nnodes,
                                      const int *nodes, int ndofs, const int *dofs,
                                      int response, int echo_time, double dT, int precision) {
  Harness *h = (Harness *)hp;
  if (!h || !path || nnodes < 1 || ndofs < 1 || response < 0 || response > 2) return -1;
  ID nid(nnodes), did(ndofs);
  for (int i = 0; i < nnodes; i++) nid(i) = nodes[i];
  for (int i = 0; i < ndofs; i++) did(i) = dofs[i];
  const NodeData flag = response == 0 ? NodeData::DisplTrial
                        : response == 1 ? NodeData::VelocTrial : NodeData::AccelTrial;
  OPS_Stream *out = new DataFileStream(path, openMode::OVERWRITE, 2, 0, false, precision, false);
  Recorder *rec;
  if (envelope)
    rec = new EnvelopeNodeRecorder(did, &nid, flag, -1, *h->domain, *out, dT, 1e-5,
                                   echo_time != 0, nullptr);
  else
    rec = new NodeRecorder(did, &nid, -1, flag, -1, *h->domain, *out, dT, 1e-5,
                           echo_time != 0, nullptr);
  return h->domain->addRecorder(*rec) == 0 ? 0 : -1;
}

extern "C" int xref_close_recorders(void *hp) {
  Harness *h = (Harness *)hp;
  if (!h) return -1;
  h->domain->removeRecorders();
  return 0;
}

// Add load pattern p (its nodal loads and imposed SP values) to the domain.
static void add_pattern(Harness *h, int p) {
  const xg_model_desc &d = h->d;
  if (p < 0 || p >= (int)h->patterns.size() || h->patterns[p] != nullptr) return;
  LoadPattern *lp = new LoadPattern(p + 1);
  lp->setTimeSeries(new LinearSeries());
  h->domain->addLoadPattern(lp);
  h->patterns[p] = lp;
  int tag = 1000000 * (p + 1);
  for (int i = 0; i < d.num_sp; i++) {
    if (d.sp_pattern[i] == p) {
      SP_Constraint *sp = new SP_Constraint(d.sp_node[i], d.sp_dof[i], d.sp_value[i], false);
      h->domain->addSP_Constraint(sp, p + 1);
    }
  }
  for (int i = 0; i < d.num_loads; i++) {
    if (d.load_pattern[i] == p) {
      Vector v(d.ndf);
      for (int j = 0; j < d.ndf; j++) v(j) = d.load_value[(size_t)i * d.ndf + j];
      NodalLoad *nl = new NodalLoad(tag++, d.load_node[i], v);
      h->domain->addNodalLoad(nl, p + 1);
    }
  }
}

// Run one phase of the analysis.  Steps whose global index lies in
// [cap_begin, cap_end) have every solve captured (up to cap_solves solves).
// step_u[num_steps*num_nodes*ndf], step_lambda[num_steps] and
// step_iters[num_steps] receive the committed state after each step.
int xref_run_phase(void *hp, const xg_phase_desc *ph, int cap_begin, int cap_end,
                   int cap_solves, double *step_u, double *step_lambda, int *step_iters) {
  Harness *h = (Harness *)hp;
  const xg_model_desc &d = h->d;
  add_pattern(h, ph->pattern);

  ConvergenceTest *test = nullptr;
  const int print_flag = getenv("XREF_TEST_PRINT") ? 1 : 0;   // the test's own trace
  if (ph->test == XG_TEST_NORM_DISP_INCR)
    test = new CTestNormDispIncr(ph->tol, ph->max_iter, print_flag);
  else
    test = new CTestNormUnbalance(ph->tol, ph->max_iter, print_flag);
  NewtonRaphson *algo = new NewtonRaphson(*test);
  IncrementalIntegrator *integ = nullptr;
  TransientIntegrator *transient = nullptr;
  if (ph->integrator == XG_INT_LOAD_CONTROL)
    integ = new LoadControl(ph->d_lambda, 1, ph->d_lambda, ph->d_lambda);
  else if (ph->integrator == XG_INT_DISP_CONTROL)
    integ = new DisplacementControl(ph->dc_node, ph->dc_dof, ph->dc_incr, h->domain, 1,
                                    ph->dc_incr, ph->dc_incr);
  else if (ph->integrator == XG_INT_NEWMARK) {
    // `integrator Newmark gamma beta`, `rayleigh ...`, and one
    // `pattern UniformExcitation` over a `timeSeries Path -dt` record
    transient = new Newmark(ph->gamma, ph->beta);
    integ = transient;
    if (h->ddm.active) {
      // `sensitivityAlgorithm -computeAtEachStep`
      // (runtime/commands/analysis/sensitivity.cpp:124-139)
      transient->setComputeType(1);
      transient->activateSensitivityKey();
    }
    h->domain->setRayleighDampingFactors(ph->alpha_m, ph->beta_k, ph->beta_k_init,
                                         ph->beta_k_comm);
    if (ph->gm_npts > 0) {
      if (ph->gm_node_record || ph->gm_count > 1) {
        fprintf(stderr, "xref_run_phase: one ground-motion record for all nodes only\n");
        return -1;
      }
      Vector path(ph->gm_npts);
      for (int k = 0; k < ph->gm_npts; k++) path(k) = ph->gm_accel[k];
      PathSeries *series = new PathSeries(1, path, ph->gm_dt);
      GroundMotion *motion = new GroundMotion(nullptr, nullptr, series);
      UniformExcitation *ue = new UniformExcitation(*motion, ph->gm_dof, 900 + ph->pattern);
      h->domain->addLoadPattern(ue);
    }
  } else {
    fprintf(stderr, "xref_run_phase: integrator %d not supported\n", ph->integrator);
    return -1;
  }

  if (!h->model) {
    h->model = new AnalysisModel();
    if (d.handler == XG_HANDLER_TRANSFORMATION)
      h->handler = new TransformationConstraintHandler();
    else
      h->handler = new PlainHandler();
    h->numberer = new DOF_Numberer(*(new RCM(false)));
    h->soe = new CaptureSOE(h);
    h->soe->obs = h->observer;
    h->soe->on_solve = h->on_solve;
    h->soe->on_solve_ctx = h->on_solve_ctx;
  }
  // wiring as BasicAnalysisBuilder::setLinks(STATIC_ANALYSIS)
  h->soe->setLinks(*h->model);
  h->model->setLinks(*h->domain, *h->handler);
  h->numberer->setLinks(*h->model);
  h->handler->setLinks(*h->domain, *h->model, *integ);
  algo->setLinks(*h->model, *integ, *h->soe, test);
  integ->setLinks(*h->model, *h->soe, test);

  // domainChanged (BasicAnalysisBuilder.cpp:225-300)
  h->model->clearAll();
  h->handler->clearAll();
  if (h->handler->handle() < 0) return -2;
  if (h->numberer->numberDOF() < 0) return -3;
  if (h->handler->doneNumberingDOF() < 0) return -3;
  Graph &g = h->model->getDOFGraph();
  if (h->soe->setSize(g) < 0) return -4;
  h->model->clearDOFGraph();
  if (integ->domainChanged() < 0) return -5;
  h->numbered = 1;

  int nu = d.num_nodes * d.ndf;
  Capture &c = h->cap;
  c.cap = cap_solves;
  for (int s = 0; s < ph->num_steps; s++) {
    int gstep = h->totalSteps;
    c.enabled = (gstep >= cap_begin && gstep < cap_end);
    c.step = gstep;
    c.iter = 0;
    auto t0 = clk::now();
    double solve0 = h->soe->solveSeconds;
    const int ns = transient ? transient->newStep(ph->dt)
                             : static_cast<StaticIntegrator *>(integ)->newStep();
    if (ns < 0) return -10 - s;
    int r = algo->solveCurrentStep();
    if (r < 0) {
      fprintf(stderr, "xref_run_phase: step %d failed (%d)\n", gstep, r);
      return -1000 - s;
    }
    if (transient && h->ddm.active) {
      // BasicAnalysisBuilder::analyzeTransient (runtime/runtime/
      // BasicAnalysisBuilder.cpp:502-511): the sensitivities of the
      // converged step before its commit; then dJ/dtheta += 2 w u du/dtheta
      if (transient->computeSensitivities() < 0) return -30;
      Harness::Ddm &dd = h->ddm;
      for (size_t k = 0; k < dd.w.size(); k++) {
        Node *nd = h->nodes[dd.node_index[k]];
        const double u = nd->getTrialDisp()(dd.dof[k]);
        dd.J += dd.w[k] * u * u;
        for (size_t g = 0; g < dd.grad.size(); g++)
          dd.grad[g] += 2.0 * dd.w[k] * u * nd->getDispSensitivity(dd.dof[k] + 1, (int)g);
      }
    }
    if (integ->commit() < 0) return -20;
    double dt = std::chrono::duration<double>(clk::now() - t0).count();
    h->stepSeconds += dt;
    h->elemSeconds += dt - (h->soe->solveSeconds - solve0);
    if (step_u) {
      for (int i = 0; i < d.num_nodes; i++) {
        const Vector &u = h->nodes[i]->getDisp();
        for (int j = 0; j < d.ndf; j++) step_u[(size_t)s * nu + i * d.ndf + j] = u(j);
      }
    }
    if (step_lambda) step_lambda[s] = h->domain->getCurrentTime();
    if (step_iters) step_iters[s] = algo->getNumIterations();
    h->totalSteps++;
  }
  if (ph->load_const) {
    h->domain->setLoadConstant();
    h->domain->setCurrentTime(0.0);
    h->domain->setCommittedTime(0.0);
  }
  return 0;
}

// DDM set-up before the first phase: one Parameter per (element tag,
// name), name 0 "fy", 1 "E", 2 "b" (Steel01), 3 "fc", 4 "epsco", 5 "fcu"
// (Concrete01), reaching every fiber material of the element that has it
// (ForceBeamColumn2d::setParameter -> FiberSection2d::setParameter
// -> the materials' setParameter, ForceBeamColumn2d.cpp:2763-2846,
// FiberSection2d.cpp:877-960), added to the Domain in order (gradient index
// = position); the objective's terms by node tag and 0-based dof.
extern "C" int xref_ddm_setup(void *hp, int nparam, const int *elem_tag, const int *name,
                              int nterm, const int *node_tag, const int *dof,
                              const double *w) {
  Harness *h = (Harness *)hp;
  if (h->soe) return -1;
  static const char *names[6] = {"fy", "E", "b", "fc", "epsco", "fcu"};
  for (int k = 0; k < nparam; k++) {
    Element *el = h->domain->getElement(elem_tag[k]);
    if (!el || name[k] < 0 || name[k] > 5) return -2;
    const char *argv[1] = {names[name[k]]};
    Parameter *p = new Parameter(k + 1, el, argv, 1);
    if (!h->domain->addParameter(p)) return -3;
  }
  Harness::Ddm &dd = h->ddm;
  dd.active = 1;
  dd.grad.assign(nparam, 0.0);
  dd.J = 0.0;
  for (int k = 0; k < nterm; k++) {
    int idx = -1;
    for (size_t i = 0; i < h->nodes.size(); i++)
      if (h->nodes[i]->getTag() == node_tag[k]) idx = (int)i;
    if (idx < 0) return -4;
    dd.node_index.push_back(idx);
    dd.dof.push_back(dof[k]);
    dd.w.push_back(w[k]);
  }
  return 0;
}

extern "C" int xref_ddm_result(void *hp, double *grad, double *J) {
  Harness *h = (Harness *)hp;
  for (size_t g = 0; g < h->ddm.grad.size(); g++) grad[g] = h->ddm.grad[g];
  *J = h->ddm.J;
  return (int)h->ddm.grad.size();
}

// Equation numbers per (node, dof) after the first phase was set up.
int xref_numbering(void *hp, int *eqn, int *num_eqn, int *nnz) {
  Harness *h = (Harness *)hp;
  if (!h->numbered) return -1;
  int ndf = h->d.ndf;
  for (size_t i = 0; i < h->nodes.size(); i++) {
    DOF_Group *g = h->nodes[i]->getDOF_GroupPtr();
    const ID &id = g->getID();
    for (int j = 0; j < ndf; j++) eqn[i * ndf + j] = (j < id.Size()) ? id(j) : -1;
    // TransformationDOF_Group keeps a reduced ID; map it back per dof
    if (id.Size() != ndf) {
      for (int j = 0; j < ndf; j++) eqn[i * ndf + j] = -1;
    }
  }
  *num_eqn = h->soe->gen().n();
  *nnz = h->soe->gen().nz();
  return 0;
}

int xref_pattern(void *hp, int *colstart, int *rowidx) {
  Harness *h = (Harness *)hp;
  GenAccess &g = h->soe->gen();
  memcpy(colstart, g.colStart(), sizeof(int) * (g.n() + 1));
  memcpy(rowidx, g.rows(), sizeof(int) * g.nz());
  return 0;
}

// Feed every LinearSOE call of the analysis also to `soe` (a LinearSOE*)
// and run on_solve(ctx) before each solve.  Before the first phase only.
int xref_set_observer(void *hp, void *soe, void (*on_solve)(void *), void *ctx) {
  Harness *h = (Harness *)hp;
  if (h->soe) return -1;
  h->observer = (LinearSOE *)soe;
  h->on_solve = on_solve;
  h->on_solve_ctx = ctx;
  return 0;
}

// Calls the observer answered with a negative status.
int xref_observer_errors(void *hp) {
  Harness *h = (Harness *)hp;
  return h->soe ? h->soe->obs_errors : 0;
}

int xref_num_captured(void *hp) { return ((Harness *)hp)->cap.count; }

// The reference Domain the harness built (for shims that work on it, before
// the first phase).
extern "C" void *xref_domain(void *hp) { return ((Harness *)hp)->domain; }

// Keep ProfileSPDLinSOE's own profile A at every captured solve as well
// (before the first phase).
extern "C" int xref_capture_profile(void *hp, int on) {
  ((Harness *)hp)->cap.profile = on;
  return 0;
}

// The profile layout (iDiagLoc[n], 1-based as the reference keeps it) and
// size, then the captured profiles [count][size].
extern "C" int xref_profile_layout(void *hp, int *diag_loc, int *size) {
  Harness *h = (Harness *)hp;
  if (!h->soe) return -1;
  const int n = h->soe->getNumEqn();
  const ProfAccess &p = h->soe->profile();
  if (diag_loc) memcpy(diag_loc, p.diagLoc(), sizeof(int) * n);
  if (size) *size = p.psize();
  return 0;
}

extern "C" int xref_captured_profile(void *hp, double *out) {
  Capture &c = ((Harness *)hp)->cap;
  if (out) memcpy(out, c.P.data(), sizeof(double) * c.P.size());
  return (int)c.P.size();
}

int xref_captured(void *hp, int *step, int *iter, double *B, double *A, double *X, double *U) {
  Capture &c = ((Harness *)hp)->cap;
  int n = c.count;
  if (step) memcpy(step, c.stepOf.data(), sizeof(int) * n);
  if (iter) memcpy(iter, c.iterOf.data(), sizeof(int) * n);
  if (B) memcpy(B, c.B.data(), sizeof(double) * c.B.size());
  if (A) memcpy(A, c.A.data(), sizeof(double) * c.A.size());
  if (X) memcpy(X, c.X.data(), sizeof(double) * c.X.size());
  if (U) memcpy(U, c.U.data(), sizeof(double) * c.U.size());
  return n;
}

void xref_times(void *hp, double *elem_s, double *solve_s, double *step_s) {
  Harness *h = (Harness *)hp;
  *elem_s = h->elemSeconds;
  *solve_s = h->soe->solveSeconds;
  *step_s = h->stepSeconds;
}

// Material-point driver: J2 plane strain (dim 2) or 3D (dim 3) through a
// strain path; commit[k] != 0 commits after point k.  stress/tangent out:
// [npts*nstress], [npts*nstress*nstress].
int xref_j2_path(int dim, const double *param, int npts, const double *strain,
                 const int *commit, double *stress, double *tangent) {
  NDMaterial *m;
  int ns;
  if (dim == 2) {
    m = new J2PlaneStrain(1, param[0], param[1], param[2], param[3], param[4], param[5], param[6], param[7]);
    ns = 3;
  } else {
    m = new J2ThreeDimensional(1, param[0], param[1], param[2], param[3], param[4], param[5], param[6], param[7]);
    ns = 6;
  }
  Vector eps(ns);
  for (int k = 0; k < npts; k++) {
    for (int i = 0; i < ns; i++) eps(i) = strain[k * ns + i];
    m->setTrialStrain(eps);
    const Vector &s = m->getStress();
    const Matrix &t = m->getTangent();
    for (int i = 0; i < ns; i++) stress[k * ns + i] = s(i);
    for (int i = 0; i < ns; i++)
      for (int j = 0; j < ns; j++) tangent[(k * ns + i) * ns + j] = t(i, j);
    if (commit[k]) m->commitState();
  }
  delete m;
  return 0;
}

}  // extern "C"

// Domain time (the load factor of LinearSeries patterns) at every captured solve.
extern "C" int xref_captured_lambda(void *hp, double *lam) {
  Capture &c = ((Harness *)hp)->cap;
  memcpy(lam, c.lam.data(), sizeof(double) * c.lam.size());
  return (int)c.lam.size();
}

// Uniaxial material path (Steel02 / Concrete02): stress and tangent at each
// trial strain; commit[k] != 0 commits after point k.
extern "C" int xref_uniaxial_path(int type, const double *param, int npts, const double *strain,
                                  const int *commit, double *stress, double *tangent) {
  UniaxialMaterial *m = make_uniaxial(type, param, 1);
  if (!m) return -1;
  for (int k = 0; k < npts; k++) {
    double s = 0, t = 0;
    m->setTrial(strain[k], s, t);
    stress[k] = s;
    tangent[k] = t;
    if (commit[k]) m->commitState();
  }
  delete m;
  return 0;
}

// Element response at trial displacements U[num_nodes*ndf]: optionally
// Domain::revertToLastCommit first, then Node::setTrialDisp on every node,
// Domain::update, and each element's global tangent and resisting force
// (element order of the description; K[ne*ned*ned] row major, P[ne*ned]).
extern "C" int xref_elem_response(void *hp, const double *U, int revert_first, double *K,
                                  double *P) {
  Harness *h = (Harness *)hp;
  const xg_model_desc &d = h->d;
  if (revert_first && h->domain->revertToLastCommit() < 0) return -1;
  for (int i = 0; i < d.num_nodes; i++) {
    Vector u(d.ndf);
    for (int j = 0; j < d.ndf; j++) u(j) = U[(size_t)i * d.ndf + j];
    h->nodes[i]->setTrialDisp(u);
  }
  if (h->domain->update() < 0) return -2;
  const int ned = nen_of(d.elem_type) * d.ndf;
  for (int e = 0; e < d.num_elems; e++) {
    Element *ele = h->domain->getElement(d.elem_tag[e]);
    const Matrix &k = ele->getTangentStiff();
    const Vector &p = ele->getResistingForce();
    for (int a = 0; a < ned; a++) {
      P[(size_t)e * ned + a] = p(a);
      for (int b = 0; b < ned; b++) K[((size_t)e * ned + a) * ned + b] = k(a, b);
    }
  }
  return 0;
}
