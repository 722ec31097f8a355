// CudaLinSOE: the reference's LinearSOE interface over libxara_gpu's
// standalone device system (xg_linsoe_*), the common body of the two
// `system` classes that use it:
//
//   * CudaBJPCGLinSOE (CudaBJPCGLinSOE.h): `system CudaBJPCG <rtol> <maxit>`,
//     SparseGenColLinSOE's assembly and block-Jacobi PCG on the device;
//   * CudaProfileSPDLinSOE (CudaProfileSPDLinSOE.h): `system ProfileSPD` on
//     the device, ProfileSPDLinSOE's assembly and the device LDL'.
//
// Maintainer-side source: it compiles inside the reference's tree, against
// its headers (system_of_eqn/linearSOE/LinearSOE.h, graph/graph/Graph.h,
// matrix/{Matrix,Vector,ID}.h, analysis/model/AnalysisModel.h), and links
// against libxara_gpu.so.  Registered in the `system` command's table
// (runtime/commands/analysis/solver.hpp:113-187):
//
//   * setSize builds the scalar pattern from the DOF graph the way
//     SparseGenColLinSOE::setSize does (sparseGEN/SparseGenColLinSOE.cpp:161-250:
//     each equation's adjacency plus its diagonal, ascending), and the node
//     blocks of the block-Jacobi preconditioner from the AnalysisModel's
//     DOF groups (the contiguous equations of one node);
//   * addA / addB / setB / zeroA / zeroB accumulate on the host in the order
//     the integrator calls them (SparseGenColLinSOE.cpp:262-350 or
//     ProfileSPDLinSOE.cpp:214-410: an equation number outside 0..n-1 is
//     skipped, fact == 0 returns at once), so the assembled values equal
//     the reference's bit for bit;
//   * solve runs on the device and copies X back; a negative return is what
//     NewtonRaphson maps to BadLinearSolve
//     (analysis/algorithm/equiSolnAlgo/NewtonRaphson.cpp:194).
//
// The reference is single-threaded and so is this class: one handle per
// analysis, not reentrant.  sendSelf / recvSelf (parallel channels) are not
// supported and return -1.
#ifndef XARA_CUDA_LINSOE_H
#define XARA_CUDA_LINSOE_H

#include <AnalysisModel.h>
#include <DOF_Group.h>
#include <DOF_GrpIter.h>
#include <Graph.h>
#include <ID.h>
#include <LinearSOE.h>
#include <Matrix.h>
#include <Vector.h>
#include <Vertex.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "xara_gpu.h"

class CudaLinSOE : public LinearSOE {
 public:
  // system: XG_SYSTEM_BJPCG or XG_SYSTEM_PROFILE_SPD (xara_gpu.h)
  CudaLinSOE(int system, double rtol, int maxit, int classTag)
      : LinearSOE(classTag), system_(system), rtol_(rtol), maxit_(maxit) {}
  ~CudaLinSOE() override { xg_linsoe_destroy(h_); }

  int setSize(Graph &graph) override {
    n_ = graph.getNumVertex();
    rowptr_.assign(n_ + 1, 0);
    colidx_.clear();
    for (int i = 0; i < n_; i++) {
      Vertex *v = graph.getVertexPtr(i);
      if (v == nullptr) { n_ = 0; return -1; }     // as SparseGenColLinSOE::setSize
      const ID &adj = v->getAdjacency();
      const size_t row0 = colidx_.size();
      colidx_.push_back(v->getTag());
      for (int k = 0; k < adj.Size(); k++) colidx_.push_back(adj(k));
      std::sort(colidx_.begin() + row0, colidx_.end());
      rowptr_[i + 1] = (int)colidx_.size();
    }
    node_blocks();
    xg_linsoe_destroy(h_);
    h_ = nullptr;
    B_.resize(n_);
    B_.Zero();
    X_.resize(n_);
    X_.Zero();
    const int r = xg_linsoe_create(n_, rowptr_.data(), colidx_.data(),
                                   blk_.empty() ? nullptr : blk_.data(),
                                   blk_.empty() ? 0 : (int)blk_.size() - 1, &h_);
    if (r < 0) return r;
    return xg_linsoe_set_system(h_, system_);
  }
  int getNumEqn() const override { return n_; }

  int addA(const Matrix &m, const ID &id, double fact = 1.0) override {
    const int nd = id.Size();
    if (fact == 0.0 || nd == 0) return 0;
    rm_.resize((size_t)nd * nd);                   // Matrix is column-major
    for (int i = 0; i < nd; i++)
      for (int j = 0; j < nd; j++) rm_[(size_t)i * nd + j] = m(i, j);
    ids_.assign(nd, 0);
    for (int i = 0; i < nd; i++) ids_[i] = id(i);
    return xg_linsoe_add_a(h_, rm_.data(), ids_.data(), nd, fact);
  }
  int addB(const Vector &v, const ID &id, double fact = 1.0) override {
    const int nd = id.Size();
    if (fact == 0.0 || nd == 0) return 0;
    rm_.resize(nd);
    ids_.assign(nd, 0);
    for (int i = 0; i < nd; i++) { rm_[i] = v(i); ids_[i] = id(i); }
    return xg_linsoe_add_b(h_, rm_.data(), ids_.data(), nd, fact);
  }
  int setB(const Vector &v, double fact = 1.0) override {
    if (v.Size() != n_) return -1;
    rm_.resize(n_);
    for (int i = 0; i < n_; i++) rm_[i] = v(i);
    return xg_linsoe_set_b(h_, rm_.data(), fact);
  }
  void zeroA() override { xg_linsoe_zero_a(h_); }
  void zeroB() override { xg_linsoe_zero_b(h_); }

  int solve() override {
    if (n_ == 0) return 0;
    int it = 0;
    double rr = 0.0;
    const int r = xg_linsoe_solve(h_, rtol_, maxit_, &it, &rr);
    xg_linsoe_get_x(h_, &X_(0));
    iters_ = it;
    relres_ = rr;
    return r < 0 ? -1 : 0;
  }

  const Vector &getX() override { return X_; }
  const Vector &getB() override {
    if (n_ > 0) xg_linsoe_get_b(h_, &B_(0));
    return B_;
  }
  double normRHS() override {
    getB();
    double s = 0.0;
    for (int i = 0; i < n_; i++) s += B_(i) * B_(i);
    return std::sqrt(s);
  }
  void setX(int loc, double value) override {
    if (loc >= 0 && loc < n_) X_(loc) = value;
  }
  void setX(const Vector &x) override {
    if (x.Size() == n_) X_ = x;
  }

  int sendSelf(int, Channel &) override { return -1; }
  int recvSelf(int, Channel &, FEM_ObjectBroker &) override { return -1; }

  // the last solve's PCG iterations and relative residual (0 for the LDL')
  int iterations() const { return iters_; }
  double relativeResidual() const { return relres_; }
  // the scalar CSR pattern setSize built, and the assembled values
  const std::vector<int> &rowptr() const { return rowptr_; }
  const std::vector<int> &colidx() const { return colidx_; }
  int values(double *out) const { return xg_linsoe_get_a(h_, out); }
  // preconditioner block starts (empty: point Jacobi)
  const std::vector<int> &blocks() const { return blk_; }

 private:
  // Preconditioner blocks: the equations of one DOF group when they are
  // contiguous, number 1 to 6 and belong to no other group (DOF_Numberer
  // gives a node's free dofs consecutive numbers).  The equations of a group
  // that breaks the rule -- a node tied to another by equalDOF shares the
  // retained node's equation -- and equations of no group are blocks of
  // their own.
  void node_blocks() {
    blk_.clear();
    if (theModel == nullptr || n_ == 0) return;
    std::vector<int> claims(n_, 0);
    std::vector<std::pair<int, int>> runs;     // [lo, hi] of the contiguous groups
    DOF_GrpIter &groups = theModel->getDOFs();
    DOF_Group *g;
    while ((g = groups()) != nullptr) {
      const ID &eq = g->getID();
      int lo = -1, hi = -1, cnt = 0;
      for (int k = 0; k < eq.Size(); k++) {
        const int e = eq(k);
        if (e < 0 || e >= n_) continue;
        claims[e]++;
        lo = (lo < 0 || e < lo) ? e : lo;
        hi = e > hi ? e : hi;
        cnt++;
      }
      if (cnt > 0 && cnt <= 6 && hi - lo + 1 == cnt) runs.emplace_back(lo, hi);
    }
    std::vector<int> len(n_, 0);   // len[lo] > 0: a node block starts at lo
    for (const auto &r : runs) {
      bool own = true;
      for (int e = r.first; e <= r.second; e++) own = own && claims[e] == 1;
      if (own) len[r.first] = r.second - r.first + 1;
    }
    std::vector<int> blk{0};
    for (int e = 0; e < n_;) {
      e += len[e] > 0 ? len[e] : 1;
      blk.push_back(e);
    }
    blk_.swap(blk);
  }

  xg_linsoe *h_ = nullptr;
  int system_;
  double rtol_;
  int maxit_;
  int n_ = 0;
  int iters_ = 0;
  double relres_ = 0.0;
  std::vector<int> rowptr_, colidx_, blk_, ids_;
  std::vector<double> rm_;
  Vector B_, X_;
};

#endif  // XARA_CUDA_LINSOE_H
