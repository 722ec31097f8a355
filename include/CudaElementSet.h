// CudaElementSet: the element loop of a reference Domain on the device.
//
// Maintainer-side source, like CudaLinSOE.h: it compiles inside the
// reference's tree against its headers (element/Element.h,
// domain/domain/Domain.h, domain/node/Node.h, matrix/{Matrix,Vector,ID}.h)
// and links against libxara_gpu.so.  It replaces, for the elements the
// device path covers (FourNodeQuad, Brick, ForceBeamColumn2d/3d; one element
// type per set), the per-element virtual calls of the reference's analysis:
//
//   * claim(domain, desc) is called where BasicAnalysisBuilder::domainChanged
//     (runtime/runtime/BasicAnalysisBuilder.cpp:225-300) would build the
//     FE_Elements.  The description is the one the modelling commands built
//     the Domain from (xg_model_desc: nodes, elements, material and section
//     tables).  Every described element must be in the Domain with the
//     class the description names (Element::getClassType), the same node
//     tags and nodes at the described coordinates; each one is then taken
//     out of the Domain (kept by the set) and a CudaElementProxy with the
//     same tag and nodes put in its place.
//   * Domain::update (domain/domain/Domain.cpp:1988-2006) calls update() on
//     every element in tag order.  The first proxy's update gathers the
//     nodes' trial displacements (Node::getTrialDisp), and runs the state
//     determination of every claimed element at once
//     (xg_elemset_set_trial_disp + xg_elemset_update), then reads back every
//     element's tangent and resisting force (xg_elemset_element_matrices);
//     the other proxies' updates find their results there.
//   * Domain::commit and Domain::revertToLastCommit (Domain.cpp:1893-1960)
//     call commitState / revertToLastCommit on every element: the first
//     proxy forwards them once to xg_elemset_commit / xg_elemset_revert.
//   * FE_Element (analysis/fe_ele/FE_Element.cpp:266-430) then assembles
//     the proxies' getTangentStiff / getResistingForce into any LinearSOE,
//     exactly as it assembles the reference's own elements; getInitialStiff
//     is the tangent of the first state determination (at the Domain's
//     displacements when claimed: zero for a fresh model), so Rayleigh
//     damping on the initial stiffness works too (Element::getDamp).
//   * getResponse("force" | "forces" | "globalForce" | "globalForces") is
//     the element's resisting force.
//
// The reference is single-threaded and so is this set: one set per Domain,
// not reentrant.  The proxies hold no state of their own; sendSelf /
// recvSelf (parallel channels) return -1.
#ifndef XARA_CUDA_ELEMENT_SET_H
#define XARA_CUDA_ELEMENT_SET_H

#include <Domain.h>
#include <Element.h>
#include <ElementResponse.h>
#include <ID.h>
#include <Information.h>
#include <Matrix.h>
#include <Node.h>
#include <OPS_Stream.h>
#include <Vector.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "xara_gpu.h"

class CudaElementSet;

class CudaElementProxy : public Element {
 public:
  CudaElementProxy(int tag, const ID &nodes, int index, int ned, CudaElementSet &set)
      : Element(tag, 0), nodes_(nodes), ptrs_(nodes.Size(), nullptr), index_(index),
        ned_(ned), set_(set) {}

  const char *getClassType() const { return "CudaElementProxy"; }
  int getNumExternalNodes() const override { return nodes_.Size(); }
  const ID &getExternalNodes() override { return nodes_; }
  Node **getNodePtrs() override { return ptrs_.data(); }
  int getNumDOF() override { return ned_; }
  void setDomain(Domain *d) override {
    for (int a = 0; a < nodes_.Size(); a++) ptrs_[a] = d ? d->getNode(nodes_(a)) : nullptr;
    DomainComponent::setDomain(d);
  }

  inline int update() override;
  inline int commitState() override;
  inline int revertToLastCommit() override;
  inline int revertToStart() override;
  inline const Matrix &getTangentStiff() override;
  inline const Matrix &getInitialStiff() override;
  inline const Vector &getResistingForce() override;
  // the resisting force with the Rayleigh damping forces, as the claimed
  // elements add them (e.g. ForceBeamColumn2d.cpp:1337-1366; the elements of
  // the device path carry no element mass)
  const Vector &getResistingForceIncInertia() override {
    const Vector &p = this->getResistingForce();
    if (alphaM == 0.0 && betaK == 0.0 && betaK0 == 0.0 && betaKc == 0.0) return p;
    inertia_ = p;
    inertia_ += this->getRayleighDampingForces();
    return inertia_;
  }

  int sendSelf(int, Channel &) override { return -1; }
  int recvSelf(int, Channel &, FEM_ObjectBroker &) override { return -1; }
  void Print(OPS_Stream &s, int = 0) override {
    s << "CudaElementProxy " << this->getTag() << " (element " << index_
      << " of a device element set)\n";
  }
  Response *setResponse(const char **argv, int argc, OPS_Stream &s) override {
    if (argc >= 1 && (strcmp(argv[0], "force") == 0 || strcmp(argv[0], "forces") == 0 ||
                      strcmp(argv[0], "globalForce") == 0 ||
                      strcmp(argv[0], "globalForces") == 0))
      return new ElementResponse(this, 1, Vector(ned_));
    return Element::setResponse(argv, argc, s);
  }
  int getResponse(int id, Information &info) override {
    if (id == 1) return info.setVector(this->getResistingForce());
    return Element::getResponse(id, info);
  }

 private:
  ID nodes_;
  std::vector<Node *> ptrs_;
  Vector inertia_;
  int index_, ned_;
  CudaElementSet &set_;
};

class CudaElementSet {
 public:
  CudaElementSet() = default;
  CudaElementSet(const CudaElementSet &) = delete;
  CudaElementSet &operator=(const CudaElementSet &) = delete;
  ~CudaElementSet() {
    if (m_) xg_model_destroy(m_);
  }

  // Claim the described elements of the domain (see the file comment).
  // Returns 0, or < 0 with nothing changed in the domain when an element is
  // missing, of another class, on other nodes, or the device model cannot
  // be built (xg_last_error() tells).
  int claim(Domain &domain, const xg_model_desc &desc) {
    if (m_ != nullptr) return -1;
    const char *cls = class_name(desc.elem_type);
    if (cls == nullptr) return -1;
    nen_ = desc.elem_type == XG_ELE_QUAD ? 4 : desc.elem_type == XG_ELE_BRICK ? 8 : 2;
    ndf_ = desc.ndf;
    ned_ = nen_ * ndf_;
    ne_ = desc.num_elems;
    nn_ = desc.num_nodes;
    // the nodes of the description, at its coordinates
    nodes_.assign(nn_, nullptr);
    for (int i = 0; i < nn_; i++) {
      Node *nd = domain.getNode(desc.node_tag[i]);
      if (nd == nullptr || nd->getNumberDOF() != ndf_) return -2;
      const Vector &x = nd->getCrds();
      if (x.Size() != desc.ndm) return -2;
      for (int k = 0; k < desc.ndm; k++) {
        const double want = desc.node_crd[(size_t)i * desc.ndm + k];
        if (std::fabs(x(k) - want) > 1e-12 * (1.0 + std::fabs(want))) return -2;
      }
      nodes_[i] = nd;
    }
    // the elements: class and nodes
    for (int e = 0; e < ne_; e++) {
      Element *el = domain.getElement(desc.elem_tag[e]);
      if (el == nullptr || strcmp(el->getClassType(), cls) != 0) return -3;
      const ID &c = el->getExternalNodes();
      if (c.Size() != nen_) return -3;
      for (int a = 0; a < nen_; a++)
        if (c(a) != desc.elem_conn[(size_t)e * nen_ + a]) return -3;
    }
    if (xg_model_create(&desc, &m_) < 0) {
      m_ = nullptr;
      return -4;
    }
    U_.assign((size_t)nn_ * ndf_, 0.0);
    K_.assign((size_t)ne_ * ned_ * ned_, 0.0);
    P_.assign((size_t)ne_ * ned_, 0.0);
    // the first state determination, at the Domain's displacements: its
    // tangents are the initial stiffness
    if (device_update() < 0) return -4;
    K0_ = K_;
    for (int e = 0; e < ne_; e++) {
      Element *el = domain.removeElement(desc.elem_tag[e]);
      originals_.emplace_back(el);
      const ID &c = el->getExternalNodes();
      auto *proxy = new CudaElementProxy(desc.elem_tag[e], c, e, ned_, *this);
      if (!domain.addElement(proxy)) return -5;   // Domain::addElement runs update()
    }
    K_matrix_ = Matrix(ned_, ned_);
    P_vector_ = Vector(ned_);
    return 0;
  }

  int num_elements() const { return ne_; }
  xg_model *model() const { return m_; }
  // counts of the forwarded calls, for checks
  long updates() const { return n_update_; }
  long commits() const { return n_commit_; }
  long reverts() const { return n_revert_; }

  // ---- called by the proxies ----
  int on_update(int index) { return index == 0 ? device_update() : 0; }
  int on_commit(int index) {
    if (index != 0) return 0;
    n_commit_++;
    return xg_elemset_commit(m_) < 0 ? -1 : 0;
  }
  int on_revert(int index) {
    if (index != 0) return 0;
    n_revert_++;
    return xg_elemset_revert(m_) < 0 ? -1 : 0;
  }
  int on_revert_to_start(int index) {
    if (index != 0) return 0;
    return xg_elemset_revert_to_start(m_) < 0 ? -1 : 0;
  }
  const Matrix &tangent(int index) { return fill(K_, index); }
  const Matrix &initial(int index) { return fill(K0_, index); }
  const Vector &force(int index) {
    for (int i = 0; i < ned_; i++) P_vector_(i) = P_[(size_t)index * ned_ + i];
    return P_vector_;
  }

 private:
  static const char *class_name(int type) {
    switch (type) {
      case XG_ELE_QUAD: return "FourNodeQuad";
      case XG_ELE_BRICK: return "Brick";
      case XG_ELE_FBC2D: return "ForceBeamColumn2d";
      case XG_ELE_FBC3D: return "ForceBeamColumn3d";
    }
    return nullptr;
  }

  // Domain::update's work for every claimed element at once.
  int device_update() {
    n_update_++;
    for (int i = 0; i < nn_; i++) {
      const Vector &u = nodes_[i]->getTrialDisp();
      for (int j = 0; j < ndf_; j++) U_[(size_t)i * ndf_ + j] = u(j);
    }
    if (xg_elemset_set_trial_disp(m_, U_.data()) < 0) return -1;
    // a negative count of failed elements is passed on, as Domain::update
    // passes on an element's failure
    const int r = xg_elemset_update(m_, nullptr, nullptr);
    if (xg_elemset_element_matrices(m_, K_.data(), P_.data()) < 0) return -1;
    return r < 0 ? -1 : 0;
  }

  const Matrix &fill(const std::vector<double> &src, int index) {
    const double *k = src.data() + (size_t)index * ned_ * ned_;
    for (int i = 0; i < ned_; i++)
      for (int j = 0; j < ned_; j++) K_matrix_(i, j) = k[(size_t)i * ned_ + j];
    return K_matrix_;
  }

  xg_model *m_ = nullptr;
  int ne_ = 0, nn_ = 0, nen_ = 0, ndf_ = 0, ned_ = 0;
  std::vector<Node *> nodes_;
  std::vector<double> U_, K_, K0_, P_;
  std::vector<std::unique_ptr<Element>> originals_;
  Matrix K_matrix_;
  Vector P_vector_;
  long n_update_ = 0, n_commit_ = 0, n_revert_ = 0;
};

inline int CudaElementProxy::update() { return set_.on_update(index_); }
inline int CudaElementProxy::commitState() {
  Element::commitState();              // keeps Kc for betaKc damping
  return set_.on_commit(index_);
}
inline int CudaElementProxy::revertToLastCommit() { return set_.on_revert(index_); }
inline int CudaElementProxy::revertToStart() { return set_.on_revert_to_start(index_); }
inline const Matrix &CudaElementProxy::getTangentStiff() { return set_.tangent(index_); }
inline const Matrix &CudaElementProxy::getInitialStiff() { return set_.initial(index_); }
inline const Vector &CudaElementProxy::getResistingForce() { return set_.force(index_); }

#endif  // XARA_CUDA_ELEMENT_SET_H
