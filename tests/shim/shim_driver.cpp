// Test driver: the `system` shims (include/CudaBJPCGLinSOE.h,
// include/CudaProfileSPDLinSOE.h) attached to the reference's own analysis
// loop in oracle/_ref/libxara_ref.so.
//
// The harness feeds every LinearSOE call of the analysis (setLinks, setSize,
// zeroA/zeroB, FE_Element's addA/addB through the integrator, setB) to the
// shim as well as to the reference's SparseGenColLinSOE; before each solve
// this driver copies the shim's assembled CSR values and right-hand side,
// for the test to compare with the reference's.  Host work only: the shim's
// device solve is never called here.
#include <memory>
#include <vector>

#include "CudaBJPCGLinSOE.h"
#include "CudaProfileSPDLinSOE.h"

extern "C" int xref_set_observer(void *hp, void *soe, void (*on_solve)(void *), void *ctx);

namespace {

struct Record {
  std::unique_ptr<CudaLinSOE> soe;
  int cap = 0;
  int count = 0;
  std::vector<double> A, B;
};

void on_solve(void *ctx) {
  Record *r = static_cast<Record *>(ctx);
  if (r->count >= r->cap) return;
  const size_t nnz = r->soe->colidx().size();
  const size_t off = r->A.size();
  r->A.resize(off + nnz);
  r->soe->values(r->A.data() + off);
  const Vector &b = r->soe->getB();
  for (int i = 0; i < b.Size(); i++) r->B.push_back(b(i));
  r->count++;
}

}  // namespace

extern "C" {

// system: XG_SYSTEM_BJPCG or XG_SYSTEM_PROFILE_SPD
void *shim_attach(void *harness, int cap, int system) {
  Record *r = new Record();
  r->cap = cap;
  if (system == XG_SYSTEM_PROFILE_SPD)
    r->soe.reset(new CudaProfileSPDLinSOE());
  else
    r->soe.reset(new CudaBJPCGLinSOE());
  if (xref_set_observer(harness, r->soe.get(), on_solve, r) < 0) {
    delete r;
    return nullptr;
  }
  return r;
}

void shim_free(void *rp) { delete static_cast<Record *>(rp); }

int shim_sizes(void *rp, int *neq, int *nnz, int *nblk, int *count) {
  Record *r = static_cast<Record *>(rp);
  *neq = r->soe->getNumEqn();
  *nnz = (int)r->soe->colidx().size();
  *nblk = r->soe->blocks().empty() ? 0 : (int)r->soe->blocks().size() - 1;
  *count = r->count;
  return 0;
}

int shim_pattern(void *rp, int *rowptr, int *colidx, int *blocks) {
  Record *r = static_cast<Record *>(rp);
  const auto &rp_ = r->soe->rowptr();
  const auto &ci = r->soe->colidx();
  const auto &bk = r->soe->blocks();
  for (size_t i = 0; i < rp_.size(); i++) rowptr[i] = rp_[i];
  for (size_t i = 0; i < ci.size(); i++) colidx[i] = ci[i];
  for (size_t i = 0; i < bk.size(); i++) blocks[i] = bk[i];
  return 0;
}

int shim_captured(void *rp, double *A, double *B) {
  Record *r = static_cast<Record *>(rp);
  for (size_t i = 0; i < r->A.size(); i++) A[i] = r->A[i];
  for (size_t i = 0; i < r->B.size(); i++) B[i] = r->B[i];
  return r->count;
}

}  // extern "C"
