// Test driver: the element-set shim (include/CudaElementSet.h) claiming the
// elements of a Domain built by the reference harness (oracle/_ref), so that
// the reference's own analysis loop runs on the proxies.  Linked here
// against tests/shim/oracle_elemset.c (the C oracle behind the element-set C
// ABI) so the whole loop runs on the host.
#include "CudaElementSet.h"

extern "C" void *xref_domain(void *hp);

namespace {
CudaElementSet *g_set = nullptr;
}

extern "C" {

// Claim the described elements of the harness's Domain (before its first
// phase).  Returns claim()'s status.
int elemset_claim(void *harness, const xg_model_desc *desc) {
  Domain *d = static_cast<Domain *>(xref_domain(harness));
  if (d == nullptr || desc == nullptr) return -10;
  delete g_set;
  g_set = new CudaElementSet();
  return g_set->claim(*d, *desc);
}

// Forwarded calls so far: device updates, commits, reverts.
void elemset_counts(long *updates, long *commits, long *reverts) {
  *updates = g_set ? g_set->updates() : 0;
  *commits = g_set ? g_set->commits() : 0;
  *reverts = g_set ? g_set->reverts() : 0;
}

// The class of the element the Domain holds under tag (a proxy after a
// claim), copied into out.
int elemset_class_of(void *harness, int tag, char *out, int cap) {
  Domain *d = static_cast<Domain *>(xref_domain(harness));
  Element *e = d ? d->getElement(tag) : nullptr;
  if (e == nullptr || cap < 1) return -1;
  strncpy(out, e->getClassType(), cap - 1);
  out[cap - 1] = 0;
  return 0;
}

}  // extern "C"
