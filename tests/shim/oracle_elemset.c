/* Test double of the element-set entry points of libxara_gpu.so
 * (include/xara_gpu.h: xg_model_create / destroy, xg_elemset_set_trial_disp,
 * xg_elemset_update, xg_elemset_element_matrices, xg_elemset_commit /
 * revert / revert_to_start, xg_last_error) computed on the host by the C
 * oracle (oracle/xara_oracle.c), so that the element-set shim
 * (include/CudaElementSet.h) can run inside the reference's own analysis
 * loop on a machine without a GPU.  Every call is logged (one letter each:
 * M create, T trial displacements, U update, K element matrices, C commit,
 * R revert, S revert to start) for the test to check the order in which the
 * shim forwards the Domain's calls.  Test infrastructure only. */
#include <stdlib.h>
#include <string.h>

#include "xara_gpu.h"

typedef struct xo_model xo_model;
xo_model *xo_create(const xg_model_desc *desc);
void xo_destroy(xo_model *m);
int xo_elem_state(xo_model *m, const double *U, double *vals, double *resid);
void xo_commit(xo_model *m);
void xo_revert(xo_model *m);
void xo_keep_element_matrices(xo_model *m, double *K, double *P);

struct xg_model {
  xo_model *o;
  int nu, ne, ned;
  double *U, *K, *P;
};

static char g_log[1 << 16];
static int g_nlog = 0;

static void logc(char c) {
  if (g_nlog < (int)sizeof g_log - 1) g_log[g_nlog++] = c;
  g_log[g_nlog] = 0;
}

/* The call log so far (reset by oelem_log_reset). */
const char *oelem_log(void) { return g_log; }
void oelem_log_reset(void) { g_nlog = 0; g_log[0] = 0; }

const char *xg_last_error(void) { return ""; }

int xg_model_create(const xg_model_desc *desc, xg_model **out) {
  if (!desc || !out) return XG_EINVAL;
  xg_model *m = (xg_model *)calloc(1, sizeof *m);
  m->o = xo_create(desc);
  if (!m->o) { free(m); return XG_EINVAL; }
  const int nen = desc->elem_type == XG_ELE_QUAD ? 4 : desc->elem_type == XG_ELE_BRICK ? 8 : 2;
  m->nu = desc->num_nodes * desc->ndf;
  m->ne = desc->num_elems;
  m->ned = nen * desc->ndf;
  m->U = (double *)calloc(m->nu, sizeof(double));
  m->K = (double *)calloc((size_t)m->ne * m->ned * m->ned, sizeof(double));
  m->P = (double *)calloc((size_t)m->ne * m->ned, sizeof(double));
  xo_keep_element_matrices(m->o, m->K, m->P);
  logc('M');
  *out = m;
  return 0;
}

int xg_model_destroy(xg_model *m) {
  if (!m) return 0;
  xo_destroy(m->o);
  free(m->U); free(m->K); free(m->P); free(m);
  return 0;
}

int xg_elemset_set_trial_disp(xg_model *m, const double *u) {
  if (!m || !u) return XG_EINVAL;
  memcpy(m->U, u, sizeof(double) * m->nu);
  logc('T');
  return 0;
}

int xg_elemset_update(xg_model *m, double *csr_vals, double *resid) {
  if (!m) return XG_EINVAL;
  logc('U');
  return xo_elem_state(m->o, m->U, csr_vals, resid);
}

int xg_elemset_element_matrices(const xg_model *m, double *K, double *P) {
  if (!m) return XG_EINVAL;
  if (K) memcpy(K, m->K, sizeof(double) * (size_t)m->ne * m->ned * m->ned);
  if (P) memcpy(P, m->P, sizeof(double) * (size_t)m->ne * m->ned);
  logc('K');
  return 0;
}

int xg_elemset_commit(xg_model *m) {
  if (!m) return XG_EINVAL;
  xo_commit(m->o);
  logc('C');
  return 0;
}

int xg_elemset_revert(xg_model *m) {
  if (!m) return XG_EINVAL;
  xo_revert(m->o);
  logc('R');
  return 0;
}

int xg_elemset_revert_to_start(xg_model *m) {
  (void)m;
  logc('S');
  return XG_EINVAL;   /* the oracle keeps no initial state; no test reverts to start */
}
