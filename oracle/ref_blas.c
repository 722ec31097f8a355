/*
 * ref_blas.c -- test infrastructure: the few Fortran BLAS/LAPACK entry points
 * the reference's Matrix/MatrixND classes call (dgemv, dgemm, dgesv, dgetrf,
 * dgetri), written as plain column-major loops with the reference BLAS /
 * LAPACK semantics.  Linked only into oracle/_ref/libxara_ref.so; the image
 * has no system BLAS.
 */
#include <math.h>
#include <stddef.h>

static int lsame(const char *c, char u) { return *c == u || *c == (char)(u + 32); }

void dgemv_(const char *trans, const int *m, const int *n, const double *alpha,
            const double *A, const int *lda, const double *x, const int *incx,
            const double *beta, double *y, const int *incy) {
  const int M = *m, N = *n, ld = *lda, ix = *incx, iy = *incy;
  const int leny = lsame(trans, 'N') ? M : N, lenx = lsame(trans, 'N') ? N : M;
  int ky = iy > 0 ? 0 : -(leny - 1) * iy, kx = ix > 0 ? 0 : -(lenx - 1) * ix;
  for (int i = 0; i < leny; i++) {
    double *yi = y + ky + i * iy;
    *yi = (*beta == 0.0) ? 0.0 : *beta * *yi;
  }
  if (*alpha == 0.0) return;
  if (lsame(trans, 'N')) {
    for (int j = 0; j < N; j++) {
      double t = *alpha * x[kx + j * ix];
      for (int i = 0; i < M; i++) y[ky + i * iy] += t * A[i + (size_t)j * ld];
    }
  } else {
    for (int j = 0; j < N; j++) {
      double t = 0.0;
      for (int i = 0; i < M; i++) t += A[i + (size_t)j * ld] * x[kx + i * ix];
      y[ky + j * iy] += *alpha * t;
    }
  }
}

void dgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k,
            const double *alpha, const double *A, const int *lda, const double *B,
            const int *ldb, const double *beta, double *Cm, const int *ldc) {
  const int M = *m, N = *n, K = *k;
  const int nta = lsame(ta, 'N'), ntb = lsame(tb, 'N');
  for (int j = 0; j < N; j++)
    for (int i = 0; i < M; i++) {
      double t = 0.0;
      for (int l = 0; l < K; l++) {
        double a = nta ? A[i + (size_t)l * *lda] : A[l + (size_t)i * *lda];
        double b = ntb ? B[l + (size_t)j * *ldb] : B[j + (size_t)l * *ldb];
        t += a * b;
      }
      double *c = Cm + i + (size_t)j * *ldc;
      *c = (*beta == 0.0 ? 0.0 : *beta * *c) + *alpha * t;
    }
}

void dgetrf_(const int *m, const int *n, double *A, const int *lda, int *ipiv, int *info) {
  const int M = *m, N = *n, ld = *lda, mn = M < N ? M : N;
  *info = 0;
  for (int j = 0; j < mn; j++) {
    int p = j;
    for (int i = j + 1; i < M; i++)
      if (fabs(A[i + (size_t)j * ld]) > fabs(A[p + (size_t)j * ld])) p = i;
    ipiv[j] = p + 1;
    if (A[p + (size_t)j * ld] == 0.0) {
      if (*info == 0) *info = j + 1;
      continue;
    }
    if (p != j)
      for (int c = 0; c < N; c++) {
        double t = A[j + (size_t)c * ld];
        A[j + (size_t)c * ld] = A[p + (size_t)c * ld];
        A[p + (size_t)c * ld] = t;
      }
    double inv = 1.0 / A[j + (size_t)j * ld];
    for (int i = j + 1; i < M; i++) A[i + (size_t)j * ld] *= inv;
    for (int c = j + 1; c < N; c++) {
      double t = A[j + (size_t)c * ld];
      for (int i = j + 1; i < M; i++) A[i + (size_t)c * ld] -= A[i + (size_t)j * ld] * t;
    }
  }
}

static void getrs(int n, const double *A, int ld, const int *ipiv, double *b) {
  for (int i = 0; i < n; i++) {
    int p = ipiv[i] - 1;
    if (p != i) { double t = b[i]; b[i] = b[p]; b[p] = t; }
  }
  for (int i = 0; i < n; i++)
    for (int k = 0; k < i; k++) b[i] -= A[i + (size_t)k * ld] * b[k];
  for (int i = n - 1; i >= 0; i--) {
    for (int k = i + 1; k < n; k++) b[i] -= A[i + (size_t)k * ld] * b[k];
    b[i] /= A[i + (size_t)i * ld];
  }
}

void dgesv_(const int *n, const int *nrhs, double *A, const int *lda, int *ipiv, double *B,
            const int *ldb, int *info) {
  dgetrf_(n, n, A, lda, ipiv, info);
  if (*info) return;
  for (int r = 0; r < *nrhs; r++) getrs(*n, A, *lda, ipiv, B + (size_t)r * *ldb);
}

void dgetri_(const int *n, double *A, const int *lda, const int *ipiv, double *work,
             const int *lwork, int *info) {
  const int N = *n, ld = *lda;
  *info = 0;
  if (*lwork < N * N) {   /* workspace: an N x N copy */
    *info = -7;
    return;
  }
  for (int j = 0; j < N; j++) {
    double *col = work + (size_t)j * N;
    for (int i = 0; i < N; i++) col[i] = (i == j) ? 1.0 : 0.0;
    getrs(N, A, ld, ipiv, col);
  }
  for (int j = 0; j < N; j++)
    for (int i = 0; i < N; i++) A[i + (size_t)j * ld] = work[i + (size_t)j * N];
}
