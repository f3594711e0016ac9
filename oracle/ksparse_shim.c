/* ksparse_shim.c — test-only bridge to Kundert Sparse 1.3 as compiled from
 * the reference's own sources (src/LinearAlgebraServicesPKG/ksparse).  It
 * mirrors the call sequence of Epetra_CrsKundertSparse.C:66-184: spCreate,
 * spGetElement per CSR entry, spOrderAndFactor, spSolve with 1-based vectors.
 * Used by tests to pin the oracle's sparse LU; never linked by the product. */
#include <stdlib.h>
#include "spmatrix.h"

int ks_solve(int n, const int *row_ptr, const int *col_idx, const double *vals,
             const double *b, double *x) {
  int err = 0;
  char *m = spCreate(n, 0, &err);
  if (err) return -1;
  for (int i = 0; i < n; ++i)
    for (int p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
      double *e = (double *)spGetElement(m, i + 1, col_idx[p] + 1);
      *e += vals[p];
    }
  double *rhs = (double *)malloc(sizeof(double) * (n + 1));
  double *sol = (double *)malloc(sizeof(double) * (n + 1));
  for (int i = 0; i < n; ++i) rhs[i + 1] = b[i];
  /* RelThreshold 1e-3, AbsThreshold 1e-13, DiagPivoting: the defaults of
   * Epetra_CrsKundertSparse.h:130-132 */
  int st = spOrderAndFactor(m, NULL, 1.0e-3, 1.0e-13, 1, 1);
  if (st == 0) {
    spSolve(m, rhs, sol, NULL, NULL);
    for (int i = 0; i < n; ++i) x[i] = sol[i + 1];
  }
  free(rhs); free(sol);
  spDestroy(m);
  return st;
}
