/* Direct linear solve for the reference-as-oracle build (test
 * infrastructure).  It stands in for the reference's lu() entry point
 * (src/sl_lu.c:41, "Solution Algorithm = lu"), which needs the Sparse 1.3
 * library that is absent here.  The MSR system (a = diagonal then
 * off-diagonal values, ija = row pointers then column indices, as built by
 * src/mm_fill_util.c:2865) is copied into a dense band and solved by
 * Gaussian elimination with partial pivoting.  Only the converged Newton
 * solution is compared downstream, so any accurate direct solve serves. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int first_time = 1;

void lu(const int N, const int NExt, const int M, double a[], int ija[], double x[],
        const int factor_flag) {
  (void)NExt;
  (void)M;
  (void)factor_flag;
  int kl = 0, ku = 0;
  for (int i = 0; i < N; i++)
    for (int k = ija[i]; k < ija[i + 1]; k++) {
      int j = ija[k];
      if (j < i && i - j > kl) kl = i - j;
      if (j > i && j - i > ku) ku = j - i;
    }
  /* band storage: row i holds columns [i-kl, i+kl+ku] (fill from pivoting) */
  const int w = 2 * kl + ku + 1;
  double *B = (double *)calloc((size_t)N * (size_t)w, sizeof(double));
  if (!B) {
    fprintf(stderr, "band_lu: cannot allocate %d x %d band\n", N, w);
    abort();
  }
#define BAND(i, j) B[(size_t)(i) * (size_t)w + (size_t)((j) - (i) + kl)]
  for (int i = 0; i < N; i++) {
    BAND(i, i) = a[i];
    for (int k = ija[i]; k < ija[i + 1]; k++) BAND(i, ija[k]) += a[k];
  }
  for (int c = 0; c < N; c++) {
    int last = c + kl < N - 1 ? c + kl : N - 1;
    int p = c;
    double best = fabs(BAND(c, c));
    for (int r = c + 1; r <= last; r++)
      if (fabs(BAND(r, c)) > best) {
        best = fabs(BAND(r, c));
        p = r;
      }
    if (best == 0.0) {
      fprintf(stderr, "band_lu: singular at column %d\n", c);
      abort();
    }
    int cmax = c + kl + ku < N - 1 ? c + kl + ku : N - 1;
    if (p != c) {
      for (int j = c; j <= cmax; j++) {
        double t = BAND(c, j);
        BAND(c, j) = BAND(p, j);
        BAND(p, j) = t;
      }
      double t = x[c];
      x[c] = x[p];
      x[p] = t;
    }
    double piv = BAND(c, c);
    for (int r = c + 1; r <= last; r++) {
      double f = BAND(r, c) / piv;
      if (f == 0.0) continue;
      BAND(r, c) = 0.0;
      for (int j = c + 1; j <= cmax; j++) BAND(r, j) -= f * BAND(c, j);
      x[r] -= f * x[c];
    }
  }
  for (int i = N - 1; i >= 0; i--) {
    int cmax = i + kl + ku < N - 1 ? i + kl + ku : N - 1;
    double s = x[i];
    for (int j = i + 1; j <= cmax; j++) s -= BAND(i, j) * x[j];
    x[i] = s / BAND(i, i);
  }
#undef BAND
  free(B);
}
