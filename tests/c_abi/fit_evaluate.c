/* A plain C program against include/polatory_gpu.h: fits 2,000 points (biharmonic3d, degree 1)
 * through pgpu_interpolant_fit, evaluates the interpolant at its own data points and at a few
 * queries, and checks that the data are reproduced within the tolerance. Exit status 0 = ok. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "polatory_gpu.h"

static double next_uniform(unsigned long long* s) {
  *s = *s * 6364136223846793005ULL + 1442695040888963407ULL;
  return (double)(*s >> 11) / 9007199254740992.0;
}

#define CHECK(call)                                                        \
  do {                                                                     \
    int rc_ = (call);                                                      \
    if (rc_ != PGPU_OK) {                                                  \
      fprintf(stderr, "%s failed: %d %s\n", #call, rc_, pgpu_last_error()); \
      return 1;                                                            \
    }                                                                      \
  } while (0)

int main(void) {
  const int64_t n = 2000;
  const double tol = 1e-6;
  double* pts = malloc(sizeof(double) * 3 * n);
  double* vals = malloc(sizeof(double) * n);
  double* out = malloc(sizeof(double) * n);
  unsigned long long s = 12345;
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) pts[3 * i + k] = next_uniform(&s);
    vals[i] = sin(6.283185307179586 * pts[3 * i]) * cos(6.283185307179586 * pts[3 * i + 1]) +
              pts[3 * i + 2] * pts[3 * i + 2];
  }
  pgpu_model model = {0};
  model.n_rbfs = 1;
  model.poly_degree = 1;
  model.rbfs[0].kind = PGPU_RBF_BH3;
  model.rbfs[0].params[0] = 1.0;
  model.rbfs[0].aniso[0] = model.rbfs[0].aniso[4] = model.rbfs[0].aniso[8] = 1.0;
  CHECK(pgpu_model_validate(&model));
  pgpu_interpolant* it = NULL;
  CHECK(pgpu_interpolant_create(&model, &it));
  CHECK(pgpu_interpolant_fit(it, pts, n, NULL, 0, vals, tol, INFINITY, 100, INFINITY, INFINITY,
                             NULL));
  CHECK(pgpu_interpolant_evaluate(it, pts, n, NULL, 0, INFINITY, INFINITY, out));
  double err = 0.0;
  for (int64_t i = 0; i < n; ++i) err = fmax(err, fabs(out[i] - vals[i]));
  pgpu_fit_stats st;
  CHECK(pgpu_interpolant_fit_stats(it, &st));
  int64_t nw = 0;
  CHECK(pgpu_interpolant_num_weights(it, &nw));
  CHECK(pgpu_interpolant_destroy(it));
  printf("iterations %d weights %lld max_error %.3e\n", st.iterations, (long long)nw, err);
  free(pts);
  free(vals);
  free(out);
  return (err <= 2 * tol && nw == n + 4) ? 0 : 2;
}
