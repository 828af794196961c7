/* A C caller of libmpsq's FINUFFT replacements in the form gfortran gives mp_sqom's call
 * (code/src/mp_sqom56.f90:1148): an implicit-interface external, so every argument by
 * reference, opts an unallocated allocatable (NULL) and ier written back; fk column-major,
 * k1 fastest.  Built by tests/test_abi.py against include/mpsq.h (which must compile as C).
 * Prints one line per call: "<case> ier=<n>" and, for a call that succeeded, the modes. */
#include <stdint.h>
#include <stdio.h>

#include "mpsq.h"

static void show(const char* name, int ier, const double* fk, int n) {
  printf("%s ier=%d", name, ier);
  if (ier == 0)
    for (int i = 0; i < 2 * n; ++i) printf(" %.17g", fk[i]);
  printf("\n");
}

int main(void) {
  int64_t nj = 3, ms = 4, mt = 3, mu = 2;
  double x[3] = {0.1, -1.2, 2.5}, y[3] = {-2.0, 0.7, 3.0}, z[3] = {1.5, -0.3, -3.1};
  double c[6] = {1.0, 0.0, 0.5, -0.5, -1.0, 2.0};
  double fk[2 * 4 * 3 * 2];
  int iflag = -1, ier = -7;
  double eps = 1e-9;
  finufft2d1_(&nj, x, y, c, &iflag, &eps, &ms, &mt, fk, NULL, &ier);
  show("2d", ier, fk, (int)(ms * mt));
  ier = -7;
  finufft3d1_(&nj, x, y, z, c, &iflag, &eps, &ms, &mt, &mu, fk, NULL, &ier);
  show("3d", ier, fk, (int)(ms * mt * mu));
  ier = -7;
  finufft2d1_(&nj, x, y, c, NULL, &eps, &ms, &mt, fk, NULL, &ier);
  show("null", ier, fk, 0);
  return 0;
}
