/* The C ABI used from plain C99, as a C or Fortran (iso_c_binding) caller
 * would: only entry points that need no GPU are called. Prints one line per
 * check; exits non-zero on the first failure. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "qcxgpu.h"

static int fail(const char* what) {
  fprintf(stderr, "FAIL %s: %s\n", what, qcx_last_error());
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  if (qcx_version() < 100) return fail("version");
  /* boltz: two fragments 2 eV apart at 3000 K (Fortran order ip(2,1)) */
  double ip[2] = {8.0, 10.0}, w[2];
  if (qcx_boltz(2, 2, 1, 3000.0, ip, w) != 0) return fail("boltz");
  double f = 3000.0 * 3.166808578545117e-06 * 27.21138505, r = exp(-2.0 / f);
  if (fabs(w[0] - 1.0 / (1.0 + r)) > 1e-14 || fabs(w[0] + w[1] - 1.0) > 1e-15) return fail("boltz values");
  /* start files of the fixture ensemble: size query, then the arrays */
  char path[4096];
  int32_t nat = 0, itrj = 0;
  snprintf(path, sizeof(path), "%s/TMP.1/start.xyz", argv[1]);
  if (qcx_read_xyz(path, 0, &nat, NULL, NULL) != 0 || nat < 1) return fail("read_xyz size");
  int32_t* num = malloc(sizeof(int32_t) * nat);
  double* xyz = malloc(sizeof(double) * 3 * nat);
  double* vel = malloc(sizeof(double) * 3 * nat);
  double* velof = malloc(sizeof(double) * nat);
  double eimp = 0.0, tadd = 0.0;
  if (qcx_read_xyz(path, nat, &nat, num, xyz) != 0) return fail("read_xyz");
  snprintf(path, sizeof(path), "%s/TMP.1/qcxms.start", argv[1]);
  if (qcx_read_start(path, nat, &itrj, &eimp, &tadd, vel, velof) != 0 || itrj != 1) return fail("read_start");
  /* a batch call on a NULL handle is rejected on the host */
  if (qcx_batch_set_md_rules(NULL, 2, 250, 100) != -1) return fail("null handle");
  printf("ok nat=%d itrj=%d eimp=%.14e tadd=%.14e Z0=%d\n", (int)nat, (int)itrj, eimp, tadd, (int)num[0]);
  free(num);
  free(xyz);
  free(vel);
  free(velof);
  return 0;
}
