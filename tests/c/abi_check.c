/* A plain C11 caller of the C ABI (include/sfd.h), as a C, cgo or FFI user
 * would write it.  Without touching a device it checks the defaults and that
 * bad arguments come back as SFD_ERR_INVALID with a message:
 *   abi_check    prints "ok" and exits 0, or prints the first mismatch and exits 1 */
#include <stdio.h>
#include <string.h>

#include "sfd.h"

static int fail(const char* what) {
  printf("mismatch: %s\n", what);
  return 1;
}

int main(void) {
  sfd_options o;
  sfd_default_options(&o);
  if (o.precision != SFD_PRECISION_MIXED || o.use_graphs != 1 || o.refactor_lag != 0) return fail("default options");
  if (o.extra_iters != 2 || o.refine_tol != 1e-10) return fail("default refinement options");
  sfd_problem p;
  sfd_default_problem(&p);
  if (p.physics != SFD_WATER || p.gravity != 1.0) return fail("default problem");
  sfd_engine* e = NULL;
  const int n64[1] = {64};
  o.extra_iters = 5;
  if (sfd_create(n64, 1, &p, 1, &o, &e) != SFD_ERR_INVALID || e != NULL) return fail("extra_iters > 4 refused");
  o.extra_iters = 2;
  if (sfd_create(NULL, 1, &p, 1, &o, &e) != SFD_ERR_INVALID || e != NULL) return fail("null sizes refused");
  if (strlen(sfd_last_error()) == 0) return fail("error message set");
  if (sfd_rk4_steps(NULL, 0.01, 1) != SFD_ERR_INVALID) return fail("null engine refused");
  if (sfd_set_default_precision(7) != SFD_ERR_INVALID) return fail("unknown precision refused");
  double x[256] = {0}, y[256] = {0}, phi[256] = {0};
  if (calculatePerturbedStates256(x, y, phi, NULL, 1.0, 0.0, 0.0, 1.0, 1e-6) != SFD_ERR_INVALID)
    return fail("null output refused");
  if (calculateRHS256FromFile(NULL, "out.h5", 1e-6, 145.0, 0.0, 1e-8) != SFD_ERR_INVALID)
    return fail("null file name refused");
  printf("ok\n");
  return 0;
}
