/* Host-only use of the C ABI from C (no GPU needed): the calling pattern of
   the C example in the integration notes -- describe the problem, create a
   plan, size its workspace, read the launch geometry -- and the error
   contract (status code plus thread-local message) for a bad request.
   Prints one line per check; exits non-zero on the first failure. */
#include <stdio.h>
#include <string.h>

#include "pjzfdtd.h"

static int fail(const char* what) {
  char msg[512];
  pjzfdtd_last_error(msg, sizeof msg);
  printf("FAIL %s: %s\n", what, msg);
  return 1;
}

int main(void) {
  enum { X = 64, Y = 48, Z = 32, TT = 40 };
  float kappa[Z * 2], sigma[Z * 2], alpha[Z * 2];
  for (int i = 0; i < Z * 2; ++i) {
    kappa[i] = 1.f;
    sigma[i] = 0.f;
    alpha[i] = 0.f;
  }
  pjzfdtd_problem p;
  memset(&p, 0, sizeof p);
  p.xx = X; p.yy = Y; p.zz = Z;
  p.ox = 2; p.oy = 2; p.oz = 2;
  p.rx = X - 4; p.ry = Y - 4; p.rz = Z - 4;
  p.tt = TT; p.dt = 0.5f; p.pml_lo = 4; p.pml_hi = 4;
  p.src_x0 = 9; p.src_nx = 2; p.src_ny = Y; p.src_nz = Z; p.src_ncols = 2;
  p.out_start = 20; p.out_stop = TT; p.out_step = 5;
  p.out_mode = PJZFDTD_OUT_SNAPSHOTS;

  if (pjzfdtd_abi_version() != PJZFDTD_ABI_VERSION) return fail("abi version");
  printf("ok abi version %d\n", pjzfdtd_abi_version());

  pjzfdtd_plan* plan = NULL;
  if (pjzfdtd_plan_create(&p, kappa, sigma, alpha, NULL, &plan)) return fail("plan");
  size_t ws = 0;
  if (pjzfdtd_plan_workspace_bytes(plan, &ws) || ws == 0) return fail("workspace");
  int32_t ns = 0;
  if (pjzfdtd_plan_num_samples(plan, &ns) || ns != 4) return fail("samples");
  int32_t ty, sx, th, spp, kern, st;
  if (pjzfdtd_plan_launch_config(plan, &ty, &sx, &th, &spp, &kern, &st))
    return fail("launch config");
  if (kern != 2 || spp != 1 || ty <= 0 || th <= 0) return fail("launch values");
  printf("ok plan: workspace %zu bytes, %d samples, kernel %d, tile_y %d, "
         "%d threads, %d steps per pass\n", ws, ns, kern, ty, th, spp);
  pjzfdtd_plan_destroy(plan);

  p.steps_per_pass = 2;  /* two steps per HBM pass on request */
  if (pjzfdtd_plan_create(&p, kappa, sigma, alpha, NULL, &plan)) return fail("plan 2");
  if (pjzfdtd_plan_launch_config(plan, NULL, NULL, NULL, &spp, NULL, NULL) || spp != 2)
    return fail("two-step plan");
  printf("ok two-step plan\n");
  pjzfdtd_plan_destroy(plan);

  p.steps_per_pass = 0;
  p.rx = X + 1;  /* region larger than the domain */
  plan = NULL;
  const int32_t rc = pjzfdtd_plan_create(&p, kappa, sigma, alpha, NULL, &plan);
  char msg[512];
  pjzfdtd_last_error(msg, sizeof msg);
  if (rc != PJZFDTD_ERR_INVALID || plan != NULL || msg[0] == 0) {
    printf("FAIL bad region: rc %d\n", rc);
    return 1;
  }
  printf("ok bad region -> PJZFDTD_ERR_INVALID: %s\n", msg);
  return 0;
}
