/* Host-only use of the C ABI from C (no GPU needed): the calling pattern of
   the C example in the integration notes -- describe the problem, create a
   plan, size its workspace, read the launch geometry, restrict the output
   to monitor boxes, batch plans of different domains -- and the error
   contract (status code plus thread-local message) for bad requests.
   Prints one line per check; exits non-zero on the first failure. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "pjzfdtd.h"

static int fail(const char* what) {
  char msg[512];
  pjzfdtd_last_error(msg, sizeof msg);
  printf("FAIL %s: %s\n", what, msg);
  return 1;
}

static int expect_rc(int32_t got, int32_t want, const char* what) {
  if (got == want) return 0;
  printf("FAIL %s: rc %d, expected %d\n", what, got, want);
  return 1;
}

/* Batches: creation from streamed plans of different domains, the
   workspace they need, refusal of a register-marching plan, and the
   argument checks of a run that happen before any device work. */
static int batch_checks(const pjzfdtd_problem* pa, pjzfdtd_plan* a,
                        const float* kappa, const float* sigma, const float* alpha) {
  pjzfdtd_problem q = *pa;
  q.xx = 40; q.yy = 32; q.zz = 16;
  q.rx = 36; q.ry = 28; q.rz = 12;
  q.src_ny = 32; q.src_nz = 16;
  pjzfdtd_plan* b = NULL;
  if (pjzfdtd_plan_create(&q, kappa, sigma, alpha, NULL, &b)) return fail("plan b");
  q.zz = 6; q.pml_lo = 1; q.pml_hi = 1;
  q.oz = 1; q.rz = 4; q.src_nz = 6;
  pjzfdtd_plan* c = NULL;
  if (pjzfdtd_plan_create(&q, kappa, sigma, alpha, NULL, &c)) return fail("plan c");
  int32_t kern = 0;
  if (pjzfdtd_plan_launch_config(c, NULL, NULL, NULL, NULL, &kern, NULL) || kern != 1)
    return fail("zz 6 takes the register-marching kernel");

  pjzfdtd_batch* bt = NULL;
  pjzfdtd_plan* ac[2] = {a, c};
  if (expect_rc(pjzfdtd_batch_create(ac, 0, &bt), PJZFDTD_ERR_INVALID, "empty batch") ||
      expect_rc(pjzfdtd_batch_create(ac, 2, &bt), PJZFDTD_ERR_UNSUPPORTED,
                "batch with a register-marching plan") || bt != NULL)
    return 1;
  pjzfdtd_plan* ab[2] = {a, b};
  if (pjzfdtd_batch_create(ab, 2, &bt) || bt == NULL) return fail("batch");
  size_t wa = 0, wb = 0, wbt = 0;
  if (pjzfdtd_plan_workspace_bytes(a, &wa) || pjzfdtd_plan_workspace_bytes(b, &wb) ||
      pjzfdtd_batch_workspace_bytes(bt, &wbt) || wbt < wa + wb)
    return fail("batch workspace");
  pjzfdtd_buffers bufs[2];
  memset(bufs, 0, sizeof bufs);
  if (expect_rc(pjzfdtd_batch_run(bt, bufs, NULL, 0, 0, NULL), PJZFDTD_ERR_WORKSPACE,
                "batch without workspace") ||
      expect_rc(pjzfdtd_batch_run(bt, bufs, (void*)(uintptr_t)264, wbt, 0, NULL),
                PJZFDTD_ERR_WORKSPACE, "misaligned batch workspace") ||
      expect_rc(pjzfdtd_batch_run(bt, bufs, (void*)(uintptr_t)4096, wbt, 1, NULL),
                PJZFDTD_ERR_INVALID, "graph capture on the legacy stream"))
    return 1;
  printf("ok batch: %zu workspace bytes for plans of %zu + %zu\n", wbt, wa, wb);
  pjzfdtd_batch_destroy(bt);
  pjzfdtd_plan_destroy(b);
  pjzfdtd_plan_destroy(c);
  return 0;
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
  /* auto: the streamed (2) or, where a compile-time shape applies, the lean
     (3) kernel */
  if (kern < 2 || kern > 3 || spp != 1 || ty <= 0 || th <= 0)
    return fail("launch values");
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

  /* Output size of the whole region, then of two monitor boxes. */
  if (pjzfdtd_plan_create(&p, kappa, sigma, alpha, NULL, &plan)) return fail("plan 3");
  size_t nf = 0;
  if (pjzfdtd_plan_output_floats(plan, &nf) ||
      nf != (size_t)4 * 3 * (X - 4) * (Y - 4) * (Z - 4))
    return fail("region output floats");
  const int32_t boxes[12] = {0, 0, 0, 4, 5, 6, 10, 2, 3, 2, 3, 4};
  if (pjzfdtd_plan_set_monitors(plan, 2, boxes)) return fail("monitors");
  if (pjzfdtd_plan_output_floats(plan, &nf) || nf != (size_t)4 * 3 * (120 + 24))
    return fail("monitor output floats");
  const int32_t outside[6] = {X - 2, 0, 0, 4, 1, 1};
  if (pjzfdtd_plan_set_monitors(plan, 1, outside) != PJZFDTD_ERR_INVALID)
    return fail("monitor outside the domain accepted");
  printf("ok monitors: %zu output floats\n", nf);

  if (batch_checks(&p, plan, kappa, sigma, alpha)) return 1;
  pjzfdtd_plan_destroy(plan);

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
