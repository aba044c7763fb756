// Host side of the pjzfdtd C ABI (include/pjzfdtd.h): plan validation,
// CPML coefficient set-up, workspace layout and the time loop that launches
// the sm_103a step kernels.
//
// Replaces the fdtdz engine call of src/pjz/_field.py:254-269 and, in
// PHASORS mode, the pinv projection of src/pjz/_field.py:271-279 too.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/pjzfdtd.h"
// This translation unit defines the small set-up kernels and the
// register-marching step kernel; the streamed kernels live in kern_*.cu.
#define PJZ_HOST_KERNELS
#include "step_kernel.cuh"
#include "stream_kernel.cuh"
#include "stream2_kernel.cuh"
#include "lean_kernel.cuh"
#include "lean2_kernel.cuh"
#include "record_kernel.cuh"
#include "smatrix_kernel.cuh"
#include "kernel_table.cuh"

using namespace pjzfdtd;

namespace {

thread_local char g_err[512] = "";
thread_local int32_t g_err_code = PJZFDTD_OK;

int32_t fail(int32_t code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  g_err_code = code;
  return code;
}

#define CUDA_TRY(expr)                                                   \
  do {                                                                   \
    cudaError_t e_ = (expr);                                             \
    if (e_ != cudaSuccess)                                               \
      return fail(PJZFDTD_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_)); \
  } while (0)

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

}  // namespace

// The resolved launch geometry of a plan (the fields the resolvers set).
struct LaunchState {
  int tile_y, seg_x, threads, steps_per_pass, kernel, stages, threads2, stages2,
      src_ring, src_rows;
  size_t smem, smem2;
};

struct pjzfdtd_plan {
  pjzfdtd_problem p;
  int ns = 0;
  int P = 0;
  long long N = 0;
  std::vector<float> zc;       // [6][Z]
  std::vector<float> weights;  // [rows][ns]
  // Resolved launch geometry.
  int tile_y = 0, seg_x = 0, threads = 0, steps_per_pass = 1;
  int kernel = 1;   // 1 register-marching, 2 bulk-copy streamed, 3 lean streamed
  int esz = 4;      // bytes per stored state value (4 FP32, 2 binary16)
  int stages = 0;   // streamed ring depth
  size_t smem = 0;  // dynamic shared memory per CTA
  // Two-step kernel (steps_per_pass == 2): CTA size, ring depths (ring A in
  // the low byte, ring B above) and shared memory; same tile as above.
  int threads2 = 0, stages2 = 0;
  size_t smem2 = 0;
  int cur = 0;      // state buffer (0: A, 1: B) holding the current step
  // Ring-carried source rows (single-step kernel): floats per ring slot
  // (0: the source is read from global memory) and rows per block.
  int src_ring = 0, src_rows = 0;
  // Recorded boxes (x0, y0, z0, nx, ny, nz) and their offsets in `out`.
  std::vector<std::array<int32_t, 6>> boxes;
  std::vector<size_t> box_off;
  size_t out_floats = 0;
  // Workspace layout (byte offsets).
  size_t off_fa = 0, off_fb = 0, off_cb = 0, off_pa = 0, off_pb = 0,
         off_zc = 0, off_comp = 0, off_comph = 0, off_status = 0, off_mask = 0,
         off_srcws = 0, bytes = 0;
  int Pp = 0;  // PML state row stride (P rounded up to 4)
  int Yp = 0;  // padded y length of the streamed kernel's absorber copy
  // When auto selection chose a lean kernel: the streamed plan it replaced
  // (same workspace layout), which a batch falls back to.
  bool has_streamed = false;
  LaunchState streamed = {};
};

namespace {

void pml_coeff(double kappa, double sigma, double alpha, double dt, double* ik,
               double* b, double* c) {
  if (std::isinf(kappa)) {
    *ik = 0.0;
    *b = std::exp(-alpha * dt);
    *c = 0.0;
    return;
  }
  *ik = 1.0 / kappa;
  *b = std::exp(-(sigma / kappa + alpha) * dt);
  *c = (sigma == 0.0) ? 0.0
                      : sigma * (*b - 1.0) / (sigma * kappa + kappa * kappa * alpha);
}

int32_t validate(const pjzfdtd_problem& p) {
  if (p.xx <= 0 || p.yy <= 0 || p.zz <= 0)
    return fail(PJZFDTD_ERR_INVALID, "domain must be positive, got (%d, %d, %d)",
                p.xx, p.yy, p.zz);
  if (p.rx <= 0 || p.ry <= 0 || p.rz <= 0)
    return fail(PJZFDTD_ERR_INVALID, "epsilon shape must be positive");
  if (p.ox < 0 || p.oy < 0 || p.oz < 0 || p.ox + p.rx > p.xx ||
      p.oy + p.ry > p.yy || p.oz + p.rz > p.zz)
    return fail(PJZFDTD_ERR_INVALID,
                "epsilon (%d, %d, %d) at offset (%d, %d, %d) does not fit the "
                "(%d, %d, %d) domain",
                p.rx, p.ry, p.rz, p.ox, p.oy, p.oz, p.xx, p.yy, p.zz);
  if (p.tt < 0) return fail(PJZFDTD_ERR_INVALID, "tt must be >= 0");
  if (p.pml_lo < 0 || p.pml_hi < 0 || p.pml_lo + p.pml_hi > p.zz)
    return fail(PJZFDTD_ERR_INVALID, "pml_widths (%d, %d) do not fit zz=%d",
                p.pml_lo, p.pml_hi, p.zz);
  if (!(p.dt > 0.f) || !std::isfinite(p.dt))
    return fail(PJZFDTD_ERR_INVALID, "dt must be positive and finite");
  if (p.src_ncols < 0 || p.src_ncols > 64)
    return fail(PJZFDTD_ERR_INVALID, "source columns must be in [0, 64]");
  if (p.src_ncols > 0) {
    if (p.src_nx <= 0 || p.src_ny <= 0 || p.src_nz <= 0 || p.src_x0 < 0 ||
        p.src_y0 < 0 || p.src_z0 < 0 || p.src_x0 + p.src_nx > p.xx ||
        p.src_y0 + p.src_ny > p.yy || p.src_z0 + p.src_nz > p.zz)
      return fail(PJZFDTD_ERR_INVALID,
                  "source box (%d, %d, %d)+(%d, %d, %d) outside the domain",
                  p.src_x0, p.src_y0, p.src_z0, p.src_nx, p.src_ny, p.src_nz);
  }
  if (p.out_mode < PJZFDTD_OUT_NONE || p.out_mode > PJZFDTD_OUT_GRADIENT)
    return fail(PJZFDTD_ERR_INVALID, "unknown out_mode %d", p.out_mode);
  if (p.out_mode != PJZFDTD_OUT_NONE) {
    if (p.out_step <= 0)
      return fail(PJZFDTD_ERR_INVALID, "output step must be positive");
    // Steps before 0 are allowed (pjz asks for them when tt is short,
    // src/pjz/_field.py:216): the field there is the zero initial state.
    if (p.out_stop > p.tt || p.out_stop <= p.out_start)
      return fail(PJZFDTD_ERR_INVALID,
                  "output_steps (%d, %d, %d) must end within tt=%d",
                  p.out_start, p.out_stop, p.out_step, p.tt);
  }
  if (p.out_mode == PJZFDTD_OUT_PHASORS || p.out_mode == PJZFDTD_OUT_GRADIENT) {
    if (p.out_rows <= 0 || p.out_rows > kMaxRows)
      return fail(PJZFDTD_ERR_INVALID, "out_rows must be in [1, %d]", kMaxRows);
  }
  if (p.out_mode == PJZFDTD_OUT_GRADIENT) {
    if (p.grad_nx <= 0 || p.grad_ny <= 0 || p.grad_nz <= 0 || p.grad_x0 < 0 ||
        p.grad_y0 < 0 || p.grad_z0 < 0 || p.grad_x0 + p.grad_nx > p.xx ||
        p.grad_y0 + p.grad_ny > p.yy || p.grad_z0 + p.grad_nz > p.zz)
      return fail(PJZFDTD_ERR_INVALID, "gradient box outside the domain");
    if (p.record_h)
      return fail(PJZFDTD_ERR_INVALID, "record_h is not defined for GRADIENT");
  }
  if (p.tile_y < 0 || p.seg_x < 0 || p.steps_per_pass < 0 || p.warps < 0 ||
      p.wait_limit_kcycles < 0 || p.test_stall_bytes < 0 ||
      p.test_stall_bytes % 16)
    return fail(PJZFDTD_ERR_INVALID, "launch params must be >= 0");
  if (p.steps_per_pass > 2)
    return fail(PJZFDTD_ERR_INVALID, "steps_per_pass must be 0 (auto), 1 or 2");
  if (p.storage != PJZFDTD_STORAGE_F32 && p.storage != PJZFDTD_STORAGE_F16)
    return fail(PJZFDTD_ERR_INVALID, "storage must be 0 (FP32) or 1 (binary16)");
  return PJZFDTD_OK;
}

constexpr size_t kSmemBudget = 220 * 1024;  // of the 227 KB per CTA
// Dynamic shared memory a CTA may request: 227 KB less a margin for the
// kernels' static shared memory (abort flag, waveform row cache; the batch
// kernel holds one per inlined tile shape, 1.3 KB).
constexpr size_t kSmemMax = 227 * 1024 - 2048;
constexpr int kStreamThreads = 512;

// Two-step kernel geometry for tile height ty: rows per pass the CTA can
// hold (one compute thread per z-pair, at most kStream2Threads - 32 compute
// threads) and the ring depths that fit shared memory (3 each when they
// fit, else 2), or 0 when nothing fits.
int stream2_rows_cap(int Z) { return (kStream2Threads - 32) / (Z / 2); }
int stream2_stages(int ty, int Z, int P, int want) {
  for (int s = want > 0 ? want : 3; s >= 2; --s) {
    if (Stream2Geom(ty, Z, P).bytes(s, s) <= kSmemBudget) return s;
    if (want > 0) break;
  }
  return 0;
}

// Streamed kernel: zz % 4 == 0, one compute thread per z-pair of a row,
// compute threads = (zz / 2) * rows-per-pass rounded up to whole warps, one
// extra producer warp, and a tile height whose ring fits shared memory.
// With steps_per_pass 2 (or auto) the tile height is the two-step kernel's
// (rows y0-2..y0+TY in one pass, its rings in shared memory) and the
// single-step kernel, used for steps whose state is sampled, shares it.
int32_t resolve_stream(pjzfdtd_plan* pl) {
  const int Z = pl->p.zz;
  const int P = pl->p.pml_lo + pl->p.pml_hi;
  const int rpt = std::max(1, (kStreamThreads - 32) / (Z / 2));
  const int S = pl->p.stages > 0 ? pl->p.stages : 4;
  if (S < 2 || S > 8)
    return fail(PJZFDTD_ERR_INVALID, "stages must be in [2, 8], got %d", S);
  int ty = pl->p.tile_y;
  int spp = pl->p.steps_per_pass;
  int s2 = 0;
  if (spp != 1) {
    const int cap = stream2_rows_cap(Z);
    int t2 = ty;
    if (t2 == 0)
      for (int t = std::min(cap - 3, 64); t >= 1; --t)
        if (stream2_stages(t, Z, P, pl->p.stages) > 0) {
          t2 = std::min(t, pl->p.yy);
          break;
        }
    s2 = t2 > 0 ? stream2_stages(t2, Z, P, pl->p.stages) : 0;
    bool use = t2 > 0 && s2 > 0 && StreamGeom(t2, Z, P).bytes(S) <= kSmemBudget;
    // The streamed kernels keep one step per pass when it is automatic: the
    // streamed two-step kernel moves about half the HBM bytes per
    // cell-update but issues ~1.3x the instructions, and on GB300 its time
    // is set on the SM side, not by HBM (512x512x64: 0.192 ms per step with
    // one step per launch, 0.224 ms with two).  Auto selection takes two
    // steps per pass on the lean two-step kernel instead (resolve_tile).
    if (spp == 0) use = false;
    if (use) {
      ty = t2;
      spp = 2;
    } else if (spp == 2) {
      return fail(PJZFDTD_ERR_INVALID,
                  "two-step tile (tile_y=%d, zz=%d) exceeds shared memory", t2, Z);
    } else {
      spp = 1;
    }
  }
  if (ty == 0) {
    int best = 0;
    for (int t = 1; t <= 64; ++t) {
      if (StreamGeom(t, Z, P).bytes(S) > kSmemBudget) break;
      // Prefer heights whose H rows split evenly over the row groups.
      if ((t + 1) % rpt == 0 || t + 1 < rpt || best == 0) best = t;
    }
    ty = std::min(best, pl->p.yy);
  }
  if (ty <= 0 || StreamGeom(ty, Z, P).bytes(S) > kSmemBudget)
    return fail(PJZFDTD_ERR_INVALID,
                "streamed tile (tile_y=%d, zz=%d, stages=%d) exceeds shared "
                "memory", ty, Z, S);
  pl->tile_y = ty;
  pl->stages = S;
  int ncomp = ((Z / 2) * std::min(rpt, ty + 1) + 31) / 32 * 32;
  if (pl->p.warps > 0) {
    if (pl->p.warps * 32 < Z / 2 || pl->p.warps > 15)
      return fail(PJZFDTD_ERR_INVALID,
                  "warps=%d must cover one z column (%d threads) and be <= 15",
                  pl->p.warps, Z / 2);
    ncomp = pl->p.warps * 32;
  }
  pl->threads = ncomp + 32;
  pl->smem = StreamGeom(ty, Z, P).bytes(S);
  pl->kernel = 2;
  // Carry the source box rows in the ring (the box re-laid out as
  // [x][y][column][component][z] in the workspace, so a tile's rows of one
  // plane are one bulk copy, `stages` planes ahead like the fields) when a
  // re-laid row is whole 16-byte units and the slots still fit; a box of
  // many rows (a plane crossing the whole tile) keeps the global loads --
  // it is crossed by few planes.
  pl->src_ring = pl->src_rows = 0;
  const pjzfdtd_problem& q = pl->p;
  if (q.src_ncols > 0 && (q.src_ncols * 3 * q.src_nz) % 4 == 0) {
    const int rows = std::min(ty, q.src_ny);
    const int sw = q.src_ncols * 3 * rows * q.src_nz;
    if (rows > 0 && StreamGeom(ty, Z, P, sw).bytes(S) <= kSmemMax) {
      pl->src_ring = sw;
      pl->src_rows = rows;
      pl->smem = StreamGeom(ty, Z, P, sw).bytes(S);
    }
  }
  pl->steps_per_pass = spp;
  if (spp == 2) {
    const int rows = std::min(stream2_rows_cap(Z), ty + 3);
    pl->threads2 = ((Z / 2) * rows + 31) / 32 * 32 + 32;
    bool special = false;
#define PJZ_IS2(ZC, TYC) special |= (Z == ZC && ty == TYC);
    PJZ_STREAM2_SHAPES(PJZ_IS2)
#undef PJZ_IS2
    if (special) pl->threads2 = std::min(pl->threads2, stream2_bound(Z, ty));
    pl->stages2 = s2 | (s2 << 8);
    pl->smem2 = Stream2Geom(ty, Z, P).bytes(s2, s2);
  }
  return PJZFDTD_OK;
}

// Whether auto selection takes the lean kernels where they apply (FP32
// storage; binary16 always runs on them): the two-step kernel when the
// steps per pass are automatic, else the one-step kernel at zz 64.
constexpr bool kLeanAuto = true;
constexpr bool kLean2Auto = true;

LaunchState save_launch(const pjzfdtd_plan* pl) {
  return LaunchState{pl->tile_y,   pl->seg_x,   pl->threads,  pl->steps_per_pass,
                     pl->kernel,   pl->stages,  pl->threads2, pl->stages2,
                     pl->src_ring, pl->src_rows, pl->smem,    pl->smem2};
}

void load_launch(pjzfdtd_plan* pl, const LaunchState& s) {
  pl->tile_y = s.tile_y;
  pl->seg_x = s.seg_x;
  pl->threads = s.threads;
  pl->steps_per_pass = s.steps_per_pass;
  pl->kernel = s.kernel;
  pl->stages = s.stages;
  pl->threads2 = s.threads2;
  pl->stages2 = s.stages2;
  pl->src_ring = s.src_ring;
  pl->src_rows = s.src_rows;
  pl->smem = s.smem;
  pl->smem2 = s.smem2;
}
// Whether auto selection takes the tall binary16 lean tile where it applies
// (c1, binary16: 0.145 ms per step against 0.162 at tile_y 14).
constexpr bool kLeanTallAuto = true;

// Lean streamed kernel (lean_kernel.cuh) on top of a resolved streamed
// plan: a compile-time (zz, tile_y) shape, one step per launch, z-PML slab
// widths that are multiples of 4 (PML quads are whole), the source read
// from global memory.  `required`: fail when it does not apply, else keep
// the streamed plan.
int32_t resolve_lean(pjzfdtd_plan* pl, bool required) {
  const pjzfdtd_problem& p = pl->p;
  const int Z = p.zz, ty = pl->tile_y;
  const bool shape = lean_kernel_ptr(Z, ty, p.storage) != nullptr;
  const bool ok = shape && (required || pl->steps_per_pass == 1) &&
                  p.pml_lo % 4 == 0 && p.pml_hi % 4 == 0 &&
                  (required || pl->src_ring == 0);
  if (!ok) {
    if (!required) return PJZFDTD_OK;
    return fail(PJZFDTD_ERR_UNSUPPORTED,
                "the lean kernel needs (zz, tile_y) in {(64, 14), (48, 19), "
                "(32, 29), (32, 28)}, or (64, 28) with binary16 storage (got "
                "(%d, %d)), and z-PML widths that are multiples of 4 (got %d, "
                "%d)",
                Z, ty, p.pml_lo, p.pml_hi);
  }
  const int warps = lean_warps(Z, ty + 1, p.pml_lo, p.pml_hi, pl->esz);
  const int bound = lean_kernel_threads(Z, ty, p.storage);
  if (warps * 32 + 32 > bound)
    return required ? fail(PJZFDTD_ERR_UNSUPPORTED, "lean tile needs %d warps",
                           warps)
                    : PJZFDTD_OK;
  // The lean layout holds a third new-H buffer: drop ring stages (not
  // below two, and only those picked automatically) where the streamed
  // plan's depth no longer fits.
  auto bytes = [&](int s) {
    return p.storage == PJZFDTD_STORAGE_F16 ? LeanGeom<__half>(ty, Z, pl->P).bytes(s)
                                            : LeanGeom<float>(ty, Z, pl->P).bytes(s);
  };
  int stages = pl->stages;
  while (p.stages == 0 && stages > 2 && bytes(stages) > kSmemMax) --stages;
  if (bytes(stages) > kSmemMax)
    return required ? fail(PJZFDTD_ERR_UNSUPPORTED,
                           "lean tile needs %zu bytes of shared memory",
                           bytes(stages))
                    : PJZFDTD_OK;
  pl->kernel = 3;
  pl->threads = warps * 32 + 32;
  pl->src_ring = pl->src_rows = 0;
  pl->stages = stages;
  pl->smem = bytes(stages);
  return PJZFDTD_OK;
}

// Lean two-step kernel (lean2_kernel.cuh) on a plan already resolved for
// the lean one-step kernel with two steps per pass: its compile-time shape,
// block and shared memory (the ring depths of the streamed two-step plan).
int32_t resolve_lean2(pjzfdtd_plan* pl) {
  const pjzfdtd_problem& p = pl->p;
  const int Z = p.zz, ty = pl->tile_y;
  if (!lean2_kernel_ptr(Z, ty, p.storage))
    return fail(PJZFDTD_ERR_UNSUPPORTED,
                "the lean two-step kernel needs (zz, tile_y) = (64, 14), got "
                "(%d, %d)", Z, ty);
  const int warps = lean2_warps(Z, ty, p.pml_lo, p.pml_hi, pl->esz);
  if (warps * 32 + 32 > kLeanThreads)
    return fail(PJZFDTD_ERR_UNSUPPORTED, "lean two-step tile needs %d warps", warps);
  const int s2 = pl->stages2 & 0xff;
  pl->threads2 = warps * 32 + 32;
  pl->smem2 = p.storage == PJZFDTD_STORAGE_F16
                  ? Lean2Geom<__half>(ty, Z, pl->P).bytes(s2, s2)
                  : Lean2Geom<float>(ty, Z, pl->P).bytes(s2, s2);
  return PJZFDTD_OK;
}

// Whether the lean two-step kernel takes a plan resolved for the streamed
// two-step kernel: a compile-time shape of both lean kernels, z-PML slabs of
// whole quads, no ring-carried source rows, blocks within their bounds.
bool lean2_applies(const pjzfdtd_plan* pl) {
  const pjzfdtd_problem& p = pl->p;
  const int Z = p.zz, ty = pl->tile_y;
  if (pl->steps_per_pass != 2 || pl->src_ring != 0 || p.pml_lo % 4 != 0 ||
      p.pml_hi % 4 != 0 || !lean_kernel_ptr(Z, ty, p.storage) ||
      !lean2_kernel_ptr(Z, ty, p.storage))
    return false;
  return lean2_warps(Z, ty, p.pml_lo, p.pml_hi, pl->esz) * 32 + 32 <= kLeanThreads &&
         lean_warps(Z, ty + 1, p.pml_lo, p.pml_hi, pl->esz) * 32 + 32 <=
             lean_kernel_threads(Z, ty, p.storage);
}

// Resolves the CTA tile.  Register-marching kernel: (tile_y + 2) * zz
// cells, one thread each, at most kMaxThreads threads.
int32_t resolve_tile(pjzfdtd_plan* pl) {
  const int Z = pl->p.zz;
  if (pl->p.kernel < 0 || pl->p.kernel > 3)
    return fail(PJZFDTD_ERR_INVALID, "unknown kernel %d", pl->p.kernel);
  const int zmax = 2 * (kStreamThreads - 32);
  if (pl->p.kernel >= 2 && (Z % 4 != 0 || Z > zmax))
    return fail(PJZFDTD_ERR_INVALID,
                "the streamed kernels need zz %% 4 == 0 and zz <= %d", zmax);
  if (pl->p.storage == PJZFDTD_STORAGE_F16 && pl->p.kernel != 0 &&
      pl->p.kernel != 3)
    return fail(PJZFDTD_ERR_UNSUPPORTED,
                "binary16 storage is served by the lean kernel (kernel 0 or 3)");
  if (pl->p.kernel == 3 || pl->p.storage == PJZFDTD_STORAGE_F16) {
    if (Z % 4 != 0 || Z > zmax)
      return fail(PJZFDTD_ERR_UNSUPPORTED,
                  "binary16 storage needs the lean kernel (zz %% 4 == 0)");
    // The tall binary16 tile (one step per launch): resolved like the
    // streamed plan at the automatic height, then given the tall height.
    const int tall = pl->p.storage == PJZFDTD_STORAGE_F16 && pl->p.steps_per_pass != 2
                         ? lean_tall_tile_y(Z)
                         : 0;
    const bool asked = tall > 0 && pl->p.tile_y == tall;
    if (asked || (tall > 0 && pl->p.tile_y == 0 && kLeanTallAuto)) {
      const int req_ty = pl->p.tile_y;
      pl->p.tile_y = 0;
      int32_t rc = resolve_stream(pl);
      pl->p.tile_y = req_ty;
      if (rc) return rc;
      pl->tile_y = tall;
      if ((rc = resolve_lean(pl, asked))) return rc;
      if (pl->kernel == 3) return PJZFDTD_OK;
      pl->seg_x = 0;  // not applicable: the plan below starts over
    }
    int32_t rc = resolve_stream(pl);
    if (rc) return rc;
    if ((rc = resolve_lean(pl, true))) return rc;
    return pl->steps_per_pass == 2 ? resolve_lean2(pl) : PJZFDTD_OK;
  }
  if (pl->p.kernel == 2 || (pl->p.kernel == 0 && Z % 4 == 0 && Z <= zmax)) {
    int32_t rc = resolve_stream(pl);
    if (rc || pl->p.kernel == 2 || !kLeanAuto) return rc;
    // Auto: the lean two-step kernel, else the lean one-step kernel, where
    // they apply; the streamed plan is kept for batches.
    const LaunchState streamed = save_launch(pl);
    if (kLean2Auto && pl->p.steps_per_pass == 0 && pl->src_ring == 0) {
      pl->p.steps_per_pass = 2;
      rc = resolve_stream(pl);
      pl->p.steps_per_pass = 0;
      if (rc == PJZFDTD_OK && lean2_applies(pl) &&
          resolve_lean(pl, true) == PJZFDTD_OK && resolve_lean2(pl) == PJZFDTD_OK) {
        pl->has_streamed = true;
        pl->streamed = streamed;
        return PJZFDTD_OK;
      }
      load_launch(pl, streamed);
    }
    // The one-step lean kernel only where it measured faster than the
    // streamed kernel (zz 64: 0.184 against 0.192 ms per step on
    // 512x512x64; zz 32: 0.117 against 0.111 on 512x512x32).
    if (Z != 64) return PJZFDTD_OK;
    if ((rc = resolve_lean(pl, false))) return rc;
    if (pl->kernel == 3) {
      pl->has_streamed = true;
      pl->streamed = streamed;
    }
    return PJZFDTD_OK;
  }
  pl->kernel = 1;
  if (pl->p.steps_per_pass == 2)
    return fail(PJZFDTD_ERR_UNSUPPORTED,
                "two steps per pass need the streamed kernel (zz %% 4 == 0)");
  int ty = pl->p.tile_y;
  const int max_rows = kMaxThreads / Z;
  if (max_rows < 3)
    return fail(PJZFDTD_ERR_UNSUPPORTED,
                "zz=%d exceeds the thin-z limit of this kernel (zz <= %d)", Z,
                kMaxThreads / 3);
  if (ty == 0) ty = max_rows - 2;
  if (ty + 2 > max_rows)
    return fail(PJZFDTD_ERR_INVALID, "tile_y=%d too large for zz=%d (max %d)",
                ty, Z, max_rows - 2);
  pl->tile_y = ty;
  pl->threads = ((ty + 2) * Z + 31) / 32 * 32;
  pl->steps_per_pass = 1;
  pl->smem = 6 * (size_t)(ty + 2) * Z * sizeof(float);
  return PJZFDTD_OK;
}

// Recorded boxes: the region (or the gradient box) unless monitors were set.
// `out` holds the boxes one after another, each shaped like a single-region
// output ((ns,3,box) snapshots, (rows,3,box) phasors, (3,box) gradient).
void set_boxes(pjzfdtd_plan* pl) {
  const pjzfdtd_problem& p = pl->p;
  if (pl->boxes.empty()) {
    if (p.out_mode == PJZFDTD_OUT_GRADIENT)
      pl->boxes.push_back({p.grad_x0, p.grad_y0, p.grad_z0, p.grad_nx, p.grad_ny,
                           p.grad_nz});
    else if (p.out_mode != PJZFDTD_OUT_NONE)
      pl->boxes.push_back({p.ox, p.oy, p.oz, p.rx, p.ry, p.rz});
  }
  const size_t per = p.out_mode == PJZFDTD_OUT_SNAPSHOTS ? (size_t)pl->ns * 3
                     : p.out_mode == PJZFDTD_OUT_PHASORS ? (size_t)p.out_rows * 3
                                                         : 3;
  pl->box_off.clear();
  size_t o = 0;
  for (const auto& bx : pl->boxes) {
    pl->box_off.push_back(o);
    o += per * (size_t)bx[3] * bx[4] * bx[5];
  }
  pl->out_floats = o;
}

void layout(pjzfdtd_plan* pl) {
  const pjzfdtd_problem& p = pl->p;
  const size_t N = (size_t)pl->N;
  // PML state rows are whole 16-byte units (4 FP32 or 8 binary16 values).
  pl->Pp = pl->esz == 2 ? (pl->P + 7) / 8 * 8 : round4(pl->P);
  pl->Yp = round4(p.yy);
  set_boxes(pl);
  const size_t XYP = (size_t)p.xx * p.yy * std::max(pl->Pp, 1);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o = align256(o + bytes);
    return at;
  };
  const size_t es = (size_t)pl->esz;
  pl->off_fa = take(6 * N * es);
  pl->off_fb = take(6 * N * es);
  pl->off_cb = take(3 * N * es);
  pl->off_pa = take(4 * XYP * es);
  pl->off_pb = take(4 * XYP * es);
  pl->off_zc = take(6 * (size_t)p.zz * sizeof(float));
  const size_t comp = (p.out_mode == PJZFDTD_OUT_PHASORS ||
                       p.out_mode == PJZFDTD_OUT_GRADIENT) ? pl->out_floats : 0;
  pl->off_comp = take(std::max<size_t>(comp, 1) * sizeof(float));
  pl->off_comph = take(std::max<size_t>(p.record_h ? comp : 0, 1) * sizeof(float));
  pl->off_status = take(sizeof(int));
  pl->off_mask = take((pl->kernel >= 2 ? (size_t)p.xx * 3 * pl->Yp : 1) * sizeof(float));
  pl->off_srcws = take((pl->src_ring > 0 ? (size_t)p.src_ncols * 3 * p.src_nx *
                                               p.src_ny * p.src_nz
                                         : 1) * sizeof(float));
  pl->bytes = o;
}

// The streamed kernel for a plan: its (zz, tile_y) specialisation when one
// exists, else the generic instantiation; `sr` selects the instantiation
// whose ring carries the source rows.
StreamKernel stream_kernel_for(const pjzfdtd_plan* pl, bool sr) {
  return stream_kernel_ptr(pl->p.zz, pl->tile_y, sr);
}

cudaError_t set_stream_smem(const pjzfdtd_plan* pl, bool sr) {
  return cudaFuncSetAttribute(stream_kernel_for(pl, sr),
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)pl->smem);
}

cudaError_t set_lean_smem(const pjzfdtd_plan* pl) {
  return cudaFuncSetAttribute(lean_kernel_ptr(pl->p.zz, pl->tile_y, pl->p.storage),
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)pl->smem);
}

// The two-step kernel for a plan, by the same rule (the lean one for lean
// plans).
StreamKernel stream2_kernel_for(const pjzfdtd_plan* pl) {
  if (pl->kernel == 3) return lean2_kernel_ptr(pl->p.zz, pl->tile_y, pl->p.storage);
  return stream2_kernel_ptr(pl->p.zz, pl->tile_y);
}

cudaError_t set_stream2_smem(const pjzfdtd_plan* pl) {
  return cudaFuncSetAttribute(stream2_kernel_for(pl),
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)pl->smem2);
}

int32_t resolve_seg_x(pjzfdtd_plan* pl) {
  if (pl->seg_x > 0) return PJZFDTD_OK;
  if (pl->p.seg_x > 0) {
    pl->seg_x = pl->p.seg_x;
    return PJZFDTD_OK;
  }
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int per_sm = 1;
  if (pl->kernel >= 2 && pl->steps_per_pass == 2) {
    CUDA_TRY(set_stream2_smem(pl));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, stream2_kernel_for(pl), pl->threads2, pl->smem2));
  } else if (pl->kernel == 3) {
    CUDA_TRY(set_lean_smem(pl));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, lean_kernel_ptr(pl->p.zz, pl->tile_y, pl->p.storage), pl->threads,
        pl->smem));
  } else if (pl->kernel == 2) {
    CUDA_TRY(set_stream_smem(pl, pl->src_ring > 0));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, stream_kernel_for(pl, pl->src_ring > 0), pl->threads, pl->smem));
  } else {
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, yee_step_kernel, pl->threads, pl->smem));
  }
  per_sm = std::max(per_sm, 1);
  const int tiles_y = (pl->p.yy + pl->tile_y - 1) / pl->tile_y;
  const int slots = sms * per_sm;
  int nseg = std::max(1, slots / tiles_y);
  int seg = (pl->p.xx + nseg - 1) / nseg;
  // At least 4 planes per segment: each segment re-reads one halo plane,
  // and small domains (c0: 128x128x32) need short segments to fill the
  // SMs at all.
  seg = std::max(seg, std::min(pl->p.xx, 4));
  pl->seg_x = seg;
  return PJZFDTD_OK;
}

template <typename T>
T* at(void* ws, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(ws) + off);
}

int32_t check_buffers(const pjzfdtd_plan* pl, const pjzfdtd_buffers* b,
                      void* ws, size_t ws_bytes) {
  if (!b) return fail(PJZFDTD_ERR_INVALID, "buffers is NULL");
  if (!ws || ws_bytes < pl->bytes)
    return fail(PJZFDTD_ERR_WORKSPACE, "workspace of %zu bytes needed, got %zu",
                pl->bytes, ws ? ws_bytes : (size_t)0);
  if (reinterpret_cast<uintptr_t>(ws) % 256)
    return fail(PJZFDTD_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  if (!b->epsilon || !b->absorption_mask)
    return fail(PJZFDTD_ERR_INVALID, "epsilon and absorption_mask are required");
  if (pl->p.src_ncols > 0 && (!b->source || !b->waveform))
    return fail(PJZFDTD_ERR_INVALID, "source and waveform are required");
  if (pl->p.out_mode != PJZFDTD_OUT_NONE && !b->out)
    return fail(PJZFDTD_ERR_INVALID, "out is required for this out_mode");
  if (pl->p.record_h && !b->out_h)
    return fail(PJZFDTD_ERR_INVALID, "out_h is required when record_h is set");
  if (pl->p.out_mode == PJZFDTD_OUT_GRADIENT && !b->q)
    return fail(PJZFDTD_ERR_INVALID, "q is required for GRADIENT");
  return PJZFDTD_OK;
}

// Device pointers of one plan's workspace.
struct RunPtrs {
  float *fa, *fb, *cb, *pa, *pb, *zc, *comp, *comph, *mask_ws, *srcws;
  int* status;
  RunPtrs(const pjzfdtd_plan* pl, void* ws)
      : fa(at<float>(ws, pl->off_fa)), fb(at<float>(ws, pl->off_fb)),
        cb(at<float>(ws, pl->off_cb)), pa(at<float>(ws, pl->off_pa)),
        pb(at<float>(ws, pl->off_pb)), zc(at<float>(ws, pl->off_zc)),
        comp(at<float>(ws, pl->off_comp)), comph(at<float>(ws, pl->off_comph)),
        mask_ws(at<float>(ws, pl->off_mask)), srcws(at<float>(ws, pl->off_srcws)),
        status(at<int>(ws, pl->off_status)) {}
};

// Ring-carried source rows: the source box re-laid out in the workspace
// (stream-ordered, capturable).  Done by every run call, so a chained call
// sees the source buffer it is given.
int32_t relayout_source(const pjzfdtd_plan* pl, const pjzfdtd_buffers* b,
                        void* ws, cudaStream_t st) {
  if (pl->src_ring <= 0 || !b->source) return PJZFDTD_OK;
  const pjzfdtd_problem& p = pl->p;
  RunPtrs w(pl, ws);
  const long long n = (long long)p.src_ncols * 3 * p.src_nx * p.src_ny * p.src_nz;
  source_rows_kernel<<<(int)std::min<long long>((n + 255) / 256, 1 << 16), 256, 0,
                       st>>>(b->source, w.srcws, p.src_ncols, p.src_nx, p.src_ny,
                             p.src_nz);
  CUDA_TRY(cudaGetLastError());
  return PJZFDTD_OK;
}

// Start-of-run work (stream-ordered, capturable unless copy_zc): zero the
// state, outputs and status word, load the initial fields, build the
// coefficient and absorber arrays.  The CPML table is a pageable host copy,
// done here only when copy_zc.
int32_t run_init(pjzfdtd_plan* pl, const pjzfdtd_buffers* b, void* ws,
                 cudaStream_t st, bool copy_zc) {
  const pjzfdtd_problem& p = pl->p;
  const long long N = pl->N;
  const size_t XYP = (size_t)p.xx * p.yy * std::max(pl->Pp, 1);
  RunPtrs w(pl, ws);
  if (p.out_mode != PJZFDTD_OUT_NONE) {
    // Snapshots before step 0 are zero; accumulators start at zero.
    CUDA_TRY(cudaMemsetAsync(b->out, 0, pl->out_floats * sizeof(float), st));
    if (p.record_h)
      CUDA_TRY(cudaMemsetAsync(b->out_h, 0, pl->out_floats * sizeof(float), st));
  }
  if (p.out_mode == PJZFDTD_OUT_PHASORS || p.out_mode == PJZFDTD_OUT_GRADIENT) {
    CUDA_TRY(cudaMemsetAsync(w.comp, 0, pl->out_floats * sizeof(float), st));
    if (p.record_h)
      CUDA_TRY(cudaMemsetAsync(w.comph, 0, pl->out_floats * sizeof(float), st));
  }
  if (copy_zc)
    CUDA_TRY(cudaMemcpyAsync(w.zc, pl->zc.data(), pl->zc.size() * sizeof(float),
                             cudaMemcpyHostToDevice, st));
  const bool f16 = pl->esz == 2;
  const int threads = 256;
  if (b->fields && f16) {
    const long long n = 6 * N;
    narrow_f16_kernel<<<(int)std::min<long long>((n + 255) / 256, 1 << 20), 256, 0,
                        st>>>(b->fields, reinterpret_cast<__half*>(w.fa), n);
    CUDA_TRY(cudaGetLastError());
  } else if (b->fields) {
    CUDA_TRY(cudaMemcpyAsync(w.fa, b->fields, 6 * N * sizeof(float),
                             cudaMemcpyDeviceToDevice, st));
  } else {
    CUDA_TRY(cudaMemsetAsync(w.fa, 0, 6 * N * pl->esz, st));
  }
  CUDA_TRY(cudaMemsetAsync(w.pa, 0, 4 * XYP * pl->esz, st));
  CUDA_TRY(cudaMemsetAsync(w.pb, 0, 4 * XYP * pl->esz, st));
  CUDA_TRY(cudaMemsetAsync(w.status, 0, sizeof(int), st));
  const long long total = 3 * N;
  const int blocks = (int)std::min<long long>((total + threads - 1) / threads, 1 << 20);
  if (f16)
    precompute_cb_kernel<__half><<<blocks, threads, 0, st>>>(
        b->epsilon, b->absorption_mask, reinterpret_cast<__half*>(w.cb), p.xx,
        p.yy, p.zz, p.ox, p.oy, p.oz, p.rx, p.ry, p.rz, p.dt);
  else
    precompute_cb_kernel<float><<<blocks, threads, 0, st>>>(
        b->epsilon, b->absorption_mask, w.cb, p.xx, p.yy, p.zz, p.ox, p.oy, p.oz,
        p.rx, p.ry, p.rz, p.dt);
  CUDA_TRY(cudaGetLastError());
  if (pl->kernel >= 2) {
    const long long nm = (long long)p.xx * 3 * pl->Yp;
    pad_mask_kernel<<<(int)std::min<long long>((nm + 255) / 256, 1 << 16), 256, 0,
                      st>>>(b->absorption_mask, w.mask_ws, p.xx, p.yy, pl->Yp);
    CUDA_TRY(cudaGetLastError());
  }
  return relayout_source(pl, b, ws, st);
}

// Step arguments of a launch starting at step n with the state in buffer
// `cur` (0: A, 1: B); the launch writes the other buffer.
StepArgs step_args(const pjzfdtd_plan* pl, const pjzfdtd_buffers* b, void* ws,
                   int n, int cur) {
  const pjzfdtd_problem& p = pl->p;
  RunPtrs w(pl, ws);
  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.X = p.xx;
  a.Y = p.yy;
  a.Z = p.zz;
  a.P = pl->P;
  a.Pst = std::max(pl->Pp, 1);
  a.plo = p.pml_lo;
  a.phi = p.pml_hi;
  a.N = pl->N;
  a.dt = p.dt;
  a.tile_y = pl->tile_y;
  a.seg_x = pl->seg_x;
  a.cb = w.cb;
  a.mask = b->absorption_mask;
  a.zc = w.zc;
  a.sx0 = p.src_x0;
  a.sy0 = p.src_y0;
  a.sz0 = p.src_z0;
  a.snx = p.src_ncols > 0 ? p.src_nx : 0;
  a.sny = p.src_ncols > 0 ? p.src_ny : 0;
  a.snz = p.src_ncols > 0 ? p.src_nz : 0;
  a.snc = p.src_ncols;
  a.src = b->source;
  const bool in_a = cur == 0;
  a.fin = in_a ? w.fa : w.fb;
  a.fout = in_a ? w.fb : w.fa;
  a.psi_in = in_a ? w.pa : w.pb;
  a.psi_out = in_a ? w.pb : w.pa;
  a.wave = p.src_ncols > 0 ? b->waveform + (size_t)n * p.src_ncols : nullptr;
  return a;
}

StreamArgs stream_args(const pjzfdtd_plan* pl, void* ws, const StepArgs& a) {
  RunPtrs w(pl, ws);
  StreamArgs sa;
  std::memset(&sa, 0, sizeof(sa));
  sa.s = a;
  sa.stages = pl->stages;
  sa.stages2 = pl->stages2;
  sa.status = w.status;
  sa.Yp = pl->Yp;
  sa.mask_ws = w.mask_ws;
  sa.wait_cycles = pl->p.wait_limit_kcycles > 0
                       ? 1000LL * pl->p.wait_limit_kcycles : kWaitCycles;
  sa.stall_bytes = (unsigned)pl->p.test_stall_bytes;
  sa.src_ring = pl->src_ring;
  sa.src_rows = pl->src_rows;
  sa.src_tma = pl->src_ring > 0 && a.src;
  sa.src_ws = w.srcws;
  return sa;
}

bool is_sample(const pjzfdtd_problem& p, int n) {
  return p.out_mode != PJZFDTD_OUT_NONE && n >= p.out_start && n < p.out_stop &&
         (n - p.out_start) % p.out_step == 0;
}

// Record pass of step n (a sample step) over every box, from state `f`.
int32_t record_step(const pjzfdtd_plan* pl, const pjzfdtd_buffers* b, void* ws,
                    int n, const float* f, cudaStream_t st) {
  const pjzfdtd_problem& p = pl->p;
  RunPtrs w(pl, ws);
  const int j = (n - p.out_start) / p.out_step;
  RecordArgs ra;
  std::memset(&ra, 0, sizeof(ra));
  ra.f = f;
  ra.N = pl->N;
  ra.X = p.xx;
  ra.Y = p.yy;
  ra.Z = p.zz;
  ra.record_h = p.record_h;
  ra.rows = p.out_rows;
  ra.q = b->q;
  if (p.out_mode != PJZFDTD_OUT_SNAPSHOTS)
    for (int r = 0; r < p.out_rows; ++r) ra.w[r] = pl->weights[(size_t)r * pl->ns + j];
  for (size_t k = 0; k < pl->boxes.size(); ++k) {
    const auto& bx = pl->boxes[k];
    ra.bx0 = bx[0];
    ra.by0 = bx[1];
    ra.bz0 = bx[2];
    ra.bnx = bx[3];
    ra.bny = bx[4];
    ra.bnz = bx[5];
    const long long nb = (long long)bx[3] * bx[4] * bx[5];
    size_t o = pl->box_off[k];
    if (p.out_mode == PJZFDTD_OUT_SNAPSHOTS) o += (size_t)j * 3 * nb;
    ra.out = b->out + o;
    ra.out_h = p.record_h ? b->out_h + o : nullptr;
    ra.comp = w.comp + pl->box_off[k];
    ra.comp_h = w.comph + pl->box_off[k];
    const int rblocks = (int)std::min<long long>((nb + 255) / 256, 1 << 20);
    const bool f16 = pl->esz == 2;
    switch (p.out_mode) {
      case PJZFDTD_OUT_SNAPSHOTS:
        if (f16) record_kernel<kRecSnap, __half><<<rblocks, 256, 0, st>>>(ra);
        else record_kernel<kRecSnap, float><<<rblocks, 256, 0, st>>>(ra);
        break;
      case PJZFDTD_OUT_PHASORS:
        if (f16) record_kernel<kRecProj, __half><<<rblocks, 256, 0, st>>>(ra);
        else record_kernel<kRecProj, float><<<rblocks, 256, 0, st>>>(ra);
        break;
      default:
        if (f16) record_kernel<kRecGrad, __half><<<rblocks, 256, 0, st>>>(ra);
        else record_kernel<kRecGrad, float><<<rblocks, 256, 0, st>>>(ra);
        break;
    }
    CUDA_TRY(cudaGetLastError());
  }
  return PJZFDTD_OK;
}

int32_t run_finish(const pjzfdtd_plan* pl, const pjzfdtd_buffers* b, void* ws,
                   cudaStream_t st, int cur) {
  if (!b->fields) return PJZFDTD_OK;
  RunPtrs w(pl, ws);
  float* fin = cur == 0 ? w.fa : w.fb;
  if (pl->esz == 2) {
    const long long n = 6 * pl->N;
    widen_f16_kernel<<<(int)std::min<long long>((n + 255) / 256, 1 << 20), 256, 0,
                       st>>>(reinterpret_cast<const __half*>(fin), b->fields, n);
    CUDA_TRY(cudaGetLastError());
    return PJZFDTD_OK;
  }
  CUDA_TRY(cudaMemcpyAsync(b->fields, fin, 6 * pl->N * sizeof(float),
                           cudaMemcpyDeviceToDevice, st));
  return PJZFDTD_OK;
}

// Launch schedule of steps [n0, n1): two steps per launch where the plan
// allows it and the state between them is not sampled, one step otherwise.
// Each entry is (first step, steps).
std::vector<std::pair<int, int>> schedule(const pjzfdtd_plan* pl, int n0, int n1) {
  std::vector<std::pair<int, int>> out;
  for (int n = n0; n < n1;) {
    const bool pair =
        pl->steps_per_pass == 2 && n + 1 < n1 && !is_sample(pl->p, n);
    out.emplace_back(n, pair ? 2 : 1);
    n += pair ? 2 : 1;
  }
  return out;
}

int32_t run_range(pjzfdtd_plan* pl, const pjzfdtd_buffers* b, void* ws,
                  size_t ws_bytes, int n0, int n1, cudaStream_t st) {
  int32_t rc = check_buffers(pl, b, ws, ws_bytes);
  if (rc) return rc;
  if (n0 < 0 || n1 > pl->p.tt || n0 > n1)
    return fail(PJZFDTD_ERR_INVALID, "step range [%d, %d) outside [0, %d)", n0,
                n1, pl->p.tt);
  rc = resolve_seg_x(pl);
  if (rc) return rc;
  const pjzfdtd_problem& p = pl->p;
  if (n0 == 0) {
    if ((rc = run_init(pl, b, ws, st, true))) return rc;
    pl->cur = 0;
  } else if ((rc = relayout_source(pl, b, ws, st))) {
    return rc;
  }
  const dim3 grid((p.yy + pl->tile_y - 1) / pl->tile_y,
                  (p.xx + pl->seg_x - 1) / pl->seg_x);
  StreamKernel sk = nullptr, sk2 = nullptr;
  if (pl->kernel == 3) {
    CUDA_TRY(set_lean_smem(pl));
    sk = lean_kernel_ptr(p.zz, pl->tile_y, p.storage);
  } else if (pl->kernel == 2) {
    // Ring-carried source rows need an aligned source profile (fixed per run).
    const bool sr = stream_args(pl, ws, step_args(pl, b, ws, n0, pl->cur)).src_tma;
    CUDA_TRY(set_stream_smem(pl, sr));
    sk = stream_kernel_for(pl, sr);
  }
  if (pl->steps_per_pass == 2) {
    CUDA_TRY(set_stream2_smem(pl));
    sk2 = stream2_kernel_for(pl);
  }
  for (const auto& ln : schedule(pl, n0, n1)) {
    const StepArgs a = step_args(pl, b, ws, ln.first, pl->cur);
    if (ln.second == 2) {
      sk2<<<grid, pl->threads2, pl->smem2, st>>>(stream_args(pl, ws, a));
    } else if (pl->kernel >= 2) {
      sk<<<grid, pl->threads, pl->smem, st>>>(stream_args(pl, ws, a));
    } else {
      yee_step_kernel<<<grid, pl->threads, pl->smem, st>>>(a);
    }
    CUDA_TRY(cudaGetLastError());
    pl->cur ^= 1;
    const int last = ln.first + ln.second - 1;
    if (is_sample(p, last) && (rc = record_step(pl, b, ws, last, a.fout, st)))
      return rc;
  }
  if (n1 == p.tt) return run_finish(pl, b, ws, st, pl->cur);
  return PJZFDTD_OK;
}

}  // namespace

struct pjzfdtd_batch {
  std::vector<pjzfdtd_plan*> plans;
  std::vector<size_t> off;  // workspace offset of each plan
  size_t off_args = 0, off_work = 0, off_sched = 0, bytes = 0;
  int max_work = 0;
  int tt_max = 0;
  size_t smem = 0;
  size_t smem2 = 0;       // two-step kernel's shared memory (0: none)
  // Per launch: the prefix of the work table that runs and which kernels it
  // needs (bit 0: one step, bit 1: two steps); per problem the launches of
  // its own schedule (first step, steps).
  std::vector<int> active, kinds;
  std::vector<std::vector<std::pair<int, int>>> sched;
  // Cached CUDA graph of a whole run and the buffers it was captured with.
  cudaGraphExec_t exec = nullptr;
  std::vector<pjzfdtd_buffers> gbufs;
  void* gws = nullptr;
  cudaStream_t gstream = nullptr;
  ~pjzfdtd_batch() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

namespace {

bool same_buffers(const pjzfdtd_buffers& a, const pjzfdtd_buffers& b) {
  return std::memcmp(&a, &b, sizeof(a)) == 0;
}

// Enqueues one whole batched run on `st` (capturable: no host copies).
int32_t batch_enqueue(pjzfdtd_batch* bt, const pjzfdtd_buffers* bufs, void* ws,
                      cudaStream_t st) {
  const int n = (int)bt->plans.size();
  int32_t rc;
  for (int i = 0; i < n; ++i)
    if ((rc = run_init(bt->plans[i], &bufs[i], at<char>(ws, bt->off[i]), st, false)))
      return rc;
  BatchArgs ba;
  ba.args = at<const StreamArgs>(ws, bt->off_args);
  ba.work = at<const int4>(ws, bt->off_work);
  ba.sched = at<const int2>(ws, bt->off_sched);
  ba.nsim = n;
  for (int j = 0; j < (int)bt->active.size(); ++j) {
    ba.launch = j;
    if (bt->active[j] > 0 && (bt->kinds[j] & 2)) {
      batch_kernel_ptr(2)<<<bt->active[j], kStream2Threads, bt->smem2, st>>>(ba);
      CUDA_TRY(cudaGetLastError());
    }
    if (bt->active[j] > 0 && (bt->kinds[j] & 1)) {
      batch_kernel_ptr(1)<<<bt->active[j], kStreamThreads, bt->smem, st>>>(ba);
      CUDA_TRY(cudaGetLastError());
    }
    for (int i = 0; i < n; ++i) {
      const pjzfdtd_plan* pl = bt->plans[i];
      if (j >= (int)bt->sched[i].size()) continue;
      const auto& ln = bt->sched[i][j];
      const int last = ln.first + ln.second - 1;
      if (!is_sample(pl->p, last)) continue;
      void* wsi = at<char>(ws, bt->off[i]);
      RunPtrs w(pl, wsi);
      const float* fout = (j % 2 == 0) ? w.fb : w.fa;
      if ((rc = record_step(pl, &bufs[i], wsi, last, fout, st))) return rc;
    }
  }
  for (int i = 0; i < n; ++i)
    if ((rc = run_finish(bt->plans[i], &bufs[i], at<char>(ws, bt->off[i]), st,
                         (int)(bt->sched[i].size() & 1))))
      return rc;
  return PJZFDTD_OK;
}

}  // namespace

extern "C" {

int32_t pjzfdtd_abi_version(void) { return PJZFDTD_ABI_VERSION; }

int32_t pjzfdtd_last_error(char* buf, size_t len) {
  if (buf && len) {
    std::strncpy(buf, g_err, len - 1);
    buf[len - 1] = 0;
  }
  return g_err_code;
}

int32_t pjzfdtd_plan_create(const pjzfdtd_problem* problem,
                            const float* pml_kappa, const float* pml_sigma,
                            const float* pml_alpha, const float* weights,
                            pjzfdtd_plan** plan) {
  if (!problem || !plan) return fail(PJZFDTD_ERR_INVALID, "NULL argument");
  *plan = nullptr;
  int32_t rc = validate(*problem);
  if (rc) return rc;
  if (!pml_kappa || !pml_sigma || !pml_alpha)
    return fail(PJZFDTD_ERR_INVALID, "pml_kappa/sigma/alpha are required");
  pjzfdtd_plan* pl = new (std::nothrow) pjzfdtd_plan();
  if (!pl) return fail(PJZFDTD_ERR_INVALID, "out of host memory");
  pl->p = *problem;
  const pjzfdtd_problem& p = pl->p;
  pl->N = (long long)p.xx * p.yy * p.zz;
  pl->esz = p.storage == PJZFDTD_STORAGE_F16 ? 2 : 4;
  pl->P = p.pml_lo + p.pml_hi;
  pl->ns = (p.out_mode != PJZFDTD_OUT_NONE && p.out_stop > p.out_start)
               ? (p.out_stop - p.out_start + p.out_step - 1) / p.out_step
               : 0;
  pl->zc.assign(6 * (size_t)p.zz, 0.f);
  for (int z = 0; z < p.zz; ++z)
    for (int col = 0; col < 2; ++col) {
      const double k = pml_kappa[2 * z + col], s = pml_sigma[2 * z + col],
                   al = pml_alpha[2 * z + col];
      if (!(k > 0.0) || !(s >= 0.0) || !(al >= 0.0) || std::isnan(k) ||
          std::isinf(s) || std::isinf(al)) {
        delete pl;
        return fail(PJZFDTD_ERR_INVALID,
                    "pml coefficients at z=%d column %d must have kappa > 0 "
                    "(inf allowed), finite sigma >= 0, alpha >= 0",
                    z, col);
      }
      double ik, b, c;
      pml_coeff(k, s, al, (double)p.dt, &ik, &b, &c);
      pl->zc[(3 * col + 0) * p.zz + z] = (float)ik;
      pl->zc[(3 * col + 1) * p.zz + z] = (float)b;
      pl->zc[(3 * col + 2) * p.zz + z] = (float)c;
    }
  if (p.out_mode == PJZFDTD_OUT_PHASORS || p.out_mode == PJZFDTD_OUT_GRADIENT) {
    if (!weights) {
      delete pl;
      return fail(PJZFDTD_ERR_INVALID, "weights are required for this out_mode");
    }
    pl->weights.assign(weights, weights + (size_t)p.out_rows * pl->ns);
  }
  rc = resolve_tile(pl);
  if (rc) {
    delete pl;
    return rc;
  }
  layout(pl);
  *plan = pl;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_workspace_bytes(const pjzfdtd_plan* plan, size_t* bytes) {
  if (!plan || !bytes) return fail(PJZFDTD_ERR_INVALID, "NULL argument");
  *bytes = plan->bytes;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_num_samples(const pjzfdtd_plan* plan, int32_t* ns) {
  if (!plan || !ns) return fail(PJZFDTD_ERR_INVALID, "NULL argument");
  *ns = plan->ns;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_launch_config(const pjzfdtd_plan* plan, int32_t* tile_y,
                                   int32_t* seg_x, int32_t* threads,
                                   int32_t* steps_per_pass, int32_t* kernel,
                                   int32_t* stages) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (tile_y) *tile_y = plan->tile_y;
  if (seg_x) *seg_x = plan->seg_x > 0 ? plan->seg_x : plan->p.seg_x;
  if (threads) *threads = plan->threads;
  if (steps_per_pass) *steps_per_pass = plan->steps_per_pass;
  if (kernel) *kernel = plan->kernel;
  if (stages) *stages = plan->stages;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_status(pjzfdtd_plan* plan, void* workspace,
                            size_t workspace_bytes, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (!workspace || workspace_bytes < plan->bytes)
    return fail(PJZFDTD_ERR_WORKSPACE, "workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int* dev = at<int>(workspace, plan->off_status);
  int host = 0;
  CUDA_TRY(cudaMemcpyAsync(&host, dev, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (host != 0) {
    CUDA_TRY(cudaMemsetAsync(dev, 0, sizeof(int), st));
    return fail(PJZFDTD_ERR_TIMEOUT,
                "a device-side wait exceeded its limit (status %d)", host);
  }
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_destroy(pjzfdtd_plan* plan) {
  delete plan;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_forward(pjzfdtd_plan* plan, const pjzfdtd_buffers* buffers,
                        void* workspace, size_t workspace_bytes, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (plan->p.out_mode == PJZFDTD_OUT_GRADIENT)
    return fail(PJZFDTD_ERR_INVALID, "GRADIENT plans run through pjzfdtd_adjoint");
  return run_range(plan, buffers, workspace, workspace_bytes, 0, plan->p.tt,
                   static_cast<cudaStream_t>(stream));
}

int32_t pjzfdtd_adjoint(pjzfdtd_plan* plan, const pjzfdtd_buffers* buffers,
                        void* workspace, size_t workspace_bytes, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (plan->p.out_mode != PJZFDTD_OUT_GRADIENT)
    return fail(PJZFDTD_ERR_INVALID, "pjzfdtd_adjoint needs a GRADIENT plan");
  return run_range(plan, buffers, workspace, workspace_bytes, 0, plan->p.tt,
                   static_cast<cudaStream_t>(stream));
}

int32_t pjzfdtd_run_steps(pjzfdtd_plan* plan, const pjzfdtd_buffers* buffers,
                          void* workspace, size_t workspace_bytes,
                          int32_t step_begin, int32_t step_end, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  return run_range(plan, buffers, workspace, workspace_bytes, step_begin,
                   step_end, static_cast<cudaStream_t>(stream));
}

int32_t pjzfdtd_plan_set_monitors(pjzfdtd_plan* plan, int32_t n,
                                  const int32_t* boxes) {
  if (!plan || n < 1 || !boxes)
    return fail(PJZFDTD_ERR_INVALID, "need a plan and at least one box");
  const pjzfdtd_problem& p = plan->p;
  if (p.out_mode != PJZFDTD_OUT_SNAPSHOTS && p.out_mode != PJZFDTD_OUT_PHASORS)
    return fail(PJZFDTD_ERR_INVALID, "monitors apply to SNAPSHOTS and PHASORS plans");
  std::vector<std::array<int32_t, 6>> v;
  for (int k = 0; k < n; ++k) {
    const int32_t* b = boxes + 6 * k;
    if (b[0] < 0 || b[1] < 0 || b[2] < 0 || b[3] <= 0 || b[4] <= 0 || b[5] <= 0 ||
        b[0] + b[3] > p.xx || b[1] + b[4] > p.yy || b[2] + b[5] > p.zz)
      return fail(PJZFDTD_ERR_INVALID,
                  "monitor %d (%d, %d, %d)+(%d, %d, %d) outside the domain", k,
                  b[0], b[1], b[2], b[3], b[4], b[5]);
    v.push_back({b[0], b[1], b[2], b[3], b[4], b[5]});
  }
  plan->boxes = v;
  layout(plan);
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_output_floats(const pjzfdtd_plan* plan, size_t* floats) {
  if (!plan || !floats) return fail(PJZFDTD_ERR_INVALID, "NULL argument");
  *floats = plan->out_floats;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_batch_create(pjzfdtd_plan* const* plans, int32_t n,
                             pjzfdtd_batch** batch) {
  if (!plans || n < 1 || !batch)
    return fail(PJZFDTD_ERR_INVALID, "need at least one plan");
  *batch = nullptr;
  pjzfdtd_batch* bt = new (std::nothrow) pjzfdtd_batch();
  if (!bt) return fail(PJZFDTD_ERR_INVALID, "out of host memory");
  size_t o = 0;
  for (int i = 0; i < n; ++i) {
    pjzfdtd_plan* pl = plans[i];
    if (pl && pl->esz != 4) {
      delete bt;
      return fail(PJZFDTD_ERR_UNSUPPORTED,
                  "plan %d stores binary16; batches run FP32 storage only", i);
    }
    if (!pl || pl->kernel < 2) {
      delete bt;
      return fail(PJZFDTD_ERR_UNSUPPORTED,
                  "plan %d is not a streamed-kernel plan (zz %% 4 == 0 needed)", i);
    }
    if (pl->kernel == 3 && !pl->has_streamed) {
      delete bt;
      return fail(PJZFDTD_ERR_UNSUPPORTED,
                  "plan %d runs the lean kernel by request; batches run the "
                  "streamed kernels (kernel 0 or 2)", i);
    }
  }
  for (int i = 0; i < n; ++i) {
    pjzfdtd_plan* pl = plans[i];
    // A lean plan chosen automatically joins on its streamed plan (same
    // workspace layout) and keeps it from now on.
    if (pl->kernel == 3) {
      load_launch(pl, pl->streamed);
      pl->has_streamed = false;
    }
    bt->plans.push_back(pl);
    bt->off.push_back(o);
    o = align256(o + pl->bytes);
    bt->tt_max = std::max(bt->tt_max, pl->p.tt);
    bt->smem = std::max(bt->smem, pl->smem);
    bt->smem2 = std::max(bt->smem2, pl->smem2);
    // Segments are the requested length, else at least 4 planes long (or
    // the whole x extent; resolve_seg_x).
    const int tiles = (pl->p.yy + pl->tile_y - 1) / pl->tile_y;
    const int minseg = pl->p.seg_x > 0 ? std::min(pl->p.xx, pl->p.seg_x)
                                       : std::min(pl->p.xx, 4);
    bt->max_work += tiles * ((pl->p.xx + minseg - 1) / minseg);
  }
  bt->off_args = o;
  o = align256(o + 2 * (size_t)n * sizeof(StreamArgs));
  bt->off_work = o;
  o = align256(o + (size_t)bt->max_work * sizeof(int4));
  bt->off_sched = o;  // at most one launch per step
  o = align256(o + (size_t)bt->tt_max * n * sizeof(int2));
  bt->bytes = o;
  *batch = bt;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_batch_workspace_bytes(const pjzfdtd_batch* batch, size_t* bytes) {
  if (!batch || !bytes) return fail(PJZFDTD_ERR_INVALID, "NULL argument");
  *bytes = batch->bytes;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_batch_run(pjzfdtd_batch* batch, const pjzfdtd_buffers* buffers,
                          void* workspace, size_t workspace_bytes,
                          int32_t use_graph, void* stream) {
  if (!batch || !buffers) return fail(PJZFDTD_ERR_INVALID, "NULL argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int n = (int)batch->plans.size();
  if (!workspace || workspace_bytes < batch->bytes)
    return fail(PJZFDTD_ERR_WORKSPACE, "batch workspace of %zu bytes needed",
                batch->bytes);
  if (reinterpret_cast<uintptr_t>(workspace) % 256)
    return fail(PJZFDTD_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  if (use_graph && st == nullptr)
    return fail(PJZFDTD_ERR_INVALID,
                "graph capture needs a stream other than the legacy default");
  int32_t rc;
  for (int i = 0; i < n; ++i) {
    pjzfdtd_plan* pl = batch->plans[i];
    if ((rc = check_buffers(pl, &buffers[i], at<char>(workspace, batch->off[i]),
                            pl->bytes)))
      return rc;
    if ((rc = resolve_seg_x(pl))) return rc;
  }
  if (use_graph && batch->exec && batch->gws == workspace && batch->gstream == st) {
    bool same = true;
    for (int i = 0; i < n && same; ++i)
      same = same_buffers(batch->gbufs[i], buffers[i]);
    if (same) {
      CUDA_TRY(cudaGraphLaunch(batch->exec, st));
      return PJZFDTD_OK;
    }
  }
  // Launch schedules; work table with the problems of most launches first,
  // so that the active entries of every launch form a prefix; per-problem
  // step arguments for both buffer parities.
  batch->sched.assign(n, {});
  for (int i = 0; i < n; ++i)
    batch->sched[i] = schedule(batch->plans[i], 0, batch->plans[i]->p.tt);
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return batch->sched[a].size() > batch->sched[b].size();
  });
  std::vector<int4> work;
  std::vector<int> prefix_end(n);
  for (int r = 0; r < n; ++r) {
    const pjzfdtd_plan* pl = batch->plans[order[r]];
    const int tiles = (pl->p.yy + pl->tile_y - 1) / pl->tile_y;
    const int segs = (pl->p.xx + pl->seg_x - 1) / pl->seg_x;
    for (int t = 0; t < tiles; ++t)
      for (int sg = 0; sg < segs; ++sg) work.push_back(make_int4(order[r], t, sg, 0));
    prefix_end[r] = (int)work.size();
  }
  if ((int)work.size() > batch->max_work)
    return fail(PJZFDTD_ERR_INVALID, "work table overflow");
  const int nl = (int)batch->sched[order[0]].size();
  batch->active.assign(nl, 0);
  batch->kinds.assign(nl, 0);
  std::vector<int2> table((size_t)nl * n, make_int2(0, 0));
  for (int r = 0; r < n; ++r) {
    const int i = order[r];
    for (int j = 0; j < (int)batch->sched[i].size(); ++j) {
      batch->active[j] = prefix_end[r];
      batch->kinds[j] |= batch->sched[i][j].second;
      table[(size_t)j * n + i] =
          make_int2(batch->sched[i][j].first, batch->sched[i][j].second);
    }
  }
  std::vector<StreamArgs> args(2 * (size_t)n);
  for (int parity = 0; parity < 2; ++parity)
    for (int i = 0; i < n; ++i) {
      void* wsi = at<char>(workspace, batch->off[i]);
      const pjzfdtd_plan* pl = batch->plans[i];
      StepArgs a = step_args(pl, &buffers[i], wsi, 0, parity);
      a.wave = buffers[i].waveform;  // row 0; the kernel adds the step
      args[(size_t)parity * n + i] = stream_args(pl, wsi, a);
    }
  // Host copies (not capturable from pageable memory) happen before capture.
  CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, batch->off_args), args.data(),
                           args.size() * sizeof(StreamArgs), cudaMemcpyHostToDevice,
                           st));
  CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, batch->off_work), work.data(),
                           work.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, batch->off_sched), table.data(),
                           table.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
  for (int i = 0; i < n; ++i) {
    pjzfdtd_plan* pl = batch->plans[i];
    RunPtrs w(pl, at<char>(workspace, batch->off[i]));
    CUDA_TRY(cudaMemcpyAsync(w.zc, pl->zc.data(), pl->zc.size() * sizeof(float),
                             cudaMemcpyHostToDevice, st));
  }
  CUDA_TRY(cudaFuncSetAttribute(batch_kernel_ptr(1),
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)batch->smem));
  if (batch->smem2 > 0)
    CUDA_TRY(cudaFuncSetAttribute(batch_kernel_ptr(2),
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)batch->smem2));
  if (!use_graph) return batch_enqueue(batch, buffers, workspace, st);

  CUDA_TRY(cudaStreamSynchronize(st));  // host copies above read pageable memory
  if (batch->exec) {
    cudaGraphExecDestroy(batch->exec);
    batch->exec = nullptr;
  }
  CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  rc = batch_enqueue(batch, buffers, workspace, st);
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(st, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ec != cudaSuccess)
    return fail(PJZFDTD_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ec));
  const cudaError_t ei = cudaGraphInstantiate(&batch->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) {
    batch->exec = nullptr;
    return fail(PJZFDTD_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei));
  }
  batch->gbufs.assign(buffers, buffers + n);
  batch->gws = workspace;
  batch->gstream = st;
  CUDA_TRY(cudaGraphLaunch(batch->exec, st));
  return PJZFDTD_OK;
}

int32_t pjzfdtd_batch_destroy(pjzfdtd_batch* batch) {
  delete batch;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plane_overlaps(int32_t nterms, const float* const* blocks,
                               const float* const* profiles,
                               const int32_t* comps, const int64_t* npts,
                               int32_t ww, double* out, void* stream) {
  if (nterms < 1 || nterms > kPlaneTermsMax)
    return fail(PJZFDTD_ERR_INVALID, "plane overlaps: 1 to %d terms, got %d",
                kPlaneTermsMax, nterms);
  if (ww < 1 || ww > kSmatFreqMax || !blocks || !profiles || !comps || !npts || !out)
    return fail(PJZFDTD_ERR_INVALID, "plane overlaps: bad arguments");
  PlaneOverlapArgs a = {};
  for (int k = 0; k < nterms; ++k) {
    if (!blocks[k] || !profiles[k] || npts[k] < 1 || comps[k] < 0 || comps[k] > 2)
      return fail(PJZFDTD_ERR_INVALID, "plane overlaps: bad term %d", k);
    a.block[k] = blocks[k];
    a.prof[k] = profiles[k];
    a.npts[k] = npts[k];
    a.comp[k] = comps[k];
  }
  a.ww = ww;
  a.out = out;
  plane_overlap_kernel<<<dim3((unsigned)nterms, (unsigned)ww), kOverlapThreads, 0,
                         static_cast<cudaStream_t>(stream)>>>(a);
  CUDA_TRY(cudaGetLastError());
  return PJZFDTD_OK;
}

int32_t pjzfdtd_smatrix_gradient(int32_t n, int32_t ww, int64_t cells,
                                 const float* const* forward,
                                 const float* const* adjoint, const float* coef,
                                 const float* q, float* grad, void* stream) {
  if (n < 1 || n > kSmatSolvesMax || ww < 1 || ww > kSmatFreqMax ||
      (long long)n * n * ww > kSmatCoefMax)
    return fail(PJZFDTD_ERR_INVALID,
                "S-matrix gradient: n <= %d, ww <= %d and n*n*ww <= %d, got "
                "n=%d ww=%d", kSmatSolvesMax, kSmatFreqMax, kSmatCoefMax, n, ww);
  if (cells < 1 || !forward || !adjoint || !coef || !q || !grad)
    return fail(PJZFDTD_ERR_INVALID, "S-matrix gradient: bad arguments");
  SmatGradArgs a = {};
  for (int i = 0; i < n; ++i) {
    if (!forward[i] || !adjoint[i])
      return fail(PJZFDTD_ERR_INVALID, "S-matrix gradient: NULL phasors %d", i);
    a.F[i] = forward[i];
    a.G[i] = adjoint[i];
  }
  for (int k = 0; k < n * n * ww; ++k) {
    a.coef[k][0] = coef[2 * k];
    a.coef[k][1] = coef[2 * k + 1];
  }
  for (int w = 0; w < ww; ++w) {
    a.q[w][0] = q[2 * w];
    a.q[w][1] = q[2 * w + 1];
  }
  a.n = n;
  a.ww = ww;
  a.cells = cells;
  a.grad = grad;
  const int blocks = (int)std::min<long long>((cells + 255) / 256, 1 << 16);
  smatrix_grad_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
  CUDA_TRY(cudaGetLastError());
  return PJZFDTD_OK;
}

int32_t pjzfdtd_render_epsilon(const float* layers, int32_t ll, int32_t xx,
                               int32_t yy, int32_t zz, int32_t magnification,
                               const float* interface_positions,
                               int32_t use_simple_averaging, float* out,
                               void* stream) {
  if (!layers || !out) return fail(PJZFDTD_ERR_INVALID, "NULL layers or out");
  if (ll < 1 || ll > kRenderMaxLayers)
    return fail(PJZFDTD_ERR_INVALID, "layers must number 1 to %d, got %d",
                kRenderMaxLayers, ll);
  if (xx < 1 || yy < 1 || zz < 1 || magnification < 1)
    return fail(PJZFDTD_ERR_INVALID,
                "xx, yy, zz and magnification must be positive, got %d, %d, %d, %d",
                xx, yy, zz, magnification);
  if (ll > 1 && !interface_positions)
    return fail(PJZFDTD_ERR_INVALID, "%d interface positions needed", ll - 1);
  // x cells per CTA (their patches share rows) and layers staged together:
  // as many as keep the CTA within 36 KB of shared memory (six CTAs per
  // SM), trading x cells first; the patches' flat indices must keep
  // t * columns below 2^32 (render_div).
  const int pcol = render_patch_cols(magnification);
  auto bytes = [&](int g, int nxb) {
    return render_smem_floats(ll, zz, magnification, g, nxb) * sizeof(float);
  };
  auto exact = [&](int g, int nxb) {
    return (uint64_t)g * render_patch_rows(magnification, nxb) * pcol * (uint64_t)pcol <
           ((uint64_t)1 << 32);
  };
  int nxb = std::min(xx, kRenderMaxXCells), group = ll;
  constexpr size_t kBudget = 36 * 1024;
  while (nxb > 1 && (bytes(1, nxb) > kBudget || !exact(1, nxb))) --nxb;
  while (group > 1 && (bytes(group, nxb) > kBudget || !exact(group, nxb))) --group;
  const int prow = render_patch_rows(magnification, nxb);
  const size_t smem = bytes(group, nxb);
  const long long yblocks = ((long long)yy + kRenderTileY - 1) / kRenderTileY;
  const bool zq_exact =
      (uint64_t)kRenderTileY * (zz / 4) * (uint64_t)(zz / 4) < ((uint64_t)1 << 32);
  const bool layer_fits =  // pixel offsets within a layer are 32-bit
      (uint64_t)(2 * magnification) * xx * (uint64_t)(2 * magnification) * yy <
      ((uint64_t)1 << 31);
  if (smem > kSmemMax || !exact(group, nxb) || !zq_exact || !layer_fits ||
      yblocks > 65535)
    return fail(PJZFDTD_ERR_INVALID,
                "zz = %d with %d layers at magnification %d (or yy = %d) "
                "exceeds one CTA's reach", zz, ll, magnification, yy);
  RenderArgs a = {};
  a.layers = layers;
  a.out = out;
  a.ll = ll;
  a.xx = xx;
  a.yy = yy;
  a.zz = zz;
  a.m = magnification;
  a.simple = use_simple_averaging != 0;
  a.group = group;
  a.nxb = nxb;
  a.sorted = 1;  // nondecreasing without NaN: owners by comparison
  for (int i = 0; i + 1 < ll; ++i)
    if (interface_positions[i] != interface_positions[i] ||
        (i > 0 && !(interface_positions[i - 1] <= interface_positions[i])))
      a.sorted = 0;
  a.col_magic = render_col_magic((uint32_t)pcol);
  a.row_magic = render_col_magic((uint32_t)prow);
  a.zq_magic = zz % 4 == 0 && zz >= 8 ? render_col_magic((uint32_t)(zz / 4)) : 0;
  for (int i = 0; i + 1 < ll; ++i) a.pos[i] = interface_positions[i];
  const RenderKernel k = render_kernel_ptr();
  if (smem > 48 * 1024)
    CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  const dim3 grid((unsigned)((xx + nxb - 1) / nxb), (unsigned)yblocks);
  k<<<grid, 256, smem, static_cast<cudaStream_t>(stream)>>>(a);
  CUDA_TRY(cudaGetLastError());
  return PJZFDTD_OK;
}

}  // extern "C"

// Scratch for pjzfdtd_forward_static: a fixed device array, so a caller
// that may not allocate device memory can still run a forward solve.  Every
// GPU that loads this library holds it until the process exits.  All calls
// on a device share it and it keeps the last call's contents; the forward
// solve clears what must start at zero (fields, PML state, accumulators,
// status word) at its first step.
namespace {
constexpr size_t kStaticScratchBytes = size_t(64) << 20;  // 64 MiB
constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_ptr[kMaxDevices] = {};
}  // namespace

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace {

// Device address of the current device's scratch array.  The host cannot use
// the array's symbol as a device address, so it is looked up with the device
// current: on every call made outside a stream capture (so an address made
// stale by cudaDeviceReset is replaced), and taken from the per-device cache
// during a capture, which therefore needs one earlier call on that device.
int32_t static_scratch(cudaStream_t st, void** out) {
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(PJZFDTD_ERR_UNSUPPORTED, "device %d beyond %d", dev, kMaxDevices);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CUDA_TRY(cudaStreamIsCapturing(st, &cap));
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
    g_static_ptr[dev] = p;
  } else if (!g_static_ptr[dev]) {
    return fail(PJZFDTD_ERR_INVALID,
                "the first static-scratch call on device %d was made during a "
                "stream capture; make one call before capturing", dev);
  }
  *out = g_static_ptr[dev];
  return PJZFDTD_OK;
}

}  // namespace

extern "C" {

int32_t pjzfdtd_forward_static(pjzfdtd_plan* plan,
                               const pjzfdtd_buffers* buffers, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (plan->p.out_mode == PJZFDTD_OUT_GRADIENT)
    return fail(PJZFDTD_ERR_INVALID, "GRADIENT plans run through pjzfdtd_adjoint");
  if (plan->bytes > kStaticScratchBytes)
    return fail(PJZFDTD_ERR_WORKSPACE,
                "this plan needs %zu bytes of scratch; pjzfdtd_forward_static "
                "has a fixed %zu-byte (64 MiB) array -- use pjzfdtd_forward "
                "with a caller-allocated workspace",
                plan->bytes, kStaticScratchBytes);
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  int32_t rc = static_scratch(st, &scratch);
  if (rc) return rc;
  return run_range(plan, buffers, scratch, kStaticScratchBytes, 0, plan->p.tt, st);
}

int32_t pjzfdtd_forward_static_status(pjzfdtd_plan* plan, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (plan->bytes > kStaticScratchBytes)
    return fail(PJZFDTD_ERR_WORKSPACE,
                "this plan needs %zu bytes of scratch, more than the %zu-byte "
                "static array; it never ran through pjzfdtd_forward_static",
                plan->bytes, kStaticScratchBytes);
  void* scratch = nullptr;
  int32_t rc = static_scratch(static_cast<cudaStream_t>(stream), &scratch);
  if (rc) return rc;
  return pjzfdtd_plan_status(plan, scratch, kStaticScratchBytes, stream);
}

}  // extern "C"
