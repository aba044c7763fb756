// Host emulation of render_epsilon_kernel (pjz_gb300/csrc/render_kernel.cuh),
// for the CPU tests: every CTA runs the kernel's phase functions, with its
// shared-memory carving, for each of 256 threads in turn between the
// kernel's barriers; every profile read is checked against its layer and
// guard zones around the output catch a write outside it.  Built with g++
// -ffp-contract=off so that its FP32 operations are the kernel's (nvcc
// -fmad=false).
#include <stdint.h>
#include <string.h>

#include <vector>

#define PJZ_RENDER_HOST_CHECK
#include "render_kernel.cuh"

namespace pjzfdtd {
size_t g_render_layer_floats = 0;
int g_render_bad = 0;
}  // namespace pjzfdtd

using namespace pjzfdtd;

namespace {
constexpr int kThreads = 256;
constexpr size_t kGuard = 4096;
constexpr uint32_t kSentinel = 0x7fc0dead;  // a NaN no output takes
}  // namespace

// Stages `group` layers at a time (0: all) for `nxb` x cells per CTA.
// Returns 0, or 1 when a read or write left its array.
extern "C" int render_host(const float* layers, int ll, int xx, int yy, int zz,
                           int m, const float* pos, int simple, int group, int nxb,
                           float* out) {
  const size_t out_floats = (size_t)3 * xx * yy * zz;
  std::vector<float> guarded(out_floats + 2 * kGuard);
  for (float& v : guarded) memcpy(&v, &kSentinel, 4);
  RenderArgs a = {};
  a.layers = layers;
  a.out = guarded.data() + kGuard;
  a.ll = ll;
  a.xx = xx;
  a.yy = yy;
  a.zz = zz;
  a.m = m;
  a.simple = simple != 0;
  a.group = group > 0 && group < ll ? group : ll;
  a.nxb = nxb > 0 ? nxb : 1;
  a.sorted = 1;
  for (int i = 0; i + 1 < ll; ++i)
    if (pos[i] != pos[i] || (i > 0 && !(pos[i - 1] <= pos[i]))) a.sorted = 0;
  a.col_magic = render_col_magic((uint32_t)render_patch_cols(m));
  a.row_magic = render_col_magic((uint32_t)render_patch_rows(m, a.nxb));
  a.zq_magic = zz % 4 == 0 && zz >= 8 ? render_col_magic((uint32_t)(zz / 4)) : 0;
  for (int i = 0; i + 1 < ll; ++i) a.pos[i] = pos[i];
  g_render_layer_floats = (size_t)(2 * m * xx) * (2 * m * yy);
  g_render_bad = 0;
  std::vector<float> sm(render_smem_floats(ll, zz, m, a.group, a.nxb));
  const RenderSmem s = render_carve(sm.data(), ll, zz, m, a.group, a.nxb);
  if (s.end != sm.data() + sm.size()) return 1;  // carving
  for (int x0 = 0; x0 < xx; x0 += a.nxb)
    for (int y0 = 0; y0 < yy; y0 += kRenderTileY) {
      const int nx = xx - x0 < a.nxb ? xx - x0 : a.nxb;
      const int ny = yy - y0 < kRenderTileY ? yy - y0 : kRenderTileY;
      for (int t = 0; t < kThreads; ++t) render_phase_setup(a, s, t, kThreads);
      for (int t = 0; t < kThreads; ++t) render_phase_occupancy(a, s, t, kThreads);
      for (int t = 0; t < kThreads; ++t) render_phase_cuts(a, s, t, kThreads);
      for (int l0 = 0; l0 < ll; l0 += a.group) {
        const int ng = a.group < ll - l0 ? a.group : ll - l0;
        for (int t = 0; t < kThreads; ++t)
          render_phase_stage(a, s, l0, ng, x0, nx, y0, ny, t, kThreads);
        for (int t = 0; t < kThreads; ++t)
          render_phase_windows(a, s, l0, ng, nx, ny, t, kThreads);
      }
      for (int t = 0; t < kThreads; ++t)
        render_phase_out(a, s, x0, nx, y0, ny, t >> 5, kThreads >> 5, t & 31, a.out);
      for (int t = 0; t < kThreads; ++t)
        render_phase_cut_cells(a, s, x0, nx, y0, ny, t, kThreads, a.out);
    }
  for (size_t i = 0; i < kGuard; ++i) {
    uint32_t lo, hi;
    memcpy(&lo, &guarded[i], 4);
    memcpy(&hi, &guarded[kGuard + out_floats + i], 4);
    if (lo != kSentinel || hi != kSentinel) g_render_bad = 1;
  }
  memcpy(out, a.out, out_floats * sizeof(float));
  return g_render_bad;
}

// Number of (component, z) cells, z in [zlo, zhi), whose owner by
// comparison differs from the owner by exact fractions, for `ll` layers
// with interface positions `pos` (nondecreasing, no NaN).
extern "C" int render_owner_mismatches(const float* pos, int ll, int zlo, int zhi) {
  RenderArgs a = {};
  a.ll = ll;
  int bad = 0;
  for (int c = 0; c < 3; ++c)
    for (int z = zlo; z < zhi; ++z)
      bad += render_owner(a, pos, c, z) != render_owner_sorted(a, pos, c, z);
  return bad;
}
