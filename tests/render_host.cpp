// Host emulation of render_epsilon_kernel (pjz_gb300/csrc/render_kernel.cuh),
// for the CPU tests: the kernel's phases (z occupancy and filling layer per
// component; per layer the staged pixel patch and the window statistics and
// one-layer values; outputs) run for every CTA with the same __host__
// __device__ functions and shared-memory carving, every profile read
// checked against its layer and every output index against the output.
// Built with g++ -ffp-contract=off so that its FP32 operations are the
// kernel's (nvcc -fmad=false).
#include <stdint.h>

#include <vector>

#define PJZ_RENDER_HOST_CHECK
#include "render_kernel.cuh"

namespace pjzfdtd {
size_t g_render_layer_floats = 0;
int g_render_bad = 0;
}  // namespace pjzfdtd

using namespace pjzfdtd;

// Returns 0, or 1 when a read or write left its array.
extern "C" int render_host(const float* layers, int ll, int xx, int yy, int zz,
                           int m, const float* pos, int simple, float* out) {
  RenderArgs a = {};
  a.layers = layers;
  a.out = out;
  a.ll = ll;
  a.xx = xx;
  a.yy = yy;
  a.zz = zz;
  a.m = m;
  a.simple = simple != 0;
  for (int i = 0; i + 1 < ll; ++i) a.pos[i] = pos[i];
  g_render_layer_floats = (size_t)(2 * m * xx) * (2 * m * yy);
  g_render_bad = 0;
  const size_t out_floats = (size_t)3 * xx * yy * zz;
  std::vector<float> sm(render_smem_floats(ll, zz, m));
  const int LZ = ll * zz, TL = kRenderTileY * ll;
  float* frac = sm.data();
  float* mid = frac + 3 * LZ;
  int* owner = reinterpret_cast<int*>(mid + 3 * LZ);
  WindowStats* st = reinterpret_cast<WindowStats*>(owner + 3 * zz);
  float* ival = reinterpret_cast<float*>(st + 3 * TL);
  int* yfin = reinterpret_cast<int*>(ival + 3 * TL);
  float* pf = reinterpret_cast<float*>(yfin + 3 * kRenderTileY);
  const int pc = render_patch_cols(m);
  const int np = render_patch_rows(m) * pc;
  float* pinv = pf + np;
  float* u = pinv + np;
  if (u + 2 * m != sm.data() + sm.size()) return 1;  // carving
  for (int x = 0; x < xx; ++x)
    for (int y0 = 0; y0 < yy; y0 += kRenderTileY) {
      const int ny = yy - y0 < kRenderTileY ? yy - y0 : kRenderTileY;
      for (int t = 0; t < 3 * zz; ++t) {
        const int c = t / zz, z = t - c * zz;
        for (int l = 0; l < ll; ++l)
          render_occupancy(a, c, l, z, &frac[c * LZ + l * zz + z],
                           &mid[c * LZ + l * zz + z]);
        owner[t] = render_owner(a, frac + c * LZ, z);
      }
      for (int t = 0; t < 3 * kRenderTileY; ++t) yfin[t] = 1;
      for (int t = 0; t < 2 * m; ++t) u[t] = render_u(a, t);
      for (int l = 0; l < ll; ++l) {
        for (int t = 0; t < np; ++t) render_stage(a, l, x, y0, ny, t, pf, pinv);
        for (int t = 0; t < 3 * ny; ++t) {
          const int c = t / ny, yl = t - c * ny;
          const int i = (c * kRenderTileY + yl) * ll + l;
          st[i] = render_window(a, c, yl, pf, pinv, pc, u);
          ival[i] = render_interior(a, c, st[i]);
          if (!render_finite(st[i])) yfin[c * kRenderTileY + yl] = 0;
        }
      }
      for (int t = 0; t < 3 * ny * zz; ++t) {
        const int c = t / (ny * zz);
        const int r = t - c * ny * zz;
        const int yl = r / zz, z = r - yl * zz;
        const int cy = c * kRenderTileY + yl;
        const size_t o = render_out_index(a, c, x, y0 + yl, z);
        if (o >= out_floats) {
          g_render_bad = 1;
          continue;
        }
        const int w = yfin[cy] ? owner[c * zz + z] : -1;
        out[o] = w >= 0 ? ival[cy * ll + w]
                        : render_value(a, c, st + cy * ll, frac + c * LZ,
                                       mid + c * LZ, z);
      }
    }
  return g_render_bad;
}
