// Host emulation of render_epsilon_kernel (pjz_gb300/csrc/render_kernel.cuh),
// for the CPU tests: the kernel's three phases (z occupancy and filling
// layer, window statistics and one-layer values, outputs) run for every CTA
// with the same __host__ __device__ functions and shared-memory carving,
// every profile read checked against its layer and every output index
// against the output.  Built with g++ -ffp-contract=off so that its FP32
// operations are the kernel's (nvcc -fmad=false).
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
  std::vector<float> sm(render_smem_floats(ll, zz));
  float* frac = sm.data();
  float* mid = frac + ll * zz;
  int* owner = reinterpret_cast<int*>(mid + ll * zz);
  WindowStats* st = reinterpret_cast<WindowStats*>(owner + zz);
  float* ival = reinterpret_cast<float*>(st + kRenderTileY * ll);
  int* yfin = reinterpret_cast<int*>(ival + kRenderTileY * ll);
  if (reinterpret_cast<float*>(yfin + kRenderTileY) != sm.data() + sm.size())
    return 1;  // carving
  for (int c = 0; c < 3; ++c)
    for (int x = 0; x < xx; ++x)
      for (int y0 = 0; y0 < yy; y0 += kRenderTileY) {
        const int ny = yy - y0 < kRenderTileY ? yy - y0 : kRenderTileY;
        for (int z = 0; z < zz; ++z) {
          for (int l = 0; l < ll; ++l)
            render_occupancy(a, c, l, z, &frac[l * zz + z], &mid[l * zz + z]);
          owner[z] = render_owner(a, frac, z);
        }
        for (int i = 0; i < kRenderTileY; ++i) yfin[i] = 1;
        for (int i = 0; i < ny * ll; ++i) {
          st[i] = render_window(a, c, i % ll, x, y0 + i / ll);
          ival[i] = render_interior(a, c, st[i]);
          if (!render_finite(st[i])) yfin[i / ll] = 0;
        }
        for (int i = 0; i < ny * zz; ++i) {
          const int yl = i / zz, z = i - yl * zz;
          const size_t o = render_out_index(a, c, x, y0 + yl, z);
          if (o >= out_floats) {
            g_render_bad = 1;
            continue;
          }
          const int w = yfin[yl] ? owner[z] : -1;
          out[o] = w >= 0 ? ival[yl * ll + w]
                          : render_value(a, c, st + yl * ll, frac, mid, z);
        }
      }
  return g_render_bad;
}
