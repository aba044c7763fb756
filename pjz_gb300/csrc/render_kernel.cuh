// Permittivity of the Yee cell from magnified layer profiles: pjz's
// `epsilon` (src/pjz/_epsilon.py:10-155) for sm_103a.
//
// Layer l of `ll` is a 2-D profile magnified 2m times in x and y, stored
// (ll, 2m*xx, 2m*yy) row-major, and lies between interfaces l-1 and l along
// z (the outer layers extend to infinity).  Each Yee component samples the
// cell it lives in:
//   * a 2m x 2m pixel window, shifted by half a cell (m pixels) along the
//     in-plane axes on which the component sits at integer positions (Ex:
//     y; Ey: x; Ez: x and y), the first m pixels repeating the edge;
//   * a z cell [z - 1/2, z + 1/2] (Ex, Ey) or [z, z + 1] (Ez).
// Per layer and window: the mean, the mean of the inverse and the
// least-squares x / y slopes (12 mean(f u), u the pixel centre's offset from
// the window centre in cells); per layer and z cell: the filled fraction and
// the filled part's offset from the cell centre, whose first moment gives
// the z slope.  With simple averaging the value is the fraction-weighted
// mean; otherwise the inverse of the mean and the mean of the inverse are
// mixed by the squared share of the component's axis in the slope vector
// (subpixel smoothing, diagonal of the interface projection only).
//
// One CTA per (x, component, block of kRenderTileY y cells): it tabulates
// the z occupancy of its component's cells and the window statistics of its
// y cells in shared memory, then writes its (y, z) outputs with z fastest.
// A z cell that lies wholly inside one layer (its fraction exactly 1, all
// others exactly 0) has the same value at every such z of a column: it is
// computed once per (y, layer) and copied, and only the cells an interface
// cuts take the full mix.  Both give the same floats when every layer's
// window statistics at that (x, y) are finite (the full mix then adds exact
// zeros to that layer's terms); where one is not (a zero pixel makes the
// mean of the inverse infinite, a NaN pixel makes everything NaN), 0 * inf
// in the full mix gives NaN as pjz's einsum does, so such columns take the
// full mix at every z.  FP32 throughout; the per-cell
// functions are __host__ __device__ so that a host emulation of the block
// loop checks the same code on the CPU.
#pragma once

#include <math.h>
#include <stddef.h>

#ifdef __CUDACC__
#define PJZ_HD __host__ __device__ __forceinline__
#else
#define PJZ_HD inline
#endif

namespace pjzfdtd {

constexpr int kRenderMaxLayers = 16;
constexpr int kRenderTileY = 32;

struct RenderArgs {
  const float* layers;  // (ll, 2m*xx, 2m*yy)
  float* out;           // (3, xx, yy, zz)
  int ll, xx, yy, zz, m, simple;
  float pos[kRenderMaxLayers - 1];  // interface positions, increasing
};

struct WindowStats {
  float mean, inv, gx, gy;
};

#ifdef PJZ_RENDER_HOST_CHECK
// Host emulation only: every profile read is checked against the layer.
extern size_t g_render_layer_floats;
extern int g_render_bad;
PJZ_HD float render_load(const float* layer, size_t i) {
  if (i >= g_render_layer_floats) {
    g_render_bad = 1;
    return 1.0f;
  }
  return layer[i];
}
#else
PJZ_HD float render_load(const float* layer, size_t i) { return layer[i]; }
#endif

PJZ_HD int render_imax(int a, int b) { return a > b ? a : b; }

// Shared-memory floats of one CTA: occupancy [2][ll][zz], the layer that
// fills each z cell [zz] (int, -1 when an interface cuts it), statistics
// [kRenderTileY][ll] of 4 floats, one-layer values [kRenderTileY][ll], and
// per y cell whether every layer's statistics are finite [kRenderTileY]
// (int).
PJZ_HD size_t render_smem_floats(int ll, int zz) {
  return 2 * (size_t)ll * zz + zz + 5 * (size_t)kRenderTileY * ll + kRenderTileY;
}

PJZ_HD bool render_finite(const WindowStats& w) {
  return isfinite(w.mean) && isfinite(w.inv) && isfinite(w.gx) && isfinite(w.gy);
}

// Filled fraction of z cell `z` of component `c` by layer `l`, and the
// offset of the filled part's midpoint from the cell centre.
PJZ_HD void render_occupancy(const RenderArgs& a, int c, int l, int z,
                             float* frac, float* mid) {
  const float lo = c == 2 ? (float)z : (float)z - 0.5f;
  const float hi = c == 2 ? (float)z + 1.0f : (float)z + 0.5f;
  const float b = l == 0 ? lo : fminf(fmaxf(a.pos[l - 1], lo), hi);
  const float t = l == a.ll - 1 ? hi : fminf(fmaxf(a.pos[l], lo), hi);
  *frac = (t - b) / (hi - lo);
  *mid = 0.5f * (b + t) - 0.5f * (lo + hi);
}

// Statistics of layer `l` over the pixel window of component `c` at (x, y).
PJZ_HD WindowStats render_window(const RenderArgs& a, int c, int l, int x, int y) {
  const int k = 2 * a.m;
  const int PX = k * a.xx, PY = k * a.yy;
  const int sx = c != 0 ? a.m : 0, sy = c != 1 ? a.m : 0;
  const float* L = a.layers + (size_t)l * PX * PY;
  const float c0 = (float)a.m - 0.5f;
  float s = 0.f, si = 0.f, sxu = 0.f, syu = 0.f;
  for (int i = 0; i < k; ++i) {
    const int px = render_imax(k * x + i - sx, 0);
    const float ui = ((float)i - c0) / (float)k;
    for (int j = 0; j < k; ++j) {
      const int py = render_imax(k * y + j - sy, 0);
      const float uj = ((float)j - c0) / (float)k;
      const float f = render_load(L, (size_t)px * PY + py);
      s += f;
      si += 1.0f / f;
      sxu += f * ui;
      syu += f * uj;
    }
  }
  const float n = (float)(k * k);
  WindowStats w;
  w.mean = s / n;
  w.inv = si / n;
  w.gx = 12.0f * sxu / n;
  w.gy = 12.0f * syu / n;
  return w;
}

// The value from the fraction-weighted sums over the layers.
PJZ_HD float render_mix(const RenderArgs& a, int c, float avg, float inv,
                        float gx, float gy, float gz) {
  if (a.simple) return avg;
  gz = 12.0f * gz;  // first moment over the unit cell's second moment 1/12
  const float norm = gx * gx + gy * gy + gz * gz;
  const float g = c == 0 ? gx : (c == 1 ? gy : gz);
  const float p = norm == 0.0f ? 0.0f : g * g / norm;
  return 1.0f / (p * inv + (1.0f - p) / avg);
}

// Value of component `c` at z from the window statistics of its (x, y)
// (st[l]) and the occupancy of its z cells (frac / mid [l * zz + z]).
PJZ_HD float render_value(const RenderArgs& a, int c, const WindowStats* st,
                          const float* frac, const float* mid, int z) {
  float avg = 0.f, inv = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
  for (int l = 0; l < a.ll; ++l) {
    const float f = frac[l * a.zz + z];
    avg += st[l].mean * f;
    inv += st[l].inv * f;
    gx += st[l].gx * f;
    gy += st[l].gy * f;
    gz += st[l].mean * f * mid[l * a.zz + z];
  }
  return render_mix(a, c, avg, inv, gx, gy, gz);
}

// Value of a z cell that one layer fills: render_value with that layer's
// fraction 1, midpoint offset 0 and every other fraction 0 (each sum then
// holds that layer's term alone, and the z moment +0).
PJZ_HD float render_interior(const RenderArgs& a, int c, const WindowStats& w) {
  return render_mix(a, c, 0.f + w.mean, 0.f + w.inv, 0.f + w.gx, 0.f + w.gy, 0.f);
}

// The layer whose fraction of z cell `z` is exactly 1, else -1.
PJZ_HD int render_owner(const RenderArgs& a, const float* frac, int z) {
  for (int l = 0; l < a.ll; ++l)
    if (frac[l * a.zz + z] == 1.0f) return l;
  return -1;
}

PJZ_HD size_t render_out_index(const RenderArgs& a, int c, int x, int y, int z) {
  return (((size_t)c * a.xx + x) * a.yy + y) * a.zz + z;
}

#if defined(__CUDACC__) && defined(PJZ_RENDER_KERNEL)  // kern_render.cu only
// grid (xx, 3, ceil(yy / kRenderTileY)); dynamic shared memory
// render_smem_floats(ll, zz) floats.
__global__ void __launch_bounds__(256) render_epsilon_kernel(const RenderArgs a) {
  extern __shared__ __align__(16) float rsm[];
  const int x = blockIdx.x, c = blockIdx.y, y0 = blockIdx.z * kRenderTileY;
  const int ny = min(kRenderTileY, a.yy - y0);
  float* frac = rsm;
  float* mid = frac + a.ll * a.zz;
  int* owner = reinterpret_cast<int*>(mid + a.ll * a.zz);
  WindowStats* st = reinterpret_cast<WindowStats*>(owner + a.zz);
  float* ival = reinterpret_cast<float*>(st + kRenderTileY * a.ll);
  int* yfin = reinterpret_cast<int*>(ival + kRenderTileY * a.ll);
  for (int z = threadIdx.x; z < a.zz; z += blockDim.x) {
    for (int l = 0; l < a.ll; ++l)
      render_occupancy(a, c, l, z, &frac[l * a.zz + z], &mid[l * a.zz + z]);
    owner[z] = render_owner(a, frac, z);
  }
  if (threadIdx.x < kRenderTileY) yfin[threadIdx.x] = 1;
  __syncthreads();
  for (int i = threadIdx.x; i < ny * a.ll; i += blockDim.x) {
    st[i] = render_window(a, c, i % a.ll, x, y0 + i / a.ll);
    ival[i] = render_interior(a, c, st[i]);
    if (!render_finite(st[i])) yfin[i / a.ll] = 0;  // every writer stores 0
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ny * a.zz; i += blockDim.x) {
    const int yl = i / a.zz, z = i - yl * a.zz;
    const int o = yfin[yl] ? owner[z] : -1;
    a.out[render_out_index(a, c, x, y0 + yl, z)] =
        o >= 0 ? ival[yl * a.ll + o] : render_value(a, c, st + yl * a.ll, frac, mid, z);
  }
}
#endif

}  // namespace pjzfdtd
