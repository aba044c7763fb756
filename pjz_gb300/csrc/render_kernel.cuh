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
// One CTA per (x, block of kRenderTileY y cells), all three components.
// It tabulates the layer that fills each component's z cells, then, a group of
// layers at a time (as many as the host fits in shared memory), stages the
// layers' pixel patches that the block's windows cover (3m rows x
// (2m*ny + m) columns each, edge pixels repeated) with each pixel's
// reciprocal computed once, computes every window's statistics from the
// patches, and finally writes the (component, y, z) outputs with z fastest,
// coalesced.  With interface positions in nondecreasing order, a z cell
// that lies wholly inside one layer (its fraction exactly 1, all others
// exactly 0) has the same value at every such z of a column: it is
// computed once per (y, layer) and copied, and only the cells an interface
// cuts take the full mix (out-of-order or NaN positions: every cell).  Both give the
// same floats when every layer's window statistics at that (x, y) are
// finite (the full mix then adds exact zeros to that layer's terms); where
// one is not (a zero pixel makes the mean of the inverse infinite, a NaN
// pixel makes everything NaN), 0 * inf in the full mix gives NaN as pjz's
// einsum does, so such columns take the full mix at every z.  FP32
// throughout, the window sums in the order of the original per-window loop
// (rows outer, columns inner).  The CTA's phases are __host__ __device__
// strided loops over (thread, thread count), with no integer division in
// their index arithmetic, so that a host emulation runs the kernel's own
// code, thread by thread, on the CPU.
#pragma once

#include <math.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __CUDACC__
#define PJZ_HD __host__ __device__ __forceinline__
#define PJZ_UNROLL _Pragma("unroll")
#else
#define PJZ_HD inline
#define PJZ_UNROLL
#endif

namespace pjzfdtd {

constexpr int kRenderMaxLayers = 16;
constexpr int kRenderTileY = 32;
// x cells per CTA at most (512x512x64, 3 layers at 2x: 0.132 ms with 2 and
// a 36 KB budget, 0.137 with 2 at 48 KB, 0.149 with 4, 0.153 with 1).
constexpr int kRenderMaxXCells = 2;

struct RenderArgs {
  const float* layers;  // (ll, 2m*xx, 2m*yy)
  float* out;           // (3, xx, yy, zz)
  int ll, xx, yy, zz, m, simple;
  int group;            // layers staged together (1 .. ll)
  int nxb;              // x cells per CTA (their patches share rows)
  int sorted;           // positions nondecreasing and free of NaN
  uint32_t col_magic;   // render_col_magic(patch columns)
  uint32_t row_magic;   // render_col_magic(patch rows)
  uint32_t zq_magic;    // render_col_magic(zz / 4), when render_quads
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

// Pixel patch of one CTA and layer: for x cells x0 .. x0 + nx - 1, rows
// k*x0 - m .. k*(x0 + nx) - 1 and columns k*y0 - m .. k*(y0 + ny) - 1 (k =
// 2m), negative indices repeating the edge pixel; cell x0 + i reads rows
// k*i .. k*i + 3m - 1 of it.
PJZ_HD int render_patch_rows(int m, int nx) { return 2 * m * nx + m; }
PJZ_HD int render_patch_cols(int m) { return 2 * m * kRenderTileY + m; }

// t / d for the patches' flat indices: floor(t * ceil(2^32 / d) / 2^32)
// equals floor(t / d) while t * d < 2^32, which the host's limits keep.
// d >= 2, so the magic fits 32 bits.
PJZ_HD uint32_t render_col_magic(uint32_t d) {
  return (uint32_t)((((uint64_t)1 << 32) + d - 1) / d);
}
PJZ_HD int render_div(int t, uint32_t magic) {
#ifdef __CUDA_ARCH__
  return (int)__umulhi((uint32_t)t, magic);
#else
  return (int)(((uint64_t)(uint32_t)t * magic) >> 32);
#endif
}

// Shared-memory floats of one CTA staging `group` layers at once: the layer
// that fills each z cell [3][zz] (int, -1 when an interface cuts it),
// window statistics [3][kRenderTileY][ll] of 4
// floats, one-layer values [3][kRenderTileY][ll], per (component, y)
// whether every layer's statistics are finite [3][kRenderTileY] (int), the
// pixel patches and their reciprocals [2][group][3m][2m*kRenderTileY + m],
// the pixel offsets u [2m], the interface positions [kRenderMaxLayers], and
// per component the z cells an interface cuts [3][zz] (int) and their
// count [4] (int).
PJZ_HD size_t render_smem_floats(int ll, int zz, int m, int group, int nxb) {
  return 3 * (size_t)zz + 15 * (size_t)nxb * kRenderTileY * ll +
         3 * (size_t)nxb * kRenderTileY +
         2 * (size_t)group * render_patch_rows(m, nxb) * render_patch_cols(m) +
         2 * m + kRenderMaxLayers + 3 * (size_t)zz + 4;
}

// The regions of one CTA's shared memory (render_smem_floats floats).
struct RenderSmem {
  int* owner;       // [3][zz]
  WindowStats* st;  // [nxb][3][kRenderTileY][ll]
  float* ival;      // [nxb][3][kRenderTileY][ll]
  int* yfin;        // [nxb][3][kRenderTileY]
  float* pf;        // [group][2m*nxb + m][pc]
  float* pinv;      // [group][2m*nxb + m][pc]
  float* u;         // [2m]
  float* pos;       // [kRenderMaxLayers]
  int* cut;         // [3][zz]: z cells no single layer fills
  int* ncut;        // [4]: their number per component
  float* end;
};

PJZ_HD RenderSmem render_carve(float* sm, int ll, int zz, int m, int group,
                              int nxb) {
  const int TL = nxb * kRenderTileY * ll;
  const int np = group * render_patch_rows(m, nxb) * render_patch_cols(m);
  RenderSmem s;
  s.owner = reinterpret_cast<int*>(sm);
  s.st = reinterpret_cast<WindowStats*>(s.owner + 3 * zz);
  s.ival = reinterpret_cast<float*>(s.st + 3 * TL);
  s.yfin = reinterpret_cast<int*>(s.ival + 3 * TL);
  s.pf = reinterpret_cast<float*>(s.yfin + 3 * nxb * kRenderTileY);
  s.pinv = s.pf + np;
  s.u = s.pinv + np;
  s.pos = s.u + 2 * m;
  s.cut = reinterpret_cast<int*>(s.pos + kRenderMaxLayers);
  s.ncut = s.cut + 3 * zz;
  s.end = reinterpret_cast<float*>(s.ncut + 4);
  return s;
}

PJZ_HD bool render_finite(const WindowStats& w) {
  return isfinite(w.mean) && isfinite(w.inv) && isfinite(w.gx) && isfinite(w.gy);
}

// Filled fraction of z cell `z` of component `c` by layer `l`, and the
// offset of the filled part's midpoint from the cell centre.
// `pos` holds the interface positions.
// Clamp to [lo, hi] that keeps NaN (as pjz's jnp.clip does).
PJZ_HD float render_clip(float v, float lo, float hi) {
  return v != v ? v : fminf(fmaxf(v, lo), hi);
}

PJZ_HD void render_occupancy(const RenderArgs& a, const float* pos, int c, int l,
                             int z, float* frac, float* mid) {
  const float lo = c == 2 ? (float)z : (float)z - 0.5f;
  const float hi = c == 2 ? (float)z + 1.0f : (float)z + 0.5f;
  const float b = l == 0 ? lo : render_clip(pos[l - 1], lo, hi);
  const float t = l == a.ll - 1 ? hi : render_clip(pos[l], lo, hi);
  *frac = (t - b) / (hi - lo);
  *mid = 0.5f * (b + t) - 0.5f * (lo + hi);
}

// Offset of pixel i of a window from the window centre, in cells.
PJZ_HD float render_u(const RenderArgs& a, int i) {
  const float c0 = (float)a.m - 0.5f;
  return ((float)i - c0) / (float)(2 * a.m);
}

// Statistics of one layer over the pixel window of component `c` at tile
// row yl, from the staged patch `pf` (pixels) and `pinv` (their
// reciprocals) with row stride `pc`; `u` holds render_u of 0 .. 2m-1.
// MC > 0: the magnification as a compile-time constant (same operations
// in the same order, loops unrolled); MC = 0 takes a.m.
template <int MC>
PJZ_HD WindowStats render_window_m(const RenderArgs& a, int c, int yl,
                                   const float* pf, const float* pinv, int pc,
                                   const float* u) {
  const int m = MC > 0 ? MC : a.m;
  const int k = 2 * m;
  const int ioff = c == 0 ? m : 0;           // rows shifted unless Ex
  const int joff = k * yl + (c == 1 ? m : 0);  // columns shifted unless Ey
  float s = 0.f, si = 0.f, sxu = 0.f, syu = 0.f;
PJZ_UNROLL
  for (int i = 0; i < k; ++i) {
    const float ui = u[i];
    const float* rf = pf + (i + ioff) * pc + joff;
    const float* ri = pinv + (i + ioff) * pc + joff;
PJZ_UNROLL
    for (int j = 0; j < k; ++j) {
      const float f = rf[j];
      s += f;
      si += ri[j];
      sxu += f * ui;
      syu += f * u[j];
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

PJZ_HD WindowStats render_window(const RenderArgs& a, int c, int yl,
                                 const float* pf, const float* pinv, int pc,
                                 const float* u) {
  switch (a.m) {
    case 1: return render_window_m<1>(a, c, yl, pf, pinv, pc, u);
    case 2: return render_window_m<2>(a, c, yl, pf, pinv, pc, u);
    case 3: return render_window_m<3>(a, c, yl, pf, pinv, pc, u);
    case 4: return render_window_m<4>(a, c, yl, pf, pinv, pc, u);
    default: return render_window_m<0>(a, c, yl, pf, pinv, pc, u);
  }
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
// (st[l]) and the occupancy of its z cell by each layer (interface
// positions `pos`).
PJZ_HD float render_value(const RenderArgs& a, const float* pos, int c,
                          const WindowStats* st, int z) {
  float avg = 0.f, inv = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
  for (int l = 0; l < a.ll; ++l) {
    float f, mid;
    render_occupancy(a, pos, c, l, z, &f, &mid);
    avg += st[l].mean * f;
    inv += st[l].inv * f;
    gx += st[l].gx * f;
    gy += st[l].gy * f;
    gz += st[l].mean * f * mid;
  }
  return render_mix(a, c, avg, inv, gx, gy, gz);
}

// Value of a z cell that one layer fills: render_value with that layer's
// fraction 1, midpoint offset 0 and every other fraction 0 (each sum then
// holds that layer's term alone, and the z moment +0).
PJZ_HD float render_interior(const RenderArgs& a, int c, const WindowStats& w) {
  return render_mix(a, c, 0.f + w.mean, 0.f + w.inv, 0.f + w.gx, 0.f + w.gy, 0.f);
}

// The layer whose fraction of z cell `z` of component `c` is exactly 1,
// else -1 (the definition render_owner_sorted is tested against).
PJZ_HD int render_owner(const RenderArgs& a, const float* pos, int c, int z) {
  for (int l = 0; l < a.ll; ++l) {
    float f, mid;
    render_occupancy(a, pos, c, l, z, &f, &mid);
    if (f == 1.0f) return l;
  }
  return -1;
}

// render_owner for nondecreasing positions without NaN, by comparisons:
// with no interface strictly inside the cell (lo, hi) the layer above the
// k interfaces at or below lo spans it (fraction (hi - lo) / (hi - lo) = 1,
// every other layer 0); with one inside, every layer stops short of lo or
// hi and the fractions are exact differences below 1.
PJZ_HD int render_owner_sorted(const RenderArgs& a, const float* pos, int c, int z) {
  const float lo = c == 2 ? (float)z : (float)z - 0.5f;
  const float hi = c == 2 ? (float)z + 1.0f : (float)z + 0.5f;
  int k = 0;
  bool cut = false;
  for (int i = 0; i + 1 < a.ll; ++i) {
    k += pos[i] <= lo;
    cut |= pos[i] > lo && pos[i] < hi;
  }
  return cut ? -1 : k;
}

PJZ_HD size_t render_out_index(const RenderArgs& a, int c, int x, int y, int z) {
  return (((size_t)c * a.xx + x) * a.yy + y) * a.zz + z;
}

// Whether the outputs go out four z cells at a time (16-byte stores): zz a
// multiple of 4 (at least 8) and a 16-byte aligned output.
PJZ_HD bool render_quads(const RenderArgs& a, const float* out) {
  return a.zz % 4 == 0 && a.zz >= 8 && reinterpret_cast<uintptr_t>(out) % 16 == 0;
}

// Four consecutive owners (16-byte aligned: zz % 4 == 0 and z % 4 == 0).
PJZ_HD void render_owner4(const int* p, int o[4]) {
#ifdef __CUDA_ARCH__
  const int4 v = *reinterpret_cast<const int4*>(p);
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
  o[3] = v.w;
#else
  for (int j = 0; j < 4; ++j) o[j] = p[j];
#endif
}

PJZ_HD void render_store4(float* p, const float v[4]) {
#ifdef __CUDA_ARCH__
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
#else
  for (int j = 0; j < 4; ++j) p[j] = v[j];
#endif
}

// The CTA's phases, each a strided loop of thread `tid` of `nthr` (a
// barrier between consecutive phases), shared by the kernel and its host
// emulation.  Phase 1: interface positions, pixel offsets, finiteness
// flags.
PJZ_HD void render_phase_setup(const RenderArgs& a, const RenderSmem& s, int tid,
                               int nthr) {
  if (tid == 0) {  // constant indices: the arguments stay in parameter space
PJZ_UNROLL
    for (int i = 0; i < kRenderMaxLayers - 1; ++i)
      s.pos[i] = i < a.ll - 1 ? a.pos[i] : 0.f;
    s.pos[kRenderMaxLayers - 1] = 0.f;
  }
  for (int t = tid; t < 2 * a.m; t += nthr) s.u[t] = render_u(a, t);
  for (int t = tid; t < 3 * a.nxb * kRenderTileY; t += nthr) s.yfin[t] = 1;
}

// Phase 2 (after the positions are in shared memory): the filling layer of
// every component's z cells.  Out-of-order (or NaN) positions make some
// layers' fractions negative or NaN, so no cell has a single owner there:
// every cell takes the full mix.
PJZ_HD void render_phase_occupancy(const RenderArgs& a, const RenderSmem& s,
                                   int tid, int nthr) {
  for (int t = tid; t < 3 * a.zz; t += nthr) {
    const int c = t >= 2 * a.zz ? 2 : (t >= a.zz ? 1 : 0), z = t - c * a.zz;
    s.owner[t] = a.sorted ? render_owner_sorted(a, s.pos, c, z) : -1;
  }
}

// Phase 3 (beside the first group's staging, after a barrier that follows
// phase 2): per component, the z cells no single layer fills, in increasing
// z.  On the device warp c (c < 3) compacts component c with ballots; the
// host walks z in order, which gives the same list.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ void render_phase_cuts(const RenderArgs& a,
                                                  const RenderSmem& s, int tid,
                                                  int nthr) {
  const int c = tid >> 5, lane = tid & 31;
  if (c >= 3) return;
  int n = 0;
  for (int z0 = 0; z0 < a.zz; z0 += 32) {
    const int z = z0 + lane;
    const bool f = z < a.zz && s.owner[c * a.zz + z] < 0;
    const unsigned m = __ballot_sync(0xffffffffu, f);
    if (f) s.cut[c * a.zz + n + __popc(m & ((1u << lane) - 1u))] = z;
    n += __popc(m);
  }
  if (lane == 0) s.ncut[c] = n;
}
#else
inline void render_phase_cuts(const RenderArgs& a, const RenderSmem& s, int tid,
                              int nthr) {
  for (int c = tid; c < 3; c += nthr) {
    int n = 0;
    for (int z = 0; z < a.zz; ++z)
      if (s.owner[c * a.zz + z] < 0) s.cut[c * a.zz + n++] = z;
    s.ncut[c] = n;
  }
}
#endif

// Phase 4, per group of layers l0 .. l0 + ng - 1: their pixel patches for
// the CTA at (x, y0) with ny tile rows (the columns its windows cover:
// 2m*ny + m), one flat index over (layer, row, column).  Each thread
// issues the loads of kRenderStageBatch of its pixels before it uses any,
// so their memory latencies overlap instead of adding up.
constexpr int kRenderStageBatch = 8;

PJZ_HD void render_phase_stage(const RenderArgs& a, const RenderSmem& s, int l0,
                               int ng, int x0, int nx, int y0, int ny, int tid,
                               int nthr) {
  const int k = 2 * a.m, pc = render_patch_cols(a.m);
  const int PR = render_patch_rows(a.m, a.nxb);  // rows per layer's patch
  const int cols = k * ny + a.m, rows = ng * PR;
  const int live_rows = render_patch_rows(a.m, nx);
  const int PX = k * a.xx, PY = k * a.yy;
  const int n = rows * pc;
  const float* L0 = a.layers + (size_t)l0 * PX * PY;
  for (int t0 = tid; t0 < n; t0 += kRenderStageBatch * nthr) {
    float f[kRenderStageBatch];
    unsigned live = 0;  // bit b: pixel t0 + b * nthr is staged
PJZ_UNROLL
    for (int b = 0; b < kRenderStageBatch; ++b) {
      const int t = t0 + b * nthr;
      const int gr = render_div(t, a.col_magic);  // (layer, row) of the group
      const int cc = t - gr * pc;
      f[b] = 0.f;
      const int g = render_div(gr, a.row_magic);  // layer of the group
      const int r = gr - g * PR;
      if (t < n && cc < cols && r < live_rows) {
        const int px = render_imax(k * x0 - a.m + r, 0);
        const int py = render_imax(k * y0 - a.m + cc, 0);
        // One layer holds fewer than 2^31 pixels (checked by the host).
        f[b] = render_load(L0 + (size_t)g * PX * PY, (size_t)(px * PY + py));
        live |= 1u << b;
      }
    }
PJZ_UNROLL
    for (int b = 0; b < kRenderStageBatch; ++b) {
      const int t = t0 + b * nthr;
      if (live >> b & 1u) {
        s.pf[t] = f[b];
        s.pinv[t] = 1.0f / f[b];
      }
    }
  }
}

// Row of the (x cell, component, y cell) statistics of a CTA.
PJZ_HD int render_cy(int xi, int c, int yl) { return (3 * xi + c) * kRenderTileY + yl; }

// Phase 5, per group: window statistics and one-layer values of the
// (x cell, layer, component, row) windows of the staged patches.
PJZ_HD void render_phase_windows(const RenderArgs& a, const RenderSmem& s, int l0,
                                 int ng, int nx, int ny, int tid, int nthr) {
  const int pc = render_patch_cols(a.m);
  const int np1 = render_patch_rows(a.m, a.nxb) * pc;  // one layer's patch
  const int per = 3 * ny * ng;                         // items per x cell
  for (int t = tid; t < nx * per; t += nthr) {
    int xi = 0, r = t;
    while (r >= per) {  // nx is small: at most a.nxb
      r -= per;
      ++xi;
    }
    int g = 0;
    while (r >= 3 * ny) {  // ng is small: at most kRenderMaxLayers
      r -= 3 * ny;
      ++g;
    }
    const int c = r >= 2 * ny ? 2 : (r >= ny ? 1 : 0), yl = r - c * ny;
    const int cy = render_cy(xi, c, yl);
    const int i = cy * a.ll + l0 + g;
    const int off = g * np1 + 2 * a.m * xi * pc;  // cell xi's rows of the patch
    s.st[i] = render_window(a, c, yl, s.pf + off, s.pinv + off, pc, s.u);
    s.ival[i] = render_interior(a, c, s.st[i]);
    if (!render_finite(s.st[i])) s.yfin[cy] = 0;  // any writer stores 0
  }
}

// Phase 6: outputs of the cells one layer fills.  With zz % 4 == 0 and a
// 16-byte aligned output each thread writes four consecutive z cells at a
// time (interface-cut cells among them get a placeholder that phase 7
// overwrites after a barrier), z fastest over the CTA's threads: coalesced
// 16-byte stores.  Otherwise warp `w` takes whole (component, y) rows, lane
// `lane` along z, skipping cut cells.  A row whose statistics are not all
// finite takes the full mix at every z here.
PJZ_HD void render_phase_out(const RenderArgs& a, const RenderSmem& s, int x0,
                             int nx, int y0, int ny, int w, int nw, int lane,
                             float* out) {
  const int tid = w * 32 + lane, nthr = nw * 32;
  if (render_quads(a, out)) {
    const int zq = a.zz >> 2;
    for (int xi = 0; xi < nx; ++xi)
    for (int c = 0; c < 3; ++c)
      for (int t = tid; t < ny * zq; t += nthr) {
        const int yl = render_div(t, a.zq_magic), z = 4 * (t - yl * zq);
        const int cy = render_cy(xi, c, yl);
        const int x = x0 + xi;
        float v[4];
        if (s.yfin[cy]) {
          const float* iv = s.ival + cy * a.ll;
          int o[4];
          render_owner4(s.owner + c * a.zz + z, o);
PJZ_UNROLL
          for (int j = 0; j < 4; ++j) v[j] = o[j] >= 0 ? iv[o[j]] : 0.f;
        } else {
PJZ_UNROLL
          for (int j = 0; j < 4; ++j)
            v[j] = render_value(a, s.pos, c, s.st + cy * a.ll, z + j);
        }
        render_store4(out + render_out_index(a, c, x, y0 + yl, z), v);
      }
    return;
  }
  for (int xi = 0; xi < nx; ++xi)
  for (int c = 0; c < 3; ++c)
    for (int yl = w; yl < ny; yl += nw) {
      const int cy = render_cy(xi, c, yl);
      const int x = x0 + xi;
      const WindowStats* st = s.st + cy * a.ll;
      float* row = out + render_out_index(a, c, x, y0 + yl, 0);
      if (s.yfin[cy]) {
        const float* iv = s.ival + cy * a.ll;
        for (int z = lane; z < a.zz; z += 32) {
          const int o = s.owner[c * a.zz + z];
          if (o >= 0) row[z] = iv[o];
        }
      } else {
        for (int z = lane; z < a.zz; z += 32)
          row[z] = render_value(a, s.pos, c, st, z);
      }
    }
}

// Phase 7 (after a barrier): the interface-cut cells of every row with
// finite statistics, shared over the CTA's threads (the same few z for
// every row).
PJZ_HD void render_phase_cut_cells(const RenderArgs& a, const RenderSmem& s, int x0,
                                   int nx, int y0, int ny, int tid, int nthr,
                                   float* out) {
  for (int xi = 0; xi < nx; ++xi)
  for (int c = 0; c < 3; ++c)
    for (int t = tid; t < s.ncut[c] * kRenderTileY; t += nthr) {
      const int yl = t % kRenderTileY, z = s.cut[c * a.zz + t / kRenderTileY];
      const int cy = render_cy(xi, c, yl);
      if (yl < ny && s.yfin[cy])
        out[render_out_index(a, c, x0 + xi, y0 + yl, z)] =
            render_value(a, s.pos, c, s.st + cy * a.ll, z);
    }
}

#if defined(__CUDACC__) && defined(PJZ_RENDER_KERNEL)  // kern_render.cu only
// grid (ceil(xx / nxb), ceil(yy / kRenderTileY)), a multiple of 32
// threads (at least 96); dynamic shared memory
// render_smem_floats(ll, zz, m, group, nxb) floats.
__global__ void __launch_bounds__(256, 6) render_epsilon_kernel(const RenderArgs a) {
  extern __shared__ __align__(16) float rsm[];
  const int x0 = blockIdx.x * a.nxb, y0 = blockIdx.y * kRenderTileY;
  const int nx = min(a.nxb, a.xx - x0), ny = min(kRenderTileY, a.yy - y0);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const RenderSmem s = render_carve(rsm, a.ll, a.zz, a.m, a.group, a.nxb);
  render_phase_setup(a, s, tid, nthr);
  __syncthreads();
  render_phase_occupancy(a, s, tid, nthr);
  for (int l0 = 0; l0 < a.ll; l0 += a.group) {
    const int ng = min(a.group, a.ll - l0);
    __syncthreads();  // the previous group's windows are done with the patches
    if (l0 == 0) render_phase_cuts(a, s, tid, nthr);
    render_phase_stage(a, s, l0, ng, x0, nx, y0, ny, tid, nthr);
    __syncthreads();
    render_phase_windows(a, s, l0, ng, nx, ny, tid, nthr);
  }
  __syncthreads();
  render_phase_out(a, s, x0, nx, y0, ny, tid >> 5, nthr >> 5, tid & 31, a.out);
  __syncthreads();  // placeholders of cut cells are written before phase 7
  render_phase_cut_cells(a, s, x0, nx, y0, ny, tid, nthr, a.out);
}
#endif

}  // namespace pjzfdtd
