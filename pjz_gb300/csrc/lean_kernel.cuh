// Lean streamed Yee step kernel for sm_103a (one time step per launch).
//
// Same data movement as yee_stream_kernel (stream_kernel.cuh): a producer
// warp fills a ring of shared-memory slots with bulk copies of the x-plane
// tile pieces (E rows -1..TY, H rows -1..TY-1, coefficient rows, absorber
// row, z-PML state rows) `stages` planes ahead, and bulk-stores the results
// from staging buffers; the shared-memory layout (StreamGeom) and the
// producer's copies are those of the streamed kernel.  What differs is the
// compute side, written for few instructions per cell-update:
//
//  * zz and tile_y are compile-time, so every shared-memory offset of a
//    thread is fixed before the plane loop;
//  * a compute thread owns one z-quad (4 adjacent z cells, 128-bit shared
//    accesses) of one buffer row for the whole launch: in the H phase row
//    rH (y = y0 - 1 + rH), in the E phase tile row rH (y = y0 + rH);
//  * quads inside the z-PML slabs (the slab widths must be multiples of 4)
//    belong to their own warps, which carry the CPML state; the other warps
//    never branch on it;
//  * the source current is added only on planes the source box crosses
//    (a plane-uniform test), from global memory as in the streamed kernel.
//
// Per cell the arithmetic is the explicit round-to-nearest FP32 sequence of
// the streamed kernel and of the CPU oracle, so results are bit-identical.
// Barriers and bounded waits follow the streamed kernel's protocol.
#pragma once

#include <cuda_fp16.h>
#include <string.h>

#include "stream_kernel.cuh"
#include "kernel_table.cuh"

namespace pjzfdtd {

// Quads per row outside / inside the z-PML slabs.
__host__ __device__ inline int lean_quads_interior(int Z, int plo, int phi) {
  return (Z - plo - phi) / 4;
}
__host__ __device__ inline int lean_quads_pml(int plo, int phi) {
  return (plo + phi) / 4;
}

// Items of the lean kernels: one (buffer row, z-quad) per compute thread
// over `rows` buffer rows.
//
// Split mapping (FP32 storage, zz 64, plo + phi <= 32): a 128-bit shared
// access of a warp is served 8 lanes at a time, and quad q of any row sits
// in bank group q % 8 (rows are 256 bytes).  Each row's 16 quads split into
// an edge set -- quads [0, 8 - ph) and [16 - ph, 16), ph = phi / 4, which
// holds every z-PML quad -- and an interior set [8 - ph, 16 - ph); each
// set has one quad per bank group.  Edge warps take the edge sets of four
// rows (8 lanes per row), interior warps the interior sets, so every quad
// access is free of bank conflicts; edge warps branch per lane on the
// z-PML update.
//
// Row-major mapping (binary16 storage, or zz 32): consecutive lanes hold
// consecutive quads of the row-major (row, quad) order, i.e. consecutive
// 8-byte (binary16) or 16-byte (FP32) pieces of every shared region, so no
// pass (16 lanes of 8 bytes, 8 lanes of 16 bytes) repeats a bank; every
// warp branches per lane on the z-PML update.  For binary16 at zz 64 a
// 64-bit pass must cover a whole 128-byte row to be conflict-free, which
// no split of interior and slab quads gives; at zz 32 that split left
// every pass 2-way conflicted.
//
// Otherwise: interior warps first (the quads between the slabs, row-major),
// then z-PML warps (the slab quads), so the z-PML branch is warp-uniform.
struct LeanItem {
  int row;   // buffer row (rows and beyond: idle)
  int z0;    // first z of the quad
  int col;   // z-PML state column of z0 (z-PML quads)
  bool pml;  // a z-PML quad
};

__host__ __device__ inline bool lean_split(int Z, int plo, int phi, int esz) {
  return esz == 4 && Z == 64 && plo + phi <= 32;
}

__host__ __device__ inline bool lean_rows(int Z, int esz) {
  return esz == 2 || Z == 32;
}

__host__ __device__ inline int lean_warps(int Z, int rows, int plo, int phi, int esz) {
  if (lean_split(Z, plo, phi, esz)) return 2 * ((rows + 3) / 4);
  if (lean_rows(Z, esz)) return (rows * (Z / 4) + 31) / 32;
  return (rows * lean_quads_interior(Z, plo, phi) + 31) / 32 +
         (rows * lean_quads_pml(plo, phi) + 31) / 32;
}

__host__ __device__ inline LeanItem lean_item(int tid, int Z, int rows, int plo,
                                              int phi, int esz) {
  const int lq = plo / 4, pq = phi / 4, nq = Z / 4;
  LeanItem it;
  int q;
  if (lean_split(Z, plo, phi, esz)) {
    const int ne = (rows + 3) / 4;  // edge warps
    const int w = tid >> 5, j = tid & 7;
    const bool edge = w < ne;
    it.row = 4 * (edge ? w : w - ne) + ((tid >> 3) & 3);
    q = edge ? (j < 8 - pq ? j : j + 8) : 8 - pq + j;
  } else if (lean_rows(Z, esz)) {
    it.row = tid / nq;
    q = tid - it.row * nq;
  } else {
    const int QI = lean_quads_interior(Z, plo, phi), QP = lean_quads_pml(plo, phi);
    const int nwi = (rows * QI + 31) / 32;
    const bool pw = (tid >> 5) >= nwi;
    const int i = pw ? tid - 32 * nwi : tid;
    const int Qn = pw ? QP : QI;
    it.row = Qn > 0 ? i / Qn : rows;
    const int qi = i - it.row * Qn;
    q = pw ? (qi < lq ? qi : nq - QP + qi) : lq + qi;
  }
  it.pml = q < lq || q >= nq - pq;
  it.z0 = 4 * q;
  it.col = 4 * (q < lq ? q : lq + q - (nq - pq));
  return it;
}

// Shared-memory geometry of one lean CTA for storage type T (bytes).  The
// ring slot holds E rows -1..TY, H rows -1..TY-1, E-coefficient rows
// 0..TY-1 (all T), the absorber window (FP32) and the z-PML state rows (T,
// row stride Pp = P rounded up to 16 bytes); every region starts on a
// 16-byte boundary, as the bulk copies need.  After the ring: new H
// [3][3][RH*Z] (planes x - 1, x, x + 1: the E phase of plane x shares its
// barrier interval with the H phase of plane x + 1), new E [2][3][TY*Z],
// new PML state [2][4][TY*Pp] (T), the z coefficient table [6][Z] (FP32:
// 1/kappa and the CPML b, c of E, then of H), then the mbarriers.
template <typename T>
struct LeanGeom {
  int TY, Z, Pp, RE, RH, MT;
  int e_off, h_off, c_off, m_off, p_off, stage;  // bytes within a slot
  __host__ __device__ LeanGeom(int ty, int z, int p) {
    constexpr int per16 = 16 / (int)sizeof(T);
    TY = ty;
    Z = z;
    Pp = (p + per16 - 1) / per16 * per16;
    RE = ty + 2;
    RH = ty + 1;
    MT = round4(ty) + 8;
    e_off = 0;
    h_off = e_off + 3 * RE * z * (int)sizeof(T);
    c_off = h_off + 3 * RH * z * (int)sizeof(T);
    m_off = c_off + 3 * ty * z * (int)sizeof(T);
    p_off = m_off + 3 * MT * 4;
    stage = p_off + 4 * RH * Pp * (int)sizeof(T);
  }
  __host__ __device__ size_t hn_bytes() const { return 3 * 3 * (size_t)RH * Z * sizeof(T); }
  __host__ __device__ size_t en_bytes() const { return 2 * 3 * (size_t)TY * Z * sizeof(T); }
  __host__ __device__ size_t pn_bytes() const { return 2 * 4 * (size_t)TY * Pp * sizeof(T); }
  __host__ __device__ size_t zc_bytes() const { return 6 * (size_t)Z * sizeof(float); }
  __host__ __device__ size_t bytes(int stages) const {
    return (size_t)stages * stage + hn_bytes() + en_bytes() + pn_bytes() +
           zc_bytes() + (size_t)(2 * stages + 2) * sizeof(uint64_t) + 16;
  }
};

// Four consecutive stored values to FP32 and back (128-bit accesses for
// float, 64-bit for binary16; conversions to binary16 round to nearest
// even, widening is exact).
template <typename T>
struct Quad;
template <>
struct Quad<float> {
  static __device__ __forceinline__ void ld(const float* p, float o[4]) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
  }
  static __device__ __forceinline__ void st(float* p, const float v[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
  static __device__ __forceinline__ float ld1(const float* p) { return *p; }
};
template <>
struct Quad<__half> {
  static __device__ __forceinline__ void ld(const __half* p, float o[4]) {
    const uint2 u = *reinterpret_cast<const uint2*>(p);
    __half2 lo, hi;
    memcpy(&lo, &u.x, 4);
    memcpy(&hi, &u.y, 4);
    const float2 a = __half22float2(lo), b = __half22float2(hi);
    o[0] = a.x;
    o[1] = a.y;
    o[2] = b.x;
    o[3] = b.y;
  }
  static __device__ __forceinline__ void st(__half* p, const float v[4]) {
    const __half2 lo = __floats2half2_rn(v[0], v[1]);
    const __half2 hi = __floats2half2_rn(v[2], v[3]);
    uint2 u;
    memcpy(&u.x, &lo, 4);
    memcpy(&u.y, &hi, 4);
    *reinterpret_cast<uint2*>(p) = u;
  }
  static __device__ __forceinline__ float ld1(const __half* p) {
    return __half2float(*p);
  }
};

// (zz, tile_y) shapes of the lean kernel: the streamed kernel's tile heights
// for these zz with 4 ring stages (zz 32 with a 16-cell z-PML: 28).
#define PJZ_LEAN_SHAPES(X_) X_(64, 14) X_(48, 19) X_(32, 29) X_(32, 28)
// Taller binary16 tiles (half the shared memory per row): 16 warps per CTA
// hide more latency than 9 and the y halo is half as large per cell
// (auto selection takes them for one step per pass).
#define PJZ_LEAN_SHAPES_F16(X_) X_(64, 28)

// Block bound of a lean kernel instantiation: one CTA per SM (the ring and
// staging buffers take most of the shared memory), 12 warps, or 16 for the
// tall binary16 tiles (whose registers are capped at 128 by that).
constexpr bool lean_tall_shape(int zc, int tyc) {
#define PJZ_IS_TALL(ZC, TYC) (zc == ZC && tyc == TYC) ||
  return PJZ_LEAN_SHAPES_F16(PJZ_IS_TALL) false;
#undef PJZ_IS_TALL
}
template <int ZC, int TYC, typename T>
struct LeanBounds {
  static constexpr int threads = sizeof(T) == 2 && lean_tall_shape(ZC, TYC) ? 512 : 384;
  static constexpr int blocks = 1;
};

// One CTA of the lean kernel: tile `tile` of y rows, segment `seg` of x
// planes.  ZC / TYC: zz and tile_y (compile-time); T: storage type of the
// fields, coefficients and z-PML state in HBM and shared memory (float, or
// __half for reduced-precision storage); arithmetic is FP32 either way.
template <int ZC, int TYC, typename T>
__device__ __forceinline__ void lean_tile(const StreamArgs& sa, int tile, int seg,
                                          unsigned char* sm) {
  using Q = Quad<T>;
  constexpr int Z = ZC, TY = TYC;
  constexpr int RE = TY + 2, RH = TY + 1;
  constexpr int REZ = RE * Z, RHZ = RH * Z, TYZ = TY * Z;
  constexpr uint32_t ES = sizeof(T);
  const StepArgs& a = sa.s;
  const int X = a.X, Y = a.Y;
  const int S = sa.stages;
  const LeanGeom<T> g(TY, Z, a.plo + a.phi);
  const int Pp = g.Pp;
  T* hn = reinterpret_cast<T*>(sm + (size_t)S * g.stage);  // [3][3][RH*Z]
  T* en = hn + 3 * 3 * RHZ;                                // [2][3][TY*Z]
  T* pn = en + 2 * 3 * TYZ;                                // [2][4][TY*Pp]
  float* zcs = reinterpret_cast<float*>(pn + 2 * 4 * TY * Pp);  // [6][Z]
  uint64_t* full = reinterpret_cast<uint64_t*>(zcs + 6 * Z);
  uint64_t* done = full + S;
  uint64_t* freeb = done + S;
  __shared__ int abort_flag;
  const T* fin = reinterpret_cast<const T*>(a.fin);
  T* fout = reinterpret_cast<T*>(a.fout);
  const T* cbg = reinterpret_cast<const T*>(a.cb);
  const T* psi_in = reinterpret_cast<const T*>(a.psi_in);
  T* psi_out = reinterpret_cast<T*>(a.psi_out);

  const int tid = threadIdx.x;
  const int ncomp = blockDim.x - 32;
  const int nwarps = ncomp >> 5;
  const bool producer = tid >= ncomp;
  const int y0 = tile * TY;
  const int xs = seg * a.seg_x;
  const int xe = min(X, xs + a.seg_x);
  const int x0 = xs > 0 ? xs - 1 : 0;
  const int xlast = min(xe, X - 1);  // last plane whose E is read
  const long long N = a.N;
  const long long YZ = (long long)Y * Z;
  const long long PXY = (long long)X * Y * Pp;
  const int ey_lo = max(y0 - 1, 0), ey_hi = min(y0 + TY + 1, Y);
  const int hy_hi = min(y0 + TY, Y);
  const int nrows = hy_hi - y0;
  const int erow0 = ey_lo - (y0 - 1);
  const int ma = y0 & ~3;
  const int mb = min(round4(y0 + TY), sa.Yp);
  const int moff = y0 - ma;

  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&done[s], nwarps);
    }
    mbar_init(&freeb[0], 1);
    mbar_init(&freeb[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  {
    uint32_t* w = reinterpret_cast<uint32_t*>(sm);
    const size_t nw = ((size_t)S * g.stage + g.hn_bytes() + g.en_bytes() +
                       g.pn_bytes()) / 4;
    for (size_t i = tid; i < nw; i += blockDim.x) w[i] = 0u;
    for (int i = tid; i < 6 * Z; i += blockDim.x) zcs[i] = a.zc[i];
  }
  fence_async_smem();
  __syncthreads();

  if (producer) {
    if ((tid & 31) != 0) return;
    // ---------------- producer (one lane) ----------------
    auto fill = [&](int xp, int slot, bool fullp) {
      unsigned char* st = sm + (size_t)slot * g.stage;
      const uint32_t eb = (uint32_t)((ey_hi - ey_lo) * Z) * ES;
      const uint32_t hb = (uint32_t)((hy_hi - ey_lo) * Z) * ES;
      const uint32_t cbb = (uint32_t)(nrows * Z) * ES;
      const uint32_t mbb = (uint32_t)((mb - ma) * 4);
      const uint32_t pb = (uint32_t)((hy_hi - ey_lo) * Pp) * ES;
      const uint32_t total = sa.stall_bytes + 3 * eb +
          (fullp ? 3 * (hb + cbb + mbb) + (Pp > 0 ? 4 * pb : 0) : 0);
      mbar_expect_tx(&full[slot], total);
      const long long base = (long long)xp * YZ;
      T* se = reinterpret_cast<T*>(st + g.e_off);
      T* sh = reinterpret_cast<T*>(st + g.h_off);
      T* sc = reinterpret_cast<T*>(st + g.c_off);
      float* smk = reinterpret_cast<float*>(st + g.m_off);
      T* sp = reinterpret_cast<T*>(st + g.p_off);
      for (int c = 0; c < 3; ++c)
        bulk_g2s(se + c * REZ + erow0 * Z,
                 fin + c * N + base + (long long)ey_lo * Z, eb, &full[slot]);
      if (!fullp) return;
      for (int c = 0; c < 3; ++c) {
        bulk_g2s(sh + c * RHZ + erow0 * Z,
                 fin + (3 + c) * N + base + (long long)ey_lo * Z, hb, &full[slot]);
        bulk_g2s(sc + c * TYZ, cbg + c * N + base + (long long)y0 * Z, cbb,
                 &full[slot]);
        bulk_g2s(smk + c * g.MT,
                 sa.mask_ws + ((long long)xp * 3 + c) * sa.Yp + ma, mbb, &full[slot]);
      }
      if (Pp > 0)
        for (int c = 0; c < 4; ++c)
          bulk_g2s(sp + c * RH * Pp + erow0 * Pp,
                   psi_in + c * PXY + ((long long)xp * Y + ey_lo) * Pp, pb,
                   &full[slot]);
    };
    int nfill = 0;  // planes issued so far (x0 + nfill is the next one)
    while (nfill < S && x0 + nfill <= xlast) {
      fill(x0 + nfill, nfill, x0 + nfill < xe);
      ++nfill;
    }
    bool ok = true;
    int slot = 0;        // ring slot of plane x
    uint32_t round = 0;  // fills of that slot before plane x's
    for (int x = x0; x < xe && ok; ++x) {
      const int k = x - x0;
      const int b = k & 1;
      ok = mbar_wait_or_abort(&done[slot], round & 1, sa.status, &abort_flag,
                              sa.wait_cycles);
      if (!ok) break;
      if (x >= xs) {
        T* hcur = hn + (size_t)(k % 3) * 3 * RHZ;
        T* ecur = en + (size_t)b * 3 * TYZ;
        T* pcur = pn + (size_t)b * 4 * TY * Pp;
        const long long base = (long long)x * YZ + (long long)y0 * Z;
        const uint32_t fb = (uint32_t)(nrows * Z) * ES;
        for (int c = 0; c < 3; ++c) {
          bulk_s2g(fout + (3 + c) * N + base, hcur + c * RHZ + Z, fb);
          bulk_s2g(fout + c * N + base, ecur + c * TYZ, fb);
        }
        if (Pp > 0) {
          const uint32_t pb = (uint32_t)(nrows * Pp) * ES;
          const long long pbase = ((long long)x * Y + y0) * Pp;
          for (int c = 0; c < 4; ++c)
            bulk_s2g(psi_out + c * PXY + pbase, pcur + c * TY * Pp, pb);
        }
        bulk_commit();
      }
      if (x0 + nfill <= xlast) {
        fill(x0 + nfill, slot, x0 + nfill < xe);
        ++nfill;
      }
      bulk_wait_read_all();
      mbar_arrive(&freeb[b]);
      if (++slot == S) {
        slot = 0;
        ++round;
      }
    }
    for (int j = max(0, nfill - S); j < nfill; ++j)
      mbar_wait(&full[j % S], (uint32_t)(j / S) & 1, sa.status, sa.wait_cycles);
    bulk_wait_all();
    return;
  }

  // ---------------- compute warps ----------------
  // Item of this thread: interior warps first, then PML warps; item i is
  // (buffer row i / Qn, quad i % Qn of the warp kind's quads).
  const LeanItem item = lean_item(tid, Z, RH, a.plo, a.phi, (int)ES);
  const bool pml = item.pml;
  const int rH = item.row;
  const int z0 = item.z0;
  const int col = item.col;  // z-PML state column of z0 (z-PML quads)
  const bool doH = rH < RH && y0 - 1 + rH >= 0 && y0 - 1 + rH < Y;
  const int yE = y0 + rH;
  const bool doE = rH < TY && yE < Y;
  const bool zhi = z0 + 4 < Z;  // a z + 1 neighbour inside the domain
  const bool zlo = z0 > 0;      // a z - 1 neighbour inside the domain

  // z coefficients of the quad (z0 + 3 < Z for every item, idle or not):
  // 1/kappa, b, c of E then of H.
  const float* zq = zcs + z0;
  // Register-capped shapes read them from the table; the others hold them.
  constexpr bool kZcShared = LeanBounds<ZC, TYC, T>::threads > 384;
  float rz[6][4];
  if constexpr (!kZcShared) {
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int j = 0; j < 4; ++j) rz[r][j] = a.zc[r * Z + z0 + j];
  }
  auto zload = [&](int r, float o[4]) {
    if constexpr (kZcShared) {
      Quad<float>::ld(zq + r * Z, o);
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) o[j] = rz[r][j];
    }
  };
  const float mdt = -a.dt;
  // Source box rows and z range of this item (the plane test is separate).
  const bool src_row = a.snc > 0 && yE >= a.sy0 && yE < a.sy0 + a.sny &&
                       z0 + 4 > a.sz0 && z0 < a.sz0 + a.snz;
  const long long sb = (long long)a.snx * a.sny * a.snz;

  const int ieH = rH * Z + z0;        // H-phase row rH, E rows rH / rH + 1
  const int ihE = (rH + 1) * Z + z0;  // E-phase buffer row rH + 1
  const int icE = rH * Z + z0;        // coefficient / staging row rH
  const int pH = rH * Pp + col;
  const int pE = (rH + 1) * Pp + col;

  // H^{n+1/2} of the quad at buffer row rH (y = y0 - 1 + rH) of the plane in
  // ring slot `sl` (E of the next plane in slot `sl1`, or zero), into hcur /
  // pcur (PML state comps 0, 1).
  auto h_phase = [&](int sl, int sl1, bool has_x1, T* hcur, T* pcur) {
    const unsigned char* st = sm + (size_t)sl * g.stage;
    const T* Es = reinterpret_cast<const T*>(st + g.e_off);
    const T* E1 = reinterpret_cast<const T*>(sm + (size_t)sl1 * g.stage + g.e_off);
    const T* Hs = reinterpret_cast<const T*>(st + g.h_off);
    const T* Ps = reinterpret_cast<const T*>(st + g.p_off);
    {
      float ex[4], ey[4], ez[4], exy[4], ezy[4], e1y[4], e1z[4], ho[3][4];
      Q::ld(Es + ieH, ex);
      Q::ld(Es + REZ + ieH, ey);
      Q::ld(Es + 2 * REZ + ieH, ez);
      Q::ld(Es + ieH + Z, exy);
      Q::ld(Es + 2 * REZ + ieH + Z, ezy);
      const float exz = zhi ? Q::ld1(Es + ieH + 4) : 0.f;
      const float eyz = zhi ? Q::ld1(Es + REZ + ieH + 4) : 0.f;
      if (has_x1) {
        Q::ld(E1 + REZ + ieH, e1y);
        Q::ld(E1 + 2 * REZ + ieH, e1z);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) e1y[j] = e1z[j] = 0.f;
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) Q::ld(Hs + c * RHZ + ieH, ho[c]);
      float pa[4], pb[4], ikh[4], bh[4], ch[4];
      zload(3, ikh);
      if (pml) {
        Q::ld(Ps + pH, pa);
        Q::ld(Ps + RH * Pp + pH, pb);
        zload(4, bh);
        zload(5, ch);
      }
      float hx[4], hy[4], hz[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float ey1 = j < 3 ? ey[j + 1] : eyz;
        const float ex1 = j < 3 ? ex[j + 1] : exz;
        const float dEz_y = fsub(ezy[j], ez[j]), dEy_z = fsub(ey1, ey[j]);
        const float dEx_z = fsub(ex1, ex[j]), dEz_x = fsub(e1z[j], ez[j]);
        const float dEy_x = fsub(e1y[j], ey[j]), dEx_y = fsub(exy[j], ex[j]);
        float zEy, zEx;
        if (pml) {
          const float na = ffma(ch[j], dEy_z, fmul(bh[j], pa[j]));
          const float nb = ffma(ch[j], dEx_z, fmul(bh[j], pb[j]));
          pa[j] = na;
          pb[j] = nb;
          zEy = ffma(dEy_z, ikh[j], na);
          zEx = ffma(dEx_z, ikh[j], nb);
        } else {
          zEy = fmul(dEy_z, ikh[j]);
          zEx = fmul(dEx_z, ikh[j]);
        }
        hx[j] = ffma(mdt, fsub(dEz_y, zEy), ho[0][j]);
        hy[j] = ffma(mdt, fsub(zEx, dEz_x), ho[1][j]);
        hz[j] = ffma(mdt, fsub(dEy_x, dEx_y), ho[2][j]);
      }
      Q::st(hcur + ieH, hx);
      Q::st(hcur + RHZ + ieH, hy);
      Q::st(hcur + 2 * RHZ + ieH, hz);
      if (pml && rH > 0) {
        Q::st(pcur + (rH - 1) * Pp + col, pa);
        Q::st(pcur + TY * Pp + (rH - 1) * Pp + col, pb);
      }
    }
  };

  // E^{n+1} of the quad at tile row rH (y = y0 + rH) of plane x in ring slot
  // `sl`, from the new H of planes x (hcur) and x - 1 (hprev), into ecur /
  // pcur (PML state comps 2, 3).
  auto e_phase = [&](int x, int sl, const T* hcur, const T* hprev, T* ecur,
                     T* pcur) {
    const unsigned char* st = sm + (size_t)sl * g.stage;
    const T* Es = reinterpret_cast<const T*>(st + g.e_off);
    const T* Cs = reinterpret_cast<const T*>(st + g.c_off);
    const float* Ms = reinterpret_cast<const float*>(st + g.m_off) + moff;
    const T* Ps = reinterpret_cast<const T*>(st + g.p_off);
    {
      float hx[4], hy[4], hz[4], hxm[4], hzm[4], hyp[4], hzp[4], eo[3][4], cb[3][4];
      Q::ld(hcur + ihE, hx);
      Q::ld(hcur + RHZ + ihE, hy);
      Q::ld(hcur + 2 * RHZ + ihE, hz);
      Q::ld(hcur + ihE - Z, hxm);
      Q::ld(hcur + 2 * RHZ + ihE - Z, hzm);
      const float hxz = zlo ? Q::ld1(hcur + ihE - 1) : 0.f;
      const float hyz = zlo ? Q::ld1(hcur + RHZ + ihE - 1) : 0.f;
      Q::ld(hprev + RHZ + ihE, hyp);
      Q::ld(hprev + 2 * RHZ + ihE, hzp);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        Q::ld(Es + c * REZ + ihE, eo[c]);
        Q::ld(Cs + c * TYZ + icE, cb[c]);
      }
      const float sig[3] = {Ms[rH], Ms[g.MT + rH], Ms[2 * g.MT + rH]};
      float pa[4], pb[4], ike[4], be[4], ce[4];
      zload(0, ike);
      if (pml) {
        Q::ld(Ps + 2 * RH * Pp + pE, pa);
        Q::ld(Ps + 3 * RH * Pp + pE, pb);
        zload(1, be);
        zload(2, ce);
      }
      const bool src = src_row && x >= a.sx0 && x < a.sx0 + a.snx;
      float enew[3][4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float hy0 = j > 0 ? hy[j - 1] : hyz;
        const float hx0 = j > 0 ? hx[j - 1] : hxz;
        const float dHz_y = fsub(hz[j], hzm[j]), dHy_z = fsub(hy[j], hy0);
        const float dHx_z = fsub(hx[j], hx0), dHz_x = fsub(hz[j], hzp[j]);
        const float dHy_x = fsub(hy[j], hyp[j]), dHx_y = fsub(hx[j], hxm[j]);
        float zHy, zHx;
        if (pml) {
          const float na = ffma(ce[j], dHy_z, fmul(be[j], pa[j]));
          const float nb = ffma(ce[j], dHx_z, fmul(be[j], pb[j]));
          pa[j] = na;
          pb[j] = nb;
          zHy = ffma(dHy_z, ike[j], na);
          zHx = ffma(dHx_z, ike[j], nb);
        } else {
          zHy = fmul(dHy_z, ike[j]);
          zHx = fmul(dHx_z, ike[j]);
        }
        float cur[3] = {fsub(dHz_y, zHy), fsub(zHx, dHz_x), fsub(dHy_x, dHx_y)};
        if (src) {
          const int z = z0 + j;
          if (z >= a.sz0 && z < a.sz0 + a.snz) {
            const long long si =
                ((long long)(x - a.sx0) * a.sny + (yE - a.sy0)) * a.snz + (z - a.sz0);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              float jc = 0.f;
              for (int w = 0; w < a.snc; ++w)
                jc = ffma(a.src[((long long)w * 3 + c) * sb + si], a.wave[w], jc);
              cur[c] = fsub(cur[c], jc);
            }
          }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float rr = ffma(-sig[c], eo[c][j], cur[c]);
          enew[c][j] = ffma(cb[c][j], rr, eo[c][j]);
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) Q::st(ecur + c * TYZ + icE, enew[c]);
      if (pml) {
        Q::st(pcur + 2 * TY * Pp + rH * Pp + col, pa);
        Q::st(pcur + 3 * TY * Pp + rH * Pp + col, pb);
      }
    }
  };

  // Ring position (slot, fill round) of a plane, advanced plane by plane.
  struct RingPos {
    int slot;
    uint32_t round;
  };
  auto next = [&](RingPos p) {
    if (++p.slot == S) {
      p.slot = 0;
      ++p.round;
    }
    return p;
  };
  // Planes x, x + 1, x + 2 of the loop below.
  RingPos p0 = {0, 0u};
  RingPos p1 = next(p0);
  RingPos p2 = next(p1);
  // New-H buffer (0, 1, 2) of plane x: plane x - 1's is the one before it
  // and plane x + 1's the one after, cyclically.
  int hb = 0;
  auto hbuf = [&](int i) { return hn + (size_t)i * 3 * RHZ; };

  // Plane x0: its H phase.
  {
    bool ok = mbar_wait_or_abort(&full[p0.slot], p0.round & 1, sa.status,
                                 &abort_flag, sa.wait_cycles);
    if (ok && x0 + 1 < X)
      ok = mbar_wait_or_abort(&full[p1.slot], p1.round & 1, sa.status, &abort_flag,
                              sa.wait_cycles);
    if (ok && doH) h_phase(p0.slot, p1.slot, x0 + 1 < X, hbuf(0), pn);
  }
  // Each iteration: barrier (H of plane x done by every warp), E of plane x,
  // release plane x to the producer, then H of plane x + 1 -- which needs
  // no result of E(x), so the two share one barrier interval; three H
  // buffers keep H(x + 1) off the H(x) and H(x - 1) that E(x) reads.
  for (int x = x0; x < xe; ++x) {
    const int k = x - x0;
    const int hb1 = hb == 2 ? 0 : hb + 1;  // plane x + 1's buffer
    const int hb0 = hb == 0 ? 2 : hb - 1;  // plane x - 1's buffer
    compute_sync(ncomp);
    if (abort_flag) break;
    if (x >= xs && doE)
      e_phase(x, p0.slot, hbuf(hb), hbuf(hb0), en + (size_t)(k & 1) * 3 * TYZ,
              pn + (size_t)(k & 1) * 4 * TY * Pp);
    // Publish this plane's results to the producer and release its slot.
    fence_async_smem();
    __syncwarp();
    if ((tid & 31) == 0) mbar_arrive(&done[p0.slot]);
    if (x + 1 < xe) {
      const int k1 = k + 1;
      bool ok = true;
      if (x + 2 < X)
        ok = mbar_wait_or_abort(&full[p2.slot], p2.round & 1, sa.status,
                                &abort_flag, sa.wait_cycles);
      // The staging buffers of plane x + 1 held plane x - 1's results: wait
      // until the producer's stores of them have read them.
      if (ok && k1 >= 2)
        ok = mbar_wait_or_abort(&freeb[k1 & 1], (uint32_t)((k1 >> 1) - 1) & 1,
                                sa.status, &abort_flag, sa.wait_cycles);
      if (ok && doH)
        h_phase(p1.slot, p2.slot, x + 2 < X, hbuf(hb1),
                pn + (size_t)(k1 & 1) * 4 * TY * Pp);
    }
    hb = hb1;
    p0 = p1;
    p1 = p2;
    p2 = next(p2);
  }
}

template <int ZC, int TYC, typename T>
__global__ void __launch_bounds__(LeanBounds<ZC, TYC, T>::threads,
                                  LeanBounds<ZC, TYC, T>::blocks)
    yee_lean_kernel(const StreamArgs sa) {
  extern __shared__ __align__(16) unsigned char lean_sm[];
  lean_tile<ZC, TYC, T>(sa, blockIdx.x, blockIdx.y, lean_sm);
}

}  // namespace pjzfdtd
