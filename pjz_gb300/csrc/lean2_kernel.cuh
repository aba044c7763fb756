// Lean two-step (temporally blocked) streamed Yee kernel for sm_103a.
//
// One launch advances the state by two time steps, n and n + 1, reading the
// fields, coefficients and z-PML state from HBM once and writing them once
// -- the data movement, ring protocol and barriers of yee_stream2_kernel
// (stream2_kernel.cuh), whose header describes the two-level wavefront:
// level 1 computes H and E of plane x over rows y0-2..y0+TY (H) and
// y0-1..y0+TY (E); level 2 computes H and E of plane x-1 over rows
// y0-1..y0+TY-1 and y0..y0+TY-1 from level 1's planes x-1 and x, and stores
// rows y0..y0+TY-1 to HBM.
//
// The compute side is the lean kernel's (lean_kernel.cuh): compile-time zz
// and tile_y, one z-quad per thread with 128-bit (FP32) or 64-bit
// (binary16) shared-memory accesses, interior and z-PML quads on separate
// warps.  A thread keeps the same (buffer row, quad) in all four phases, so
// the z-PML state level 1 hands to level 2 is read back by its writer.  T
// is the storage type (float, or __half for reduced-precision storage: the
// level-1 results are rounded to it exactly where a single step would store
// them).  Per cell the arithmetic is the explicit RN FP32 sequence of the
// one-step kernels and of the CPU oracle, so results are bit-identical.
#pragma once

#include "lean_kernel.cuh"

namespace pjzfdtd {

// Shared-memory geometry of a lean two-step CTA for storage type T (bytes):
// ring A slot: E [3][NE*Z], H [3][NR*Z], PML state [4][NR*Pp] (T);
// ring B slot: coefficients [3][NR*Z] (T), absorber [3][MT] (FP32);
// after the rings: H1 [2][3][NR*Z], E1 [2][3][NR*Z], H2x [NR*Z],
// H2yz [2][2][NR*Z], P1 [2][4][NR*Pp] (T), then the mbarriers.  Every
// region starts on a 16-byte boundary.  For T = float this is Stream2Geom's
// layout.
template <typename T>
struct Lean2Geom {
  int TY, Z, Pp, NR, NE, MT;
  int a_e, a_h, a_p, a_stage, b_c, b_m, b_stage;  // bytes
  __host__ __device__ Lean2Geom(int ty, int z, int p) {
    constexpr int per16 = 16 / (int)sizeof(T);
    constexpr int es = (int)sizeof(T);
    TY = ty;
    Z = z;
    Pp = (p + per16 - 1) / per16 * per16;
    NR = ty + 3;
    NE = ty + 4;
    MT = round4(ty + 2) + 8;
    a_e = 0;
    a_h = a_e + 3 * NE * z * es;
    a_p = a_h + 3 * NR * z * es;
    a_stage = a_p + 4 * NR * Pp * es;
    b_c = 0;
    b_m = b_c + 3 * NR * z * es;
    b_stage = b_m + 3 * MT * 4;
  }
  __host__ __device__ size_t inter_bytes() const {
    return ((size_t)17 * NR * Z + 8 * (size_t)NR * Pp) * sizeof(T);
  }
  __host__ __device__ size_t bytes(int sa, int sb) const {
    return (size_t)sa * a_stage + (size_t)sb * b_stage + inter_bytes() +
           (size_t)(2 * sa + 2 * sb) * sizeof(uint64_t) + 16;
  }
};

// Warps of the lean two-step kernel: one item per (buffer row, quad) over
// the NR = tile_y + 3 rows of level 1 (lean_item).
__host__ __device__ inline int lean2_warps(int Z, int ty, int plo, int phi, int esz) {
  return lean_warps(Z, ty + 3, plo, phi, esz);
}

template <int ZC, int TYC, typename T>
__device__ __forceinline__ void lean2_tile(const StreamArgs& sa, int tile, int seg,
                                           unsigned char* sm) {
  using Q = Quad<T>;
  constexpr int Z = ZC, TY = TYC;
  constexpr int NR = TY + 3, NE = TY + 4;
  constexpr int NRZ = NR * Z, NEZ = NE * Z;
  constexpr uint32_t ES = sizeof(T);
  const StepArgs& a = sa.s;
  const int X = a.X, Y = a.Y;
  const int SA = sa.stages2 & 0xff, SB = (sa.stages2 >> 8) & 0xff;
  const Lean2Geom<T> g(TY, Z, a.plo + a.phi);
  const int Pp = g.Pp;
  const int NRP = NR * Pp;
  unsigned char* ringA = sm;
  unsigned char* ringB = ringA + (size_t)SA * g.a_stage;
  T* H1 = reinterpret_cast<T*>(ringB + (size_t)SB * g.b_stage);  // [2][3][NRZ]
  T* E1 = H1 + 6 * (size_t)NRZ;                                  // [2][3][NRZ]
  T* H2x = E1 + 6 * (size_t)NRZ;                                 // [NRZ]
  T* H2yz = H2x + NRZ;                                           // [2][2][NRZ]
  T* P1 = H2yz + 4 * (size_t)NRZ;                                // [2][4][NRP]
  uint64_t* fullA = reinterpret_cast<uint64_t*>(P1 + 8 * (size_t)NRP);
  uint64_t* doneA = fullA + SA;
  uint64_t* fullB = doneA + SA;
  uint64_t* doneB = fullB + SB;
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
  const int a1 = max(xs - 2, 0);          // first level-1 plane
  const int a2 = max(xs - 1, 0);          // first level-2 plane
  const int last1 = min(xe, X - 1);       // last level-1 plane (ring B)
  const int lastA = min(xe + 1, X - 1);   // last plane whose E is read
  const long long N = a.N;
  const long long YZ = (long long)Y * Z;
  const long long PXY = (long long)X * Y * Pp;
  const int ylo = max(y0 - 2, 0);
  const int e_hi = min(y0 + TY + 2, Y);   // E rows [ylo, e_hi)
  const int h_hi = min(y0 + TY + 1, Y);   // H, PML rows [ylo, h_hi)
  const int clo = max(y0 - 1, 0);         // cb rows [clo, h_hi)
  const int ma = clo & ~3;                // absorber window [ma, mb)
  const int mb = min(round4(y0 + TY + 1), sa.Yp);

  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < SA; ++s) {
      mbar_init(&fullA[s], 1);
      mbar_init(&doneA[s], nwarps);
    }
    for (int s = 0; s < SB; ++s) {
      mbar_init(&fullB[s], 1);
      mbar_init(&doneB[s], nwarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  {
    uint32_t* w = reinterpret_cast<uint32_t*>(sm);
    const size_t nw = ((size_t)SA * g.a_stage + (size_t)SB * g.b_stage +
                       g.inter_bytes()) / 4;
    for (size_t i = tid; i < nw; i += blockDim.x) w[i] = 0u;
  }
  fence_async_smem();
  __syncthreads();

  if (producer) {
    if ((tid & 31) != 0) return;
    // ---------------- producer (one lane) ----------------
    const uint32_t eb = (uint32_t)((e_hi - ylo) * Z) * ES;
    const uint32_t hb = (uint32_t)((h_hi - ylo) * Z) * ES;
    const uint32_t pb = (uint32_t)((h_hi - ylo) * Pp) * ES;
    const uint32_t cbb = (uint32_t)((h_hi - clo) * Z) * ES;
    const uint32_t mbb = (uint32_t)((mb - ma) * 4);
    const int r0 = ylo - (y0 - 2);  // buffer row of the first copied row
    auto fillA = [&](int xp, int slot) {
      unsigned char* st = ringA + (size_t)slot * g.a_stage;
      T* se = reinterpret_cast<T*>(st + g.a_e);
      T* sh = reinterpret_cast<T*>(st + g.a_h);
      T* sp = reinterpret_cast<T*>(st + g.a_p);
      const bool fullp = xp <= last1;
      const uint32_t total = sa.stall_bytes + 3 * eb +
                             (fullp ? 3 * hb + (Pp > 0 ? 4 * pb : 0) : 0);
      mbar_expect_tx(&fullA[slot], total);
      const long long base = (long long)xp * YZ + (long long)ylo * Z;
      for (int c = 0; c < 3; ++c)
        bulk_g2s(se + c * NEZ + r0 * Z, fin + c * N + base, eb, &fullA[slot]);
      if (!fullp) return;
      for (int c = 0; c < 3; ++c)
        bulk_g2s(sh + c * NRZ + r0 * Z, fin + (3 + c) * N + base, hb, &fullA[slot]);
      if (Pp > 0)
        for (int c = 0; c < 4; ++c)
          bulk_g2s(sp + c * NRP + r0 * Pp,
                   psi_in + c * PXY + ((long long)xp * Y + ylo) * Pp, pb,
                   &fullA[slot]);
    };
    auto fillB = [&](int xp, int slot) {
      unsigned char* st = ringB + (size_t)slot * g.b_stage;
      T* sc = reinterpret_cast<T*>(st + g.b_c);
      float* smk = reinterpret_cast<float*>(st + g.b_m);
      mbar_expect_tx(&fullB[slot], sa.stall_bytes + 3 * (cbb + mbb));
      const long long base = (long long)xp * YZ + (long long)clo * Z;
      for (int c = 0; c < 3; ++c) {
        bulk_g2s(sc + c * NRZ + (clo - (y0 - 2)) * Z, cbg + c * N + base, cbb,
                 &fullB[slot]);
        bulk_g2s(smk + c * g.MT, sa.mask_ws + ((long long)xp * 3 + c) * sa.Yp + ma,
                 mbb, &fullB[slot]);
      }
    };
    int nA = 0, nB = 0;  // planes issued (a1 + n is the next one)
    while (nA < SA && a1 + nA <= lastA) {
      fillA(a1 + nA, nA);
      ++nA;
    }
    while (nB < SB && a1 + nB <= last1) {
      fillB(a1 + nB, nB);
      ++nB;
    }
    bool ok = true;
    int sA = 0, sB = 0;       // slots of plane x (ring A) / x-1 (ring B)
    uint32_t rA = 0, rB = 0;  // their fill rounds
    for (int x = a1; x <= xe && ok; ++x) {
      if (x <= last1) {
        ok = mbar_wait_or_abort(&doneA[sA], rA & 1, sa.status, &abort_flag,
                                sa.wait_cycles);
        if (!ok) break;
        if (a1 + nA <= lastA) {
          fillA(a1 + nA, sA);
          ++nA;
        }
        if (++sA == SA) {
          sA = 0;
          ++rA;
        }
      }
      if (x > a1 && x - 1 <= last1) {
        ok = mbar_wait_or_abort(&doneB[sB], rB & 1, sa.status, &abort_flag,
                                sa.wait_cycles);
        if (!ok) break;
        if (a1 + nB <= last1) {
          fillB(a1 + nB, sB);
          ++nB;
        }
        if (++sB == SB) {
          sB = 0;
          ++rB;
        }
      }
    }
    // Drain: every issued fill must land before shared memory is released.
    for (int j = max(0, nA - SA); j < nA; ++j)
      mbar_wait(&fullA[j % SA], (uint32_t)(j / SA) & 1, sa.status, sa.wait_cycles);
    for (int j = max(0, nB - SB); j < nB; ++j)
      mbar_wait(&fullB[j % SB], (uint32_t)(j / SB) & 1, sa.status, sa.wait_cycles);
    return;
  }

  // ---------------- compute warps ----------------
  const LeanItem item = lean_item(tid, Z, NR, a.plo, a.phi, (int)ES);
  const bool pml = item.pml;
  const int ra = item.row;  // buffer row (y = y0 - 2 + ra)
  const int z0 = item.z0;
  const int col = item.col;
  const int y = y0 - 2 + ra;
  const bool in_y = ra < NR && y >= 0 && y < Y;
  const bool do_h1 = in_y;                          // rows 0 .. NR-1
  const bool do_e1 = in_y && ra >= 1;               // rows 1 .. NR-1
  const bool do_h2 = in_y && ra >= 1 && ra <= NR - 2;
  const bool do_e2 = in_y && ra >= 2 && ra <= NR - 2;
  const bool zhi = z0 + 4 < Z, zlo = z0 > 0;

  float ike[4], ikh[4], be[4], ce[4], bh[4], ch[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int z = min(z0 + k, Z - 1);
    ike[k] = a.zc[z];
    ikh[k] = a.zc[3 * Z + z];
    be[k] = pml ? a.zc[Z + z] : 0.f;
    ce[k] = pml ? a.zc[2 * Z + z] : 0.f;
    bh[k] = pml ? a.zc[4 * Z + z] : 0.f;
    ch[k] = pml ? a.zc[5 * Z + z] : 0.f;
  }
  const float mdt = -a.dt;
  const bool src_row = a.snc > 0 && y >= a.sy0 && y < a.sy0 + a.sny &&
                       z0 + 4 > a.sz0 && z0 < a.sz0 + a.snz;
  const long long sbox = (long long)a.snx * a.sny * a.snz;
  const float* wave1 = a.wave;
  const float* wave2 = a.snc > 0 ? a.wave + a.snc : nullptr;
  const int ie = ra * Z + z0;   // row ra of every NR-row buffer (and ring A E)
  const int pi = ra * Pp + col;

  // H update of the quad: E (stride es, rows ra / ra+1, z+1), E of the next
  // plane (E1, or zero), old H (stride hs), PML state comps 0/1 (stride ps).
  auto h_quad = [&](const T* E, int es, const T* E1, int e1s, const T* Ho, int hs,
                    const T* Pin, int ps, float hn[3][4], float pa[4], float pb[4]) {
    float ex[4], ey[4], ez[4], exy[4], ezy[4], e1y[4], e1z[4], ho[3][4];
    Q::ld(E + ie, ex);
    Q::ld(E + es + ie, ey);
    Q::ld(E + 2 * es + ie, ez);
    Q::ld(E + ie + Z, exy);
    Q::ld(E + 2 * es + ie + Z, ezy);
    const float exz = zhi ? Q::ld1(E + ie + 4) : 0.f;
    const float eyz = zhi ? Q::ld1(E + es + ie + 4) : 0.f;
    if (E1) {
      Q::ld(E1 + e1s + ie, e1y);
      Q::ld(E1 + 2 * e1s + ie, e1z);
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) e1y[j] = e1z[j] = 0.f;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) Q::ld(Ho + c * hs + ie, ho[c]);
    if (pml) {
      Q::ld(Pin + pi, pa);
      Q::ld(Pin + ps + pi, pb);
    }
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
      hn[0][j] = ffma(mdt, fsub(dEz_y, zEy), ho[0][j]);
      hn[1][j] = ffma(mdt, fsub(zEx, dEz_x), ho[1][j]);
      hn[2][j] = ffma(mdt, fsub(dEy_x, dEx_y), ho[2][j]);
    }
  };

  // E update of the quad: new H of the plane (Hx, Hy, Hz; rows ra, ra-1,
  // z-1), new Hy/Hz of the previous plane, old E (stride es), coefficients
  // (stride cs), absorber of the row, PML state comps 2/3 (stride ps), the
  // source current of plane xp (waveform row wave) when `src`.
  auto e_quad = [&](const T* Hx, const T* Hy, const T* Hz, const T* Hyp,
                    const T* Hzp, const T* Eo, int es, const T* Cb, int cs,
                    const float sig[3], const T* Pin, int ps, bool src, int xp,
                    const float* wave, float en[3][4], float pa[4], float pb[4]) {
    float hx[4], hy[4], hz[4], hxm[4], hzm[4], hyp[4], hzp[4], eo[3][4], cb[3][4];
    Q::ld(Hx + ie, hx);
    Q::ld(Hy + ie, hy);
    Q::ld(Hz + ie, hz);
    Q::ld(Hx + ie - Z, hxm);
    Q::ld(Hz + ie - Z, hzm);
    const float hxz = zlo ? Q::ld1(Hx + ie - 1) : 0.f;
    const float hyz = zlo ? Q::ld1(Hy + ie - 1) : 0.f;
    Q::ld(Hyp + ie, hyp);
    Q::ld(Hzp + ie, hzp);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Q::ld(Eo + c * es + ie, eo[c]);
      Q::ld(Cb + c * cs + ie, cb[c]);
    }
    if (pml) {
      Q::ld(Pin + pi, pa);
      Q::ld(Pin + ps + pi, pb);
    }
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
              ((long long)(xp - a.sx0) * a.sny + (y - a.sy0)) * a.snz + (z - a.sz0);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float jc = 0.f;
            for (int w = 0; w < a.snc; ++w)
              jc = ffma(a.src[((long long)w * 3 + c) * sbox + si], wave[w], jc);
            cur[c] = fsub(cur[c], jc);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float rr = ffma(-sig[c], eo[c][j], cur[c]);
        en[c][j] = ffma(cb[c][j], rr, eo[c][j]);
      }
    }
  };

  int sA = 0, sA1 = SA > 1 ? 1 : 0;   // ring A slots of planes x, x+1
  uint32_t rA = 0, rA1 = SA > 1 ? 0 : 1;
  int sB = 0, sBm = 0;                // ring B slots of planes x, x-1
  uint32_t rB = 0;
  for (int x = a1; x <= xe; ++x) {
    const bool l1 = x <= last1;
    const bool l2 = x - 1 >= a2;
    const bool st2 = x - 1 >= xs;     // level-2 plane is stored
    const int b = x & 1;
    bool ok = true;
    if (l1) {
      ok = mbar_wait_or_abort(&fullA[sA], rA & 1, sa.status, &abort_flag,
                              sa.wait_cycles);
      if (ok && x + 1 <= lastA)
        ok = mbar_wait_or_abort(&fullA[sA1], rA1 & 1, sa.status, &abort_flag,
                                sa.wait_cycles);
      if (ok)
        ok = mbar_wait_or_abort(&fullB[sB], rB & 1, sa.status, &abort_flag,
                                sa.wait_cycles);
    }
    const unsigned char* As = ringA + (size_t)sA * g.a_stage;
    const unsigned char* A1s = ringA + (size_t)sA1 * g.a_stage;
    const unsigned char* Bs = ringB + (size_t)sB * g.b_stage;
    const unsigned char* Bm = ringB + (size_t)sBm * g.b_stage;
    const T* AE = reinterpret_cast<const T*>(As + g.a_e);
    const T* AH = reinterpret_cast<const T*>(As + g.a_h);
    const T* AP = reinterpret_cast<const T*>(As + g.a_p);
    T* h1c = H1 + (size_t)b * 3 * NRZ;
    const T* h1p = H1 + (size_t)(b ^ 1) * 3 * NRZ;
    T* e1c = E1 + (size_t)b * 3 * NRZ;
    const T* e1p = E1 + (size_t)(b ^ 1) * 3 * NRZ;
    T* p1c = P1 + (size_t)b * 4 * NRP;
    const T* p1p = P1 + (size_t)(b ^ 1) * 4 * NRP;
    // Level 2 works on plane x - 1: its H2 y/z buffer has parity b ^ 1 and
    // the previous plane's (x - 2) parity b.
    T* h2yz = H2yz + (size_t)(b ^ 1) * 2 * NRZ;
    const T* h2yzp = H2yz + (size_t)b * 2 * NRZ;

    // ---- level 1, H^{n+1/2}(x), rows y0-2 .. y0+TY ----
    if (ok && l1 && do_h1) {
      const T* e1n = x + 1 < X ? reinterpret_cast<const T*>(A1s + g.a_e) : nullptr;
      float hn[3][4], pa[4], pb[4];
      h_quad(AE, NEZ, e1n, NEZ, AH, NRZ, AP, NRP, hn, pa, pb);
#pragma unroll
      for (int c = 0; c < 3; ++c) Q::st(h1c + c * NRZ + ie, hn[c]);
      if (pml) {
        Q::st(p1c + pi, pa);
        Q::st(p1c + NRP + pi, pb);
      }
    }
    compute_sync(ncomp);
    if (abort_flag) break;

    // ---- level 1, E^{n+1}(x), rows y0-1 .. y0+TY ----
    if (l1 && do_e1) {
      const float* Ms = reinterpret_cast<const float*>(Bs + g.b_m) + (y0 - 2 - ma);
      const float sig[3] = {Ms[ra], Ms[g.MT + ra], Ms[2 * g.MT + ra]};
      const bool src = src_row && x >= a.sx0 && x < a.sx0 + a.snx;
      float en[3][4], pa[4], pb[4];
      e_quad(h1c, h1c + NRZ, h1c + 2 * NRZ, h1p + NRZ, h1p + 2 * NRZ, AE, NEZ,
             reinterpret_cast<const T*>(Bs + g.b_c), NRZ, sig, AP + 2 * NRP, NRP,
             src, x, wave1, en, pa, pb);
#pragma unroll
      for (int c = 0; c < 3; ++c) Q::st(e1c + c * NRZ + ie, en[c]);
      if (pml) {
        Q::st(p1c + 2 * NRP + pi, pa);
        Q::st(p1c + 3 * NRP + pi, pb);
      }
    }
    // Ring A slot of plane x is no longer read.
    if (l1) {
      __syncwarp();
      if ((tid & 31) == 0) mbar_arrive(&doneA[sA]);
    }
    compute_sync(ncomp);
    if (abort_flag) break;

    // ---- level 2, H^{n+3/2}(x-1), rows y0-1 .. y0+TY-1 ----
    const int xm = x - 1;
    if (l2 && do_h2) {
      const T* e2n = x < X ? e1c : nullptr;
      float hn[3][4], pa[4], pb[4];
      h_quad(e1p, NRZ, e2n, NRZ, h1p, NRZ, p1p, NRP, hn, pa, pb);
      Q::st(H2x + ie, hn[0]);
      Q::st(h2yz + ie, hn[1]);
      Q::st(h2yz + NRZ + ie, hn[2]);
      if (st2 && ra >= 2) {
        const long long o = (long long)xm * YZ + (long long)y * Z + z0;
#pragma unroll
        for (int c = 0; c < 3; ++c) Q::st(fout + (3 + c) * N + o, hn[c]);
        if (pml) {
          const long long po = ((long long)xm * Y + y) * Pp + col;
          Q::st(psi_out + po, pa);
          Q::st(psi_out + PXY + po, pb);
        }
      }
    }
    compute_sync(ncomp);
    if (abort_flag) break;

    // ---- level 2, E^{n+2}(x-1), rows y0 .. y0+TY-1 ----
    if (st2 && do_e2) {
      const float* Ms = reinterpret_cast<const float*>(Bm + g.b_m) + (y0 - 2 - ma);
      const float sig[3] = {Ms[ra], Ms[g.MT + ra], Ms[2 * g.MT + ra]};
      const bool src = src_row && xm >= a.sx0 && xm < a.sx0 + a.snx;
      float en[3][4], pa[4], pb[4];
      e_quad(H2x, h2yz, h2yz + NRZ, h2yzp, h2yzp + NRZ, e1p, NRZ,
             reinterpret_cast<const T*>(Bm + g.b_c), NRZ, sig, p1p + 2 * NRP, NRP,
             src, xm, wave2, en, pa, pb);
      const long long o = (long long)xm * YZ + (long long)y * Z + z0;
#pragma unroll
      for (int c = 0; c < 3; ++c) Q::st(fout + c * N + o, en[c]);
      if (pml) {
        const long long po = ((long long)xm * Y + y) * Pp + col;
        Q::st(psi_out + 2 * PXY + po, pa);
        Q::st(psi_out + 3 * PXY + po, pb);
      }
    }
    // Ring B slot of plane x - 1 is no longer read.
    if (x > a1 && x - 1 <= last1) {
      __syncwarp();
      if ((tid & 31) == 0) mbar_arrive(&doneB[sBm]);
    }
    // Advance the ring positions to plane x + 1.
    if (l1) {
      sA = sA1;
      rA = rA1;
      if (++sA1 == SA) {
        sA1 = 0;
        ++rA1;
      }
      sBm = sB;
      if (++sB == SB) {
        sB = 0;
        ++rB;
      }
    } else {
      sBm = sB;
    }
  }
}

// (zz, tile_y) shapes of the lean two-step kernel: the two-step tile heights
// the host picks for these zz.
#define PJZ_LEAN2_SHAPES(X_) X_(64, 14)

template <int ZC, int TYC, typename T>
__global__ void __launch_bounds__(384, 1) yee_lean2_kernel(const StreamArgs sa) {
  extern __shared__ __align__(16) unsigned char lean2_sm[];
  lean2_tile<ZC, TYC, T>(sa, blockIdx.x, blockIdx.y, lean2_sm);
}

}  // namespace pjzfdtd
