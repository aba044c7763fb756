// Two-step (temporally blocked) streamed Yee kernel for sm_103a.
//
// One launch advances the whole state by two time steps, n and n + 1,
// reading every field, coefficient and PML state from HBM once and writing
// the results once: about 60 B per cell per launch plus tile halos, against
// 60 B per cell per step for the single-step kernel.
//
// A CTA owns `tile_y` rows of y (all of z) and the x-planes [xs, xe) of a
// segment, and marches x as a two-level wavefront.  In iteration x:
//   level 1 computes H^{n+1/2} and E^{n+1} of plane x over rows y0-2..y0+TY
//   (H) and y0-1..y0+TY (E) -- the tile plus the halo level 2 needs;
//   level 2 computes H^{n+3/2} and E^{n+2} of plane x-1 over rows
//   y0-1..y0+TY-1 and y0..y0+TY-1 from level 1's planes x-1 and x, and
//   stores rows y0..y0+TY-1 straight to HBM (one 256-byte row per warp for
//   zz = 64, fully coalesced).
// Level 1 starts two planes before the segment and level 2 one plane before
// it, so every plane of [xs, xe) sees correct neighbours; those halo planes
// are computed but not stored.
//
// Inputs arrive through two rings of shared-memory slots filled by a
// producer warp with bulk copies (cp.async.bulk, completion on mbarriers):
//   ring A, one slot per plane: E rows y0-2..y0+TY+1, H rows y0-2..y0+TY and
//     the z-PML state rows -- released after level 1's E phase of the plane;
//   ring B, one slot per plane: the E coefficient and absorber rows --
//     released after level 2's E phase of the plane, one iteration later.
// Level-1 results live in shared memory (two planes of H and E); level-2 H
// keeps planes x-1 and x-2 (the x-neighbour of the next E phase).
//
// Every buffer row is indexed by ra = y - (y0 - 2), and a compute thread
// keeps the same (row, z-pair) in every phase, so the z-PML state that level
// 1 hands to level 2 is read back by the thread that wrote it.  Three named
// barriers per plane separate the phases; rows outside the domain are never
// written and read as the zero boundary.
//
// Per cell and step the arithmetic is the explicit RN FP32 sequence of the
// single-step kernels and of the CPU oracle, so results are bit-identical
// to them.  Waits are bounded as in the single-step kernel.
#pragma once

#include "stream_kernel.cuh"

namespace pjzfdtd {

constexpr int kStream2Threads = 576;  // up to 17 compute warps + 1 producer

// Shared-memory geometry of one two-level CTA (floats unless noted).
struct Stream2Geom {
  int TY, Z, Pp, NR, NE, MT;
  int a_e, a_h, a_p, a_stage;  // ring A slot: E [3][NE*Z], H [3][NR*Z], psi [4][NR*Pp]
  int b_c, b_m, b_stage;       // ring B slot: cb [3][NR*Z], absorber [3][MT]
  __host__ __device__ Stream2Geom(int ty, int z, int p) {
    TY = ty;
    Z = z;
    Pp = round4(p);
    NR = ty + 3;                // rows y0-2 .. y0+TY
    NE = ty + 4;                // E rows y0-2 .. y0+TY+1
    MT = round4(ty + 2) + 8;    // 4-aligned absorber window around y0-1..y0+TY
    a_e = 0;
    a_h = a_e + 3 * NE * z;
    a_p = a_h + 3 * NR * z;
    a_stage = a_p + 4 * NR * Pp;
    b_c = 0;
    b_m = b_c + 3 * NR * z;
    b_stage = b_m + 3 * MT;
  }
  // After the rings: H1 [2][3][NR*Z], E1 [2][3][NR*Z], H2x [NR*Z],
  // H2yz [2][2][NR*Z], P1 [2][4][NR*Pp].
  __host__ __device__ size_t inter_floats() const {
    return (size_t)(6 + 6 + 5) * NR * Z + 8 * (size_t)NR * Pp;
  }
  __host__ __device__ size_t bytes(int sa, int sb) const {
    return ((size_t)sa * a_stage + (size_t)sb * b_stage + inter_floats()) *
               sizeof(float) +
           (size_t)(2 * sa + 2 * sb) * sizeof(uint64_t) + 16;
  }
};

// Per-thread z data of the thread's z-pair.  The CPML decay and coupling
// coefficients (b, c) are read from `zc` ([6][Z]: ik_e, b_e, c_e, ik_h, b_h,
// c_h) only inside the slabs, which keeps them out of the register budget.
struct ZPair {
  int z0;
  int pz[2];  // PML-state column of z0 + k, -1 outside the slabs
  float ike[2], ikh[2];
  bool zpml;
  const float* zc;
};

// H^{n+1/2} of the z-pair at row ra (stride Z per row).  E: plane x with
// component stride es (rows ra, ra + 1 read); E1: plane x + 1 (null at the
// last plane, read as zero) with stride e1s; Ho: old H, stride hs; Pin:
// PML state comps 0, 1 (stride ps per comp).  New PML state goes to pn.
__device__ __forceinline__ void h_pair(const ZPair& zp, int Z, int ra,
                                       const float* E, int es, const float* E1,
                                       int e1s, const float* Ho, int hs,
                                       const float* Pin, int ps, int Pp,
                                       float mdt, float hn[3][2], float pn[2][2]) {
  const int z0 = zp.z0;
  const int ie = ra * Z + z0;
  const float2 ex = *reinterpret_cast<const float2*>(E + ie);
  const float2 ey = *reinterpret_cast<const float2*>(E + es + ie);
  const float2 ez = *reinterpret_cast<const float2*>(E + 2 * es + ie);
  const float2 ex_y1 = *reinterpret_cast<const float2*>(E + ie + Z);
  const float2 ez_y1 = *reinterpret_cast<const float2*>(E + 2 * es + ie + Z);
  const bool zin = z0 + 2 < Z;
  const float ex_z2 = zin ? E[ie + 2] : 0.f;
  const float ey_z2 = zin ? E[es + ie + 2] : 0.f;
  float2 e1y = make_float2(0.f, 0.f), e1z = make_float2(0.f, 0.f);
  if (E1) {
    e1y = *reinterpret_cast<const float2*>(E1 + e1s + ie);
    e1z = *reinterpret_cast<const float2*>(E1 + 2 * e1s + ie);
  }
  const float2 hox = *reinterpret_cast<const float2*>(Ho + ie);
  const float2 hoy = *reinterpret_cast<const float2*>(Ho + hs + ie);
  const float2 hoz = *reinterpret_cast<const float2*>(Ho + 2 * hs + ie);
  const float exs[2] = {ex.x, ex.y}, eys[2] = {ey.x, ey.y}, ezs[2] = {ez.x, ez.y};
  const float exy1[2] = {ex_y1.x, ex_y1.y}, ezy1[2] = {ez_y1.x, ez_y1.y};
  const float exz1[2] = {ex.y, ex_z2}, eyz1[2] = {ey.y, ey_z2};
  const float e1ys[2] = {e1y.x, e1y.y}, e1zs[2] = {e1z.x, e1z.y};
  const float hos[3][2] = {{hox.x, hox.y}, {hoy.x, hoy.y}, {hoz.x, hoz.y}};
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const float dEz_y = fsub(ezy1[q], ezs[q]), dEy_z = fsub(eyz1[q], eys[q]);
    const float dEx_z = fsub(exz1[q], exs[q]), dEz_x = fsub(e1zs[q], ezs[q]);
    const float dEy_x = fsub(e1ys[q], eys[q]), dEx_y = fsub(exy1[q], exs[q]);
    float zEy, zEx;
    if (zp.zpml && zp.pz[q] >= 0) {
      const int pi = ra * Pp + zp.pz[q];
      const float bh = zp.zc[4 * Z + z0 + q], ch = zp.zc[5 * Z + z0 + q];
      const float na = ffma(ch, dEy_z, fmul(bh, Pin[pi]));
      const float nb = ffma(ch, dEx_z, fmul(bh, Pin[ps + pi]));
      pn[0][q] = na;
      pn[1][q] = nb;
      zEy = ffma(dEy_z, zp.ikh[q], na);
      zEx = ffma(dEx_z, zp.ikh[q], nb);
    } else {
      zEy = fmul(dEy_z, zp.ikh[q]);
      zEx = fmul(dEx_z, zp.ikh[q]);
    }
    hn[0][q] = ffma(mdt, fsub(dEz_y, zEy), hos[0][q]);
    hn[1][q] = ffma(mdt, fsub(zEx, dEz_x), hos[1][q]);
    hn[2][q] = ffma(mdt, fsub(dEy_x, dEx_y), hos[2][q]);
  }
}

// E^{n+1} of the z-pair at row ra.  Hx/Hy/Hz: new H of plane x (rows ra,
// ra - 1); Hyp/Hzp: new H of plane x - 1; Eo: old E, component stride es;
// Cb: coefficient rows, stride cs; sig: absorber of the row; Pin: PML state
// comps 2, 3; J: source current of the cells (already summed, zero outside).
__device__ __forceinline__ void e_pair(const ZPair& zp, int Z, int ra,
                                       const float* Hx, const float* Hy,
                                       const float* Hz, const float* Hyp,
                                       const float* Hzp, const float* Eo, int es,
                                       const float* Cb, int cs, const float sig[3],
                                       const float* Pin, int ps, int Pp,
                                       const float J[3][2], bool src,
                                       float en[3][2], float pn[2][2]) {
  const int z0 = zp.z0;
  const int ih = ra * Z + z0;
  const float2 hx = *reinterpret_cast<const float2*>(Hx + ih);
  const float2 hy = *reinterpret_cast<const float2*>(Hy + ih);
  const float2 hz = *reinterpret_cast<const float2*>(Hz + ih);
  const float2 hx_ym = *reinterpret_cast<const float2*>(Hx + ih - Z);
  const float2 hz_ym = *reinterpret_cast<const float2*>(Hz + ih - Z);
  const bool zin = z0 > 0;
  const float hx_zm = zin ? Hx[ih - 1] : 0.f;
  const float hy_zm = zin ? Hy[ih - 1] : 0.f;
  const float2 hyp = *reinterpret_cast<const float2*>(Hyp + ih);
  const float2 hzp = *reinterpret_cast<const float2*>(Hzp + ih);
  const float2 eox = *reinterpret_cast<const float2*>(Eo + ih);
  const float2 eoy = *reinterpret_cast<const float2*>(Eo + es + ih);
  const float2 eoz = *reinterpret_cast<const float2*>(Eo + 2 * es + ih);
  const float2 cbx = *reinterpret_cast<const float2*>(Cb + ih);
  const float2 cby = *reinterpret_cast<const float2*>(Cb + cs + ih);
  const float2 cbz = *reinterpret_cast<const float2*>(Cb + 2 * cs + ih);
  const float hxs[2] = {hx.x, hx.y}, hys[2] = {hy.x, hy.y}, hzs[2] = {hz.x, hz.y};
  const float hxym[2] = {hx_ym.x, hx_ym.y}, hzym[2] = {hz_ym.x, hz_ym.y};
  const float hxzm[2] = {hx_zm, hx.x}, hyzm[2] = {hy_zm, hy.x};
  const float hyps[2] = {hyp.x, hyp.y}, hzps[2] = {hzp.x, hzp.y};
  const float eo[3][2] = {{eox.x, eox.y}, {eoy.x, eoy.y}, {eoz.x, eoz.y}};
  const float cbs[3][2] = {{cbx.x, cbx.y}, {cby.x, cby.y}, {cbz.x, cbz.y}};
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const float dHz_y = fsub(hzs[q], hzym[q]), dHy_z = fsub(hys[q], hyzm[q]);
    const float dHx_z = fsub(hxs[q], hxzm[q]), dHz_x = fsub(hzs[q], hzps[q]);
    const float dHy_x = fsub(hys[q], hyps[q]), dHx_y = fsub(hxs[q], hxym[q]);
    float zHy, zHx;
    if (zp.zpml && zp.pz[q] >= 0) {
      const int pi = ra * Pp + zp.pz[q];
      const float be = zp.zc[Z + z0 + q], ce = zp.zc[2 * Z + z0 + q];
      const float na = ffma(ce, dHy_z, fmul(be, Pin[pi]));
      const float nb = ffma(ce, dHx_z, fmul(be, Pin[ps + pi]));
      pn[0][q] = na;
      pn[1][q] = nb;
      zHy = ffma(dHy_z, zp.ike[q], na);
      zHx = ffma(dHx_z, zp.ike[q], nb);
    } else {
      zHy = fmul(dHy_z, zp.ike[q]);
      zHx = fmul(dHx_z, zp.ike[q]);
    }
    float cur[3] = {fsub(dHz_y, zHy), fsub(zHx, dHz_x), fsub(dHy_x, dHx_y)};
    if (src) {
#pragma unroll
      for (int c = 0; c < 3; ++c) cur[c] = fsub(cur[c], J[c][q]);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float rr = ffma(-sig[c], eo[c][q], cur[c]);
      en[c][q] = ffma(cbs[c][q], rr, eo[c][q]);
    }
  }
}

// Source current of the z-pair at (x, y) for the waveform row `wave`, summed
// over the columns in the oracle's order; returns false when the pair has
// no source cell (J untouched).
__device__ __forceinline__ bool source_pair(const StepArgs& a, int x, int y,
                                            int z0, const float* wave,
                                            float J[3][2]) {
  if (x < a.sx0 || x >= a.sx0 + a.snx || y < a.sy0 || y >= a.sy0 + a.sny)
    return false;
  bool any = false;
  const long long sb = (long long)a.snx * a.sny * a.snz;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int z = z0 + q;
    const bool in = z >= a.sz0 && z < a.sz0 + a.snz;
    any |= in;
    const long long si =
        ((long long)(x - a.sx0) * a.sny + (y - a.sy0)) * a.snz + (z - a.sz0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float j = 0.f;
      if (in)
        for (int w = 0; w < a.snc; ++w)
          j = ffma(a.src[((long long)w * 3 + c) * sb + si], wave[w], j);
      J[c][q] = j;
    }
  }
  return any;
}


// One CTA of the two-step kernel: tile `tile` of y rows, segment `seg` of x
// planes.  ZC / TYC fix zz / tile_y at compile time (0: from the arguments).
// sa.stages2 packs the ring depths: ring A in the low byte, ring B above.
template <int ZC, int TYC>
__device__ __forceinline__ void stream2_tile(const StreamArgs& sa, int tile,
                                             int seg, float* sm) {
  const StepArgs& a = sa.s;
  const int X = a.X, Y = a.Y;
  const int Z = ZC ? ZC : a.Z;
  const int TY = TYC ? TYC : a.tile_y;
  const int SA = sa.stages2 & 0xff, SB = (sa.stages2 >> 8) & 0xff;
  const Stream2Geom g(TY, Z, a.plo + a.phi);
  const int Pp = g.Pp, NR = g.NR, NE = g.NE;
  const int NRZ = NR * Z, NEZ = NE * Z, NRP = NR * Pp;
  float* ringA = sm;
  float* ringB = ringA + (size_t)SA * g.a_stage;
  float* H1 = ringB + (size_t)SB * g.b_stage;  // [2][3][NRZ]
  float* E1 = H1 + 6 * (size_t)NRZ;            // [2][3][NRZ]
  float* H2x = E1 + 6 * (size_t)NRZ;           // [NRZ]
  float* H2yz = H2x + NRZ;                     // [2][2][NRZ]
  float* P1 = H2yz + 4 * (size_t)NRZ;          // [2][4][NRP]
  uint64_t* fullA = reinterpret_cast<uint64_t*>(P1 + 8 * (size_t)NRP);
  uint64_t* doneA = fullA + SA;
  uint64_t* fullB = doneA + SA;
  uint64_t* doneB = fullB + SB;
  __shared__ int abort_flag;

  const int tid = threadIdx.x;
  const int ncomp = blockDim.x - 32;
  const int nwarps = ncomp >> 5;
  const bool producer = tid >= ncomp;
  const int Zh = Z >> 1;
  const int rpt = ncomp / Zh;
  const int rt = tid / Zh;
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
  for (size_t i = tid; i < (size_t)SA * g.a_stage + (size_t)SB * g.b_stage +
                               g.inter_floats();
       i += blockDim.x)
    sm[i] = 0.f;
  fence_async_smem();
  __syncthreads();

  if (producer) {
    if ((tid & 31) != 0) return;
    // ---------------- producer (one lane) ----------------
    const uint32_t eb = (uint32_t)((e_hi - ylo) * Z * 4);
    const uint32_t hb = (uint32_t)((h_hi - ylo) * Z * 4);
    const uint32_t pb = (uint32_t)((h_hi - ylo) * Pp * 4);
    const uint32_t cbb = (uint32_t)((h_hi - clo) * Z * 4);
    const uint32_t mbb = (uint32_t)((mb - ma) * 4);
    const int r0 = ylo - (y0 - 2);  // buffer row of the first copied row
    auto fillA = [&](int xp, int slot) {
      float* st = ringA + (size_t)slot * g.a_stage;
      const bool fullp = xp <= last1;
      const uint32_t total = sa.stall_bytes + 3 * eb +
                             (fullp ? 3 * hb + (Pp > 0 ? 4 * pb : 0) : 0);
      mbar_expect_tx(&fullA[slot], total);
      const long long base = (long long)xp * YZ + (long long)ylo * Z;
      for (int c = 0; c < 3; ++c)
        bulk_g2s(st + g.a_e + c * NEZ + r0 * Z, a.fin + c * N + base, eb,
                 &fullA[slot]);
      if (!fullp) return;
      for (int c = 0; c < 3; ++c)
        bulk_g2s(st + g.a_h + c * NRZ + r0 * Z, a.fin + (3 + c) * N + base, hb,
                 &fullA[slot]);
      if (Pp > 0)
        for (int c = 0; c < 4; ++c)
          bulk_g2s(st + g.a_p + c * NRP + r0 * Pp,
                   a.psi_in + c * PXY + ((long long)xp * Y + ylo) * Pp, pb,
                   &fullA[slot]);
    };
    auto fillB = [&](int xp, int slot) {
      float* st = ringB + (size_t)slot * g.b_stage;
      mbar_expect_tx(&fullB[slot], sa.stall_bytes + 3 * (cbb + mbb));
      const long long base = (long long)xp * YZ + (long long)clo * Z;
      for (int c = 0; c < 3; ++c) {
        bulk_g2s(st + g.b_c + c * NRZ + (clo - (y0 - 2)) * Z, a.cb + c * N + base,
                 cbb, &fullB[slot]);
        bulk_g2s(st + g.b_m + c * g.MT,
                 sa.mask_ws + ((long long)xp * 3 + c) * sa.Yp + ma, mbb,
                 &fullB[slot]);
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
    int sA = 0, sB = 0;          // slots of plane x (ring A) / x-1 (ring B)
    uint32_t rA = 0, rB = 0;     // their fill rounds
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
  ZPair zp;
  zp.z0 = 2 * (tid % Zh);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int z = zp.z0 + k;
    zp.pz[k] = z < a.plo ? z : (z >= Z - a.phi ? z - (Z - a.phi) + a.plo : -1);
    zp.ike[k] = a.zc[z];
    zp.ikh[k] = a.zc[3 * Z + z];
  }
  zp.zpml = zp.pz[0] >= 0 || zp.pz[1] >= 0;
  zp.zc = a.zc;
  const float mdt = -a.dt;
  const bool active = rt < rpt;
  const int z0 = zp.z0;
  const float* wave1 = a.wave;
  const float* wave2 = a.snc > 0 ? a.wave + a.snc : nullptr;

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
    const float* As = ringA + (size_t)sA * g.a_stage;
    const float* A1s = ringA + (size_t)sA1 * g.a_stage;
    const float* Bs = ringB + (size_t)sB * g.b_stage;
    const float* Bm = ringB + (size_t)sBm * g.b_stage;
    float* h1c = H1 + (size_t)b * 3 * NRZ;
    const float* h1p = H1 + (size_t)(b ^ 1) * 3 * NRZ;
    float* e1c = E1 + (size_t)b * 3 * NRZ;
    const float* e1p = E1 + (size_t)(b ^ 1) * 3 * NRZ;
    float* p1c = P1 + (size_t)b * 4 * NRP;
    const float* p1p = P1 + (size_t)(b ^ 1) * 4 * NRP;
    // Level 2 works on plane x - 1: its H2 y/z buffer has parity b ^ 1 and
    // the previous plane's (x - 2) parity b.
    float* h2yz = H2yz + (size_t)(b ^ 1) * 2 * NRZ;
    const float* h2yzp = H2yz + (size_t)b * 2 * NRZ;

    // ---- level 1, H^{n+1/2}(x), rows y0-2 .. y0+TY ----
    if (ok && l1 && active) {
      const float* e1n = x + 1 < X ? A1s + g.a_e : nullptr;
      for (int ra = rt; ra < NR; ra += rpt) {
        const int y = y0 - 2 + ra;
        if (y < 0 || y >= Y) continue;
        float hn[3][2], pn[2][2];
        h_pair(zp, Z, ra, As + g.a_e, NEZ, e1n, NEZ, As + g.a_h, NRZ,
               As + g.a_p, NRP, Pp, mdt, hn, pn);
        const int ie = ra * Z + z0;
#pragma unroll
        for (int c = 0; c < 3; ++c)
          *reinterpret_cast<float2*>(h1c + c * NRZ + ie) = make_float2(hn[c][0], hn[c][1]);
        if (zp.zpml) {
#pragma unroll
          for (int q = 0; q < 2; ++q)
            if (zp.pz[q] >= 0) {
              p1c[ra * Pp + zp.pz[q]] = pn[0][q];
              p1c[NRP + ra * Pp + zp.pz[q]] = pn[1][q];
            }
        }
      }
    }
    compute_sync(ncomp);
    if (abort_flag) break;

    // ---- level 1, E^{n+1}(x), rows y0-1 .. y0+TY ----
    if (l1 && active) {
      const float* Ms = Bs + g.b_m + (y0 - 2 - ma);  // absorber of row ra at [ra]
      for (int ra = rt; ra < NR; ra += rpt) {
        const int y = y0 - 2 + ra;
        if (ra < 1 || y < 0 || y >= Y) continue;
        const float sig[3] = {Ms[ra], Ms[g.MT + ra], Ms[2 * g.MT + ra]};
        float J[3][2];
        const bool src = a.snc > 0 && source_pair(a, x, y, z0, wave1, J);
        float en[3][2], pn[2][2];
        e_pair(zp, Z, ra, h1c, h1c + NRZ, h1c + 2 * NRZ, h1p + NRZ, h1p + 2 * NRZ,
               As + g.a_e, NEZ, Bs + g.b_c, NRZ, sig, As + g.a_p + 2 * NRP, NRP,
               Pp, J, src, en, pn);
        const int ie = ra * Z + z0;
#pragma unroll
        for (int c = 0; c < 3; ++c)
          *reinterpret_cast<float2*>(e1c + c * NRZ + ie) = make_float2(en[c][0], en[c][1]);
        if (zp.zpml) {
#pragma unroll
          for (int q = 0; q < 2; ++q)
            if (zp.pz[q] >= 0) {
              p1c[2 * NRP + ra * Pp + zp.pz[q]] = pn[0][q];
              p1c[3 * NRP + ra * Pp + zp.pz[q]] = pn[1][q];
            }
        }
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
    if (l2 && active) {
      const float* e2n = x < X ? e1c : nullptr;
      for (int ra = rt; ra < NR; ra += rpt) {
        const int y = y0 - 2 + ra;
        if (ra < 1 || ra >= NR - 1 || y < 0 || y >= Y) continue;
        float hn[3][2], pn[2][2];
        h_pair(zp, Z, ra, e1p, NRZ, e2n, NRZ, h1p, NRZ, p1p, NRP, Pp, mdt, hn, pn);
        const int ie = ra * Z + z0;
        *reinterpret_cast<float2*>(H2x + ie) = make_float2(hn[0][0], hn[0][1]);
        *reinterpret_cast<float2*>(h2yz + ie) = make_float2(hn[1][0], hn[1][1]);
        *reinterpret_cast<float2*>(h2yz + NRZ + ie) = make_float2(hn[2][0], hn[2][1]);
        if (st2 && ra >= 2) {
          const long long o = (long long)xm * YZ + (long long)y * Z + z0;
#pragma unroll
          for (int c = 0; c < 3; ++c)
            *reinterpret_cast<float2*>(a.fout + (3 + c) * N + o) =
                make_float2(hn[c][0], hn[c][1]);
          if (zp.zpml) {
            const long long po = ((long long)xm * Y + y) * Pp;
#pragma unroll
            for (int q = 0; q < 2; ++q)
              if (zp.pz[q] >= 0) {
                a.psi_out[po + zp.pz[q]] = pn[0][q];
                a.psi_out[PXY + po + zp.pz[q]] = pn[1][q];
              }
          }
        }
      }
    }
    compute_sync(ncomp);
    if (abort_flag) break;

    // ---- level 2, E^{n+2}(x-1), rows y0 .. y0+TY-1 ----
    if (st2 && active) {
      const float* Ms = Bm + g.b_m + (y0 - 2 - ma);
      for (int ra = rt; ra < NR; ra += rpt) {
        const int y = y0 - 2 + ra;
        if (ra < 2 || ra >= NR - 1 || y >= Y) continue;
        const float sig[3] = {Ms[ra], Ms[g.MT + ra], Ms[2 * g.MT + ra]};
        float J[3][2];
        const bool src = a.snc > 0 && source_pair(a, xm, y, z0, wave2, J);
        float en[3][2], pn[2][2];
        e_pair(zp, Z, ra, H2x, h2yz, h2yz + NRZ, h2yzp, h2yzp + NRZ, e1p, NRZ,
               Bm + g.b_c, NRZ, sig, p1p + 2 * NRP, NRP, Pp, J, src, en, pn);
        const long long o = (long long)xm * YZ + (long long)y * Z + z0;
#pragma unroll
        for (int c = 0; c < 3; ++c)
          *reinterpret_cast<float2*>(a.fout + c * N + o) = make_float2(en[c][0], en[c][1]);
        if (zp.zpml) {
          const long long po = ((long long)xm * Y + y) * Pp;
#pragma unroll
          for (int q = 0; q < 2; ++q)
            if (zp.pz[q] >= 0) {
              a.psi_out[2 * PXY + po + zp.pz[q]] = pn[0][q];
              a.psi_out[3 * PXY + po + zp.pz[q]] = pn[1][q];
            }
        }
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

// (zz, tile_y) pairs with a compile-time specialisation of the two-step
// kernel: the tile heights the host picks for these zz.
#define PJZ_STREAM2_SHAPES(X_) X_(64, 14) X_(64, 11) X_(64, 10) X_(48, 15)

// CTA size bound of a specialisation: 16 warps (128 registers per thread)
// when its rows y0-2..y0+TY fit 15 compute warps in one pass, else 18 warps.
constexpr int stream2_bound(int zc, int tyc) {
  return zc > 0 && (tyc + 3) * (zc / 2) <= 480 ? 512 : kStream2Threads;
}

template <int ZC, int TYC>
__global__ void __launch_bounds__(stream2_bound(ZC, TYC), 1)
    yee_stream2_kernel(const StreamArgs sa) {
  extern __shared__ __align__(16) float sm[];
  stream2_tile<ZC, TYC>(sa, blockIdx.x, blockIdx.y, sm);
}

// Batched two-step tiles: the zz = 64 / tile_y 14 specialisation, else the
// generic body (each inlined shape costs compile time).
__device__ __forceinline__ void stream2_tile_any(const StreamArgs& sa, int tile,
                                                 int seg, float* sm) {
  if (sa.s.Z == 64 && sa.s.tile_y == 14) return stream2_tile<64, 14>(sa, tile, seg, sm);
  stream2_tile<0, 0>(sa, tile, seg, sm);
}

// Batched launches: block b runs entry work[b] = (sim, tile, seg) when
// that problem's launch `launch` of its schedule has the kernel's step count
// (sched[launch * nsim + sim] = (first step, steps)); args[(launch & 1) *
// nsim + sim] holds its arguments for the buffer parity of this launch with
// the waveform row pointer at step 0.  A launch whose problems mix one- and
// two-step entries runs both kernels over the same work prefix.
#ifdef PJZ_BATCH2_KERNEL  // defined in kern_batch2.cu only
__global__ void __launch_bounds__(kStream2Threads, 1)
    yee_stream_batch2_kernel(const BatchArgs ba) {
  extern __shared__ __align__(16) float sm[];
  const int4 w = ba.work[blockIdx.x];
  const int2 sc = ba.sched[(size_t)ba.launch * ba.nsim + w.x];
  if (sc.y != 2) return;
  StreamArgs sa = ba.args[(ba.launch & 1) * ba.nsim + w.x];
  if (sa.s.snc > 0) sa.s.wave += (long long)sc.x * sa.s.snc;
  stream2_tile_any(sa, w.y, w.z, sm);
}

#endif  // PJZ_BATCH2_KERNEL

}  // namespace pjzfdtd
