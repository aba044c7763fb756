// Streamed Yee step kernel for sm_103a: the same single-step update as
// yee_step_kernel, with every x-plane tile moved by the bulk-copy engine.
//
// A CTA owns `tile_y` rows of y (all of z) and marches through `seg_x`
// x-planes.  For plane x the tile needs E rows -1..TY, H rows -1..TY-1, the
// E coefficient rows 0..TY-1, the absorber row and the z-PML state rows; in
// the workspace layouts ([c][x][y][z] fields, [x][c][Yp] absorber,
// [c][x][y][Pp] PML state, Yp and Pp padded to multiples of 4) each piece is
// one contiguous 16-byte aligned span, so one thread fills a ring slot with
// bulk copies (cp.async.bulk, completion on the slot's mbarrier) `stages`-1
// planes ahead.  Results go the same way: new H stays in shared memory (it
// is also the x-1 neighbour of the next plane), new E and PML state are
// written to shared staging buffers, and one thread bulk-stores them.  No
// compute thread issues a global load or store on the main path.
//
// Each thread updates a pair of adjacent z cells with 64-bit shared-memory
// accesses; for zz = 64 a warp covers one full z column of one y row.
//
// Requires zz % 4 == 0; the host falls back to yee_step_kernel otherwise.
// Arithmetic is the same explicit RN sequence as the CPU oracle, so results
// are bit-identical to it.
//
// The last warp of the CTA is a producer that issues every bulk copy and
// store; the other warps only compute, synchronised with the producer by
// mbarriers and among themselves by a named barrier, so the serial issue of
// copies never sits between two compute phases.
//
// Every wait is bounded: an mbarrier wait that exceeds kWaitCycles sets the
// status word and the abort flag, the compute warps leave together at their
// next named barrier, and the producer drains the copies it issued (again
// with bounded waits) before the CTA exits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "step_kernel.cuh"

namespace pjzfdtd {

constexpr long long kWaitCycles = 4000000000LL;  // default bound, ~2 s at 2 GHz
constexpr int kWaveCache = 64;  // waveform columns kept in shared memory
constexpr int kStatusTimeout = 4;

struct StreamArgs {
  StepArgs s;
  int stages;                             // single-step ring depth
  int stages2;                            // two-step rings: A | B << 8
  int Yp;                                 // padded y length of mask_ws rows
  const float* __restrict__ mask_ws;      // [X][3][Yp]
  int* status;                            // device status word (0 = ok)
  long long wait_cycles;                  // bound of every wait (SM cycles)
  unsigned stall_bytes;                   // test hook: unfilled expected bytes
  // Source rows carried in the ring: floats per slot reserved for them (0:
  // none), rows per (column, component) block, and whether the producer
  // fills them (else the E update reads the source from global memory).
  int src_ring;
  int src_rows;
  int src_tma;
  // The source box re-laid out as [x][y][column][component][z] in the
  // workspace, so that a tile's box rows of one plane are one span.
  const float* __restrict__ src_ws;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait; returns false (and sets *status) if the phase never flips.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          int* status, long long limit) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (clock64() - t0 > limit) {
      atomicExch(status, kStatusTimeout);
      return false;
    }
  }
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_s2g(void* dst, const void* src,
                                         uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(
                   dst),
               "r"(smem_u32(src)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__host__ __device__ inline int round4(int v) { return (v + 3) & ~3; }

// Shared-memory geometry of one CTA (floats unless noted); `sw` floats per
// slot hold the source rows of the plane when the ring carries them.
struct StreamGeom {
  int TY, Z, P, Pp, RE, RH, MT;
  int e_off, h_off, c_off, m_off, p_off, s_off, stage;  // within a ring slot
  __host__ __device__ StreamGeom(int ty, int z, int p, int sw = 0) {
    TY = ty;
    Z = z;
    P = p;
    Pp = round4(p);
    RE = ty + 2;
    RH = ty + 1;
    MT = round4(ty) + 8;  // 4-aligned window around rows y0..y0+TY-1
    e_off = 0;
    h_off = e_off + 3 * RE * z;
    c_off = h_off + 3 * RH * z;
    m_off = c_off + 3 * ty * z;
    p_off = m_off + 3 * MT;
    s_off = p_off + 4 * RH * Pp;
    stage = s_off + sw;
  }
  // CTA buffers after the ring: new H [2][3][RH*Z], new E [2][3][TY*Z],
  // new PML state [2][4][TY*Pp].
  __host__ __device__ size_t hn_floats() const { return 2 * 3 * (size_t)RH * Z; }
  __host__ __device__ size_t en_floats() const { return 2 * 3 * (size_t)TY * Z; }
  __host__ __device__ size_t pn_floats() const { return 2 * 4 * (size_t)TY * Pp; }
  __host__ __device__ size_t bytes(int stages) const {
    return ((size_t)stages * stage + hn_floats() + en_floats() + pn_floats()) *
               sizeof(float) +
           (size_t)(2 * stages + 2) * sizeof(uint64_t) + 16;
  }
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Bounded wait that also gives up when another thread of the CTA already
// did (`*abort` set); returns false in either case.
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, uint32_t parity,
                                                   int* status,
                                                   volatile int* abort,
                                                   long long limit) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (clock64() - t0 > limit) {
      atomicExch(status, kStatusTimeout);
      *abort = 1;
      return false;
    }
  }
}

__device__ __forceinline__ void compute_sync(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

// Warp-specialised CTA: the last warp is the producer (bulk loads into the
// ring, bulk stores of results), all other warps compute.  Barriers:
//   full[s]  -- ring slot s holds its plane (producer expect_tx + copies);
//   done[s]  -- every compute warp finished the plane in slot s, whose
//               results sit in output buffer b = (x - x0) & 1 (count = warps);
//   free[b]  -- the producer's bulk stores finished reading buffer b.
// One CTA's work: tile `tile` of y rows and segment `seg` of x planes of the
// problem described by `sa`.  ZC / TYC fix zz / tile_y at compile time for
// the common thin-z shapes (every shared-memory offset then folds into an
// immediate); 0 means "read it from the arguments".  SR: the ring carries
// the source box rows (sa.src_tma); without it the source code path is the
// plain global-load one and adds nothing to a source-free cell.
template <int ZC, int TYC, bool SR>
__device__ __forceinline__ void stream_tile(const StreamArgs& sa, int tile,
                                            int seg, float* sm) {
  const StepArgs& a = sa.s;
  const int X = a.X, Y = a.Y;
  const int Z = ZC ? ZC : a.Z;
  const int TY = TYC ? TYC : a.tile_y;
  const int S = sa.stages;
  const StreamGeom g(TY, Z, a.plo + a.phi, sa.src_ring);
  const int Pp = g.Pp;
  float* hn = sm + (size_t)S * g.stage;   // [2][3][RH*Z]
  float* en = hn + g.hn_floats();         // [2][3][TY*Z]
  float* pn = en + g.en_floats();         // [2][4][TY*Pp]
  uint64_t* full = reinterpret_cast<uint64_t*>(pn + g.pn_floats());
  uint64_t* done = full + S;
  uint64_t* freeb = done + S;
  __shared__ int abort_flag;
  // This launch's waveform row, read once (ring-carried sources): the E
  // updates of source cells take it from here instead of global memory.
  __shared__ float wave_sm[SR ? kWaveCache : 1];
  const bool wcache = SR && a.snc > 0 && a.snc <= kWaveCache;

  const int tid = threadIdx.x;
  const int ncomp = blockDim.x - 32;      // compute threads (multiple of 32)
  const int nwarps = ncomp >> 5;
  const bool producer = tid >= ncomp;
  const int Zh = Z >> 1;
  const int rpt = ncomp / Zh;             // rows per pass
  const int z0 = 2 * (tid % Zh);
  const int rt = tid / Zh;                // >= rpt: idle compute thread
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
  const int nrows = hy_hi - y0;           // owned rows inside the domain
  const int erow0 = ey_lo - (y0 - 1);     // tile row of the first valid row
  const int ma = y0 & ~3;                 // absorber window start
  const int mb = min(round4(y0 + TY), sa.Yp);
  const int moff = y0 - ma;
  const int RHZ = g.RH * Z, REZ = g.RE * Z;
  // Source box rows of this tile (ring-carried source blocks).
  const int srow0 = max(y0, a.sy0);
  const int nsrow = min(min(y0 + TY, Y), a.sy0 + a.sny) - srow0;
  const int srowf = a.snc * 3 * a.snz;  // floats per re-laid source row

  if (wcache && tid < a.snc) wave_sm[tid] = a.wave[tid];
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
  // Rows outside the domain are never written and read as the zero boundary.
  for (size_t i = tid; i < (size_t)S * g.stage + g.hn_floats() + g.en_floats() +
                               g.pn_floats();
       i += blockDim.x)
    sm[i] = 0.f;
  fence_async_smem();
  __syncthreads();

  if (producer) {
    if ((tid & 31) != 0) return;
    // ---------------- producer (one lane) ----------------
    auto fill = [&](int xp, int slot, bool fullp) {
      float* st = sm + (size_t)slot * g.stage;
      const uint32_t eb = (uint32_t)((ey_hi - ey_lo) * Z * 4);
      const uint32_t hb = (uint32_t)((hy_hi - ey_lo) * Z * 4);
      const uint32_t cbb = (uint32_t)(nrows * Z * 4);
      const uint32_t mbb = (uint32_t)((mb - ma) * 4);
      const uint32_t pb = (uint32_t)((hy_hi - ey_lo) * Pp * 4);
      const bool srcp = SR && fullp && nsrow > 0 && xp >= a.sx0 &&
                        xp < a.sx0 + a.snx;
      const uint32_t sbb = srcp ? (uint32_t)(nsrow * srowf * 4) : 0u;
      const uint32_t total = sa.stall_bytes + 3 * eb +
          (fullp ? 3 * (hb + cbb + mbb) + (Pp > 0 ? 4 * pb : 0) : 0) + sbb;
      mbar_expect_tx(&full[slot], total);
      if (srcp)
        bulk_g2s(st + g.s_off,
                 sa.src_ws + ((long long)(xp - a.sx0) * a.sny + (srow0 - a.sy0)) * srowf,
                 sbb, &full[slot]);
      const long long base = (long long)xp * YZ;
      for (int c = 0; c < 3; ++c)
        bulk_g2s(st + g.e_off + c * REZ + erow0 * Z,
                 a.fin + c * N + base + (long long)ey_lo * Z, eb, &full[slot]);
      if (!fullp) return;
      for (int c = 0; c < 3; ++c) {
        bulk_g2s(st + g.h_off + c * RHZ + erow0 * Z,
                 a.fin + (3 + c) * N + base + (long long)ey_lo * Z, hb, &full[slot]);
        bulk_g2s(st + g.c_off + c * TY * Z, a.cb + c * N + base + (long long)y0 * Z,
                 cbb, &full[slot]);
        bulk_g2s(st + g.m_off + c * g.MT,
                 sa.mask_ws + ((long long)xp * 3 + c) * sa.Yp + ma, mbb, &full[slot]);
      }
      if (Pp > 0)
        for (int c = 0; c < 4; ++c)
          bulk_g2s(st + g.p_off + c * g.RH * Pp + erow0 * Pp,
                   a.psi_in + c * PXY + ((long long)xp * Y + ey_lo) * Pp, pb,
                   &full[slot]);
    };
    int nfill = 0;  // planes issued so far (x0 + nfill is the next one)
    while (nfill < S && x0 + nfill <= xlast) {
      fill(x0 + nfill, nfill, x0 + nfill < xe);
      ++nfill;
    }
    bool ok = true;
    int slot = 0;            // ring slot of plane x
    uint32_t round = 0;      // fills of that slot before plane x's
    for (int x = x0; x < xe && ok; ++x) {
      const int k = x - x0;
      const int b = k & 1;
      ok = mbar_wait_or_abort(&done[slot], round & 1, sa.status, &abort_flag, sa.wait_cycles);
      if (!ok) break;
      if (x >= xs) {
        float* hcur = hn + (size_t)b * 3 * RHZ;
        float* ecur = en + (size_t)b * 3 * TY * Z;
        float* pcur = pn + (size_t)b * 4 * TY * Pp;
        const long long base = (long long)x * YZ + (long long)y0 * Z;
        const uint32_t fb = (uint32_t)(nrows * Z * 4);
        for (int c = 0; c < 3; ++c) {
          bulk_s2g(a.fout + (3 + c) * N + base, hcur + c * RHZ + Z, fb);
          bulk_s2g(a.fout + c * N + base, ecur + c * TY * Z, fb);
        }
        if (Pp > 0) {
          const uint32_t pb = (uint32_t)(nrows * Pp * 4);
          const long long pbase = ((long long)x * Y + y0) * Pp;
          for (int c = 0; c < 4; ++c)
            bulk_s2g(a.psi_out + c * PXY + pbase, pcur + c * TY * Pp, pb);
        }
        bulk_commit();
      }
      // Slot of plane x is free: refill it with the next plane.
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
    // Drain: every issued fill must land before shared memory is released
    // (bounded, and regardless of an abort).
    for (int j = max(0, nfill - S); j < nfill; ++j)
      mbar_wait(&full[j % S], (uint32_t)(j / S) & 1, sa.status, sa.wait_cycles);
    bulk_wait_all();
    return;
  }

  // ---------------- compute warps ----------------
  int pz[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int z = z0 + k;
    pz[k] = z < a.plo ? z : (z >= Z - a.phi ? z - (Z - a.phi) + a.plo : -1);
  }
  float ike[2], be[2], ce[2], ikh[2], bh[2], ch[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int z = z0 + k;
    ike[k] = a.zc[z];
    be[k] = a.zc[Z + z];
    ce[k] = a.zc[2 * Z + z];
    ikh[k] = a.zc[3 * Z + z];
    bh[k] = a.zc[4 * Z + z];
    ch[k] = a.zc[5 * Z + z];
  }
  const bool zpml = pz[0] >= 0 || pz[1] >= 0;
  const float mdt = -a.dt;
  const bool active = rt < rpt;

  int slot = 0, slot1 = S > 1 ? 1 : 0;  // ring slots of planes x and x+1
  uint32_t round = 0, round1 = S > 1 ? 0 : 1;  // their fill rounds
  for (int x = x0; x < xe; ++x) {
    const int k = x - x0;
    const int b = k & 1;
    const bool has_x1 = x + 1 < X;
    bool ok = true;
    if (k == 0) ok = mbar_wait_or_abort(&full[slot], round & 1, sa.status, &abort_flag, sa.wait_cycles);
    if (ok && has_x1)
      ok = mbar_wait_or_abort(&full[slot1], round1 & 1, sa.status, &abort_flag, sa.wait_cycles);
    if (ok && k >= 2)
      ok = mbar_wait_or_abort(&freeb[b], (uint32_t)((k >> 1) - 1) & 1, sa.status,
                              &abort_flag, sa.wait_cycles);

    float* st = sm + (size_t)slot * g.stage;  // written only for source J
    const float* Es = st + g.e_off;
    const float* E1 = sm + (size_t)slot1 * g.stage + g.e_off;
    const float* Hs = st + g.h_off;
    const float* Cs = st + g.c_off;
    const float* Ms = st + g.m_off + moff;
    const float* Ps = st + g.p_off;
    float* hcur = hn + (size_t)b * 3 * RHZ;
    const float* hprev = hn + (size_t)(b ^ 1) * 3 * RHZ;
    float* ecur = en + (size_t)b * 3 * TY * Z;
    float* pcur = pn + (size_t)b * 4 * TY * Pp;
    const bool wr = x >= xs;

    // H^{n+1/2}(x) for tile rows 0..TY (y = y0-1 .. y0+TY-1).
    if (ok && active) {
#pragma unroll 2
      for (int r = rt; r < g.RH; r += rpt) {
        const int y = y0 - 1 + r;
        if (y < 0 || y >= Y) continue;
        const int ie = r * Z + z0;
        const float2 ex = *reinterpret_cast<const float2*>(Es + ie);
        const float2 ey = *reinterpret_cast<const float2*>(Es + REZ + ie);
        const float2 ez = *reinterpret_cast<const float2*>(Es + 2 * REZ + ie);
        const float2 ex_y1 = *reinterpret_cast<const float2*>(Es + ie + Z);
        const float2 ez_y1 = *reinterpret_cast<const float2*>(Es + 2 * REZ + ie + Z);
        const bool zin = z0 + 2 < Z;
        const float ex_z2 = zin ? Es[ie + 2] : 0.f;
        const float ey_z2 = zin ? Es[REZ + ie + 2] : 0.f;
        float2 e1y = make_float2(0.f, 0.f), e1z = make_float2(0.f, 0.f);
        if (has_x1) {
          e1y = *reinterpret_cast<const float2*>(E1 + REZ + ie);
          e1z = *reinterpret_cast<const float2*>(E1 + 2 * REZ + ie);
        }
        const float2 hox = *reinterpret_cast<const float2*>(Hs + ie);
        const float2 hoy = *reinterpret_cast<const float2*>(Hs + RHZ + ie);
        const float2 hoz = *reinterpret_cast<const float2*>(Hs + 2 * RHZ + ie);
        const float exs[2] = {ex.x, ex.y}, eys[2] = {ey.x, ey.y}, ezs[2] = {ez.x, ez.y};
        const float exy1[2] = {ex_y1.x, ex_y1.y}, ezy1[2] = {ez_y1.x, ez_y1.y};
        const float exz1[2] = {ex.y, ex_z2}, eyz1[2] = {ey.y, ey_z2};
        const float e1ys[2] = {e1y.x, e1y.y}, e1zs[2] = {e1z.x, e1z.y};
        const float hos[3][2] = {{hox.x, hox.y}, {hoy.x, hoy.y}, {hoz.x, hoz.y}};
        float hnew[3][2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float dEz_y = fsub(ezy1[q], ezs[q]), dEy_z = fsub(eyz1[q], eys[q]);
          const float dEx_z = fsub(exz1[q], exs[q]), dEz_x = fsub(e1zs[q], ezs[q]);
          const float dEy_x = fsub(e1ys[q], eys[q]), dEx_y = fsub(exy1[q], exs[q]);
          float zEy, zEx;
          if (zpml && pz[q] >= 0) {
            const int pi = r * Pp + pz[q];
            const float na = ffma(ch[q], dEy_z, fmul(bh[q], Ps[pi]));
            const float nb = ffma(ch[q], dEx_z, fmul(bh[q], Ps[g.RH * Pp + pi]));
            if (r > 0) {
              pcur[(r - 1) * Pp + pz[q]] = na;
              pcur[TY * Pp + (r - 1) * Pp + pz[q]] = nb;
            }
            zEy = ffma(dEy_z, ikh[q], na);
            zEx = ffma(dEx_z, ikh[q], nb);
          } else {
            zEy = fmul(dEy_z, ikh[q]);
            zEx = fmul(dEx_z, ikh[q]);
          }
          hnew[0][q] = ffma(mdt, fsub(dEz_y, zEy), hos[0][q]);
          hnew[1][q] = ffma(mdt, fsub(zEx, dEz_x), hos[1][q]);
          hnew[2][q] = ffma(mdt, fsub(dEy_x, dEx_y), hos[2][q]);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
          *reinterpret_cast<float2*>(hcur + c * RHZ + ie) =
              make_float2(hnew[c][0], hnew[c][1]);
      }
    }
    const bool src_plane = x >= a.sx0 && x < a.sx0 + a.snx;
    if constexpr (SR) {
      // Source current J_c = sum_w src[w][c] * wave[w] of every source cell
      // of this tile, shared out over all compute threads (one cell per
      // thread, columns in order): J_c replaces column 0's value of
      // component c in the ring slot, read back by the cell's E update
      // after the barrier below.
      if (ok && src_plane && nsrow > 0) {
        const int ncell = nsrow * a.snz;
        const float* wv = wcache ? wave_sm : a.wave;
        for (int t = tid; t < ncell; t += ncomp) {
          const int r = t / a.snz;
          float* sv = st + g.s_off + r * srowf + (t - r * a.snz);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float j = 0.f;
            for (int w = 0; w < a.snc; ++w) j = ffma(sv[(w * 3 + c) * a.snz], wv[w], j);
            sv[c * a.snz] = j;
          }
        }
      }
    }
    compute_sync(ncomp);
    if (abort_flag) break;

    // E^{n+1}(x) for rows 0..TY-1 (y = y0 .. y0+TY-1).
    if (wr && active) {
#pragma unroll 2
      for (int r = rt; r < TY; r += rpt) {
        const int y = y0 + r;
        if (y >= Y) continue;
        const int ih = (r + 1) * Z + z0;
        const float2 hx = *reinterpret_cast<const float2*>(hcur + ih);
        const float2 hy = *reinterpret_cast<const float2*>(hcur + RHZ + ih);
        const float2 hz = *reinterpret_cast<const float2*>(hcur + 2 * RHZ + ih);
        const float2 hx_ym = *reinterpret_cast<const float2*>(hcur + ih - Z);
        const float2 hz_ym = *reinterpret_cast<const float2*>(hcur + 2 * RHZ + ih - Z);
        const bool zin = z0 > 0;
        const float hx_zm = zin ? hcur[ih - 1] : 0.f;
        const float hy_zm = zin ? hcur[RHZ + ih - 1] : 0.f;
        const float2 hyp = *reinterpret_cast<const float2*>(hprev + RHZ + ih);
        const float2 hzp = *reinterpret_cast<const float2*>(hprev + 2 * RHZ + ih);
        const float2 eox = *reinterpret_cast<const float2*>(Es + ih);
        const float2 eoy = *reinterpret_cast<const float2*>(Es + REZ + ih);
        const float2 eoz = *reinterpret_cast<const float2*>(Es + 2 * REZ + ih);
        const int ic = r * Z + z0;
        const float2 cbx = *reinterpret_cast<const float2*>(Cs + ic);
        const float2 cby = *reinterpret_cast<const float2*>(Cs + TY * Z + ic);
        const float2 cbz = *reinterpret_cast<const float2*>(Cs + 2 * TY * Z + ic);
        const float sig[3] = {Ms[r], Ms[g.MT + r], Ms[2 * g.MT + r]};
        const float hxs[2] = {hx.x, hx.y}, hys[2] = {hy.x, hy.y}, hzs[2] = {hz.x, hz.y};
        const float hxym[2] = {hx_ym.x, hx_ym.y}, hzym[2] = {hz_ym.x, hz_ym.y};
        const float hxzm[2] = {hx_zm, hx.x}, hyzm[2] = {hy_zm, hy.x};
        const float hyps[2] = {hyp.x, hyp.y}, hzps[2] = {hzp.x, hzp.y};
        const float eo[3][2] = {{eox.x, eox.y}, {eoy.x, eoy.y}, {eoz.x, eoz.y}};
        const float cbs[3][2] = {{cbx.x, cbx.y}, {cby.x, cby.y}, {cbz.x, cbz.y}};
        float enew[3][2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int z = z0 + q;
          const float dHz_y = fsub(hzs[q], hzym[q]), dHy_z = fsub(hys[q], hyzm[q]);
          const float dHx_z = fsub(hxs[q], hxzm[q]), dHz_x = fsub(hzs[q], hzps[q]);
          const float dHy_x = fsub(hys[q], hyps[q]), dHx_y = fsub(hxs[q], hxym[q]);
          float zHy, zHx;
          if (zpml && pz[q] >= 0) {
            const int pi = (r + 1) * Pp + pz[q];
            const float na = ffma(ce[q], dHy_z, fmul(be[q], Ps[2 * g.RH * Pp + pi]));
            const float nb = ffma(ce[q], dHx_z, fmul(be[q], Ps[3 * g.RH * Pp + pi]));
            pcur[2 * TY * Pp + r * Pp + pz[q]] = na;
            pcur[3 * TY * Pp + r * Pp + pz[q]] = nb;
            zHy = ffma(dHy_z, ike[q], na);
            zHx = ffma(dHx_z, ike[q], nb);
          } else {
            zHy = fmul(dHy_z, ike[q]);
            zHx = fmul(dHx_z, ike[q]);
          }
          float cur[3] = {fsub(dHz_y, zHy), fsub(zHx, dHz_x), fsub(dHy_x, dHx_y)};
          if (src_plane && y >= a.sy0 && y < a.sy0 + a.sny && z >= a.sz0 &&
              z < a.sz0 + a.snz) {
            // Source values from the ring slot of this plane when carried
            // there, else from global memory; same values, same order.
            if constexpr (SR) {
              const float* jv = st + g.s_off + (y - srow0) * srowf + (z - a.sz0);
#pragma unroll
              for (int c = 0; c < 3; ++c) cur[c] = fsub(cur[c], jv[c * a.snz]);
            } else {
              const long long sb = (long long)a.snx * a.sny * a.snz;
              const long long si =
                  ((long long)(x - a.sx0) * a.sny + (y - a.sy0)) * a.snz + (z - a.sz0);
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                float j = 0.f;
                for (int w = 0; w < a.snc; ++w)
                  j = ffma(a.src[((long long)w * 3 + c) * sb + si], a.wave[w], j);
                cur[c] = fsub(cur[c], j);
              }
            }
          }
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float rr = ffma(-sig[c], eo[c][q], cur[c]);
            enew[c][q] = ffma(cbs[c][q], rr, eo[c][q]);
          }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
          *reinterpret_cast<float2*>(ecur + c * TY * Z + ic) =
              make_float2(enew[c][0], enew[c][1]);
      }
    }
    // Publish this plane's results to the producer (bulk stores read them
    // through the async proxy) and release its ring slot.
    fence_async_smem();
    __syncwarp();
    if ((tid & 31) == 0) mbar_arrive(&done[slot]);
    // H(x-1) (hprev) is rewritten by the next plane's H phase.
    compute_sync(ncomp);
    slot = slot1;
    round = round1;
    if (++slot1 == S) {
      slot1 = 0;
      ++round1;
    }
  }
}

// (zz, tile_y) pairs with a compile-time specialisation: the tile heights the
// host picks for these zz with 4 ring stages.
#define PJZ_STREAM_SHAPES(X_) X_(64, 14) X_(48, 19) X_(32, 29) X_(16, 59)

template <int ZC, int TYC, bool SR>
__global__ void __launch_bounds__(512) yee_stream_kernel(const StreamArgs sa) {
  extern __shared__ __align__(16) float sm[];
  stream_tile<ZC, TYC, SR>(sa, blockIdx.x, blockIdx.y, sm);
}

// Runs the specialisation matching (zz, tile_y), else the generic body.
// Batches inline every plain shape; ring-carried sources take the generic
// body (inlining a specialised one as well made the batch kernel spill).
__device__ __forceinline__ void stream_tile_any(const StreamArgs& sa, int tile,
                                                int seg, float* sm) {
  const int z = sa.s.Z, ty = sa.s.tile_y;
  if (sa.src_tma) return stream_tile<0, 0, true>(sa, tile, seg, sm);
#define PJZ_DISPATCH(ZC, TYC) \
  if (z == ZC && ty == TYC) return stream_tile<ZC, TYC, false>(sa, tile, seg, sm);
  PJZ_STREAM_SHAPES(PJZ_DISPATCH)
#undef PJZ_DISPATCH
  stream_tile<0, 0, false>(sa, tile, seg, sm);
}

// Batched launch of one step per problem: block b runs entry work[b] =
// (sim, tile, seg) when that problem's launch `launch` of its schedule is a
// single step (sched[launch * nsim + sim] = (first step, steps));
// args[(launch & 1) * nsim + sim] holds its arguments for the buffer parity
// of this launch with the waveform row pointer at step 0.
struct BatchArgs {
  const StreamArgs* __restrict__ args;  // [2][nsim]
  const int4* __restrict__ work;        // [nwork]: sim, tile, seg, unused
  const int2* __restrict__ sched;       // [launches][nsim]: step, steps
  int nsim;
  int launch;
};

#ifdef PJZ_BATCH1_KERNEL  // defined in kern_batch.cu only
__global__ void __launch_bounds__(512) yee_stream_batch_kernel(const BatchArgs ba) {
  extern __shared__ __align__(16) float sm[];
  const int4 w = ba.work[blockIdx.x];
  const int2 sc = ba.sched[(size_t)ba.launch * ba.nsim + w.x];
  if (sc.y != 1) return;
  StreamArgs sa = ba.args[(ba.launch & 1) * ba.nsim + w.x];
  if (sa.s.snc > 0) sa.s.wave += (long long)sc.x * sa.s.snc;
  stream_tile_any(sa, w.y, w.z, sm);
}

#endif  // PJZ_BATCH1_KERNEL

#ifdef PJZ_HOST_KERNELS
// Source profile [column][component][x][y][z] (box-local) re-laid out as
// [x][y][column][component][z], the order the ring carries it in.
__global__ void source_rows_kernel(const float* __restrict__ src,
                                   float* __restrict__ dst, int ncols, int nx,
                                   int ny, int nz) {
  const int nwc = 3 * ncols;
  const long long n = (long long)nwc * nx * ny * nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int bz = (int)(t % nz);
    const long long r1 = t / nz;
    const int wc = (int)(r1 % nwc);
    const long long xy = r1 / nwc;
    dst[t] = src[((long long)wc * nx * ny + xy) * nz + bz];
  }
}

// Absorber conductivity re-laid out as [x][c][Yp] (Yp % 4 == 0, zero tail)
// so each (x, c) row of a tile is one aligned span.
__global__ void pad_mask_kernel(const float* __restrict__ mask,
                                float* __restrict__ mask_ws, int X, int Y,
                                int Yp) {
  const long long n = (long long)X * 3 * Yp;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(t % Yp);
    const long long xc = t / Yp;
    const int c = (int)(xc % 3);
    const int x = (int)(xc / 3);
    mask_ws[t] = y < Y ? mask[((long long)c * X + x) * Y + y] : 0.f;
  }
}

#endif  // PJZ_HOST_KERNELS

}  // namespace pjzfdtd
