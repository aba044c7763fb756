// Streamed Yee step kernel for sm_103a: the same single-step update as
// yee_step_kernel, with every x-plane tile staged into shared memory by the
// bulk-copy engine (cp.async.bulk + mbarrier) several planes ahead.
//
// A CTA owns `tile_y` rows of y (all of z) and marches through `seg_x`
// x-planes.  For plane x the tile needs E rows -1..TY, H rows -1..TY-1 and
// the E coefficient rows 0..TY-1; in the [c][x][y][z] layout each of those
// is one contiguous span per component, so a stage is filled by nine bulk
// copies issued by one thread and tracked by one mbarrier (transaction
// bytes).  The per-column absorber conductivity and the z-PML state rows go
// through cp.async (4-byte, any alignment) in the same stage.  A ring of
// `stages` slots keeps stages-1 planes in flight while the CTA computes one,
// so DRAM latency is off the critical path.  H computed for plane x stays in
// shared memory (double-buffered) as the x-1 neighbour of the next plane.
//
// Requires zz % 4 == 0 (16-byte aligned spans); the host falls back to
// yee_step_kernel otherwise.  Arithmetic is the same explicit RN sequence,
// so results are bit-identical to the CPU oracle.
//
// Every wait is bounded: an mbarrier wait that exceeds kWaitCycles sets the
// status word and the whole CTA leaves at the next barrier.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "step_kernel.cuh"

namespace pjzfdtd {

constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz
constexpr int kStatusTimeout = 4;

struct StreamArgs {
  StepArgs s;
  int stages;
  int* status;  // device status word (0 = ok)
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
                                          int* status) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (clock64() - t0 > kWaitCycles) {
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

__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Shared-memory geometry of one CTA (floats unless noted).
struct StreamGeom {
  int TY, Z, P, RE, RH;
  int e_off, h_off, c_off, m_off, p_off, stage;  // within a stage
  __host__ __device__ StreamGeom(int ty, int z, int p) {
    TY = ty;
    Z = z;
    P = p;
    RE = ty + 2;
    RH = ty + 1;
    e_off = 0;
    h_off = e_off + 3 * RE * z;
    c_off = h_off + 3 * RH * z;
    m_off = c_off + 3 * ty * z;
    p_off = m_off + ((3 * ty + 3) & ~3);
    stage = p_off + ((4 * RH * p + 3) & ~3);
  }
  __host__ __device__ size_t hn_floats() const { return 2 * 3 * (size_t)RH * Z; }
  __host__ __device__ size_t bytes(int stages) const {
    return ((size_t)stages * stage + hn_floats()) * sizeof(float) +
           (size_t)stages * sizeof(uint64_t) + 16;
  }
};

template <int REC>
__global__ void __launch_bounds__(512) yee_stream_kernel(const StreamArgs sa) {
  extern __shared__ __align__(16) float sm[];
  const StepArgs& a = sa.s;
  const int X = a.X, Y = a.Y, Z = a.Z, TY = a.tile_y;
  const int S = sa.stages;
  const StreamGeom g(TY, Z, a.plo + a.phi);
  const int P = g.P;
  float* hn = sm + (size_t)S * g.stage;  // [2][3][RH*Z]
  uint64_t* bars = reinterpret_cast<uint64_t*>(hn + g.hn_floats());
  __shared__ int abort_flag;

  const int tid = threadIdx.x;
  const int nt = blockDim.x;
  const int z = tid % Z;
  const int rt = tid / Z;
  const int rpt = nt / Z;
  const int y0 = blockIdx.x * TY;
  const int xs = blockIdx.y * a.seg_x;
  const int xe = min(X, xs + a.seg_x);
  const int x0 = xs > 0 ? xs - 1 : 0;
  const int xlast = min(xe, X - 1);  // last plane whose E is read
  const long long N = a.N;
  const long long YZ = (long long)Y * Z;
  const long long PXY = (long long)X * Y * max(P, 1);
  // Valid y rows of the E halo tile [y0-1, y0+TY] and the H tile
  // [y0-1, y0+TY-1] and the coefficient rows [y0, y0+TY-1].
  const int ey_lo = max(y0 - 1, 0), ey_hi = min(y0 + TY + 1, Y);
  const int hy_hi = min(y0 + TY, Y);
  const int cy_hi = min(y0 + TY, Y);

  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // Zero every slot and both H buffers once: rows outside the domain are
  // never overwritten and read as the zero boundary.
  for (size_t i = tid; i < (size_t)S * g.stage + g.hn_floats(); i += nt) sm[i] = 0.f;
  __syncthreads();

  const int pz = z < a.plo ? z : (z >= Z - a.phi ? z - (Z - a.phi) + a.plo : -1);
  const float ike = a.zc[z], be = a.zc[Z + z], ce = a.zc[2 * Z + z];
  const float ikh = a.zc[3 * Z + z], bh = a.zc[4 * Z + z], ch = a.zc[5 * Z + z];
  const float mdt = -a.dt;

  // Issues the copies of plane xp into slot `slot` (E only when !full).
  auto fill = [&](int xp, int slot, bool full) {
    float* st = sm + (size_t)slot * g.stage;
    if (tid == 0) {
      const uint32_t eb = (uint32_t)((ey_hi - ey_lo) * Z * 4);
      const uint32_t hb = (uint32_t)((hy_hi - ey_lo) * Z * 4);
      const uint32_t cbb = (uint32_t)((cy_hi - y0) * Z * 4);
      uint32_t total = 3 * eb + (full ? 3 * (hb + cbb) : 0);
      mbar_expect_tx(&bars[slot], total);
      const long long base = (long long)xp * YZ;
      const int erow0 = ey_lo - (y0 - 1);
      for (int c = 0; c < 3; ++c)
        bulk_g2s(st + g.e_off + c * g.RE * Z + erow0 * Z,
                 a.fin + c * N + base + (long long)ey_lo * Z, eb, &bars[slot]);
      if (full) {
        for (int c = 0; c < 3; ++c) {
          bulk_g2s(st + g.h_off + c * g.RH * Z + erow0 * Z,
                   a.fin + (3 + c) * N + base + (long long)ey_lo * Z, hb,
                   &bars[slot]);
          bulk_g2s(st + g.c_off + c * TY * Z,
                   a.cb + c * N + base + (long long)y0 * Z, cbb, &bars[slot]);
        }
      }
    }
    if (full) {
      // Absorber conductivity of rows y0..y0+TY-1 and z-PML state of rows
      // y0-1..y0+TY-1 for plane xp.
      const long long XY = (long long)X * Y;
      for (int i = tid; i < 3 * TY; i += nt) {
        const int c = i / TY, r = i - c * TY;
        if (y0 + r < Y)
          cp_async4(st + g.m_off + i, a.mask + c * XY + (long long)xp * Y + y0 + r);
      }
      if (P > 0) {
        const int n = 4 * g.RH * P;
        for (int i = tid; i < n; i += nt) {
          const int c = i / (g.RH * P);
          const int rem = i - c * g.RH * P;
          const int r = rem / P, q = rem - r * P;
          const int y = y0 - 1 + r;
          if (y >= 0 && y < Y)
            cp_async4(st + g.p_off + i,
                      a.psi_in + c * PXY + ((long long)xp * Y + y) * P + q);
        }
      }
    }
    cp_async_commit();
  };

  // Prologue: planes x0 .. x0+S-1 (those that exist).
  for (int k = 0; k < S; ++k) {
    const int xp = x0 + k;
    if (xp <= xlast) fill(xp, k, xp < xe);
    else cp_async_commit();
  }

  int slot = 0;  // slot of plane x
  uint32_t round = 0;  // fill round of plane x's slot
  bool waited_first = false;
  for (int x = x0; x < xe; ++x) {
    const int slot1 = (slot + 1 == S) ? 0 : slot + 1;
    const uint32_t round1 = (slot + 1 == S) ? round + 1 : round;
    const bool has_x1 = x + 1 < X;
    bool ok = true;
    if (!waited_first) {
      ok = mbar_wait(&bars[slot], round & 1, sa.status);
      waited_first = true;
    }
    if (ok && has_x1) ok = mbar_wait(&bars[slot1], round1 & 1, sa.status);
    if (!ok) abort_flag = 1;

    const float* st = sm + (size_t)slot * g.stage;
    const float* st1 = sm + (size_t)slot1 * g.stage;
    const float* Es = st + g.e_off;
    const float* E1 = st1 + g.e_off;
    const float* Hs = st + g.h_off;
    const float* Cs = st + g.c_off;
    const float* Ms = st + g.m_off;
    const float* Ps = st + g.p_off;
    float* hcur = hn + (size_t)(x & 1) * 3 * g.RH * Z;
    const float* hprev = hn + (size_t)((x + 1) & 1) * 3 * g.RH * Z;
    const bool wr = x >= xs;

    // H^{n+1/2}(x) for rows -1..TY-1.
    if (ok) {
      for (int r = rt; r < g.RH; r += rpt) {
        const int y = y0 - 1 + r;
        if (y < 0 || y >= Y) continue;
        const int ie = r * Z + z;
        const float e0x = Es[ie], e0y = Es[g.RE * Z + ie], e0z = Es[2 * g.RE * Z + ie];
        const float ex_y1 = Es[ie + Z], ez_y1 = Es[2 * g.RE * Z + ie + Z];
        const float ex_z1 = (z + 1 < Z) ? Es[ie + 1] : 0.f;
        const float ey_z1 = (z + 1 < Z) ? Es[g.RE * Z + ie + 1] : 0.f;
        const float e1y = has_x1 ? E1[g.RE * Z + ie] : 0.f;
        const float e1z = has_x1 ? E1[2 * g.RE * Z + ie] : 0.f;
        const float dEz_y = fsub(ez_y1, e0z), dEy_z = fsub(ey_z1, e0y);
        const float dEx_z = fsub(ex_z1, e0x), dEz_x = fsub(e1z, e0z);
        const float dEy_x = fsub(e1y, e0y), dEx_y = fsub(ex_y1, e0x);
        float zEy, zEx;
        if (pz >= 0) {
          const float na = ffma(ch, dEy_z, fmul(bh, Ps[r * P + pz]));
          const float nb = ffma(ch, dEx_z, fmul(bh, Ps[g.RH * P + r * P + pz]));
          if (wr && r > 0) {
            const long long pi = ((long long)x * Y + y) * P + pz;
            a.psi_out[pi] = na;
            a.psi_out[PXY + pi] = nb;
          }
          zEy = ffma(dEy_z, ikh, na);
          zEx = ffma(dEx_z, ikh, nb);
        } else {
          zEy = fmul(dEy_z, ikh);
          zEx = fmul(dEx_z, ikh);
        }
        const int ih = r * Z + z;
        const float hx = ffma(mdt, fsub(dEz_y, zEy), Hs[ih]);
        const float hy = ffma(mdt, fsub(zEx, dEz_x), Hs[g.RH * Z + ih]);
        const float hz = ffma(mdt, fsub(dEy_x, dEx_y), Hs[2 * g.RH * Z + ih]);
        hcur[ih] = hx;
        hcur[g.RH * Z + ih] = hy;
        hcur[2 * g.RH * Z + ih] = hz;
        if (wr && r > 0) {
          const long long i = x * YZ + (long long)y * Z + z;
          a.fout[3 * N + i] = hx;
          a.fout[4 * N + i] = hy;
          a.fout[5 * N + i] = hz;
        }
      }
    }
    __syncthreads();
    if (abort_flag) break;

    // E^{n+1}(x) for rows 0..TY-1.
    if (wr) {
      for (int r = rt; r < TY; r += rpt) {
        const int y = y0 + r;
        if (y >= Y) continue;
        const int ih = (r + 1) * Z + z;  // H tile index of this row
        const float hx = hcur[ih], hy = hcur[g.RH * Z + ih], hz = hcur[2 * g.RH * Z + ih];
        const float hx_ym = hcur[ih - Z], hz_ym = hcur[2 * g.RH * Z + ih - Z];
        const float hx_zm = z > 0 ? hcur[ih - 1] : 0.f;
        const float hy_zm = z > 0 ? hcur[g.RH * Z + ih - 1] : 0.f;
        const float hyp = hprev[g.RH * Z + ih], hzp = hprev[2 * g.RH * Z + ih];
        const float dHz_y = fsub(hz, hz_ym), dHy_z = fsub(hy, hy_zm);
        const float dHx_z = fsub(hx, hx_zm), dHz_x = fsub(hz, hzp);
        const float dHy_x = fsub(hy, hyp), dHx_y = fsub(hx, hx_ym);
        const long long i = x * YZ + (long long)y * Z + z;
        float zHy, zHx;
        if (pz >= 0) {
          const int pr = (r + 1) * P + pz;
          const float na = ffma(ce, dHy_z, fmul(be, Ps[2 * g.RH * P + pr]));
          const float nb = ffma(ce, dHx_z, fmul(be, Ps[3 * g.RH * P + pr]));
          const long long pi = ((long long)x * Y + y) * P + pz;
          a.psi_out[2 * PXY + pi] = na;
          a.psi_out[3 * PXY + pi] = nb;
          zHy = ffma(dHy_z, ike, na);
          zHx = ffma(dHx_z, ike, nb);
        } else {
          zHy = fmul(dHy_z, ike);
          zHx = fmul(dHx_z, ike);
        }
        float cur[3] = {fsub(dHz_y, zHy), fsub(zHx, dHz_x), fsub(dHy_x, dHx_y)};
        if (x >= a.sx0 && x < a.sx0 + a.snx && y >= a.sy0 && y < a.sy0 + a.sny &&
            z >= a.sz0 && z < a.sz0 + a.snz) {
          const long long sb = (long long)a.snx * a.sny * a.snz;
          const long long si =
              ((long long)(x - a.sx0) * a.sny + (y - a.sy0)) * a.snz + (z - a.sz0);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float j = 0.f;
            for (int k = 0; k < a.snc; ++k)
              j = ffma(a.src[((long long)k * 3 + c) * sb + si], a.wave[k], j);
            cur[c] = fsub(cur[c], j);
          }
        }
        const int ie = (r + 1) * Z + z;
        const int ic = r * Z + z;
        float e_new[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float eo = Es[c * g.RE * Z + ie];
          const float rr = ffma(-Ms[c * TY + r], eo, cur[c]);
          e_new[c] = ffma(Cs[c * TY * Z + ic], rr, eo);
          a.fout[c * N + i] = e_new[c];
        }
        if (REC == kRecSnap || REC == kRecProj) {
          const int qx = x - a.ox, qy = y - a.oy, qz = z - a.oz;
          if (qx >= 0 && qx < a.rx && qy >= 0 && qy < a.ry && qz >= 0 && qz < a.rz) {
            const long long R = (long long)a.rx * a.ry * a.rz;
            const long long ri = ((long long)qx * a.ry + qy) * a.rz + qz;
            const float hnew[3] = {hx, hy, hz};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              if (REC == kRecSnap) {
                a.out[c * R + ri] = e_new[c];
                if (a.record_h) a.out_h[c * R + ri] = hnew[c];
              } else {
                for (int rr = 0; rr < a.rows; ++rr) {
                  const long long ai = ((long long)rr * 3 + c) * R + ri;
                  kahan(&a.out[ai], &a.comp[ai], a.w[rr], e_new[c]);
                  if (a.record_h) kahan(&a.out_h[ai], &a.comp_h[ai], a.w[rr], hnew[c]);
                }
              }
            }
          }
        }
        if (REC == kRecGrad) {
          const int gx = x - a.gx0, gy = y - a.gy0, gz = z - a.gz0;
          if (gx >= 0 && gx < a.gnx && gy >= 0 && gy < a.gny && gz >= 0 && gz < a.gnz) {
            const long long G = (long long)a.gnx * a.gny * a.gnz;
            const long long gi = ((long long)gx * a.gny + gy) * a.gnz + gz;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              float coef = 0.f;
              for (int rr = 0; rr < a.rows; ++rr)
                coef = ffma(a.w[rr], a.q[((long long)rr * 3 + c) * G + gi], coef);
              kahan(&a.out[c * G + gi], &a.comp[c * G + gi], coef, e_new[c]);
            }
          }
        }
      }
    }
    // Plane x+1's cp.async pieces must land before anyone reads them.
    cp_async_wait<0>();
    __syncthreads();
    // Slot of plane x is free: refill it with plane x+S.
    const int xn = x + S;
    if (xn <= xlast) {
      if (tid == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      fill(xn, slot, xn < xe);
    }
    slot = slot1;
    round = round1;
  }
  cp_async_wait<0>();
}

}  // namespace pjzfdtd
