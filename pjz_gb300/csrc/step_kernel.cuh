// Fused Yee step kernel for sm_103a: one time step (H then E) per HBM pass.
//
// Replaces the update inside fdtdz (the engine pjz calls at
// src/pjz/_field.py:254-269).  Conventions, restated from pjz's own code:
// Ex(x+1/2,y,z), Ey(x,y+1/2,z), Ez(x,y,z+1/2) (src/pjz/_epsilon.py:10-25);
// H from forward differences of E and E from backward differences of H
// (src/pjz/_mode.py:15-19, 61-68); absorption_mask is a conductivity on E
// (src/pjz/_field.py:239-241); z-CPML columns 0/1 at integer/half-integer z
// (src/pjz/_field.py:98-106, 243-251).  Fields outside the domain are zero.
//
// Layout in HBM: six float planes-major arrays [c][x][y][z] (z fastest), so
// a CTA reading a run of (y,z) cells of one x-plane reads one contiguous
// span.  Each CTA owns `tile_y` rows of y (all of z) and marches through
// `seg_x` x-planes; E(x+1) and H(x-1) stay in registers, y/z neighbours go
// through shared memory.  The tile carries one halo row below (its H is
// recomputed) and one above (E is only read), plus one halo plane before
// the segment.  State is ping-ponged (read fin/psi_in, write fout/psi_out)
// so neighbouring CTAs never race on halo cells.
//
// Every floating-point operation is an explicit round-to-nearest intrinsic
// (no contraction), in the same order as the CPU oracle, so results are
// bit-identical to it.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pjzfdtd {

constexpr int kMaxRows = 32;      // weight rows (2 * ww)
constexpr int kMaxThreads = 1024;

enum RecordMode { kRecNone = 0, kRecSnap = 1, kRecProj = 2, kRecGrad = 3 };

struct StepArgs {
  int X, Y, Z, P, plo, phi;
  int Pst;  // row stride of the PML state arrays (P rounded up to 4)
  long long N;  // X * Y * Z
  float dt;
  int tile_y, seg_x;
  const float* __restrict__ fin;   // [6][N]   E^n, H^{n-1/2}
  float* __restrict__ fout;        // [6][N]   E^{n+1}, H^{n+1/2}
  const float* __restrict__ cb;    // [3][N]   dt / (eps + sigma dt / 2)
  const float* __restrict__ mask;  // [3][X][Y] absorber conductivity
  const float* __restrict__ zc;    // [6][Z]   ik_e, b_e, c_e, ik_h, b_h, c_h
  const float* __restrict__ psi_in;  // [4][X][Y][Pst] hx, hy, ex, ey
  float* __restrict__ psi_out;
  // Source box: J_c = sum_k src[k][c][box] * wave[k].
  int sx0, sy0, sz0, snx, sny, snz, snc;
  const float* __restrict__ src;
  const float* __restrict__ wave;  // row of the waveform for this step
};

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) {
  return __fmaf_rn(a, b, c);
}

// Compensated (Kahan) accumulation s += w * e, FP32 throughout.
__device__ __forceinline__ void kahan(float* s, float* c, float w, float e) {
  const float cs = *c, ss = *s;
  const float yv = ffma(w, e, -cs);
  const float t = fadd(ss, yv);
  *c = fsub(fsub(t, ss), yv);
  *s = t;
}

#ifdef PJZ_HOST_KERNELS  // defined in the host translation unit only
__global__ void __launch_bounds__(kMaxThreads)
    yee_step_kernel(const StepArgs a) {
  extern __shared__ float smem[];
  const int X = a.X, Y = a.Y, Z = a.Z, TY = a.tile_y;
  const int cells = (TY + 2) * Z;
  float* Es = smem;              // [3][cells], rows -1..TY
  float* Hs = smem + 3 * cells;  // [3][cells], rows -1..TY-1
  const int tid = threadIdx.x;
  const bool act = tid < cells;
  const int row = tid / Z - 1;
  const int z = tid - (row + 1) * Z;
  const int y = blockIdx.x * TY + row;
  const bool in_y = act && y >= 0 && y < Y;
  const bool hrow = in_y && row < TY;
  const bool own = in_y && row >= 0 && row < TY;
  const int xs = blockIdx.y * a.seg_x;
  const int xe = min(X, xs + a.seg_x);
  const int x0 = xs > 0 ? xs - 1 : 0;
  const long long N = a.N;
  const long long YZ = (long long)Y * Z;
  const long long colz = (long long)y * Z + z;
  const int pz = !act ? -1
                      : (z < a.plo ? z : (z >= Z - a.phi ? z - (Z - a.phi) + a.plo : -1));
  const long long PXY = (long long)X * Y * a.Pst;

  float ike = 0.f, be = 0.f, ce = 0.f, ikh = 0.f, bh = 0.f, ch = 0.f;
  if (act) {
    ike = a.zc[z];
    be = a.zc[Z + z];
    ce = a.zc[2 * Z + z];
    ikh = a.zc[3 * Z + z];
    bh = a.zc[4 * Z + z];
    ch = a.zc[5 * Z + z];
  }
  const float mdt = -a.dt;

  float e0x = 0.f, e0y = 0.f, e0z = 0.f, e1x = 0.f, e1y = 0.f, e1z = 0.f;
  if (in_y) {
    const long long i = x0 * YZ + colz;
    e0x = a.fin[i];
    e0y = a.fin[N + i];
    e0z = a.fin[2 * N + i];
    if (x0 + 1 < X) {
      e1x = a.fin[i + YZ];
      e1y = a.fin[N + i + YZ];
      e1z = a.fin[2 * N + i + YZ];
    }
  }
  float hyp = 0.f, hzp = 0.f;  // H^{n+1/2}(x-1): Hy, Hz

  const bool src_yz = in_y && y >= a.sy0 && y < a.sy0 + a.sny && z >= a.sz0 &&
                      z < a.sz0 + a.snz;

  for (int x = x0; x < xe; ++x) {
    const long long i = x * YZ + colz;
    float e2x = 0.f, e2y = 0.f, e2z = 0.f;
    if (in_y && x + 2 < X) {
      e2x = a.fin[i + 2 * YZ];
      e2y = a.fin[N + i + 2 * YZ];
      e2z = a.fin[2 * N + i + 2 * YZ];
    }
    float hx = 0.f, hy = 0.f, hz = 0.f;
    if (hrow) {
      hx = a.fin[3 * N + i];
      hy = a.fin[4 * N + i];
      hz = a.fin[5 * N + i];
    }
    if (act) {
      Es[tid] = e0x;
      Es[cells + tid] = e0y;
      Es[2 * cells + tid] = e0z;
    }
    __syncthreads();

    const bool write = own && x >= xs;
    if (hrow) {
      const float ex_y1 = Es[tid + Z];
      const float ez_y1 = Es[2 * cells + tid + Z];
      const float ex_z1 = (z + 1 < Z) ? Es[tid + 1] : 0.f;
      const float ey_z1 = (z + 1 < Z) ? Es[cells + tid + 1] : 0.f;
      const float dEz_y = fsub(ez_y1, e0z), dEy_z = fsub(ey_z1, e0y);
      const float dEx_z = fsub(ex_z1, e0x), dEz_x = fsub(e1z, e0z);
      const float dEy_x = fsub(e1y, e0y), dEx_y = fsub(ex_y1, e0x);
      float zEy, zEx;
      if (pz >= 0) {
        const long long pi = ((long long)x * Y + y) * a.Pst + pz;
        const float na = ffma(ch, dEy_z, fmul(bh, a.psi_in[pi]));
        const float nb = ffma(ch, dEx_z, fmul(bh, a.psi_in[PXY + pi]));
        if (write) {
          a.psi_out[pi] = na;
          a.psi_out[PXY + pi] = nb;
        }
        zEy = ffma(dEy_z, ikh, na);
        zEx = ffma(dEx_z, ikh, nb);
      } else {
        zEy = fmul(dEy_z, ikh);
        zEx = fmul(dEx_z, ikh);
      }
      hx = ffma(mdt, fsub(dEz_y, zEy), hx);
      hy = ffma(mdt, fsub(zEx, dEz_x), hy);
      hz = ffma(mdt, fsub(dEy_x, dEx_y), hz);
      if (write) {
        a.fout[3 * N + i] = hx;
        a.fout[4 * N + i] = hy;
        a.fout[5 * N + i] = hz;
      }
    }
    if (act && row < TY) {
      Hs[tid] = hx;
      Hs[cells + tid] = hy;
      Hs[2 * cells + tid] = hz;
    }
    __syncthreads();

    if (write) {
      const float hx_ym = Hs[tid - Z];
      const float hz_ym = Hs[2 * cells + tid - Z];
      const float hx_zm = z > 0 ? Hs[tid - 1] : 0.f;
      const float hy_zm = z > 0 ? Hs[cells + tid - 1] : 0.f;
      const float dHz_y = fsub(hz, hz_ym), dHy_z = fsub(hy, hy_zm);
      const float dHx_z = fsub(hx, hx_zm), dHz_x = fsub(hz, hzp);
      const float dHy_x = fsub(hy, hyp), dHx_y = fsub(hx, hx_ym);
      float zHy, zHx;
      if (pz >= 0) {
        const long long pi = ((long long)x * Y + y) * a.Pst + pz;
        const float na = ffma(ce, dHy_z, fmul(be, a.psi_in[2 * PXY + pi]));
        const float nb = ffma(ce, dHx_z, fmul(be, a.psi_in[3 * PXY + pi]));
        a.psi_out[2 * PXY + pi] = na;
        a.psi_out[3 * PXY + pi] = nb;
        zHy = ffma(dHy_z, ike, na);
        zHx = ffma(dHx_z, ike, nb);
      } else {
        zHy = fmul(dHy_z, ike);
        zHx = fmul(dHx_z, ike);
      }
      float cur[3] = {fsub(dHz_y, zHy), fsub(zHx, dHz_x), fsub(dHy_x, dHx_y)};
      if (src_yz && x >= a.sx0 && x < a.sx0 + a.snx) {
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
      const float e_old[3] = {e0x, e0y, e0z};
      float e_new[3];
      const long long mi = (long long)x * Y + y;
      const long long XY = (long long)X * Y;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float s = a.mask[c * XY + mi];
        const float r = ffma(-s, e_old[c], cur[c]);
        e_new[c] = ffma(a.cb[c * N + i], r, e_old[c]);
        a.fout[c * N + i] = e_new[c];
      }
    }
    hyp = hy;
    hzp = hz;
    e0x = e1x;
    e0y = e1y;
    e0z = e1z;
    e1x = e2x;
    e1y = e2y;
    e1z = e2z;
  }
}

__device__ __forceinline__ void store_as(float* p, float v) { *p = v; }
__device__ __forceinline__ void store_as(__half* p, float v) {
  *p = __float2half_rn(v);
}

// cb[c][x][y][z] = dt / (eps_c(clamped region index) + sigma_c(x,y) * dt/2),
// computed in FP32 and stored as T (rounded to nearest even for __half).
template <typename T>
__global__ void precompute_cb_kernel(const float* __restrict__ eps,
                                     const float* __restrict__ mask,
                                     T* __restrict__ cb, int X, int Y, int Z,
                                     int ox, int oy, int oz, int rx, int ry,
                                     int rz, float dt) {
  const long long N = (long long)X * Y * Z;
  const float hdt = 0.5f * dt;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 3 * N;
       t += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(t / N);
    const long long i = t - c * N;
    const int z = (int)(i % Z);
    const long long xy = i / Z;
    const int y = (int)(xy % Y);
    const int x = (int)(xy / Y);
    const int ex = min(max(x - ox, 0), rx - 1);
    const int ey = min(max(y - oy, 0), ry - 1);
    const int ez = min(max(z - oz, 0), rz - 1);
    const float e = eps[(((long long)c * rx + ex) * ry + ey) * rz + ez];
    const float s = mask[((long long)c * X + x) * Y + y];
    store_as(&cb[t], __fdiv_rn(dt, __fmaf_rn(s, hdt, e)));
  }
}

// FP32 state in and out of binary16 storage (round to nearest even; the
// widening is exact).
__global__ void narrow_f16_kernel(const float* __restrict__ src,
                                  __half* __restrict__ dst, long long n) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    dst[t] = __float2half_rn(src[t]);
}
__global__ void widen_f16_kernel(const __half* __restrict__ src,
                                 float* __restrict__ dst, long long n) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    dst[t] = __half2float(src[t]);
}

#endif  // PJZ_HOST_KERNELS

}  // namespace pjzfdtd
