// Sample-step recording pass: reads the state a step kernel just wrote and
// records it -- E (and H) snapshots (the fdtdz return value), the phasor
// projection of pjz's `field` (src/pjz/_field.py:271-279) as compensated
// FP32 sums `out[r] += w[r] * E`, or the adjoint's fused dL/d-eps sum
// `grad += E * (w . q)`.  It runs only at the 2ww+1 sample steps, so the
// time loop stores no snapshots; one thread per cell, z fastest, coalesced.
// Per element the operations are those of the CPU oracle, in its order.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "step_kernel.cuh"

namespace pjzfdtd {

struct RecordArgs {
  const void* __restrict__ f;   // [6][N] state after the step (storage type)
  long long N;
  int X, Y, Z;
  int bx0, by0, bz0, bnx, bny, bnz;  // recorded box (region or gradient box)
  int record_h;
  float* __restrict__ out;
  float* __restrict__ out_h;
  float* __restrict__ comp;
  float* __restrict__ comp_h;
  int rows;
  const float* __restrict__ q;
  float w[kMaxRows];
};

__device__ __forceinline__ float widen(float v) { return v; }
__device__ __forceinline__ float widen(__half v) { return __half2float(v); }

// T: storage type of the state (float, or __half for reduced-precision
// storage; the records and accumulators are FP32 either way).
template <int REC, typename T>
__global__ void record_kernel(const RecordArgs a) {
  const T* f = static_cast<const T*>(a.f);
  const long long B = (long long)a.bnx * a.bny * a.bnz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < B;
       t += (long long)gridDim.x * blockDim.x) {
    const int bz = (int)(t % a.bnz);
    const long long xy = t / a.bnz;
    const int by = (int)(xy % a.bny);
    const int bx = (int)(xy / a.bny);
    const long long i =
        ((long long)(bx + a.bx0) * a.Y + (by + a.by0)) * a.Z + (bz + a.bz0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float e = widen(f[c * a.N + i]);
      if (REC == kRecSnap) {
        a.out[c * B + t] = e;
        if (a.record_h) a.out_h[c * B + t] = widen(f[(3 + c) * a.N + i]);
      } else if (REC == kRecProj) {
        const float h = a.record_h ? widen(f[(3 + c) * a.N + i]) : 0.f;
        for (int r = 0; r < a.rows; ++r) {
          const long long ai = ((long long)r * 3 + c) * B + t;
          kahan(&a.out[ai], &a.comp[ai], a.w[r], e);
          if (a.record_h) kahan(&a.out_h[ai], &a.comp_h[ai], a.w[r], h);
        }
      } else {
        float coef = 0.f;
        for (int r = 0; r < a.rows; ++r)
          coef = ffma(a.w[r], a.q[((long long)r * 3 + c) * B + t], coef);
        kahan(&a.out[c * B + t], &a.comp[c * B + t], coef, e);
      }
    }
  }
}

}  // namespace pjzfdtd
