// S-matrix assembly on the device: port-plane overlaps of recorded phasors
// and the dL/d-eps product of forward and unit-adjoint phasors over the
// design box.  Replaces the host-side reductions of a multi-port S-matrix
// objective: pjz's scatter reads the port planes of every port's field
// (src/pjz/_field.py:305-338, 367-369) and differentiates with the
// pairwise residual products f_i f_j / a_i (src/pjz/_field.py:380-398);
// here the objective's gradient is sum_w Re(q_w sum_ij F_i c_ijw G_j) over
// the n forward phasors F_i and n unit-adjoint phasors G_j of one batched
// launch.  Both kernels accumulate in FP64 in a fixed order (deterministic).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pjzfdtd {

constexpr int kPlaneTermsMax = 64;  // overlaps per call
constexpr int kSmatSolvesMax = 16;  // forward (and adjoint) solves
constexpr int kSmatCoefMax = 1024;  // n * n * ww coefficients
constexpr int kSmatFreqMax = 32;
constexpr int kOverlapThreads = 256;

struct PlaneOverlapArgs {
  const float* block[kPlaneTermsMax];  // phasors (2 ww, 3, npts) per term
  const float* prof[kPlaneTermsMax];   // weights (npts) per term
  long long npts[kPlaneTermsMax];
  int comp[kPlaneTermsMax];            // field component of each term
  int ww;
  double* out;                         // (nterms, ww, 2): re, im
};

// grid (nterms, ww), kOverlapThreads threads: out[k][w] = sum_p
// (block_k[w][comp_k][p] + i block_k[ww + w][comp_k][p]) * prof_k[p].
__global__ void __launch_bounds__(kOverlapThreads)
    plane_overlap_kernel(const PlaneOverlapArgs a) {
  __shared__ double sr[kOverlapThreads], si[kOverlapThreads];
  const int k = blockIdx.x, w = blockIdx.y;
  const long long n = a.npts[k];
  const float* re = a.block[k] + ((long long)w * 3 + a.comp[k]) * n;
  const float* im = a.block[k] + ((long long)(a.ww + w) * 3 + a.comp[k]) * n;
  const float* pr = a.prof[k];
  double r = 0.0, i = 0.0;
  for (long long p = threadIdx.x; p < n; p += kOverlapThreads) {
    const double pv = (double)pr[p];
    r += (double)re[p] * pv;
    i += (double)im[p] * pv;
  }
  sr[threadIdx.x] = r;
  si[threadIdx.x] = i;
  __syncthreads();
  for (int s = kOverlapThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.out[((long long)k * a.ww + w) * 2] = sr[0];
    a.out[((long long)k * a.ww + w) * 2 + 1] = si[0];
  }
}

struct SmatGradArgs {
  const float* F[kSmatSolvesMax];  // forward phasors (2 ww, cells)
  const float* G[kSmatSolvesMax];  // unit-adjoint phasors (2 ww, cells)
  float coef[kSmatCoefMax][2];     // c[i][j][w]: re, im
  float q[kSmatFreqMax][2];        // q[w]: re, im
  int n, ww;
  long long cells;
  float* grad;                     // (cells)
};

// grad[t] = sum_w Re(q_w sum_i F_i,w[t] sum_j c_ijw G_j,w[t]), FP64 sums.
__global__ void smatrix_grad_kernel(const SmatGradArgs a) {
  const long long C = a.cells;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < C;
       t += (long long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int w = 0; w < a.ww; ++w) {
      double gr[kSmatSolvesMax], gi[kSmatSolvesMax];
      for (int j = 0; j < a.n; ++j) {
        gr[j] = (double)a.G[j][(long long)w * C + t];
        gi[j] = (double)a.G[j][(long long)(a.ww + w) * C + t];
      }
      double sr = 0.0, si = 0.0;  // sum_i F_i (sum_j c_ij G_j)
      for (int i = 0; i < a.n; ++i) {
        double cr = 0.0, ci = 0.0;
        for (int j = 0; j < a.n; ++j) {
          const int ix = (i * a.n + j) * a.ww + w;
          const double ar = (double)a.coef[ix][0], ai = (double)a.coef[ix][1];
          cr += ar * gr[j] - ai * gi[j];
          ci += ar * gi[j] + ai * gr[j];
        }
        const double fr = (double)a.F[i][(long long)w * C + t];
        const double fi = (double)a.F[i][(long long)(a.ww + w) * C + t];
        sr += fr * cr - fi * ci;
        si += fr * ci + fi * cr;
      }
      acc += (double)a.q[w][0] * sr - (double)a.q[w][1] * si;
    }
    a.grad[t] = (float)acc;
  }
}

}  // namespace pjzfdtd
