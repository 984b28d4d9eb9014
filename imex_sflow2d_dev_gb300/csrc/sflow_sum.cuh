// sflow_sum.cuh -- compensated FP64 summation for the log-line sums (mass,
// volume, wet area, solid mass; IMEX_SfloW2D.f90:535-542): each thread adds
// its cells with Neumaier's compensation (A. Neumaier, ZAMM 54, 1974), the
// threads of a block combine (sum, compensation) pairs with the exact error
// of each pairwise addition, and the host or a last kernel adds the block
// results with the same compensation.
#pragma once

namespace sflow {

// s + c += x, with the rounding error of s + x kept in c
__device__ __forceinline__ void csum_add(double& s, double& c, double x) {
  const double t = s + x;
  c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
  s = t;
}

// In-block reduction of M compensated sums held by every thread (blockDim.x
// = T, a power of two): on return thread 0 holds the block's (s + c) of each
// sum in out[m].  sh_s and sh_c are shared arrays of M * T doubles.
template <int M, int T>
__device__ __forceinline__ void csum_block(const double (&s)[M], const double (&c)[M], double* sh_s,
                                           double* sh_c, double* out) {
  for (int m = 0; m < M; ++m) {
    sh_s[m * T + threadIdx.x] = s[m];
    sh_c[m * T + threadIdx.x] = c[m];
  }
  __syncthreads();
  for (int w = T / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      for (int m = 0; m < M; ++m) {
        double a = sh_s[m * T + threadIdx.x], ca = sh_c[m * T + threadIdx.x];
        csum_add(a, ca, sh_s[m * T + threadIdx.x + w]);
        sh_s[m * T + threadIdx.x] = a;
        sh_c[m * T + threadIdx.x] = ca + sh_c[m * T + threadIdx.x + w];
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int m = 0; m < M; ++m) out[m] = sh_s[m * T] + sh_c[m * T];
}

}  // namespace sflow
