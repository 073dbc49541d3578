// Kernels of the SOS-AO-MP2 Laplace batch (ll_full Z builder) that are not
// GEMMs: coefficient gathers, operand exponents, the split-K reduction of Z
// and the energy sums.  Every point t of the batch uses the same padded
// strides (hld occupied columns, vld virtual columns), so grid.y = t and a
// fixed per-point stride address all of them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbjk {

// Cg_t[r][i] = Lo_t[colmap[r]][i]: panel-column copies of every point's
// occupied factor.  grid (ceil(nrows*ld / 256), npts).
__global__ void k_mp2_gather(const double* __restrict__ Lo, long long lo_stride, int ld,
                             const int* __restrict__ colmap, int nrows,
                             double* __restrict__ Cg, long long cg_stride) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nrows * ld) return;
  const int r = (int)(idx / ld), i = (int)(idx % ld);
  const int t = blockIdx.y;
  Cg[t * cg_stride + idx] = Lo[t * lo_stride + (long long)colmap[r] * ld + i];
}

// Row exponents of the second-transform operand: row rho = (X, i) of point
// t has the values H_t[n][rho], n < nk.  e[t][rho] = (max biased FP64
// exponent over n) - 1022, or -2000 for an all-zero row.  Coalesced: one
// thread per rho, looping over n.  grid (ceil(nrho / 256), npts).
__global__ void k_mp2_colmax_exp(const double* __restrict__ H, long long h_stride, int nk,
                                 long long nrho, int* __restrict__ e, long long e_stride) {
  const long long rho = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (rho >= nrho) return;
  const int t = blockIdx.y;
  const double* p = H + t * h_stride + rho;
  unsigned int mx = 0;
  for (int n = 0; n < nk; ++n) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(p[(long long)n * nrho]);
    mx = max(mx, (unsigned int)((u >> 52) & 0x7FF));
  }
  e[t * e_stride + rho] = mx == 0 ? -2000 : (int)mx - 1022;
}

// Z_t[X][Y] = Z_t[Y][X] = sum_s part[s][t][X][Y] (s in order) for X <= Y.
// grid (ceil(n*n / 256), npts).
__global__ void k_mp2_z_reduce(const double* __restrict__ part, int nsplit, int npts, int n,
                               double* __restrict__ Z) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nn = (long long)n * n;
  if (idx >= nn) return;
  const int t = blockIdx.y;
  const int X = (int)(idx / n), Y = (int)(idx % n);
  if (Y < X) return;
  double s = 0.0;
  for (int k = 0; k < nsplit; ++k) s += part[((long long)k * npts + t) * nn + idx];
  Z[t * nn + idx] = s;
  Z[t * nn + (long long)Y * n + X] = s;
}

// Z_t[Y][X] = Z_t[X][Y] for X < Y.  grid (ceil(n*n / 256), npts).
__global__ void k_mp2_z_mirror(double* __restrict__ Z, int n) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nn = (long long)n * n;
  if (idx >= nn) return;
  const int X = (int)(idx / n), Y = (int)(idx % n);
  if (Y <= X) return;
  double* z = Z + blockIdx.y * nn;
  z[(long long)Y * n + X] = z[idx];
}

// rsq[t][X] = sum_Y Z_t[X][Y]^2: one warp per row, lane l sums Y = l, l+32,
// ... with fma, then an xor butterfly.  grid (ceil(n*32 / 256), npts).
__global__ void k_mp2_rowsq(const double* __restrict__ Z, int n, double* __restrict__ rsq) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const int t = blockIdx.y;
  const double* z = Z + (long long)t * n * n + w * n;
  double s = 0.0;
  for (int Y = lane; Y < n; Y += 32) s = fma(z[Y], z[Y], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) rsq[(long long)t * n + w] = s;
}

// e[t] = sum_X rsq[t][X] in X order (one thread per point).
__global__ void k_mp2_energy(const double* __restrict__ rsq, int n, int npts,
                             double* __restrict__ e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npts) return;
  double s = 0.0;
  for (int X = 0; X < n; ++X) s += rsq[(long long)t * n + X];
  e[t] = s;
}

}  // namespace gbjk
