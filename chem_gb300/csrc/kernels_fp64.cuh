// FP64 kernels of the DF J/K build (the plain path).
//
// The 3-center tensor lives in atom-block panels (see gbjk.h):
//   panel I = [b_I][naux][K_I] FP64 at B + panel_off[I].
// Every kernel is deterministic: each output element is produced by exactly
// one thread (or one warp) with a fixed summation order, and cross-block
// sums go through partial buffers reduced in a fixed order.
#pragma once
#include "common.cuh"

namespace gbjk {

// Pg[pg_off[I] + m*K_I + k] = P[(boff[I]+m)*ld + colmap[cmoff[I]+k]]
// grid: (ceil(maxK/128), nbf); block 128.
__global__ void k_gather_panel_rows(const double* __restrict__ P, int ld,
                                    const int* __restrict__ blk_of, const int* __restrict__ boff,
                                    const int* __restrict__ panel_K,
                                    const long long* __restrict__ pg_off,
                                    const int* __restrict__ cmoff, const int* __restrict__ colmap,
                                    double* __restrict__ Pg) {
  const int mu = blockIdx.y;
  const int I = blk_of[mu];
  const int m = mu - boff[I];
  const int KI = panel_K[I];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= KI) return;
  Pg[pg_off[I] + (long long)m * KI + k] = P[(long long)mu * ld + colmap[cmoff[I] + k]];
}

// Cg[r*n + i] = C[colmap[r]*n + i] for all panel columns r.
__global__ void k_gather_cols(const double* __restrict__ Cm, int n, const int* __restrict__ colmap,
                              int nrows, double* __restrict__ Cg) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long total = (long long)nrows * n;
  if (idx >= total) return;
  const int r = (int)(idx / n), i = (int)(idx % n);
  Cg[idx] = Cm[(long long)colmap[r] * n + i];
}

// part[mu][X] = sum_k B_I[m][X][k] * Pg_I[m][k]; one warp per (mu, X) row.
__global__ void k_j_rowdot(const double* __restrict__ B, const long long* __restrict__ panel_off,
                           const int* __restrict__ blk_of, const int* __restrict__ boff,
                           const int* __restrict__ panel_K, const long long* __restrict__ pg_off,
                           const double* __restrict__ Pg, int nbf, int naux,
                           double* __restrict__ part) {
  const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= (long long)nbf * naux) return;
  const int mu = (int)(row / naux), X = (int)(row % naux);
  const int I = blk_of[mu];
  const int m = mu - boff[I];
  const int KI = panel_K[I];
  const double* br = B + panel_off[I] + ((long long)m * naux + X) * KI;
  const double* pr = Pg + pg_off[I] + (long long)m * KI;
  double s = 0.0;
  for (int k = lane; k < KI; k += 32) s = fma(br[k], pr[k], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) part[(long long)mu * naux + X] = s;
}

// g[X] = sum_{mu} part[mu][X] (fixed order).
__global__ void k_reduce_rows(const double* __restrict__ part, int nrows, int ncols,
                              double* __restrict__ g) {
  const int X = blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= ncols) return;
  double s = 0.0;
  for (int r = 0; r < nrows; ++r) s += part[(long long)r * ncols + X];
  g[X] = s;
}

// g[X] = sum_{mu} part[mu][X] for the mixed path: warp w of a block sums
// the rows w, w + 16, ... in order (four loads in flight), then the sixteen
// partial sums are added in warp order.  A fixed order, coalesced row reads,
// and sixteen times the parallelism of one thread per column.
__global__ void __launch_bounds__(512)
    k_reduce_rows16(const double* __restrict__ part, int nrows, int ncols,
                    double* __restrict__ g) {
  __shared__ double ps[16][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int X = blockIdx.x * 32 + lane;
  double s = 0.0;
  if (X < ncols) {
    int r = w;
    for (; r + 48 < nrows; r += 64) {
      const double a0 = part[(long long)r * ncols + X];
      const double a1 = part[(long long)(r + 16) * ncols + X];
      const double a2 = part[(long long)(r + 32) * ncols + X];
      const double a3 = part[(long long)(r + 48) * ncols + X];
      s += a0;
      s += a1;
      s += a2;
      s += a3;
    }
    for (; r < nrows; r += 16) s += part[(long long)r * ncols + X];
  }
  ps[w][lane] = s;
  __syncthreads();
  if (w == 0 && X < ncols) {
    double t = ps[0][lane];
    for (int i = 1; i < 16; ++i) t += ps[i][lane];
    g[X] = t;
  }
}

// y = M x, M n x n row-major; one warp per row.
__global__ void k_gemv(const double* __restrict__ M, const double* __restrict__ x, int n,
                       double* __restrict__ y) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const double* mr = M + (long long)row * n;
  double s = 0.0;
  for (int k = lane; k < n; k += 32) s = fma(mr[k], x[k], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = s;
}

// y = L^T x for lower-triangular L (n x n row-major): y[X] = sum_{Y >= X}
// L[Y][X] x[Y], one thread per X, in increasing Y.
__global__ void k_gemv_lower_t(const double* __restrict__ L, const double* __restrict__ x, int n,
                               double* __restrict__ y) {
  const int X = blockIdx.x * blockDim.x + threadIdx.x;
  if (X >= n) return;
  double s = 0.0;
  for (int Y = X; Y < n; ++Y) s = fma(L[(long long)Y * n + X], x[Y], s);
  y[X] = s;
}

// J[mu][colmap[k]] = sum_X B_I[m][X][k] h[X]; grid (ceil(maxK/128), nbf).
__global__ void k_j_colsum(const double* __restrict__ B, const long long* __restrict__ panel_off,
                           const int* __restrict__ blk_of, const int* __restrict__ boff,
                           const int* __restrict__ panel_K, const int* __restrict__ cmoff,
                           const int* __restrict__ colmap, const double* __restrict__ h,
                           int nbf, int naux, double* __restrict__ J) {
  extern __shared__ double hs[];
  for (int x = threadIdx.x; x < naux; x += blockDim.x) hs[x] = h[x];
  __syncthreads();
  const int mu = blockIdx.y;
  const int I = blk_of[mu];
  const int m = mu - boff[I];
  const int KI = panel_K[I];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= KI) return;
  const double* b = B + panel_off[I] + (long long)m * naux * KI + k;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int X = 0;
  // eight loads in flight per thread; accumulator X % 4, in X order
  for (; X + 7 < naux; X += 8) {
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __ldg(b + (long long)(X + j) * KI);
    s0 = fma(v[0], hs[X], s0);
    s1 = fma(v[1], hs[X + 1], s1);
    s2 = fma(v[2], hs[X + 2], s2);
    s3 = fma(v[3], hs[X + 3], s3);
    s0 = fma(v[4], hs[X + 4], s0);
    s1 = fma(v[5], hs[X + 5], s1);
    s2 = fma(v[6], hs[X + 6], s2);
    s3 = fma(v[7], hs[X + 7], s3);
  }
  for (; X + 3 < naux; X += 4) {
    s0 = fma(b[(long long)X * KI], hs[X], s0);
    s1 = fma(b[(long long)(X + 1) * KI], hs[X + 1], s1);
    s2 = fma(b[(long long)(X + 2) * KI], hs[X + 2], s2);
    s3 = fma(b[(long long)(X + 3) * KI], hs[X + 3], s3);
  }
  for (; X < naux; ++X) s0 = fma(b[(long long)X * KI], hs[X], s0);
  J[(long long)mu * nbf + colmap[cmoff[I] + k]] = (s0 + s1) + (s2 + s3);
}

// x as hi + lo, two FP32 values built from the FP64 bit pattern with
// integer operations (no FP64 instruction): hi = the top 24 significand bits
// (truncated), lo = the remaining 29 bits rounded to FP32.  |x| < 2^-126
// gives (0, 0) and a lo below FP32's normal range gives lo = 0; both are
// below 2^-100 relative to the O(1) sums they enter.
__device__ __forceinline__ void f64_split_f32(double x, float& hi, float& lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((u >> 52) & 0x7FF);
  const unsigned int sgn = (unsigned int)(u >> 32) & 0x80000000u;
  const int ef = E - 896;  // FP32 biased exponent of hi (E - 1023 + 127)
  if (ef < 1 || ef > 254) {
    hi = 0.f;
    lo = 0.f;
    return;
  }
  hi = __uint_as_float(sgn | ((unsigned int)ef << 23) | (unsigned int)((u >> 29) & 0x7FFFFF));
  // lo = m29 * 2^(E - 1075): the scale 2^(E-1075) as an FP32 bit pattern
  const int es = E - 1075 + 127;
  if (es < 1) {
    lo = 0.f;
    return;
  }
  const float m29 = (float)(unsigned int)(u & 0x1FFFFFFFu);
  lo = __uint_as_float(sgn | ((unsigned int)es << 23)) * m29;
}

// Compact copy of the prefitted tensor for the mixed-path J: element x as
// hi = its sign, exponent and top 24 significand bits (FP32; 0 outside the
// FP32 normal range) and lo = the next 29 bits rounded to 16
// (lo16 = min(rint(m29 / 2^13), 65535)), so x = hi + lo16 2^(E-1062) to
// about 40 significant bits in 6 bytes.  The copy has its own layout: panel
// I's rows (m, X) with a stride of KP_I = K_I rounded up to a multiple of 8
// (zero padding), panels at cpanel_off[I], in two planes (hi FP32, lo16), so
// that four consecutive columns are one 16-byte and one 8-byte load.
// grid (naux, nbf), block 128.
__global__ void k_encode_f32i16(const double* __restrict__ B, const long long* __restrict__ panel_off,
                                const long long* __restrict__ cpanel_off,
                                const int* __restrict__ blk_of, const int* __restrict__ boff,
                                const int* __restrict__ panel_K, int naux, float* __restrict__ hi,
                                uint16_t* __restrict__ lo) {
  const int X = blockIdx.x, mu = blockIdx.y;
  const int I = blk_of[mu];
  const int m = mu - boff[I];
  const int KI = panel_K[I], KP = (KI + 7) & ~7;
  const double* src = B + panel_off[I] + ((long long)m * naux + X) * KI;
  const long long d = cpanel_off[I] + ((long long)m * naux + X) * KP;
  for (int k = threadIdx.x; k < KP; k += blockDim.x) {
    float h = 0.f;
    unsigned int l = 0;
    if (k < KI) {
      const unsigned long long u = (unsigned long long)__double_as_longlong(src[k]);
      const int E = (int)((u >> 52) & 0x7FF);
      const unsigned int sgn = (unsigned int)(u >> 32) & 0x80000000u;
      const int ef = E - 896;
      if (ef >= 1 && ef <= 254) {
        h = __uint_as_float(sgn | ((unsigned int)ef << 23) | (unsigned int)((u >> 29) & 0x7FFFFF));
        l = min(((unsigned int)(u & 0x1FFFFFFFu) + 4096u) >> 13, 65535u);
      }
    }
    hi[d + k] = h;
    lo[d + k] = (uint16_t)l;
  }
}

// The pair (hi, lo) of a compact element as FP32 values: lo = lo16 *
// 2^(ef - 39 - 127) with hi's sign (0 when that scale leaves the normal range).
__device__ __forceinline__ float f32i16_lo(float hi, unsigned int lo16) {
  const unsigned int b = __float_as_uint(hi);
  const int es = (int)((b >> 23) & 0xFF) - 39;
  const float sc = __uint_as_float((b & 0x80000000u) | ((unsigned int)max(es, 0) << 23));
  return es >= 1 ? sc * (float)lo16 : 0.f;
}

// Mixed-path J columns: J[mu][colmap[k]] = sum_X B_I[m][X][k] h[X] over
// the compact copy (6 bytes per element), with the products and the sum in
// FP32 pairs (hi/lo operands, exact product error by fma, TwoSum
// accumulation), so no FP64 arithmetic runs in the loop and the pass is
// bound by HBM rather than by GB300's FP64 rate.  The auxiliary range is cut
// into chunks of xchunk rows (blockIdx.z) so that the grid is several waves
// deep; chunk z writes its partial column sums to
// part[(z * nbf + mu) * maxK + k] and k_j_colsum_chunks adds the chunks in
// order.  Thread t of block (bx, mu, z) sums columns k = 4 (blockDim bx + t)
// .. +3.  grid (ceil(maxK/(4 blockDim)), nbf, nchunk), dynamic smem xchunk
// float2.
__global__ void k_j_colsum_f32i16(const float* __restrict__ Bhi, const uint16_t* __restrict__ Blo,
                                  const long long* __restrict__ cpanel_off,
                                  const int* __restrict__ blk_of, const int* __restrict__ boff,
                                  const int* __restrict__ panel_K, const double* __restrict__ h,
                                  int nbf, int naux, int xchunk, int maxK,
                                  double* __restrict__ part) {
  extern __shared__ float2 h2[];
  const int x0 = blockIdx.z * xchunk;
  const int nx = min(xchunk, naux - x0);
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    float a, b;
    f64_split_f32(h[x0 + x], a, b);
    h2[x] = make_float2(a, b);
  }
  __syncthreads();
  const int mu = blockIdx.y;
  const int I = blk_of[mu];
  const int m = mu - boff[I];
  const int KI = panel_K[I], KP = (KI + 7) & ~7;
  const int k0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (k0 >= KI) return;
  const long long off = cpanel_off[I] + ((long long)m * naux + x0) * KP + k0;
  const float4* bh = reinterpret_cast<const float4*>(Bhi + off);
  const uint2* bl = reinterpret_cast<const uint2*>(Blo + off);
  const int st4 = KP / 4;  // row stride in float4 / uint2 units
  float sh[4] = {0.f, 0.f, 0.f, 0.f}, sl[4] = {0.f, 0.f, 0.f, 0.f}, se[4] = {0.f, 0.f, 0.f, 0.f};
  auto acc = [](float b_h, float b_l, float2 hh, float& s_h, float& s_l, float& s_e) {
    const float p = __fmul_rn(b_h, hh.x);
    float e = fmaf(b_h, hh.x, -p);
    e = fmaf(b_h, hh.y, e);
    e = fmaf(b_l, hh.x, e);
    const float t = __fadd_rn(s_h, p);
    const float z = __fsub_rn(t, s_h);
    s_l = __fadd_rn(s_l, __fadd_rn(__fsub_rn(s_h, __fsub_rn(t, z)), __fsub_rn(p, z)));
    s_h = t;
    s_e = __fadd_rn(s_e, e);
  };
  auto row = [&](const float4 v, const uint2 w, float2 hh) {
    acc(v.x, f32i16_lo(v.x, w.x & 0xFFFFu), hh, sh[0], sl[0], se[0]);
    acc(v.y, f32i16_lo(v.y, w.x >> 16), hh, sh[1], sl[1], se[1]);
    acc(v.z, f32i16_lo(v.z, w.y & 0xFFFFu), hh, sh[2], sl[2], se[2]);
    acc(v.w, f32i16_lo(v.w, w.y >> 16), hh, sh[3], sl[3], se[3]);
  };
  // software-pipelined: the next eight rows (192 bytes per thread) are
  // loaded before the current eight are summed, so sixteen rows are in
  // flight (a plain unrolled loop of eight kept only a few: 0.55 ms against
  // 0.45 ms on n-C20H42)
  int X = 0;
  if (nx >= 8) {
    float4 v[8];
    uint2 w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      v[j] = __ldg(bh + (long long)j * st4);
      w[j] = __ldg(bl + (long long)j * st4);
    }
    for (; X + 15 < nx; X += 8) {
      float4 vn[8];
      uint2 wn[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        vn[j] = __ldg(bh + (long long)(X + 8 + j) * st4);
        wn[j] = __ldg(bl + (long long)(X + 8 + j) * st4);
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) row(v[j], w[j], h2[X + j]);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        v[j] = vn[j];
        w[j] = wn[j];
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) row(v[j], w[j], h2[X + j]);
    X += 8;
  }
  for (; X < nx; ++X) row(__ldg(bh + (long long)X * st4), __ldg(bl + (long long)X * st4), h2[X]);
  double* out = part + ((long long)blockIdx.z * nbf + mu) * maxK + k0;
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (k0 + j < KI) out[j] = (double)sh[j] + ((double)sl[j] + (double)se[j]);
}

// J[mu][colmap(k)] = sum over chunks (in order) of part[z][mu][k].
// grid (ceil(maxK/128), nbf).
__global__ void k_j_colsum_chunks(const double* __restrict__ part, int nchunk, int nbf, int maxK,
                                  const int* __restrict__ blk_of, const int* __restrict__ panel_K,
                                  const int* __restrict__ cmoff, const int* __restrict__ colmap,
                                  double* __restrict__ J) {
  const int mu = blockIdx.y;
  const int I = blk_of[mu];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= panel_K[I]) return;
  double s = 0.0;
  for (int z = 0; z < nchunk; ++z) s += part[((long long)z * nbf + mu) * maxK + k];
  J[(long long)mu * nbf + colmap[cmoff[I] + k]] = s;
}

// Dense expansion of the panel array: D[mu][X][colmap(k)] = P_I[m][X][k]
// (mu = boff[I] + m); entries outside the kept pattern are not written.
// grid (ceil(maxK/128), naux, nbf).
__global__ void k_expand_panels(const double* __restrict__ P, const long long* __restrict__ panel_off,
                                const int* __restrict__ blk_of, const int* __restrict__ boff,
                                const int* __restrict__ panel_K, const int* __restrict__ cmoff,
                                const int* __restrict__ colmap, int nbf, int naux,
                                double* __restrict__ D) {
  const int mu = blockIdx.z, X = blockIdx.y;
  const int I = blk_of[mu];
  const int KI = panel_K[I];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= KI) return;
  const int m = mu - boff[I];
  D[((long long)mu * naux + X) * nbf + colmap[cmoff[I] + k]] =
      P[panel_off[I] + ((long long)m * naux + X) * KI + k];
}

// Grouped FP64 GEMM over a tile list; 64 x TN tiles (TN = 64, 32 or 16),
// 16 * TN / 4 threads, 4x4 outputs per thread.  Every output is one in-order
// fma chain over its k range, whatever the tile shape.
// TRANSA: A is stored K x M row-major, op(A)(m, k) = A[k * lda + m].
template <bool TRANSB, bool TRANSA = false, int TN = 64>
__global__ void __launch_bounds__(TN * 4)
    k_gemm_fp64(const GemmGroup* __restrict__ groups, const GemmTile* __restrict__ tiles,
                double alpha) {
  static_assert(TN == 64 || TN == 32 || TN == 16, "tile width");
  constexpr int NT = TN * 4;   // threads
  constexpr int CW = TN / 4;   // thread columns
  __shared__ double As[16][65];
  __shared__ double Bs[16][TN + 1];
  const GemmTile t = tiles[blockIdx.x];
  const GemmGroup g = groups[t.group];
  const int tid = threadIdx.x;
  const int tx = tid % CW, ty = tid / CW;
  const int m0 = t.mt * 64, n0 = t.nt * TN;
  int kend = t.k1;
  if ((g.flags & kLowerA) && kend > m0 + 64) kend = m0 + 64;  // A[m][k] = 0 for k > m
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.0;
  for (int k0 = t.k0; k0 < kend; k0 += 16) {
#pragma unroll
    for (int r = 0; r < 1024 / NT; ++r) {
      const int idx = tid + NT * r;
      if (TRANSA) {
        const int kk = idx >> 6, row = idx & 63;
        const int gm = m0 + row, gk = k0 + kk;
        As[kk][row] = (gm < g.M && gk < kend) ? g.A[(long long)gk * g.lda + gm] : 0.0;
      } else {
        const int row = idx >> 4, kk = idx & 15;
        const int gm = m0 + row, gk = k0 + kk;
        As[kk][row] = (gm < g.M && gk < kend) ? g.A[(long long)gm * g.lda + gk] : 0.0;
      }
    }
#pragma unroll
    for (int r = 0; r < (16 * TN) / NT; ++r) {
      const int idx = tid + NT * r;
      if (TRANSB) {
        const int col = idx >> 4, kk = idx & 15;
        const int gn = n0 + col, gk = k0 + kk;
        Bs[kk][col] = (gn < g.N && gk < kend) ? g.B[(long long)gn * g.ldb + gk] : 0.0;
      } else {
        const int kk = idx / TN, col = idx % TN;
        const int gn = n0 + col, gk = k0 + kk;
        Bs[kk][col] = (gn < g.N && gk < kend) ? g.B[(long long)gk * g.ldb + gn] : 0.0;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx + CW * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
  double* C = g.C + t.coff;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int gm = m0 + ty + 16 * r;
    if (gm >= g.M) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int gn = n0 + tx + CW * c;
      if (gn >= g.N) continue;
      double v = alpha * acc[r][c];
      if (g.flags & kAccum) v += C[(long long)gm * g.ldc + gn];
      C[(long long)gm * g.ldc + gn] = v;
    }
  }
}

// Tiny problems: 16 x 16 tiles, one thread per output, each output the
// in-order fma chain over the tile's k range read straight from global
// memory.  A lower-triangular A stops at k = m: the terms beyond are exact
// zeros, so every nonzero result equals the tiled kernel's bit for bit.
// For problems so small that 64-row tiles would be mostly padding and the
// few tiles would leave most SMs' FP64 units idle.
template <bool TRANSB>
__global__ void __launch_bounds__(256)
    k_gemm_fp64_elem(const GemmGroup* __restrict__ groups, const GemmTile* __restrict__ tiles,
                     double alpha) {
  const GemmTile t = tiles[blockIdx.x];
  const GemmGroup g = groups[t.group];
  const int gm = t.mt * 16 + (threadIdx.x >> 4), gn = t.nt * 16 + (threadIdx.x & 15);
  if (gm >= g.M || gn >= g.N) return;
  int kend = t.k1;
  if ((g.flags & kLowerA) && kend > gm + 1) kend = gm + 1;
  const double* a = g.A + (long long)gm * g.lda;
  const double* b = TRANSB ? g.B + (long long)gn * g.ldb : g.B + gn;
  const long long bs = TRANSB ? 1 : g.ldb;
  double acc = 0.0;
  int k = t.k0;
  // eight loads in flight, then their fmas in order
  for (; k + 8 <= kend; k += 8) {
    double av[8], bv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      av[u] = a[k + u];
      bv[u] = b[(long long)(k + u) * bs];
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) acc = fma(av[u], bv[u], acc);
  }
  for (; k < kend; ++k) acc = fma(a[k], b[(long long)k * bs], acc);
  double* C = g.C + t.coff + (long long)gm * g.ldc + gn;
  double v = alpha * acc;
  if (g.flags & kAccum) v += *C;
  *C = v;
}

// out[m][n] = alpha * sum_s part[s][m][n] over the upper triangle (n >= m)
// when symmetric (mirrored to the lower one), else everywhere.
__global__ void k_splitk_reduce(const double* __restrict__ part, int nsplit, int n,
                                double alpha, int symmetric, double* __restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * n) return;
  const int m = (int)(idx / n), c = (int)(idx % n);
  if (symmetric && c < m) return;
  double s = 0.0;
  for (int k = 0; k < nsplit; ++k) s += part[(long long)k * n * n + idx];
  s *= alpha;
  out[idx] = s;
  if (symmetric && c != m) out[(long long)c * n + m] = s;
}

// Zero atom blocks (I, J) of the n x n matrix M with Frobenius norm < eps.
// grid (nblk, nblk), block 128.
__global__ void k_block_filter(double* __restrict__ M, int n, const int* __restrict__ boff,
                               double eps) {
  const int I = blockIdx.x, J = blockIdx.y;
  const int r0 = boff[I], nr = boff[I + 1] - r0;
  const int c0 = boff[J], nc = boff[J + 1] - c0;
  __shared__ double red[128];
  double s = 0.0;
  for (int e = threadIdx.x; e < nr * nc; e += blockDim.x) {
    const double v = M[(long long)(r0 + e / nc) * n + c0 + e % nc];
    s = fma(v, v, s);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 64; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (sqrt(red[0]) < eps)
    for (int e = threadIdx.x; e < nr * nc; e += blockDim.x)
      M[(long long)(r0 + e / nc) * n + c0 + e % nc] = 0.0;
}

}  // namespace gbjk

namespace gbjk {

// Seeded synthetic 3-center tensor in the panel layout (the synthetic DF-K
// workload): element (Y, mu, nu) = N(0,1)[seed, min(mu,nu), max(mu,nu), Y] *
// exp(-0.5 |I - J| / decay), I and J the atom blocks of mu and nu, so the
// tensor is symmetric in (mu, nu).  Normal deviates come from a splitmix64
// hash of the indices through Box-Muller.  grid (ceil(maxK/128), naux, nbf).
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void k_synthetic_panels(double* __restrict__ B, const long long* __restrict__ panel_off,
                                   const int* __restrict__ blk_of, const int* __restrict__ boff,
                                   const int* __restrict__ panel_K, const int* __restrict__ cmoff,
                                   const int* __restrict__ colmap, int nbf, int naux,
                                   unsigned long long seed, float decay) {
  const int mu = blockIdx.z;
  const int Y = blockIdx.y;
  const int I = blk_of[mu];
  const int m = mu - boff[I];
  const int KI = panel_K[I];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= KI) return;
  const int nu = colmap[cmoff[I] + k];
  const int J = blk_of[nu];
  const unsigned long long a = (unsigned long long)min(mu, nu), b = (unsigned long long)max(mu, nu);
  const unsigned long long h = splitmix64(seed ^ splitmix64((a * (unsigned long long)nbf + b) *
                                                               (unsigned long long)naux + Y));
  const float u1 = ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f);
  const float u2 = (float)((h >> 16) & 0xFFFFFF) * (1.0f / 16777216.0f);
  const float g = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
  const float w = expf(-0.5f * fabsf((float)(I - J)) / decay);
  B[panel_off[I] + ((long long)m * naux + Y) * KI + k] = (double)(g * w);
}

// out = alpha * sum_s part[s] (+ out when accumulate), upper triangle
// mirrored when symmetric; order: existing value, then splits in order.
__global__ void k_splitk_reduce_acc(const double* __restrict__ part, int nsplit, int n,
                                    double alpha, int symmetric, int accumulate,
                                    double* __restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * n) return;
  const int m = (int)(idx / n), c = (int)(idx % n);
  if (symmetric && c < m) return;
  double s = 0.0;
  for (int k = 0; k < nsplit; ++k) s += part[(long long)k * n * n + idx];
  s *= alpha;
  if (accumulate) s += out[idx];
  out[idx] = s;
  if (symmetric && c != m) out[(long long)c * n + m] = s;
}

}  // namespace gbjk
