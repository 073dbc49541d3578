// Split-precision path of the K build: FP64 operands as BF16 digit slices on
// the 5th-generation tensor cores (tcgen05.mma, accumulators in TMEM).
//
// Number format.  Row r of an FP64 operand gets an exponent e_r with
// |x| < 2^e_r for every x of the row.  x is rounded to the 39-bit integer
// X = rint(|x| 2^(39-e_r)) and written in balanced base-256 digits
//   X = sum_{j=0..4} d_j 256^j,  d_0..d_3 in [-128, 127],  d_4 in [0, 128],
// which are exact in BF16.  Slice s (s = 0 most significant) holds
// sign(x) * d_{4-s}.  The extraction uses integer operations only.
//
// Product.  sum_k x_A x_B = 2^(eA+eB-78) sum_{s,t} r_{st} 256^(8-s-t),
// r_{st} = sum_k a_s b_t.  Pairs with s+t <= 4 are kept (15 BF16 digit
// products per k).  Diagonals d = s+t = 0, 1, 2 are summed exactly: every
// digit product is at most 2^14 in magnitude, so over a chunk of 256 k every
// partial sum is an integer below 2^24, hence exact in the FP32 TMEM
// accumulator; after each chunk the epilogue converts them to integers and
// adds W = r0 256^2 + r1 256 + r2 into an int64 register.  Diagonals 3 and 4
// accumulate in FP32 over the whole k range (weights 2^-24 and 2^-32 of the
// leading term) and are folded in with 16 fractional bits:
//   value = 2^(eA+eB-46) (W 2^16 + rint(256 r3) + rint(r4)),
// where each rint is taken as 32-bit halves with FP32 arithmetic (|256 r3|
// stays below 2^38 for items of at most 8192 k); the int64 result is
// converted to FP64 (round to nearest) and 2^(eA+eB-46) is added to its
// exponent field.
//
// Pipeline (one CTA per SM, persistent over a work list):
//   warp 0      producer: 1-D bulk copies (cp.async.bulk) of pre-tiled slice
//               images into a 3-stage shared-memory ring (mbarrier tx count)
//   warp 1      TMEM allocation and the single MMA-issuing thread
//   warps 2..13 epilogue: drain exact diagonals per chunk, write results
//               (row and column exponents loaded at the item start, column
//               exponents broadcast across the warp by shuffles)
// Per k-tile the MMA thread issues the exact-diagonal pairs, commits them at
// a chunk end, then the approximate pairs (15 pairs as 9 MMAs of N = 96 or
// 192); at a chunk start it issues the approximate pairs first, so the drain
// of chunk c overlaps the approximate MMAs of two k-tiles.  Every wait is
// bounded (spin_ns, kSpinNs by default); on timeout the CTA records an error
// code, every other wait of the launch gives up, and before exiting each CTA
// waits (bounded by time only) for its own bulk copies, on the stages' full
// barriers, and its own MMAs, on a commit barrier, then frees TMEM.
//
// Shared-memory operand layout: K-major, no swizzle, 8x8 core matrices
// (128 B); within a tile of R rows x 32 k the element (r, k) sits at byte
// (r/8)*512 + (k/8)*128 + (r%8)*16 + (k%8)*2 (SBO = 512, LBO = 128).
// Global slice images hold 32 rows x 32 k in that order and are stored as
// [k-tile][slice][row block] so a tile of R rows of one slice is one
// contiguous R/32 * 2 KB run.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "common.cuh"
#include "kernels_fp64.cuh"

namespace gbjk {

constexpr int kMaxSlices = 8;
constexpr int kSlices = 5;        // digits per operand
constexpr int kTileM = 128;       // rows of A per tile (TMEM lanes)
constexpr int kTileN = 96;        // rows of B per tile (accumulator columns)
constexpr int kTileK = 32;        // k per pipeline stage
constexpr int kChunkTiles = 8;    // k-tiles per exact chunk (256 k)
constexpr int kStages = 3;
constexpr int kImage = 1024;      // bf16 elements per 32x32 slice image
constexpr int kEpiWarps = 12;      // 3 per TMEM lane quadrant, 32 columns each
constexpr int kEpiCols = kTileN / 3;
constexpr int kThreads = 32 * (2 + kEpiWarps);
constexpr int kTmemCols = 512;
constexpr unsigned long long kSpinNs = 2000000000ull;  // 2 s per wait
constexpr int kBytesA = kSlices * kTileM * kTileK * 2;  // 40 KB
constexpr int kBytesB = kSlices * kTileN * kTileK * 2;  // 30 KB
constexpr int kSmemBytes = kStages * (kBytesA + kBytesB) + 1024;

// One output tile of a split GEMM: C[r][c] = sum_k A[r][k] B[c][k] over the
// k-tiles [kt0, kt0+nkt) of the operands' slice images.
struct SplitItem {
  const uint16_t* a;  // slice images of the A operand group
  const uint16_t* b;  // slice images of the B operand group
  int a_nrb, a_rb0;   // row blocks (32 rows) in the group, first of the tile
  int b_nrb, b_rb0;
  int kt0, nkt;
  const int* ea;  // row exponents of the tile's A rows (tile-local index)
  const int* eb;  // row exponents of the tile's B rows
  double* out;    // out[r * ldr + c]
  long long ldr;
  int m_valid, n_valid;
  // optional: atomicMax of the biased FP64 exponent of row r's results into
  // emax[(emax_row0 + r) / emax_div] (row exponents of the next operand)
  unsigned int* emax;
  int emax_row0, emax_div;
  // optional: columns c0 + col >= ncol1 (c0 = first column of the tile) are
  // density columns m' = c0 + col - ncol1; the value of row r goes to
  // out2[emax_row0 + r] when m' == (emax_row0 + r) / emax_div, and is neither
  // stored in `out` nor counted in emax
  double* out2;
  int c0, ncol1;
  // Output layout.  perm_rs == 0: row-major out[r * ldr + c].  perm_rs > 0:
  // the half-transform layout.  The tile's row r is the linear panel row
  // R = emax_row0 + r = m * perm_div + y (AO function m of the panel,
  // auxiliary index y); its value in column c lands at
  //   out[m * perm_rs + (y / 32) * 32 * ldr + (c / 2) * 64 + (y % 32) * 2 + c % 2]
  // (ldr even, out 16-byte aligned), i.e. within each group of 32 auxiliary
  // indices the column pairs are outermost.  A warp holds 32 consecutive
  // rows, so each of its 16-byte column-pair stores is one contiguous
  // 512-byte run.  Rows of out are flat k-vectors of length perm_rs; a
  // consumer that contracts over the whole k range (the exchange) needs no
  // other order, provided every row uses the same one.
  long long perm_rs = 0;
  int perm_div = 1;
  // Padded A rows.  apitch > 0: the A operand holds its panel rows (m, y) at
  // R' = m * apitch + y (apitch a multiple of 32, so every 32-row block is
  // one AO function m and one group of 32 auxiliary indices); the tile's
  // row r is R' = arow0 + r, rows with y >= ay_valid are padding.  Every
  // row-indexed output then uses the unpadded row R = m * ay_valid + y: the
  // row-major `out` points at unpadded row arow0, emax/out2/perm take R.
  int apitch = 0, arow0 = 0, ay_valid = 0;
  // Half transform with digit output (k_split_gemm<true, false>): the
  // tile's rows are (m, y) of one panel, its columns i orbitals.  Instead
  // of FP64 values the epilogue writes the five digit slices of H row
  // mu = hrow0 + m into `hdig` (h_nrb row blocks, 64-byte swizzled images,
  // k-tile g * seg_nkt + i for auxiliary group g = y / 32, k = y % 32 in it)
  // with one exponent per (mu, g), eseg[mu * es_ld + g], and the maximum
  // over g into emax (biased, atomicMax).
  uint16_t* hdig = nullptr;
  int h_nrb = 0, hrow0 = 0;
  int* eseg = nullptr;
  int es_ld = 0;
  // k-tiles per exponent segment (the orbital count of the half transform)
  int seg_nkt = 0;
  // Segmented exchange (k_split_gemm<false, true>): k-tile kt belongs to
  // segment kt / seg_nkt, in which the tile's A and B rows carry the
  // exponents esa[r * es_ld + g] and esb[c * es_ld + g] (ea/eb: their
  // maxima over g).
  const int* esa = nullptr;
  const int* esb = nullptr;
};

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait; on timeout records `code` in *err and returns false, and
// it gives up as soon as another wait of the launch has recorded an error.
// The error flag and the timer are read every 1024 polls only, so a
// completed phase is seen within one try_wait.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code,
                                          unsigned long long spin_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023) == 0) {
      if (*(volatile int*)err != 0) return false;
      if (globaltimer() - t0 > spin_ns) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}
// Wait bounded by time only (not by the error flag): for the completion of
// this CTA's own bulk copies and MMAs before it exits, which always come.
__device__ __forceinline__ bool mbar_wait_own(uint64_t* bar, uint32_t parity,
                                              unsigned long long spin_ns) {
  const unsigned long long t0 = globaltimer();
  for (uint32_t i = 0;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023) == 1023 && globaltimer() - t0 > spin_ns) return false;
  }
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                        uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// smem matrix descriptor: K-major, no swizzle, LBO 128 B, SBO 512 B
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)(128 >> 4) << 16;
  d |= (uint64_t)(512 >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version (sm_100 family)
  return d;                // base offset 0, layout type 0 (no swizzle)
}
// smem matrix descriptor: K-major, 64-byte swizzle.  A row of 32 BF16 k
// values is one 64-byte line; its 16-byte chunk c sits at chunk
// c ^ ((row >> 1) & 3) (address bits 4-5 xor bits 7-8); 8-row groups are
// 512 B apart (SBO).  The leading byte offset is unused in this mode.  The
// second K = 16 step of a k-tile starts 32 B into the line.
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(512 >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version (sm_100 family)
  d |= (uint64_t)4 << 61;  // swizzle mode: 64-byte
  return d;
}
// Element offset (in BF16 units) of (row r, k) inside a 32 x 32 slice image
// in the 64-byte swizzled layout.
__host__ __device__ __forceinline__ int sw64_offset(int r, int k) {
  return r * 32 + ((((k >> 3) ^ ((r >> 1) & 3))) << 3) + (k & 7);
}
// instruction descriptor: kind::f16, BF16 x BF16 -> F32, K-major A and B
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// rint(a) = h 2^16 + l for an FP32 value a with |a| < 2^38, in FP32
// arithmetic only: h = rint(a 2^-16) by the 1.5*2^23 magic (a single fma
// rounds a 2^-16 + magic), the remainder a - h 2^16 is exact (|.| <= 2^15),
// and l = rint(remainder) by the same magic.  Ties round to even.
__device__ __forceinline__ void f32_split16(float a, int& h, int& l) {
  const float t = __fmaf_rn(a, 1.52587890625e-05f, 12582912.0f);
  h = __float_as_int(t) - 0x4B400000;
  const float hf = __fsub_rn(t, 12582912.0f);
  const float r = __fmaf_rn(-hf, 65536.0f, a);
  l = __float_as_int(__fadd_rn(r, 12582912.0f)) - 0x4B400000;
}

// v * 2^e2 rounded to nearest FP64, as a bit pattern built with integer
// operations only (|v| < 2^63); ties round away from zero.  Used where the
// scaled result leaves the normal range.
__device__ __forceinline__ double i64_scaled_to_f64_int(long long v, int e2) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
  const unsigned long long m = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  int msb = 63 - __clzll((long long)m);
  unsigned long long frac;
  if (msb <= 52) {
    frac = m << (52 - msb);
  } else {
    const int sh = msb - 52;
    unsigned long long mr = m + (1ull << (sh - 1));  // round half up
    if (msb < 63 && (mr >> (msb + 1))) {             // carry into a new top bit
      ++msb;
      frac = mr >> (sh + 1);
    } else {
      frac = mr >> sh;
    }
  }
  frac &= (1ull << 52) - 1;
  const long long ex = (long long)msb + e2 + 1023;
  if (ex <= 0) return 0.0;
  if (ex >= 2047) return __longlong_as_double((long long)(sgn | (0x7FFull << 52)));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)ex << 52) | frac));
}

// v * 2^e2 rounded to nearest FP64 (ties to even): the hardware int64 ->
// FP64 conversion (exact rounding, one instruction), then e2 added to the
// exponent field; results below the normal range flush to zero and above it
// become infinite, as in i64_scaled_to_f64_int.  The epilogue converts
// 128 x 96 results per work item; this form makes the half transform about
// 8 % faster than the integer-only one.
__device__ __forceinline__ double i64_scaled_to_f64(long long v, int e2) {
  const long long b = __double_as_longlong(__ll2double_rn(v));
  const int ex = (int)((b >> 52) & 0x7FF) + e2;
  const long long inf = (b & (1ll << 63)) | (0x7FFll << 52);
  const long long r = ex <= 0 ? 0ll : (ex >= 2047 ? inf : b + ((long long)e2 << 52));
  return __longlong_as_double(v == 0 ? 0ll : r);
}

// x * 2^-sh rounded to nearest (ties up) for sh >= 0; 0 when sh > 62.
__device__ __forceinline__ long long shr_round(long long x, int sh) {
  if (sh == 0) return x;
  if (sh > 62) return 0;
  return (x + (1ll << (sh - 1))) >> sh;
}

// ------------------------------------------------------------ split kernels
// A split job fills rows [row0, row0 + nrows) of one digit operand:
// element (r, c) = src[(r - row0)*rs + c*cs] for c < ncols, zero for
// ncols <= c < nkt*32.  Row exponents are e[r] (e_biased != 0: e holds the
// maximum biased FP64 exponent of the row, 0 for an all-zero row).  Slice
// images go to dst as [kt][s][rb][1024]; rows outside every job stay as
// allocated (zero).
struct SplitJob {
  const double* src;
  long long rs, cs;
  int row0, nrows;
  long long ncols;
  int* e;
  int e_biased;
  int nrb, nkt;
  uint16_t* dst;
};

// e[r] = (max biased exponent over row r) - 1022, so |x| < 2^e[r]; -2000 for
// an all-zero row.  grid (rows/8, njobs), one warp per row.
__global__ void k_row_maxexp(const SplitJob* __restrict__ jobs) {
  const SplitJob jb = jobs[blockIdx.y];
  const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= jb.nrows) return;
  unsigned int mx = 0;
  const double* p = jb.src + i * jb.rs;
  for (long long c = lane; c < jb.ncols; c += 32) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(p[c * jb.cs]);
    mx = max(mx, (unsigned int)((u >> 52) & 0x7FF));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) jb.e[jb.row0 + i] = mx == 0 ? -2000 : (int)mx - 1022;
}

// p[i] = v for i < n (grid-stride).
__global__ void k_fill_int(int* __restrict__ p, long long n, int v) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

// Biased FP64 exponent maxima (0 = all zero) -> row exponents in place.
__global__ void k_exp_unbias(int* __restrict__ e, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) e[i] = e[i] == 0 ? -2000 : e[i] - 1022;
}

// Zero the auxiliary slots y0 <= y' < 32 of the last 32-index group of every
// row of a column-pair-outermost H (SplitItem::perm_rs): rows of rs doubles,
// the group starting at column gbase, npairs column pairs.  Grid-stride.
__global__ void k_zero_hpad(double* __restrict__ H, int nrows, long long rs, long long gbase,
                            int y0, int npairs) {
  const int ny = 32 - y0;
  const long long per_row = (long long)npairs * ny;
  const long long n = (long long)nrows * per_row;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / per_row, t = i - r * per_row;
    const long long p = t / ny;
    const int yy = y0 + (int)(t - p * ny);
    *reinterpret_cast<double2*>(H + r * rs + gbase + p * 64 + yy * 2) = make_double2(0.0, 0.0);
  }
}

__device__ __forceinline__ uint16_t small_int_to_bf16(int d) {
  // d in [-2^22, 2^22): exact float via the 1.5*2^23 magic, then BF16 bits
  // (exact: |d| <= 128 needs at most 8 significant bits)
  const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
  return (uint16_t)(__float_as_uint(f) >> 16);
}

// Slice images.  One warp per (8-row group, k-tile): lane (rr, kc) =
// (lane & 7, lane >> 3) handles row 8g + rr, columns 32kt + 8kc .. +7, so
// each warp writes 512 contiguous bytes per slice.  grid (warps/8, njobs).
__global__ void k_split_tiles(const SplitJob* __restrict__ jobs) {
  const SplitJob jb = jobs[blockIdx.y];
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int g0 = jb.row0 >> 3, g1 = (jb.row0 + jb.nrows + 7) >> 3;
  const int ng = g1 - g0;
  if (wid >= (long long)ng * jb.nkt) return;
  const int g = g0 + (int)(wid % ng), kt = (int)(wid / ng);
  const int rr = lane & 7, kc = lane >> 3;
  const int r = 8 * g + rr;
  if (r < jb.row0 || r >= jb.row0 + jb.nrows) return;
  int er = jb.e[r];
  if (jb.e_biased) er = er == 0 ? -2000 : er - 1022;
  const double* src = jb.src + (long long)(r - jb.row0) * jb.rs;
  uint16_t out[kSlices][8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const long long c = (long long)kt * 32 + kc * 8 + j;
    const double x = c < jb.ncols ? src[c * jb.cs] : 0.0;
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((u >> 52) & 0x7FF);
    unsigned long long X = 0;
    if (E != 0 && er > -2000) {
      const unsigned long long m = (u & ((1ull << 52) - 1)) | (1ull << 52);
      const int sh = 1036 + er - E;  // X = rint(m / 2^sh); sh >= 14 since |x| < 2^er
      if (sh < 64) X = (m + (1ull << (sh - 1))) >> sh;
    }
    const bool neg = (u >> 63) != 0;
    const unsigned long long T = X + 0x80808080ull;
    int dgt[5];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) dgt[jj] = (int)((T >> (8 * jj)) & 255) - 128;
    dgt[4] = (int)(T >> 32);
#pragma unroll
    for (int s = 0; s < kSlices; ++s) {
      const int d = dgt[4 - s];
      out[s][j] = small_int_to_bf16(neg ? -d : d);
    }
  }
  const int rb = r >> 5;
  const long long off_in = (long long)((r & 31) >> 3) * 256 + kc * 64 + rr * 8;
#pragma unroll
  for (int s = 0; s < kSlices; ++s) {
    uint16_t* p = jb.dst + (((long long)kt * kSlices + s) * jb.nrb + rb) * kImage + off_in;
    uint4 v;
    v.x = (uint32_t)out[s][0] | ((uint32_t)out[s][1] << 16);
    v.y = (uint32_t)out[s][2] | ((uint32_t)out[s][3] << 16);
    v.z = (uint32_t)out[s][4] | ((uint32_t)out[s][5] << 16);
    v.w = (uint32_t)out[s][6] | ((uint32_t)out[s][7] << 16);
    *reinterpret_cast<uint4*>(p) = v;
  }
}

// ------------------------------------------------------------ the GEMM
// Pairs (s, t) are issued exact diagonals first (d = 0, 1, 2), then d = 3, 4;
// the accumulator of diagonal d sits at TMEM column d * kTileN.
//
// Variants.  kHDigits: the half transform writes H as digit slices
// (SplitItem::hdig) with one exponent per (AO function, auxiliary group)
// instead of FP64 values.  kSeg: the exchange over such digits; its
// operands are 64-byte swizzled and its k range is cut into segments of
// seg_nkt k-tiles, each with its own row exponents.  An exact chunk never
// crosses a segment boundary, the diagonals 3 and 4 are reset at every
// segment start and folded in at its end, and every chunk and fold is added
// to the int64 result in units of 2^(eA+eB-46) of the rows' maximum
// exponents eA, eB, shifted right by (eA - eA_g) + (eB - eB_g) bits with
// rounding (exact while that shift is at most 16 for a chunk, 0 for a
// fold).  Without kSeg there is one segment per item and no shift.

template <bool kHDigits, bool kSeg>
__global__ void __launch_bounds__(kThreads, 1)
    k_split_gemm(const SplitItem* __restrict__ items, int nitems, int* __restrict__ err,
                 int stop_item, unsigned long long spin_ns) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1 KB aligned operand ring, then barriers
  unsigned char* smem =
      (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = smem;                       // kStages * kBytesA
  unsigned char* sB = smem + kStages * kBytesA;   // kStages * kBytesB
  __shared__ uint64_t full_bar[kStages], empty_bar[kStages];
  __shared__ uint64_t exact_full, exact_empty, final_full, final_empty, mma_drain;
  // kHDigits: the three epilogue warps of a TMEM lane quadrant combine their
  // exponent maxima (double-buffered by item parity)
  __shared__ uint64_t grp_bar[4];
  __shared__ int grp_max[2][4][3];
  __shared__ uint32_t tmem_base_sh;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(&full_bar[i], 1);
      mbar_init(&empty_bar[i], 1);
    }
    mbar_init(&exact_full, 1);
    mbar_init(&exact_empty, kEpiWarps);
    mbar_init(&final_full, 1);
    mbar_init(&final_empty, kEpiWarps);
    mbar_init(&mma_drain, 1);
    for (int i = 0; i < 4; ++i) mbar_init(&grp_bar[i], 3);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;

  if (warp == 0) {
    // ---------------- producer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      // full-barrier parity of the last copies issued into each stage
      uint32_t last_par[kStages];
      bool issued[kStages];
#pragma unroll
      for (int i = 0; i < kStages; ++i) issued[i] = false;
      for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
        // test hook: stop producing at work item stop_item, so the
        // consumers' bounded waits run out (the launch reports a timeout)
        if (it == stop_item) break;
        const SplitItem w = items[it];
        const uint32_t a_run = (uint32_t)(kTileM / 32) * kImage * 2;
        const uint32_t b_run = (uint32_t)(kTileN / 32) * kImage * 2;
        for (int k = 0; k < w.nkt && ok; ++k) {
          ok = mbar_wait(&empty_bar[stage], phase ^ 1, err, 1, spin_ns);
          if (!ok) break;
          mbar_arrive_expect_tx(&full_bar[stage], kSlices * (a_run + b_run));
          const long long kt = w.kt0 + k;
          for (int s = 0; s < kSlices; ++s) {
            const uint16_t* ga = w.a + ((kt * kSlices + s) * w.a_nrb + w.a_rb0) * (long long)kImage;
            const uint16_t* gb = w.b + ((kt * kSlices + s) * w.b_nrb + w.b_rb0) * (long long)kImage;
            bulk_g2s(sA + stage * kBytesA + s * a_run, ga, a_run, &full_bar[stage]);
            bulk_g2s(sB + stage * kBytesB + s * b_run, gb, b_run, &full_bar[stage]);
          }
          last_par[stage] = phase;
          issued[stage] = true;
          if (++stage == kStages) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      // before the CTA can exit, every copy it issued must have landed,
      // also after a timeout: wait on the full barrier of each stage's last
      // copies (bounded by time only; copies always complete)
      for (int i = 0; i < kStages; ++i)
        if (issued[i]) mbar_wait_own(&full_bar[i], last_par[i], spin_ns);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = instr_desc(kTileM, kTileN);
      const uint32_t idesc2 = instr_desc(kTileM, 2 * kTileN);
      int stage = 0;
      uint32_t phase = 0;
      uint32_t ex_phase = 0, fin_phase = 0;
      bool ok = true;
      for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
        const SplitItem w = items[it];
        const int seg = kSeg ? w.seg_nkt : 1;
        int o = kSeg ? w.kt0 % seg : 0;  // kSeg: position of the k-tile in its segment
        for (int k = 0; k < w.nkt && ok; ++k) {
          // without segments the flags come from k alone (a loop-carried
          // segment position made the exchange 6 % slower)
          bool seg_start, chunk_start, seg_end, chunk_end;
          if constexpr (kSeg) {
            seg_start = k == 0 || o == 0;
            chunk_start = seg_start || (o % kChunkTiles) == 0;
            seg_end = k + 1 == w.nkt || o + 1 == seg;
            chunk_end = seg_end || ((o + 1) % kChunkTiles) == 0;
          } else {
            seg_start = k == 0;
            chunk_start = (k % kChunkTiles) == 0;
            seg_end = false;  // final_full is committed after the loop
            chunk_end = ((k + 1) % kChunkTiles) == 0 || k + 1 == w.nkt;
          }
          ok = mbar_wait(&full_bar[stage], phase, err, 5, spin_ns);
          if (!ok) break;
          tc_fence_after();
          const uint32_t a_addr = smem_u32(sA + stage * kBytesA);
          const uint32_t b_addr = smem_u32(sB + stage * kBytesB);
          const uint64_t adesc = kSeg ? smem_desc_sw64(a_addr) : smem_desc(a_addr);
          const uint64_t bdesc = kSeg ? smem_desc_sw64(b_addr) : smem_desc(b_addr);
          // descriptor start addresses advance in 16-byte units
          constexpr uint32_t kSliceA = kTileM * kTileK * 2 / 16, kSliceB = kTileN * kTileK * 2 / 16;
          // the second K = 16 step of the k-tile: two core matrices on
          // (256 B) unswizzled, 32 B into each 64-byte line swizzled
          constexpr uint32_t kStepK = kSeg ? 2 : 16;
          // The 15 slice pairs (s, t), s + t <= 4, as 9 MMAs: B slices t0 and
          // t0+1 are adjacent in shared memory and diagonals d and d+1 have
          // adjacent accumulators, so one N = 192 MMA updates both.  Entries:
          // {s, t0, number of B slices, reset class}; reset class 1 = first
          // write of exact diagonals (reset at a chunk start), 2 = first write
          // of d = 3, 4 (reset at a segment start).  MMAs 0..3 cover exactly
          // the diagonals 0..2, MMAs 4..8 the diagonals 3 and 4.
          auto issue = [&](int q0, int q1) {
#pragma unroll
            for (int q = 0; q < 9; ++q) {
              constexpr unsigned char qs[9] = {0, 0, 1, 2, 0, 1, 2, 3, 4};
              constexpr unsigned char qt[9] = {0, 2, 0, 0, 3, 2, 1, 0, 0};
              constexpr unsigned char qn[9] = {2, 1, 2, 1, 2, 2, 2, 2, 1};
              constexpr unsigned char qr[9] = {1, 1, 0, 0, 2, 0, 0, 0, 0};
              if (q < q0 || q >= q1) continue;
              const uint32_t dcol = tmem + (uint32_t)((qs[q] + qt[q]) * kTileN);
              const uint32_t id = qn[q] == 2 ? idesc2 : idesc;
              const bool reset = qr[q] == 1 ? chunk_start : (qr[q] == 2 ? seg_start : false);
#pragma unroll
              for (int j = 0; j < 2; ++j) {
                const uint64_t ad = adesc + (uint64_t)(qs[q] * kSliceA + j * kStepK);
                const uint64_t bd = bdesc + (uint64_t)(qt[q] * kSliceB + j * kStepK);
                mma_bf16(dcol, ad, bd, id, (reset && j == 0) ? 0u : 1u);
              }
            }
          };
          if (seg_start) {
            // segment (item) start: the exact diagonals are free once the
            // epilogue has drained the previous segment's last chunk, which
            // comes before its fold of d = 3, 4; so the exact pairs go first
            // and overlap that fold, and the d = 3, 4 pairs wait for it
            ok = mbar_wait(&exact_empty, ex_phase ^ 1, err, 4, spin_ns);
            ex_phase ^= 1;
            if (!ok) {
              mma_commit(&empty_bar[stage]);  // the ring drain still completes
              break;
            }
            issue(0, 4);
            if (chunk_end) mma_commit(&exact_full);
            ok = mbar_wait(&final_empty, fin_phase ^ 1, err, 3, spin_ns);
            fin_phase ^= 1;
            if (!ok) {
              mma_commit(&empty_bar[stage]);
              break;
            }
            issue(4, 9);
          } else if (chunk_start) {
            // d = 3, 4 first: they accumulate over the whole segment and the
            // exact drain does not read them, so they overlap the epilogue's
            // drain of the previous chunk; the exact pairs wait for it
            issue(4, 9);
            ok = mbar_wait(&exact_empty, ex_phase ^ 1, err, 4, spin_ns);
            ex_phase ^= 1;
            if (!ok) {
              mma_commit(&empty_bar[stage]);  // the ring drain still completes
              break;
            }
            issue(0, 4);
            if (chunk_end) mma_commit(&exact_full);
          } else {
            issue(0, 4);
            if (chunk_end) mma_commit(&exact_full);
            issue(4, 9);
          }
          mma_commit(&empty_bar[stage]);
          if (seg_end) mma_commit(&final_full);
          if (++stage == kStages) {
            stage = 0;
            phase ^= 1;
          }
          if constexpr (kSeg) {
            if (++o == seg) o = 0;
          }
        }
        if (!kSeg && ok) mma_commit(&final_full);
      }
      // every MMA this thread issued completes before TMEM is freed and the
      // CTA exits, also after a timeout (commit tracks all prior MMAs)
      mma_commit(&mma_drain);
      mbar_wait_own(&mma_drain, 0, spin_ns);
    }
  } else {
    // ---------------- epilogue (warps 2..13)
    const int q = warp & 3;                 // TMEM lane quadrant of this warp
    const int third = (warp - 2) >> 2;      // column third: 0, 1 or 2
    const int row = q * 32 + lane;          // tile-local row
    const uint32_t lane_addr = (uint32_t)(q * 32) << 16;
    uint32_t ex_phase = 0, fin_phase = 0, grp_phase = 0;
    bool ok = true;
    for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
      const SplitItem& w = items[it];  // fields read where used (register pressure)
      // row exponent of this thread's row and the column exponents of the
      // warp's 32 columns (one per lane, broadcast by shuffles at the store),
      // loaded now so that their latency hides behind the drains; a tile's
      // 128 A rows and 96 B rows are always allocated
      const int cbase = third * kEpiCols;
      const int er = w.ea[row];
      const int ecl = w.eb[cbase + lane];
      long long V[kEpiCols];
#pragma unroll
      for (int c = 0; c < kEpiCols; ++c) V[c] = 0;
      // exact diagonals of one chunk into V (kSeg: shifted by sh_a + sh_b)
      auto drain = [&](int sh_a, int sh_b) {
        // d0 is at most 2^22 in magnitude: converted with the 1.5*2^23 magic
        // (one FADD); d1, d2 (below 2^24) with a rounding conversion
#pragma unroll
        for (int g = 0; g < kEpiCols / 16; ++g) {
          uint32_t v0[16], v1[16], v2[16];
          const uint32_t col = (uint32_t)(third * kEpiCols + g * 16);
          tmem_ld16(tmem + lane_addr + col, v0);
          tmem_ld16(tmem + lane_addr + (uint32_t)kTileN + col, v1);
          tmem_ld16(tmem + lane_addr + (uint32_t)(2 * kTileN) + col, v2);
          tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const int r0 = __float_as_int(__uint_as_float(v0[c]) + 12582912.0f) - 0x4B400000;
            const int r1 = __float2int_rn(__uint_as_float(v1[c]));
            const int r2 = __float2int_rn(__uint_as_float(v2[c]));
            const int t01 = (r0 << 8) + r1;  // < 2^31
            const long long wc = ((long long)t01 << 8) + r2;
            if constexpr (kSeg) {
              const int sh = sh_a + __shfl_sync(0xffffffffu, sh_b, g * 16 + c);
              V[g * 16 + c] += sh <= 16 ? (wc << (16 - sh)) : shr_round(wc, sh - 16);
            } else {
              V[g * 16 + c] += wc;
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&exact_empty);
      };
      // fold the approximate diagonals in with 16 fractional bits,
      //   V = W 2^16 + rint(256 r3) + rint(r4),  value = V 2^(eA+eB-46)
      // (kSeg: the segment's part, shifted, added to V)
      auto fold = [&](int sh_a, int sh_b) {
#pragma unroll
        for (int g = 0; g < kEpiCols / 16; ++g) {
          uint32_t v3[16], v4[16];
          tmem_ld16(tmem + lane_addr + (uint32_t)(3 * kTileN + third * kEpiCols + g * 16), v3);
          tmem_ld16(tmem + lane_addr + (uint32_t)(4 * kTileN + third * kEpiCols + g * 16), v4);
          tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            int h3, l3, h4, l4;
            f32_split16(__fmul_rn(__uint_as_float(v3[c]), 256.0f), h3, l3);
            f32_split16(__uint_as_float(v4[c]), h4, l4);
            if constexpr (kSeg) {
              const int sh = sh_a + __shfl_sync(0xffffffffu, sh_b, g * 16 + c);
              const long long f = ((long long)(h3 + h4) << 16) + (long long)(l3 + l4);
              V[g * 16 + c] += shr_round(f, sh);
            } else {
              V[g * 16 + c] =
                  ((V[g * 16 + c] + (long long)(h3 + h4)) << 16) + (long long)(l3 + l4);
            }
          }
        }
        // the accumulators are free for the next segment or item
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&final_empty);
      };
      if constexpr (kSeg) {
        const int nkt = w.nkt, seg = w.seg_nkt;
        int o = w.kt0 % seg;  // position in the segment
        int sh_a = 0, sh_b = 0;  // shifts of this row and of column cbase + lane
        for (int k = 0; k < nkt && ok;) {
          const int len = min(min(kChunkTiles - o % kChunkTiles, seg - o), nkt - k);
          if (k == 0 || o == 0) {
            const int g = (w.kt0 + k) / seg;
            const int ea_g = w.esa[row * w.es_ld + g];
            const int eb_g = w.esb[(cbase + lane) * w.es_ld + g];
            sh_a = (er <= -2000 || ea_g <= -2000) ? 4096 : max(0, er - ea_g);
            sh_b = (ecl <= -2000 || eb_g <= -2000) ? 4096 : max(0, ecl - eb_g);
          }
          ok = mbar_wait(&exact_full, ex_phase, err, 6, spin_ns);
          ex_phase ^= 1;
          if (!ok) break;
          tc_fence_after();
          drain(sh_a, sh_b);
          k += len;
          o += len;
          if (k == nkt || o == seg) {
            ok = mbar_wait(&final_full, fin_phase, err, 7, spin_ns);
            fin_phase ^= 1;
            if (!ok) break;
            tc_fence_after();
            fold(sh_a, sh_b);
            if (o == seg) o = 0;
          }
        }
      } else {
        const int nchunks = (w.nkt + kChunkTiles - 1) / kChunkTiles;
        for (int ch = 0; ch < nchunks && ok; ++ch) {
          ok = mbar_wait(&exact_full, ex_phase, err, 6, spin_ns);
          ex_phase ^= 1;
          if (!ok) break;
          tc_fence_after();
          drain(0, 0);
        }
        if (!ok) break;
        ok = mbar_wait(&final_full, fin_phase, err, 7, spin_ns);
        fin_phase ^= 1;
        if (!ok) break;
        tc_fence_after();
        fold(0, 0);
      }
      if (!ok) break;
      // item fields of the store phase, loaded together so their latencies
      // overlap
      const int m_valid = w.m_valid, n_valid = w.n_valid, ncol1 = w.ncol1, c0 = w.c0;
      const int emax_row0 = w.emax_row0, emax_div = w.emax_div, perm_div = w.perm_div;
      const int apitch = w.apitch, arow0 = w.arow0, ay_valid = w.ay_valid;
      double* const out = w.out;
      double* const out2 = w.out2;
      const long long ldr = w.ldr, perm_rs = w.perm_rs;
      const bool rin = row < m_valid;  // row inside the tile
      // unpadded panel row R of this row, its offset from the row-major
      // output's first row, and whether it is a real row (not padding)
      int R = emax_row0 + row, mloc = 0, yrow = 0;
      long long rofs = row;
      bool rvalid = rin;
      if (apitch) {
        const int Rp = arow0 + row;
        mloc = Rp / apitch;
        yrow = Rp - mloc * apitch;
        rvalid = rin && yrow < ay_valid;
        R = mloc * ay_valid + yrow;
        rofs = (long long)R - arow0;
      }
      const int nstore = min(n_valid, ncol1 - c0);  // columns kept in `out`
      // density column of this row's AO function (tile-local), or -1
      int dcol = -1;
      if (out2) {
        const int cand = ncol1 + R / emax_div - c0;
        if (cand >= 0 && cand < n_valid) dcol = cand;
      }
      if constexpr (kHDigits) {
        // The warp's 32 rows are one auxiliary group g of one AO function
        // (apitch is a multiple of 32 and tiles start at multiples of 128):
        // its exponent is the maximum over these rows and the quadrant's
        // columns, eg = max (bit length of |V| + er + ec - 46), so that
        // |value| < 2^eg for every value of the group.
        int emx = -2000;
#pragma unroll
        for (int c = 0; c < kEpiCols; ++c) {
          const int ec = __shfl_sync(0xffffffffu, ecl, c);
          const int col = cbase + c;
          if (rvalid && col == dcol)
            out2[R] = (er <= -2000 || ec <= -2000) ? 0.0 : i64_scaled_to_f64(V[c], er + ec - 46);
          if (rvalid && col < nstore && V[c] != 0 && er > -2000 && ec > -2000) {
            const unsigned long long a =
                V[c] < 0 ? (unsigned long long)(-V[c]) : (unsigned long long)V[c];
            emx = max(emx, (64 - __clzll((long long)a)) + er + ec - 46);
          }
        }
        emx = __reduce_max_sync(0xffffffffu, emx);
        const int gp = (int)grp_phase;
        if (lane == 0) grp_max[gp][q][third] = emx;
        __syncwarp();
        if (lane == 0) mbar_arrive(&grp_bar[q]);
        ok = mbar_wait(&grp_bar[q], grp_phase, err, 8, spin_ns);
        grp_phase ^= 1;
        if (!ok) break;
        const int eg = max(max(grp_max[gp][q][0], grp_max[gp][q][1]), grp_max[gp][q][2]);
        const int mu = w.hrow0 + mloc;
        const int gy = yrow >> 5;
        if (third == 0 && lane == 0 && rin) {
          w.eseg[(long long)mu * w.es_ld + gy] = eg;
          if (eg > -2000 && w.emax) atomicMax(w.emax + mloc, (unsigned int)max(1, eg + 1022));
        }
        if (rin) {
          // digit slices of X = rint(|value| 2^(39-eg)) (see the number
          // format above) straight from the integer V: value = V 2^(er+ec-46)
          const long long sstride = (long long)w.h_nrb * kImage;
          const long long tstride = (long long)kSlices * sstride;
          uint16_t* const hbase =
              w.hdig + (long long)(mu >> 5) * kImage + sw64_offset(mu & 31, lane);
          const long long kt0 = (long long)gy * w.seg_nkt + c0;
#pragma unroll
          for (int c = 0; c < kEpiCols; ++c) {
            const int ec = __shfl_sync(0xffffffffu, ecl, c);
            const int col = cbase + c;
            if (col >= nstore) continue;  // the same for the whole warp
            const long long v = V[c];
            unsigned long long X = 0;
            if (rvalid && v != 0 && er > -2000 && ec > -2000 && eg > -2000) {
              const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
              const int t = eg - (er + ec - 46) - 39;
              X = t <= 0 ? (a << (-t)) : (t > 63 ? 0ull : (a + (1ull << (t - 1))) >> t);
            }
            const unsigned long long T = X + 0x80808080ull;
            uint16_t* const p = hbase + (kt0 + col) * tstride;
#pragma unroll
            for (int s = 0; s < kSlices; ++s) {
              const int d = s == 0 ? (int)(T >> 32) : (int)((T >> (8 * (4 - s))) & 255) - 128;
              p[s * sstride] = small_int_to_bf16(v < 0 ? -d : d);
            }
          }
        }
      } else {
        unsigned int emax_row = 0;
        {
          const bool perm = perm_rs != 0;
          double* orow;
          if (perm) {
            const int m = R / perm_div, y = R - m * perm_div;
            orow = out + (long long)m * perm_rs + (long long)(y & ~31) * ldr +
                   ((y & 31) * 2 + (cbase >> 1) * 64);
          } else {
            orow = out + rofs * ldr + cbase;
          }
          const bool vec = ((uintptr_t)orow & 15) == 0;
#pragma unroll
          for (int c = 0; c < kEpiCols; c += 2) {
            const int ecs0 = __shfl_sync(0xffffffffu, ecl, c);
            const int ecs1 = __shfl_sync(0xffffffffu, ecl, c + 1);
            const int col = cbase + c;
            const bool s0 = rvalid && col < nstore, s1 = rvalid && col + 1 < nstore;
            const bool d0 = rvalid && col == dcol, d1 = rvalid && col + 1 == dcol;
            if (!(s0 || s1 || d0 || d1)) continue;
            const int ec0 = (s0 || d0) ? ecs0 : -2000;
            const int ec1 = (s1 || d1) ? ecs1 : -2000;
            const double x0 =
                (er <= -2000 || ec0 <= -2000) ? 0.0 : i64_scaled_to_f64(V[c], er + ec0 - 46);
            const double x1 =
                (er <= -2000 || ec1 <= -2000) ? 0.0 : i64_scaled_to_f64(V[c + 1], er + ec1 - 46);
            if (d0) out2[R] = x0;
            if (d1) out2[R] = x1;
            if (s0) emax_row = max(emax_row, (unsigned int)((__double_as_longlong(x0) >> 52) & 0x7FF));
            if (s1) emax_row = max(emax_row, (unsigned int)((__double_as_longlong(x1) >> 52) & 0x7FF));
            if (perm) {
              // the pair's second column is the zero pad column when nstore
              // is odd (the last orbital of an odd count)
              if (s0)
                *reinterpret_cast<double2*>(orow + (c >> 1) * 64) = make_double2(x0, s1 ? x1 : 0.0);
            } else if (vec && s0 && s1) {
              *reinterpret_cast<double2*>(orow + c) = make_double2(x0, x1);
            } else {
              if (s0) orow[c] = x0;
              if (s1) orow[c + 1] = x1;
            }
          }
        }
        if (unsigned int* const emaxp = w.emax) {
          // one atomic per warp when all its rows map to the same target row
          const int target = rvalid ? R / emax_div : -1;
          const int t0 = __shfl_sync(0xffffffffu, target, 0);
          const bool same = __all_sync(0xffffffffu, target == t0);
          if (same) {
            unsigned int m = emax_row;
#pragma unroll
            for (int o2 = 16; o2 > 0; o2 >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o2));
            if (lane == 0 && t0 >= 0 && m) atomicMax(emaxp + t0, m);
          } else if (target >= 0 && emax_row) {
            atomicMax(emaxp + target, emax_row);
          }
        }
      }
    }
  }
  // teardown: everyone joins, then warp 1 frees TMEM once all MMAs are done
  __syncthreads();
  if (warp == 1) {
    // MMAs complete in order; the last commit of this CTA went to final_full
    // or an empty barrier; a fence plus a short bounded wait on the ring's
    // last-used empty barriers is covered by the producer's drain above.
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

}  // namespace gbjk
