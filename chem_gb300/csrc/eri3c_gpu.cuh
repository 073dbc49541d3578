// 3-center Coulomb integrals (X|mu nu) on the device, written straight into
// the atom-block panel layout of the resident tensor.
//
// The host engine (chem_gb300/csrc/ints, standing in for the libcint calls
// of megalochem's ints::aoloader, src/ints/integrals.cpp:250-370) computes
// the same tensor; this kernel follows its McMurchie-Davidson scheme and
// conventions (normalised contractions exported by gbints_basis_shells,
// real spherical harmonics from gbints_sph_coeffs, the primitive cut 1e-16)
// so that the two agree to rounding:
//   for a primitive pair (a_i, b_j): Hermite coefficients E^{ab}_{tuv}
//   (Helgaker, Jorgensen, Olsen eq. 9.5.6-9.5.7), for every auxiliary
//   primitive c_k the Hermite Coulomb integrals R_{tuv}(alpha, P - C)
//   (eq. 9.9.18-9.9.20, Boys function by its series and downward recursion,
//   or erf and upward recursion for large arguments), contracted with the
//   single-centre expansion of c and its spherical transform into
//   W[tuv][mc], then with E^{ab} into the cartesian (a, b) accumulators,
//   and finally transformed to spherical (a, b).
// Work: one block per AO shell pair (a in block I, b in block J, a <= b
// when I == J) of a kept block pair; its 4 warps take the auxiliary shells
// of the kept auxiliary blocks in turn.  Lanes split the Hermite indices of
// the bra (W) and the cartesian pairs (accumulators); the R table of a
// primitive triple lives in the warp's shared memory.  Supported: AO shells
// up to d and auxiliary shells up to f (la + lb + lc <= 7); the host checks.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbjk {

constexpr int kEriMaxLao = 2, kEriMaxLaux = 3;
constexpr int kEriMaxL = 2 * kEriMaxLao + kEriMaxLaux;                           // 7
constexpr int kEriNR = (kEriMaxL + 1) * (kEriMaxL + 2) * (kEriMaxL + 3) / 6;     // 120
constexpr int kEriLb = 2 * kEriMaxLao;                                           // 4
constexpr int kEriNW = (kEriLb + 1) * (kEriLb + 2) * (kEriLb + 3) / 6;           // 35
constexpr int kEriNcab = 36;  // (d cartesians)^2
constexpr int kEriMaxSph = 7;
constexpr int kEriWarps = 4;
// Boys values (-2 alpha)^n F_n(T), n <= L, of up to kEriRnChunk (bra
// primitive pair, auxiliary primitive) combinations, computed across the
// lanes of a warp before the combinations are processed one by one
constexpr int kEriRnChunk = 64;
// ket matrix M[mc][j] of an auxiliary primitive: j over the Hermite
// indices of t + u + v <= l_aux (at most 20), mc over its spherical components
constexpr int kEriNKet = (kEriMaxLaux + 1) * (kEriMaxLaux + 2) * (kEriMaxLaux + 3) / 6;  // 20
constexpr int kEriWarpDoubles = 2 * kEriNR + kEriNW * kEriMaxSph +
                                kEriRnChunk * (kEriMaxL + 1) +
                                kEriMaxSph * kEriNKet;  // R x2, W, rn, M
// cartesian -> spherical tables for l = 0..3, at offsets 0, 1, 10, 40
__constant__ double c_eri_sph[1 + 9 + 30 + 70];
// (t, u, v) of the compact Hermite index e (t + u + v <= 7): t | u << 8 | v << 16
__constant__ int c_eri_tuv[kEriNR];
// 1 / (2 j + 1) for the Boys series and recursion (no FP64 division there)
constexpr int kEriBoysTerms = 400;
__constant__ double c_eri_rodd[kEriMaxL + kEriBoysTerms + 1];

struct EriShell {
  int l, nprim, prim0, bf_off;
  double A[3];
};
struct EriItem {
  int p, a, b;
};

__device__ __forceinline__ int eri_tet(int n) { return n * (n + 1) * (n + 2) / 6; }
// compact index of (t, u, v) among all t + u + v <= L (independent of L)
__device__ __forceinline__ int eri_idx(int t, int u, int v) {
  const int s = t + u + v, r = u + v;
  return eri_tet(s) + r * (r + 1) / 2 + v;
}
__device__ __forceinline__ int eri_sph_off(int l) { return l == 0 ? 0 : l == 1 ? 1 : l == 2 ? 10 : 40; }
__device__ __forceinline__ void eri_cart(int l, int c, int* ex) {
  int idx = 0;
  for (int ix = l; ix >= 0; --ix)
    for (int iy = l - ix; iy >= 0; --iy) {
      if (idx == c) {
        ex[0] = ix;
        ex[1] = iy;
        ex[2] = l - ix - iy;
        return;
      }
      ++idx;
    }
}

// Boys function F_0..F_n at T: the host engine's algorithm (series at
// n = nmax and downward recursion, or erf and upward recursion for large T),
// with the divisions by odd integers taken as products with their
// reciprocals (a rounding-level difference from the host).
__device__ void eri_boys(int nmax, double T, double* F) {
  if (T < 1e-15) {
    for (int m = 0; m <= nmax; ++m) F[m] = c_eri_rodd[m];
    return;
  }
  const double eT = exp(-T);
  if (T > 33.0 + nmax) {
    F[0] = 0.5 * sqrt(3.14159265358979323846 / T) * erf(sqrt(T));
    const double inv2T = 0.5 / T;
    for (int m = 0; m < nmax; ++m) F[m + 1] = ((2 * m + 1) * F[m] - eT) * inv2T;
    return;
  }
  double term = c_eri_rodd[nmax];
  double sum = term;
  const double twoT = 2.0 * T;
  for (int k = 1; k < kEriBoysTerms; ++k) {
    term *= twoT * c_eri_rodd[nmax + k];
    sum += term;
    if (term < 1e-17 * sum) break;
  }
  F[nmax] = eT * sum;
  for (int m = nmax - 1; m >= 0; --m) F[m] = (twoT * F[m + 1] + eT) * c_eri_rodd[m];
}

// Ket matrix of an auxiliary primitive of exponent qq and angular momentum
// lc, computed across the lanes of a warp into M (row stride kEriNKet):
//   M[mc][j] = (-1)^(t+u+v) sum_cc sph[mc][cc] Ec[cx][t] Ec[cy][u] Ec[cz][v],
// (t, u, v) the Hermite index j, (cx, cy, cz) the cartesian exponents of cc,
// Ec the single-centre Hermite expansion.  The contraction with the R table
// is then W[tuv][mc] = pref sum_j M[mc][j] R[(t, u, v) + j].
__device__ void eri_ket_matrix(int lc, double qq, int lane, double* M) {
  double Ec[kEriMaxLaux + 1][kEriMaxLaux + 2];
  for (int i = 0; i <= kEriMaxLaux; ++i)
    for (int t = 0; t <= kEriMaxLaux + 1; ++t) Ec[i][t] = 0.0;
  Ec[0][0] = 1.0;
  const double oo2q = 0.5 / qq;
  for (int i = 0; i < lc; ++i)
    for (int t = 0; t <= i + 1; ++t) {
      double v = (t + 1) * Ec[i][t + 1];
      if (t > 0) v += oo2q * Ec[i][t - 1];
      Ec[i + 1][t] = v;
    }
  const int ncc = (lc + 1) * (lc + 2) / 2, nsc = 2 * lc + 1, nr = eri_tet(lc + 1);
  const double* sc = c_eri_sph + eri_sph_off(lc);
  for (int en = lane; en < nsc * nr; en += 32) {
    const int mc = en / nr, j = en % nr;
    const int tuv = c_eri_tuv[j];
    const int t = tuv & 255, u = (tuv >> 8) & 255, v = tuv >> 16;
    double m = 0.0;
    for (int cc = 0; cc < ncc; ++cc) {
      int ex[3];
      eri_cart(lc, cc, ex);
      if (t > ex[0] || u > ex[1] || v > ex[2]) continue;
      m += sc[mc * ncc + cc] * (Ec[ex[0]][t] * Ec[ex[1]][u] * Ec[ex[2]][v]);
    }
    M[mc * kEriNKet + j] = ((t + u + v) & 1) ? -m : m;
  }
}

// E[axis][i][j][t] of one primitive pair, i <= la, j <= lb, t <= i + j, in
// a flat array with strides ((lb+1)*(la+lb+1), (la+lb+1), 1) per axis.
__device__ void eri_hermite_pair(int la, int lb, double p, const double* PA, const double* PB,
                                 double kab, double* E) {
  const int nt = la + lb + 1, sj = nt, si = (lb + 1) * nt, sax = (la + 1) * si;
  const double oo2p = 0.5 / p;
  for (int d = 0; d < 3; ++d) {
    double* e = E + d * sax;
    for (int i = 0; i < sax; ++i) e[i] = 0.0;
    e[0] = d == 0 ? kab : 1.0;
    for (int i = 0; i < la; ++i)
      for (int t = 0; t <= i + 1; ++t) {
        double v = PA[d] * e[i * si + t] + (t + 1 < nt ? (t + 1) * e[i * si + t + 1] : 0.0);
        if (t > 0) v += oo2p * e[i * si + t - 1];
        e[(i + 1) * si + t] = v;
      }
    for (int i = 0; i <= la; ++i)
      for (int j = 0; j < lb; ++j)
        for (int t = 0; t <= i + j + 1; ++t) {
          double v = PB[d] * e[i * si + j * sj + t] +
                     (t + 1 < nt ? (t + 1) * e[i * si + j * sj + t + 1] : 0.0);
          if (t > 0) v += oo2p * e[i * si + j * sj + t - 1];
          e[i * si + (j + 1) * sj + t] = v;
        }
  }
}

// Compile-time forms of eri_idx's inverse and of the cartesian order.
__host__ __device__ constexpr int eri_tuv_of(int e) {
  int n = 0;
  for (int sum = 0; sum <= kEriMaxL; ++sum)
    for (int r = 0; r <= sum; ++r)
      for (int v = 0; v <= r; ++v) {
        if (n == e) return (sum - r) | ((r - v) << 8) | (v << 16);
        ++n;
      }
  return 0;
}
__host__ __device__ constexpr int eri_cart_of(int l, int c) {
  int idx = 0;
  for (int ix = l; ix >= 0; --ix)
    for (int iy = l - ix; iy >= 0; --iy) {
      if (idx == c) return ix | (iy << 8) | ((l - ix - iy) << 16);
      ++idx;
    }
  return 0;
}
__host__ __device__ constexpr int eri_idx_c(int t, int u, int v) {
  return (t + u + v) * (t + u + v + 1) * (t + u + v + 2) / 6 + (u + v) * (u + v + 1) / 2 + v;
}

// An s-s AO shell pair against one auxiliary shell of angular momentum LC:
// the lanes take the bra primitive pairs (the work of an s-s pair is all in
// its primitives), each with its R table in registers; per auxiliary
// primitive the warp first builds the ket matrix M (shared memory), then
// W[mc] = pref sum_j M[mc][j] R[j].  The partial sums of the spherical
// auxiliary components end in acc of every lane (butterfly sum).  Same
// terms as the general path, summed in another order.
template <int LC>
__device__ void eri_ss_aux(const double* pp, int psz, int npp, const EriShell& c,
                           const double* __restrict__ ax_alpha,
                           const double* __restrict__ ax_coef, int lane, double* M,
                           double* acc) {
  constexpr int NSC = 2 * LC + 1;
  constexpr int NR = (LC + 1) * (LC + 2) * (LC + 3) / 6;
  double part[NSC];
#pragma unroll
  for (int m = 0; m < NSC; ++m) part[m] = 0.0;
  for (int k = 0; k < c.nprim; ++k) {
    const double qq = ax_alpha[c.prim0 + k];
    __syncwarp();  // the previous primitive's M is no longer read
    eri_ket_matrix(LC, qq, lane, M);
    __syncwarp();
    for (int q = lane; q < npp; q += 32) {
      const double* o = pp + q * psz;
      if (o[5] == 0.0) continue;
      const double p = o[0];
      const double alpha = p * qq / (p + qq);
      const double pref = 2.0 * 17.493418327624862 / (p * qq * sqrt(p + qq)) * o[4] *
                          ax_coef[c.prim0 + k];  // 2 pi^{5/2}
      const double X = o[1] - c.A[0], Y = o[2] - c.A[1], Z = o[3] - c.A[2];
      double F[LC + 1];
      eri_boys(LC, alpha * (X * X + Y * Y + Z * Z), F);
      double rn[LC + 1];
      double fac = 1.0;
#pragma unroll
      for (int n = 0; n <= LC; ++n) {
        rn[n] = fac * F[n];
        fac *= -2.0 * alpha;
      }
      // R^n_{tuv} level by level, n = LC .. 0
      double R[NR], Ro[NR];
      R[0] = rn[LC];
#pragma unroll
      for (int n = LC - 1; n >= 0; --n) {
#pragma unroll
        for (int e = 0; e < NR; ++e) Ro[e] = R[e];
#pragma unroll
        for (int e = 0; e < NR; ++e) {
          const int tuv = eri_tuv_of(e);
          const int t = tuv & 255, u = (tuv >> 8) & 255, v = tuv >> 16;
          if (t + u + v > LC - n) continue;
          double val;
          if (t > 0) {
            val = X * Ro[eri_idx_c(t - 1, u, v)];
            if (t > 1) val += (t - 1) * Ro[eri_idx_c(t - 2, u, v)];
          } else if (u > 0) {
            val = Y * Ro[eri_idx_c(t, u - 1, v)];
            if (u > 1) val += (u - 1) * Ro[eri_idx_c(t, u - 2, v)];
          } else if (v > 0) {
            val = Z * Ro[eri_idx_c(t, u, v - 1)];
            if (v > 1) val += (v - 1) * Ro[eri_idx_c(t, u, v - 2)];
          } else {
            val = rn[n];
          }
          R[e] = val;
        }
      }
      const double cf = o[6] * o[7] * o[8] * pref;  // E^{00} of the three axes
#pragma unroll
      for (int mc = 0; mc < NSC; ++mc) {
        double w = 0.0;
#pragma unroll
        for (int jj = 0; jj < NR; ++jj) w += M[mc * kEriNKet + jj] * R[jj];
        part[mc] += cf * w;
      }
    }
  }
#pragma unroll
  for (int mc = 0; mc < NSC; ++mc) {
    double v = part[mc];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    acc[mc] = v;
  }
}

// SS: the launch holds only s-s shell pairs (lanes over primitive pairs),
// else only the other pairs; two kernels with half the code each keep the
// instruction working set of a block small.
template <bool SS>
__global__ void __launch_bounds__(32 * kEriWarps, 4)
    k_eri3c(const EriItem* __restrict__ items, const EriShell* __restrict__ ao,
            const EriShell* __restrict__ ax, const double* __restrict__ ao_alpha,
            const double* __restrict__ ao_coef, const double* __restrict__ ax_alpha,
            const double* __restrict__ ax_coef, const int* __restrict__ pair_I,
            const int* __restrict__ pair_J, const unsigned char* __restrict__ keep, int nablk,
            const int* __restrict__ ablk_shell_off, const int* __restrict__ blk_bf_off,
            const long long* __restrict__ panel_off, const int* __restrict__ panel_K,
            const int* __restrict__ col_IJ, const int* __restrict__ col_JI, int naux,
            double* __restrict__ B) {
  extern __shared__ double sm[];
  const EriItem it = items[blockIdx.x];
  const EriShell a = ao[it.a], b = ao[it.b];
  const int la = a.l, lb = b.l, Lb = la + lb;
  const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
  const int nsa = 2 * la + 1, nsb = 2 * lb + 1;
  const int npp = a.nprim * b.nprim;
  const int esz = 3 * (la + 1) * (lb + 1) * (Lb + 1);  // E doubles per primitive pair
  const int psz = 6 + esz;                              // p, P[3], coef, keep flag, E
  const int nW = eri_tet(Lb + 1);                       // bra Hermite indices
  double* pp = sm;                                      // npp * psz
  double* wbase = sm + npp * psz + (threadIdx.x >> 5) * kEriWarpDoubles;
  double* R0 = wbase;
  double* R1 = wbase + kEriNR;
  double* W = wbase + 2 * kEriNR;
  double* rnq = W + kEriNW * kEriMaxSph;  // kEriRnChunk x (kEriMaxL + 1)
  double* Mk = rnq + kEriRnChunk * (kEriMaxL + 1);  // kEriMaxSph x kEriNKet
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  // bra primitive pairs
  double ab2 = 0.0;
  for (int d = 0; d < 3; ++d) ab2 += (a.A[d] - b.A[d]) * (a.A[d] - b.A[d]);
  for (int q = threadIdx.x; q < npp; q += blockDim.x) {
    const int ia = q / b.nprim, ib = q % b.nprim;
    const double al = ao_alpha[a.prim0 + ia], be = ao_alpha[b.prim0 + ib];
    const double p = al + be;
    double P[3], PA[3], PB[3];
    for (int d = 0; d < 3; ++d) {
      P[d] = (al * a.A[d] + be * b.A[d]) / p;
      PA[d] = P[d] - a.A[d];
      PB[d] = P[d] - b.A[d];
    }
    const double kab = exp(-al * be / p * ab2);
    const double coef = ao_coef[a.prim0 + ia] * ao_coef[b.prim0 + ib];
    double* o = pp + q * psz;
    o[0] = p;
    o[1] = P[0];
    o[2] = P[1];
    o[3] = P[2];
    o[4] = coef;
    o[5] = fabs(coef * kab) < 1e-16 ? 0.0 : 1.0;
    eri_hermite_pair(la, lb, p, PA, PB, kab, o + 6);
  }
  __syncthreads();

  const int I = pair_I[it.p], J = pair_J[it.p];
  const int Eax = (la + 1) * (lb + 1) * (Lb + 1), Esi = (lb + 1) * (Lb + 1), Esj = Lb + 1;
  // shells of the kept auxiliary blocks, in turn over the warps
  int counter = 0;
  for (int A = 0; A < nablk; ++A) {
    if (!keep[(long long)it.p * nablk + A]) continue;
    for (int s = ablk_shell_off[A]; s < ablk_shell_off[A + 1]; ++s, ++counter) {
      if (counter % kEriWarps != warp) continue;
      const EriShell c = ax[s];
      const int lc = c.l, nsc = 2 * lc + 1;
      const int L = Lb + lc;
      double acc0[kEriMaxSph], acc1[kEriMaxSph];  // cartesian pairs lane, lane + 32
      for (int m = 0; m < kEriMaxSph; ++m) acc0[m] = acc1[m] = 0.0;
      const int nck = c.nprim;
      const int qch = kEriRnChunk / nck > 0 ? kEriRnChunk / nck : 1;
      if constexpr (SS) {
        // s-s pair: lanes over the bra primitive pairs; every lane ends
        // with the sums, lane 0 stores them as the one cartesian pair
        if (lc == 0)
          eri_ss_aux<0>(pp, psz, npp, c, ax_alpha, ax_coef, lane, Mk, acc0);
        else if (lc == 1)
          eri_ss_aux<1>(pp, psz, npp, c, ax_alpha, ax_coef, lane, Mk, acc0);
        else if (lc == 2)
          eri_ss_aux<2>(pp, psz, npp, c, ax_alpha, ax_coef, lane, Mk, acc0);
        else
          eri_ss_aux<3>(pp, psz, npp, c, ax_alpha, ax_coef, lane, Mk, acc0);
      } else if (nck == 1) {
        // one auxiliary primitive: its ket matrix serves every bra pair
        eri_ket_matrix(lc, ax_alpha[c.prim0], lane, Mk);
        __syncwarp();
      }
      for (int q0 = 0; q0 < (SS ? 0 : npp); q0 += qch) {
      const int q1 = min(npp, q0 + qch);
      // Boys functions of the chunk's (q, k) combinations, one per lane
      for (int jq = lane; jq < (q1 - q0) * nck; jq += 32) {
        const int q = q0 + jq / nck, k = jq % nck;
        const double* o = pp + q * psz;
        if (o[5] == 0.0) continue;
        const double p = o[0], qq = ax_alpha[c.prim0 + k];
        const double alpha = p * qq / (p + qq);
        const double X = o[1] - c.A[0], Y = o[2] - c.A[1], Z = o[3] - c.A[2];
        double F[kEriMaxL + 1];
        eri_boys(L, alpha * (X * X + Y * Y + Z * Z), F);
        double fac = 1.0;
        double* r = rnq + jq * (kEriMaxL + 1);
        for (int n = 0; n <= L; ++n) {
          r[n] = fac * F[n];
          fac *= -2.0 * alpha;
        }
      }
      __syncwarp();
      for (int q = q0; q < q1; ++q) {
        const double* o = pp + q * psz;
        if (o[5] == 0.0) continue;
        const double p = o[0];
        double w0[kEriMaxSph], w1[kEriMaxSph];  // W for bra indices lane, lane + 32
        for (int m = 0; m < kEriMaxSph; ++m) w0[m] = w1[m] = 0.0;
        for (int k = 0; k < c.nprim; ++k) {
          const double qq = ax_alpha[c.prim0 + k];
          const double pref = 2.0 * 17.493418327624862 / (p * qq * sqrt(p + qq)) * o[4] *
                              ax_coef[c.prim0 + k];  // 2 pi^{5/2}
          const double X = o[1] - c.A[0], Y = o[2] - c.A[1], Z = o[3] - c.A[2];
          const double* rn = rnq + ((q - q0) * nck + k) * (kEriMaxL + 1);
          // R^n_{tuv}, levels n = L .. 0; level 0 ends in Rc
          double* cur = (L & 1) ? R1 : R0;
          double* old = (L & 1) ? R0 : R1;
          if (lane == 0) cur[0] = rn[L];
          __syncwarp();
          for (int n = L - 1; n >= 0; --n) {
            double* t_ = cur;
            cur = old;
            old = t_;
            const int lt = L - n, cnt = eri_tet(lt + 1);
            for (int e = lane; e < cnt; e += 32) {
              const int tuv = c_eri_tuv[e];
              const int t = tuv & 255, u = (tuv >> 8) & 255, v = tuv >> 16;
              double val;
              if (t > 0) {
                val = X * old[eri_idx(t - 1, u, v)];
                if (t > 1) val += (t - 1) * old[eri_idx(t - 2, u, v)];
              } else if (u > 0) {
                val = Y * old[eri_idx(t, u - 1, v)];
                if (u > 1) val += (u - 1) * old[eri_idx(t, u - 2, v)];
              } else if (v > 0) {
                val = Z * old[eri_idx(t, u, v - 1)];
                if (v > 1) val += (v - 1) * old[eri_idx(t, u, v - 2)];
              } else {
                val = rn[n];
              }
              cur[e] = val;
            }
            __syncwarp();
          }
          const double* Rc = cur;
          // W[tuv][mc] += pref sum_j M[mc][j] R[(t, u, v) + j]
          if (nck > 1) {
            eri_ket_matrix(lc, qq, lane, Mk);
            __syncwarp();
          }
          const int nr = eri_tet(lc + 1);
          for (int h = 0; h < 2; ++h) {
            const int e = lane + 32 * h;
            if (e >= nW) break;
            const int tuv = c_eri_tuv[e];
            const int t = tuv & 255, u = (tuv >> 8) & 255, v = tuv >> 16;
            double* w = h ? w1 : w0;
            for (int jj = 0; jj < nr; ++jj) {
              const int kt = c_eri_tuv[jj];
              const double r =
                  pref * Rc[eri_idx(t + (kt & 255), u + ((kt >> 8) & 255), v + (kt >> 16))];
              for (int mc = 0; mc < nsc; ++mc) w[mc] += Mk[mc * kEriNKet + jj] * r;
            }
          }
          __syncwarp();  // R buffers are rewritten by the next primitive
        }
        // publish W of this primitive pair, then acc[cab] += sum_bra E W
        for (int h = 0; h < 2; ++h) {
          const int e = lane + 32 * h;
          if (e < nW)
            for (int mc = 0; mc < nsc; ++mc) W[e * kEriMaxSph + mc] = h ? w1[mc] : w0[mc];
        }
        __syncwarp();
        const double* E = o + 6;
        for (int h = 0; h < 2; ++h) {
          const int cab = lane + 32 * h;
          if (cab >= nca * ncb) break;
          int ea[3], eb[3];
          eri_cart(la, cab / ncb, ea);
          eri_cart(lb, cab % ncb, eb);
          for (int t = 0; t <= ea[0] + eb[0]; ++t) {
            const double ex = E[0 * Eax + ea[0] * Esi + eb[0] * Esj + t];
            if (ex == 0.0) continue;
            for (int u = 0; u <= ea[1] + eb[1]; ++u) {
              const double ey = E[1 * Eax + ea[1] * Esi + eb[1] * Esj + u];
              if (ey == 0.0) continue;
              for (int v = 0; v <= ea[2] + eb[2]; ++v) {
                const double ez = E[2 * Eax + ea[2] * Esi + eb[2] * Esj + v];
                if (ez == 0.0) continue;
                const double cf = ex * ey * ez;
                const double* w = W + eri_idx(t, u, v) * kEriMaxSph;
                double* ac = h ? acc1 : acc0;
                for (int mc = 0; mc < nsc; ++mc) ac[mc] += cf * w[mc];
              }
            }
          }
        }
        __syncwarp();
      }
      __syncwarp();  // the next chunk rewrites the Boys values
      }
      // spherical (a, b): stage the cartesian accumulators in the warp's
      // R/W space, then each lane writes outputs (ma, mb, mc)
      double* st = wbase;
      for (int h = 0; h < 2; ++h) {
        const int cab = lane + 32 * h;
        if (cab < nca * ncb)
          for (int mc = 0; mc < nsc; ++mc) st[cab * kEriMaxSph + mc] = h ? acc1[mc] : acc0[mc];
      }
      __syncwarp();
      const double* sa = c_eri_sph + eri_sph_off(la);
      const double* sb = c_eri_sph + eri_sph_off(lb);
      const int I0 = blk_bf_off[I], J0 = blk_bf_off[J];
      const int KI = panel_K[I], KJ = panel_K[J];
      double* PI = B + panel_off[I];
      double* PJ = B + panel_off[J];
      for (int o = lane; o < nsa * nsb * nsc; o += 32) {
        const int ma = o / (nsb * nsc), mb = (o / nsc) % nsb, mc = o % nsc;
        double v = 0.0;
        for (int ca = 0; ca < nca; ++ca) {
          const double fa = sa[ma * nca + ca];
          if (fa == 0.0) continue;
          double s2 = 0.0;
          for (int cb = 0; cb < ncb; ++cb)
            s2 += sb[mb * ncb + cb] * st[(ca * ncb + cb) * kEriMaxSph + mc];
          v += fa * s2;
        }
        const int mu = a.bf_off + ma - I0, nu = b.bf_off + mb - J0;
        const long long X = c.bf_off + mc;
        PI[((long long)mu * naux + X) * KI + col_IJ[it.p] + nu] = v;
        if (I != J)
          PJ[((long long)nu * naux + X) * KJ + col_JI[it.p] + mu] = v;
        else if (it.a != it.b)
          PI[((long long)nu * naux + X) * KI + col_IJ[it.p] + mu] = v;
      }
      __syncwarp();
    }
  }
}

}  // namespace gbjk
