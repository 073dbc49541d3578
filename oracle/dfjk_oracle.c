/* CPU oracle of the DF Fock-build hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C FP64 restatement of megalochem's density-fitted J/K builders on
 * the same atom-block panel layout the device engine uses.  It is the checker
 * for the CUDA path (tests, smoke check) and the timed CPU baseline of
 * bench.py; nothing in the product path calls it.
 *
 * Parity status: megalochem's own implementation cannot be built here (it
 * needs DBCSR, libcint, MPI, ScaLAPACK, HDF5), and megalochem ships no tests,
 * golden outputs or benchmark numbers, so this restatement is "parity
 * unpinned" against the reference.  It is checked against an independent
 * dense numpy einsum of the same formulas and against physics identities.
 *
 * Functions and the reference code they restate:
 *   oracle_df_j      fock::DF_J::compute_J      src/fock/jkdf.cpp:69-190
 *   oracle_df_j_chol the same J with the metric applied as L^-T L^-1
 *   oracle_dfmo_k    fock::DFMO_K::compute_K    src/fock/jkdf.cpp:221-462
 *   oracle_dflmo_k   fock::DFLMO_K::compute_K   src/fock/jkdf.cpp:897-1091
 *                    (symmetric branch)
 *   oracle_dfao_k    fock::DFAO_K::compute_K    src/fock/jkdf.cpp:510-648
 *   oracle_dflmo_k_asym  fock::DFLMO_K::compute_K, set_sym(false),
 *                    src/fock/jkdf.cpp:1093-1323
 *   oracle_prefit, oracle_mp2_ll_point  the SOS-AO-MP2 Laplace term
 *                    (src/mp/z_full.cpp:427-620, src/mp/mp_compute.cpp:232-382)
 *   oracle_filter    dbcsr::tensor::filter / contract .filter(eps) applied to
 *                    the result matrix (src/dbcsrx/dbcsr_tensor.hpp:678-688)
 *
 * Panel layout (see chem_gb300/layout.py): panel I is [b_I][naux][K_I] at
 * B + panel_off[I]; colmap[colmap_off[I] + k] is the AO index of column k.
 * Summation order.  DBCSR leaves the order of its sums unspecified, and the
 * metric inverse (condition number ~1e6 for cc-pVDZ-jkfit) amplifies any
 * rounding difference in g_X to ~1e-11 in J.  This file therefore fixes one
 * order for every sum, which the CUDA kernels reproduce operation for
 * operation (fused multiply-adds via fma(), 32-lane strided partial sums
 * combined by an xor butterfly, split-K partials summed in order), so the
 * FP64 device path is compared bit for bit.  Compile with
 * -ffp-contract=off so that no other product is fused.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int nbf, naux, nblk;
  const int* blk_off;        /* nblk+1 AO offsets of the atom blocks */
  const int* panel_K;        /* nblk */
  const long long* panel_off;/* nblk */
  const int* colmap_off;     /* nblk+1 */
  const int* colmap;         /* AO index of every panel column */
} oracle_layout;

/* sum_k a[k] b[k] as a 32-lane warp computes it: lane l accumulates
 * k = l, l+32, ... with fma, then for o = 16, 8, 4, 2, 1 every lane adds the
 * value of lane l^o; lane 0's value is returned. */
static double warp_dot(const double* a, const double* b, int n, long long stride_b) {
  double v[32], t[32];
  for (int l = 0; l < 32; ++l) {
    double s = 0.0;
    for (int k = l; k < n; k += 32) s = fma(a[k], b[(long long)k * stride_b], s);
    v[l] = s;
  }
  for (int o = 16; o > 0; o >>= 1) {
    for (int l = 0; l < 32; ++l) t[l] = v[l] + v[l ^ o];
    for (int l = 0; l < 32; ++l) v[l] = t[l];
  }
  return v[0];
}

static int blk_of(const oracle_layout* L, int mu) {
  int lo = 0, hi = L->nblk - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) / 2;
    if (L->blk_off[mid] <= mu) lo = mid; else hi = mid - 1;
  }
  return lo;
}

/* Zero every atom block (I, J) of the nbf x nbf matrix M whose Frobenius
 * norm is below eps (DBCSR result-block filtering). */
void oracle_filter(const oracle_layout* L, double* M, double eps) {
  if (eps <= 0) return;
  const int n = L->nbf;
#pragma omp parallel for schedule(dynamic, 1)
  for (int I = 0; I < L->nblk; ++I)
    for (int J = 0; J < L->nblk; ++J) {
      double s = 0;
      for (int m = L->blk_off[I]; m < L->blk_off[I + 1]; ++m)
        for (int v = L->blk_off[J]; v < L->blk_off[J + 1]; ++v) s += M[(size_t)m * n + v] * M[(size_t)m * n + v];
      if (sqrt(s) < eps)
        for (int m = L->blk_off[I]; m < L->blk_off[I + 1]; ++m)
          for (int v = L->blk_off[J]; v < L->blk_off[J + 1]; ++v) M[(size_t)m * n + v] = 0.0;
    }
}

/* g_X = sum_{mu nu} (X|mu nu) P_{mu nu}  (jkdf.cpp:111-128).
 * Order: per (mu, X) a warp dot over the panel columns k against
 * P[mu][colmap[k]], then g_X = sum over mu in increasing order. */
void oracle_contract_g(const oracle_layout* L, const double* B, const double* P, double* g) {
  const int naux = L->naux, n = L->nbf;
#pragma omp parallel for schedule(static)
  for (int X = 0; X < naux; ++X) {
    double acc = 0.0;
    for (int I = 0; I < L->nblk; ++I) {
      const int KI = L->panel_K[I];
      const int* cm = L->colmap + L->colmap_off[I];
      double* pg = (double*)malloc(sizeof(double) * (KI > 0 ? KI : 1));
      for (int m = 0; m < L->blk_off[I + 1] - L->blk_off[I]; ++m) {
        const double* row = B + L->panel_off[I] + ((size_t)m * naux + X) * KI;
        const double* prow = P + (size_t)(L->blk_off[I] + m) * n;
        for (int k = 0; k < KI; ++k) pg[k] = prow[cm[k]];
        acc += warp_dot(row, pg, KI, 1);
      }
      free(pg);
    }
    g[X] = acc;
  }
}

/* J_{mu nu} = sum_X (X|mu nu) h_X  (jkdf.cpp:153-170).
 * Order: four running fma sums over X = 4q+r (r = 0..3, the tail X >= 4*floor
 * (naux/4) going to r = 0), combined as (s0 + s1) + (s2 + s3). */
void oracle_contract_j(const oracle_layout* L, const double* B, const double* h, double* J) {
  const int naux = L->naux, n = L->nbf;
  memset(J, 0, sizeof(double) * (size_t)n * n);
#pragma omp parallel for schedule(dynamic, 1)
  for (int mu = 0; mu < n; ++mu) {
    const int I = blk_of(L, mu);
    const int m = mu - L->blk_off[I];
    const int KI = L->panel_K[I];
    const int* cm = L->colmap + L->colmap_off[I];
    for (int k = 0; k < KI; ++k) {
      const double* b = B + L->panel_off[I] + (size_t)m * naux * KI + k;
      double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
      int X = 0;
      for (; X + 3 < naux; X += 4) {
        s0 = fma(b[(size_t)X * KI], h[X], s0);
        s1 = fma(b[(size_t)(X + 1) * KI], h[X + 1], s1);
        s2 = fma(b[(size_t)(X + 2) * KI], h[X + 2], s2);
        s3 = fma(b[(size_t)(X + 3) * KI], h[X + 3], s3);
      }
      for (; X < naux; ++X) s0 = fma(b[(size_t)X * KI], h[X], s0);
      J[(size_t)mu * n + cm[k]] = (s0 + s1) + (s2 + s3);
    }
  }
}

/* DF-J: P_tot = 2 P_alpha (RHF) or P_alpha + P_beta is the caller's input. */
void oracle_df_j(const oracle_layout* L, const double* B, const double* Vinv,
                 const double* Ptot, double* J, double eps) {
  const int naux = L->naux;
  double* g = (double*)malloc(sizeof(double) * naux);
  double* h = (double*)malloc(sizeof(double) * naux);
  oracle_contract_g(L, B, Ptot, g);
  /* h = V^-1 g  (jkdf.cpp:137-141, "X_, XY -> Y_"); row Y of V^-1 dotted
   * with g as a warp does it */
#pragma omp parallel for schedule(static)
  for (int Y = 0; Y < naux; ++Y) h[Y] = warp_dot(Vinv + (size_t)Y * naux, g, naux, 1);
  oracle_contract_j(L, B, h, J);
  oracle_filter(L, J, eps);
  free(g);
  free(h);
}

/* DF-J through the Cholesky factor: h = L^-T (L^-1 g), with y = L^-1 g as
 * warp dots over the rows of L^-1 and h[X] = sum_{Y >= X} L^-1[Y][X] y[Y]
 * in increasing Y.  Same value as oracle_df_j in exact arithmetic; avoids
 * the conditioning error of the explicit V^-1. */
void oracle_df_j_chol(const oracle_layout* L, const double* B, const double* Linv,
                      const double* Ptot, double* J, double eps) {
  const int naux = L->naux;
  double* g = (double*)malloc(sizeof(double) * naux);
  double* y = (double*)malloc(sizeof(double) * naux);
  double* h = (double*)malloc(sizeof(double) * naux);
  oracle_contract_g(L, B, Ptot, g);
#pragma omp parallel for schedule(static)
  for (int Y = 0; Y < naux; ++Y) y[Y] = warp_dot(Linv + (size_t)Y * naux, g, naux, 1);
#pragma omp parallel for schedule(static)
  for (int X = 0; X < naux; ++X) {
    double s = 0.0;
    for (int Y = X; Y < naux; ++Y) s = fma(Linv[(size_t)Y * naux + X], y[Y], s);
    h[X] = s;
  }
  oracle_contract_j(L, B, h, J);
  oracle_filter(L, J, eps);
  free(g);
  free(y);
  free(h);
}

/* H[mu][X][i] = sum_lambda (X|mu lambda) C[lambda][i]  ("XMN, Mi -> XiN") */
void oracle_half_transform(const oracle_layout* L, const double* B, const double* Cm, int nocc,
                           double* H) {
  const int naux = L->naux;
  for (int I = 0; I < L->nblk; ++I) {
    const int KI = L->panel_K[I];
    const int bI = L->blk_off[I + 1] - L->blk_off[I];
    const int* cm = L->colmap + L->colmap_off[I];
    double* Cg = (double*)malloc(sizeof(double) * (size_t)KI * nocc);
    for (int k = 0; k < KI; ++k) memcpy(Cg + (size_t)k * nocc, Cm + (size_t)cm[k] * nocc, sizeof(double) * nocc);
    const long rows = (long)bI * naux;
    const double* P = B + L->panel_off[I];
    double* Hout = H + (size_t)L->blk_off[I] * naux * nocc;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < rows; ++r) {
      double* hr = Hout + (size_t)r * nocc;
      for (int i = 0; i < nocc; ++i) hr[i] = 0.0;
      const double* br = P + (size_t)r * KI;
      for (int k = 0; k < KI; ++k) {
        const double b = br[k];
        const double* c = Cg + (size_t)k * nocc;
        for (int i = 0; i < nocc; ++i) hr[i] = fma(b, c[i], hr[i]);
      }
    }
    free(Cg);
  }
}

/* out[mu][Y][i] = sum_X M[Y][X] H[mu][X][i]; lower != 0 uses X <= Y only. */
static void apply_metric(const oracle_layout* L, const double* M, int lower, const double* H,
                         int nocc, double* out) {
  const int naux = L->naux, n = L->nbf;
#pragma omp parallel for schedule(static)
  for (long r = 0; r < (long)n * naux; ++r) {
    const int mu = (int)(r / naux), Y = (int)(r % naux);
    double* o = out + ((size_t)mu * naux + Y) * nocc;
    for (int i = 0; i < nocc; ++i) o[i] = 0.0;
    const int xmax = lower ? Y + 1 : naux;
    for (int X = 0; X < xmax; ++X) {
      const double m = M[(size_t)Y * naux + X];
      const double* h = H + ((size_t)mu * naux + X) * nocc;
      for (int i = 0; i < nocc; ++i) o[i] = fma(m, h[i], o[i]);
    }
  }
}

/* K[mu][nu] = -sum_{X,i} A[mu][X][i] Bm[nu][X][i].  Order: the reduction
 * index t = X*nocc + i is cut into chunks of kchunk; each chunk is an
 * in-order fma sum, the chunk sums are added in order to 0.0, and the total
 * is negated (kchunk <= 0: one chunk). */
static void contract_k(const oracle_layout* L, const double* A, const double* Bm, int nocc,
                       double* K, int symmetric, long long kchunk) {
  const int n = L->nbf;
  const long long len = (long long)L->naux * nocc;
  if (kchunk <= 0) kchunk = len;
#pragma omp parallel for schedule(dynamic, 1)
  for (int mu = 0; mu < n; ++mu)
    for (int nu = symmetric ? mu : 0; nu < n; ++nu) {
      const double* a = A + (size_t)mu * len;
      const double* b = Bm + (size_t)nu * len;
      double s = 0.0;
      for (long long t0 = 0; t0 < len; t0 += kchunk) {
        const long long t1 = t0 + kchunk < len ? t0 + kchunk : len;
        double p = 0.0;
        for (long long t = t0; t < t1; ++t) p = fma(a[t], b[t], p);
        s += p;
      }
      s = -s;
      K[(size_t)mu * n + nu] = s;
      if (symmetric) K[(size_t)nu * n + mu] = s;
    }
}

/* DF-MO K: HT1 = B C, HT2 = L^-1 HT1, K = -HT2^T HT2  (jkdf.cpp:348-438).
 * Linv is the lower-triangular inverse Cholesky factor of the metric, or
 * NULL for a pre-fitted tensor (HT2 = HT1). */
int oracle_dfmo_k(const oracle_layout* L, const double* B, const double* Linv, const double* Cm,
                  int nocc, double* K, double eps, long long kchunk) {
  const size_t sz = (size_t)L->nbf * L->naux * nocc;
  double* H = (double*)malloc(sizeof(double) * sz);
  double* H2 = (double*)malloc(sizeof(double) * sz);
  if (!H || !H2) { free(H); free(H2); return 2; }
  oracle_half_transform(L, B, Cm, nocc, H);
  if (Linv)
    apply_metric(L, Linv, 1, H, nocc, H2);
  else  /* pre-fitted tensor: no metric */
    memcpy(H2, H, sizeof(double) * sz);
  contract_k(L, H2, H2, nocc, K, 1, kchunk);
  oracle_filter(L, K, eps);
  free(H);
  free(H2);
  return 0;
}

/* DF-MO K of a pre-fitted tensor with the auxiliary index in batches of xb
 * rows (the last batch shorter), as the device's batched FP64 path sums it:
 * batch b covers t in [X0*nocc, (X0+xbc)*nocc); within it the chunks of
 * kc_full (kc_last for a shorter last batch) are in-order fma sums added in
 * order to 0.0; the batch total is negated and added to K (K = -S_0 for the
 * first batch, then K = -S_b + K). */
int oracle_dfmo_k_batched(const oracle_layout* L, const double* B, const double* Cm, int nocc,
                          double* K, double eps, int xb, long long kc_full, long long kc_last) {
  const int n = L->nbf, naux = L->naux;
  const long long len = (long long)naux * nocc;
  if (xb <= 0 || kc_full <= 0 || kc_last <= 0) return 1;
  double* H = (double*)malloc(sizeof(double) * (size_t)n * len);
  if (!H) return 2;
  oracle_half_transform(L, B, Cm, nocc, H);
#pragma omp parallel for schedule(dynamic, 1)
  for (int mu = 0; mu < n; ++mu)
    for (int nu = mu; nu < n; ++nu) {
      const double* a = H + (size_t)mu * len;
      const double* b = H + (size_t)nu * len;
      double k = 0.0;
      for (int X0 = 0; X0 < naux; X0 += xb) {
        const int xbc = X0 + xb < naux ? xb : naux - X0;
        const long long kc = xbc == xb ? kc_full : kc_last;
        const long long u0 = (long long)X0 * nocc, u1 = (long long)(X0 + xbc) * nocc;
        double s = 0.0;
        for (long long t0 = u0; t0 < u1; t0 += kc) {
          const long long t1 = t0 + kc < u1 ? t0 + kc : u1;
          double p = 0.0;
          for (long long t = t0; t < t1; ++t) p = fma(a[t], b[t], p);
          s += p;
        }
        k = X0 == 0 ? -s : -s + k;
      }
      K[(size_t)mu * n + nu] = k;
      K[(size_t)nu * n + mu] = k;
    }
  oracle_filter(L, K, eps);
  free(H);
  return 0;
}

/* DF-MO (lmo = 0: HT2 = L^-1 HT, K = -HT2^T HT2) or DF-LMO (lmo = 1:
 * HTfit = V^-1 HT, K_mn = -sum HTfit_m HT_n) K with the occupied orbitals in
 * batches of ob (the last shorter), as the device's occupied-batched FP64
 * path sums it: batch b covers orbitals [i0, i0 + obc); its reduction
 * index t' = X*obc + (i - i0) runs in chunks of kc_full (kc_last for a
 * shorter last batch), each an in-order fma sum, the chunk sums added in
 * order to 0.0; the batch total is negated and added to K (K = -S_0, then
 * K = -S_b + K).  M is L^-1 (lmo = 0, lower) or V^-1 (lmo = 1). */
int oracle_dfk_occ_batched(const oracle_layout* L, const double* B, const double* M, int lmo,
                           const double* Cm, int nocc, double* K, double eps, int ob,
                           long long kc_full, long long kc_last) {
  const int n = L->nbf, naux = L->naux;
  if (ob <= 0 || kc_full <= 0 || kc_last <= 0) return 1;
  const size_t sz = (size_t)n * naux * nocc;
  double* H = (double*)malloc(sizeof(double) * sz);
  double* H2 = (double*)malloc(sizeof(double) * sz);
  if (!H || !H2) { free(H); free(H2); return 2; }
  oracle_half_transform(L, B, Cm, nocc, H);
  apply_metric(L, M, lmo ? 0 : 1, H, nocc, H2);
  const double* A = H2;                /* rows mu */
  const double* Bm = lmo ? H : H2;     /* rows nu */
#pragma omp parallel for schedule(dynamic, 1)
  for (int mu = 0; mu < n; ++mu)
    for (int nu = lmo ? 0 : mu; nu < n; ++nu) {
      const double* a = A + (size_t)mu * naux * nocc;
      const double* b = Bm + (size_t)nu * naux * nocc;
      double k = 0.0;
      for (int i0 = 0; i0 < nocc; i0 += ob) {
        const int obc = i0 + ob < nocc ? ob : nocc - i0;
        const long long kc = obc == ob ? kc_full : kc_last;
        const long long len = (long long)naux * obc;
        double s = 0.0;
        for (long long t0 = 0; t0 < len; t0 += kc) {
          const long long t1 = t0 + kc < len ? t0 + kc : len;
          double p = 0.0;
          for (long long t = t0; t < t1; ++t) {
            const long long X = t / obc, i = i0 + t % obc;
            p = fma(a[X * nocc + i], b[X * nocc + i], p);
          }
          s += p;
        }
        k = i0 == 0 ? -s : -s + k;
      }
      K[(size_t)mu * n + nu] = k;
      if (!lmo) K[(size_t)nu * n + mu] = k;
    }
  oracle_filter(L, K, eps);
  free(H);
  free(H2);
  return 0;
}

/* DF-LMO K (symmetric): HT = B C, HTfit = V^-1 HT, K_nm = -sum HT_m HTfit_n
 * (jkdf.cpp:1026-1088). */
int oracle_dflmo_k(const oracle_layout* L, const double* B, const double* Vinv, const double* Cm,
                   int nocc, double* K, double eps, long long kchunk) {
  const size_t sz = (size_t)L->nbf * L->naux * nocc;
  double* H = (double*)malloc(sizeof(double) * sz);
  double* Hf = (double*)malloc(sizeof(double) * sz);
  if (!H || !Hf) { free(H); free(Hf); return 2; }
  oracle_half_transform(L, B, Cm, nocc, H);
  apply_metric(L, Vinv, 0, H, nocc, Hf);
  /* K_nm = -sum_{X,i} HTfit[n][X][i] HT[m][X][i] */
  contract_k(L, Hf, H, nocc, K, 0, kchunk);
  oracle_filter(L, K, eps);
  free(H);
  free(Hf);
  return 0;
}

/* DF-LMO K, non-symmetric branch (jkdf.cpp:1093-1323): HTu = B U,
 * HTv = B V (V = Vt^T, nbf x nocc), HTvfit = V^-1 HTv,
 * K_mn = -sum_{X,i} HTu[m][X][i] HTvfit[n][X][i]. */
int oracle_dflmo_k_asym(const oracle_layout* L, const double* B, const double* Vinv,
                        const double* U, const double* V, int nocc, double* K, double eps,
                        long long kchunk) {
  const size_t sz = (size_t)L->nbf * L->naux * nocc;
  double* Hu = (double*)malloc(sizeof(double) * sz);
  double* Hv = (double*)malloc(sizeof(double) * sz);
  double* Hf = (double*)malloc(sizeof(double) * sz);
  if (!Hu || !Hv || !Hf) { free(Hu); free(Hv); free(Hf); return 2; }
  oracle_half_transform(L, B, U, nocc, Hu);
  oracle_half_transform(L, B, V, nocc, Hv);
  apply_metric(L, Vinv, 0, Hv, nocc, Hf);
  contract_k(L, Hu, Hf, nocc, K, 0, kchunk);
  oracle_filter(L, K, eps);
  free(Hu);
  free(Hv);
  free(Hf);
  return 0;
}

/* DF-AO K: cbar[X][M][L] = sum_N (X|MN) P_NL, c = V^-1 (X|..),
 * K_MN = -sum_{X,S} c[X][N][S] cbar[X][M][S]  (jkdf.cpp:549-615). */
int oracle_dfao_k(const oracle_layout* L, const double* B, const double* Vinv, const double* P,
                  double* K, double eps, long long kchunk) {
  const int n = L->nbf;
  /* cbar via the half transform with C := P (n columns) */
  const size_t sz = (size_t)n * L->naux * n;
  double* cbar = (double*)malloc(sizeof(double) * sz);
  double* c = (double*)malloc(sizeof(double) * sz);
  double* Bd = (double*)calloc(sz, sizeof(double));
  if (!cbar || !c || !Bd) { free(cbar); free(c); free(Bd); return 2; }
  oracle_half_transform(L, B, P, n, cbar); /* cbar[M][X][L] */
  /* dense (X|N S) as [N][X][S] */
  for (int I = 0; I < L->nblk; ++I) {
    const int KI = L->panel_K[I];
    const int* cm = L->colmap + L->colmap_off[I];
    for (int m = 0; m < L->blk_off[I + 1] - L->blk_off[I]; ++m)
      for (int X = 0; X < L->naux; ++X) {
        const double* row = B + L->panel_off[I] + ((size_t)m * L->naux + X) * KI;
        double* d = Bd + ((size_t)(L->blk_off[I] + m) * L->naux + X) * n;
        for (int k = 0; k < KI; ++k) d[cm[k]] = row[k];
      }
  }
  apply_metric(L, Vinv, 0, Bd, n, c); /* c[N][X][S] = sum_Y Vinv[X][Y] B[N][Y][S] */
  contract_k(L, cbar, c, n, K, 0, kchunk);  /* K[M][N] = -sum_{X,S} cbar[M][X][S] c[N][X][S] */
  oracle_filter(L, K, eps);
  free(cbar);
  free(c);
  free(Bd);
  return 0;
}

/* ------------------------------------------------------------------------
 * SOS-AO-MP2 Laplace term, ll_full Z builder (src/mp/z_full.cpp:427-620 and
 * the Laplace loop src/mp/mp_compute.cpp:232-382).
 *
 * Per Laplace point t, with the occupied / virtual Cholesky factors Lo
 * (nbf x r) and Lv (nbf x rv) of the pseudo-densities:
 *   B_xov(X,i,a) = sum_{m,n} Lo(m,i) (X|mn) Lv(n,a)   ("mi, Xmn -> Xin",
 *                                                      "Na, XiN -> Xia")
 *   Z(X,Y)      = sum_{i,a} B_xov(X,i,a) B_xov(Y,i,a)
 *   e_t         = tr(Z V^-1 Z V^-1)                    (mp_compute.cpp:361-381)
 * On the prefitted tensor (X|mn)~ = L^-1 (X|mn) the same Z~ = L^-1 Z L^-T and
 * e_t = sum_{XY} Z~(X,Y)^2 (the Cholesky route of the metric).
 *
 * Layouts and order follow the device path: Lo and Lv arrive zero-padded to
 * hld and vld columns; H[n][X][i] and W[X][i][a] use those strides; every
 * sum is an in-order fma chain; Z sums over t = i*vld + a in chunks of
 * kchunk added in order; e = sum_X warp_dot(Z[X], Z[X]) in X order.  Only
 * the first nx auxiliary functions are used (nx = naux: all), which bounds
 * a timed CPU sample.
 * ---------------------------------------------------------------------- */

/* Bfit_I[m][Y][c] = sum_X Linv[Y][X] B_I[m][X][c] over X < min(naux,
 * 64*(Y/64+1)) (entries above the diagonal are zero), in-order fma: the
 * order of the device's lower-triangular grouped GEMM (64-row tiles). */
void oracle_prefit(const oracle_layout* L, const double* B, const double* Linv, int nx,
                   double* Bfit) {
  const int naux = L->naux;
  if (nx <= 0 || nx > naux) nx = naux;
  for (int I = 0; I < L->nblk; ++I) {
    const int KI = L->panel_K[I];
    const int bI = L->blk_off[I + 1] - L->blk_off[I];
    const double* P = B + L->panel_off[I];
    double* Q = Bfit + L->panel_off[I];
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)bI * nx; ++r) {
      const int m = (int)(r / nx), Y = (int)(r % nx);
      int xend = 64 * (Y / 64 + 1);
      if (xend > naux) xend = naux;
      const double* lrow = Linv + (size_t)Y * naux;
      double* q = Q + ((size_t)m * naux + Y) * KI;
      for (int c = 0; c < KI; ++c) {
        double s = 0.0;
        for (int X = 0; X < xend; ++X) s = fma(lrow[X], P[((size_t)m * naux + X) * KI + c], s);
        q[c] = s;
      }
    }
  }
}

int oracle_mp2_ll_point(const oracle_layout* L, const double* Bfit, const double* Lo, int hld,
                        const double* Lv, int vld, long long kchunk, int nx, double* Z,
                        double* e) {
  const int n = L->nbf, naux = L->naux;
  if (nx <= 0 || nx > naux) nx = naux;
  const long long klen = (long long)hld * vld;
  if (kchunk <= 0) kchunk = klen;
  double* H = (double*)malloc(sizeof(double) * (size_t)n * nx * hld);
  double* W = (double*)malloc(sizeof(double) * (size_t)nx * klen);
  if (!H || !W) { free(H); free(W); return 2; }
  /* H[mu][X][i] = sum_c Bfit_I[mu][X][c] Lo[col(c)][i] */
  for (int I = 0; I < L->nblk; ++I) {
    const int KI = L->panel_K[I];
    const int bI = L->blk_off[I + 1] - L->blk_off[I];
    const int* cm = L->colmap + L->colmap_off[I];
    const double* P = Bfit + L->panel_off[I];
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)bI * nx; ++r) {
      const int m = (int)(r / nx), X = (int)(r % nx);
      double* hr = H + ((size_t)(L->blk_off[I] + m) * nx + X) * hld;
      for (int i = 0; i < hld; ++i) hr[i] = 0.0;
      const double* br = P + ((size_t)m * naux + X) * KI;
      for (int k = 0; k < KI; ++k) {
        const double b = br[k];
        const double* c = Lo + (size_t)cm[k] * hld;
        for (int i = 0; i < hld; ++i) hr[i] = fma(b, c[i], hr[i]);
      }
    }
  }
  /* W[X][i][a] = sum_n H[n][X][i] Lv[n][a] */
#pragma omp parallel for schedule(static)
  for (long r = 0; r < (long)nx * hld; ++r) {
    const int X = (int)(r / hld), i = (int)(r % hld);
    double* w = W + (size_t)r * vld;
    for (int a = 0; a < vld; ++a) w[a] = 0.0;
    for (int mu = 0; mu < n; ++mu) {
      const double h = H[((size_t)mu * nx + X) * hld + i];
      const double* lv = Lv + (size_t)mu * vld;
      for (int a = 0; a < vld; ++a) w[a] = fma(h, lv[a], w[a]);
    }
  }
  /* Z[X][Y] (X <= Y, mirrored) */
#pragma omp parallel for schedule(dynamic, 1)
  for (int X = 0; X < nx; ++X)
    for (int Y = X; Y < nx; ++Y) {
      const double* a = W + (size_t)X * klen;
      const double* b = W + (size_t)Y * klen;
      double s = 0.0;
      for (long long t0 = 0; t0 < klen; t0 += kchunk) {
        const long long t1 = t0 + kchunk < klen ? t0 + kchunk : klen;
        double p = 0.0;
        for (long long t = t0; t < t1; ++t) p = fma(a[t], b[t], p);
        s += p;
      }
      Z[(size_t)X * nx + Y] = s;
      Z[(size_t)Y * nx + X] = s;
    }
  double acc = 0.0;
  for (int X = 0; X < nx; ++X) acc += warp_dot(Z + (size_t)X * nx, Z + (size_t)X * nx, nx, 1);
  *e = acc;
  free(H);
  free(W);
  return 0;
}
