// DF-AO exchange: megalochem's fock::DFAO_K (src/fock/jkdf.cpp:464-648) with
// the fitting coefficients of ints::dfitting (src/ints/fitting.cpp:44-161).
//
//   cbar(X, M, S) = sum_N (X|MN) P(N, S)                 ("XMN, NL -> XML")
//   c(X, N, S)    = sum_Y V^-1(X, Y) (Y|NS)              ("XY, YMN -> XMN")
//   K(M, N)       = -sum_{X,S} c(X, N, S) cbar(X, M, S)  ("XNS, XMS -> MN")
//
// FP64 path (the reference route): c is fitted once per tensor in panel
// layout (grouped GEMM per panel row with V^-1) and expanded to a dense
// [N][X][S] array; per build cbar = half transform of B with the panel rows
// of P, then K = -cbar c^T over k = (X, S) with split-K partials summed in
// order, like the oracle (oracle_dfao_k).
// Split path (Cholesky route of the metric): with Bfit = L^-1 B,
//   K(M, N) = -sum_{Y,S} Bfit(Y, N, S) [L^-1 cbar](Y, M, S),
// and L^-1 cbar is the half transform of Bfit with P.  Once per tensor the
// dense digits of Bfit (rows N, k = (Y, S)); per build the P digits per
// panel, the split half transform (its epilogue max-reduces each row M's
// exponent), the digits of L^-1 cbar and the exchange over upper tiles,
// split over k.
#pragma once
#include <algorithm>
#include <string>
#include <vector>

#include "kernels_fp64.cuh"
#include "split_gemm.cuh"
#include "split_host.cuh"

namespace gbjk {

struct AoKState {
  size_t bytes = 0;
  int precision = -1;
  bool ready = false;
  long long kdim = 0;  // naux * nbf
  double *d_Pg = nullptr, *d_cbar = nullptr, *d_cd = nullptr, *d_Kpart = nullptr;
  // FP64 plan
  GemmGroup* d_groups = nullptr;
  GemmTile* d_tiles = nullptr;
  int ht_0 = 0, ht_n = 0, k_0 = 0, k_n = 0, ksplit = 1;
  // split plan
  uint16_t *d_Pdig = nullptr, *d_Cbdig = nullptr, *d_Bdig = nullptr;
  int *d_eP = nullptr, *d_eBd = nullptr;
  unsigned int* d_eCb = nullptr;
  SplitItem* d_items = nullptr;
  SplitJob* d_jobs = nullptr;
  int i_ht0 = 0, i_htn = 0, i_k0 = 0, i_kn = 0, j_p0 = 0, j_cb = 0;
  int p_nrb = 0, r_nrb = 0, r_nkt = 0, p_maxthr = 0;

  template <class T>
  cudaError_t alloc(T** p, size_t n) {
    const size_t b = std::max<size_t>(n, 1) * sizeof(T);
    cudaError_t e = cudaMalloc((void**)p, b);
    if (e == cudaSuccess)
      bytes += b;
    else
      cudaGetLastError();
    return e;
  }
  template <class T>
  void free_(T** p) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  void release() {
    free_(&d_Pg);
    free_(&d_cbar);
    free_(&d_cd);
    free_(&d_Kpart);
    free_(&d_groups);
    free_(&d_tiles);
    free_(&d_Pdig);
    free_(&d_Cbdig);
    free_(&d_Bdig);
    free_(&d_eP);
    free_(&d_eBd);
    free_(&d_eCb);
    free_(&d_items);
    free_(&d_jobs);
    bytes = 0;
    precision = -1;
    ready = false;
  }
  static int cdiv_(long long a, long long b) { return (int)((a + b - 1) / b); }

  struct Layout {
    int nbf, naux, nblk, ncols_total, maxK;
    const std::vector<int>*bsize, *boff, *panelK, *cmoff;
    const std::vector<long long>* panel_off;
    const int *d_blk_of, *d_boff, *d_panelK, *d_cmoff, *d_colmap;
    const long long* d_panel_off;
  };

  // Dense [N][X][S] copy of a panel array into `dst` (zeroed first).
  static gbjk_status expand(cudaStream_t st, const Layout& L, const double* src, double* dst,
                            int64_t* launches, std::string* err) {
    if (cudaMemsetAsync(dst, 0, (size_t)L.nbf * L.naux * L.nbf * 8, st) != cudaSuccess) {
      *err = "DF-AO K: memset failed";
      return GBJK_CUDA_ERROR;
    }
    k_expand_panels<<<dim3(cdiv_(L.maxK, 128), L.naux, L.nbf), 128, 0, st>>>(
        src, L.d_panel_off, L.d_blk_of, L.d_boff, L.d_panelK, L.d_cmoff, L.d_colmap, L.nbf,
        L.naux, dst);
    (*launches)++;
    return GBJK_OK;
  }

  // --- FP64 plan: fitted coefficients (once), half transform and exchange ---
  gbjk_status plan_fp64(cudaStream_t st, const Layout& L, const double* d_B, const double* d_Vinv,
                        int64_t* launches, std::string* err) {
    const size_t nbf = L.nbf, naux = L.naux;
    kdim = (long long)naux * nbf;
    const size_t big = nbf * naux * nbf;
    const long long nnz = L.panel_off->back() + (long long)L.bsize->back() * L.naux * L.panelK->back();
    double* d_c = nullptr;  // panel-layout coefficients, temporary
    long long kc = kdim;
    gbjk_k_split_plan(L.nbf, L.naux, L.nbf, &ksplit, &kc);
    if (alloc(&d_Pg, (size_t)L.ncols_total * nbf) || alloc(&d_cbar, big) || alloc(&d_cd, big) ||
        alloc(&d_Kpart, (size_t)ksplit * nbf * nbf) ||
        cudaMalloc((void**)&d_c, (size_t)nnz * 8) != cudaSuccess) {
      cudaGetLastError();
      if (d_c) cudaFree(d_c);
      *err = "DF-AO K: out of device memory (FP64 path needs 2 nbf^2 naux doubles)";
      return GBJK_OOM;
    }
    std::vector<GemmGroup> groups;
    std::vector<GemmTile> tiles;
    auto add = [&](int group, int M, int N, int k0, int k1, long long coff) {
      for (int mt = 0; mt < cdiv_(M, 64); ++mt)
        for (int nt = 0; nt < cdiv_(N, 64); ++nt) tiles.push_back({group, mt, nt, k0, k1, coff});
    };
    // fitting: c_I[m] = V^-1 B_I[m] (naux x K_I per AO function), once
    for (int I = 0; I < L.nblk; ++I) {
      const int K = (*L.panelK)[I];
      if (K == 0) continue;
      for (int m = 0; m < (*L.bsize)[I]; ++m) {
        GemmGroup g;
        const long long off = (*L.panel_off)[I] + (long long)m * naux * K;
        g.A = d_Vinv;
        g.B = d_B + off;
        g.C = d_c + off;
        g.M = (int)naux;
        g.N = K;
        g.K = (int)naux;
        g.lda = (int)naux;
        g.ldb = K;
        g.ldc = K;
        g.flags = 0;
        add((int)groups.size(), g.M, g.N, 0, g.K, 0);
        groups.push_back(g);
      }
    }
    const int nfit = (int)tiles.size();
    ht_0 = (int)tiles.size();
    for (int I = 0; I < L.nblk; ++I) {
      GemmGroup g;
      g.A = d_B + (*L.panel_off)[I];
      g.B = d_Pg + (long long)(*L.cmoff)[I] * nbf;
      g.C = d_cbar + (long long)(*L.boff)[I] * naux * nbf;
      g.M = (*L.bsize)[I] * (int)naux;
      g.N = (int)nbf;
      g.K = (*L.panelK)[I];
      g.lda = g.K;
      g.ldb = (int)nbf;
      g.ldc = (int)nbf;
      g.flags = 0;
      if (g.K == 0) continue;
      add((int)groups.size(), g.M, g.N, 0, g.K, 0);
      groups.push_back(g);
    }
    ht_n = (int)tiles.size() - ht_0;
    k_0 = (int)tiles.size();
    {
      GemmGroup g;
      g.A = d_cbar;
      g.B = d_cd;
      g.C = d_Kpart;
      g.M = (int)nbf;
      g.N = (int)nbf;
      g.K = (int)kdim;
      g.lda = (int)kdim;
      g.ldb = (int)kdim;
      g.ldc = (int)nbf;
      g.flags = kTransB;
      const int gi = (int)groups.size();
      groups.push_back(g);
      for (int k = 0; k < ksplit; ++k) {
        const long long k0 = (long long)k * kc, k1 = std::min<long long>(kdim, (k + 1) * kc);
        add(gi, g.M, g.N, (int)k0, (int)std::max(k0, k1), (long long)k * nbf * nbf);
      }
    }
    k_n = (int)tiles.size() - k_0;
    if (alloc(&d_groups, groups.size()) || alloc(&d_tiles, tiles.size()) ||
        cudaMemcpy(d_groups, groups.data(), groups.size() * sizeof(GemmGroup),
                   cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_tiles, tiles.data(), tiles.size() * sizeof(GemmTile),
                   cudaMemcpyHostToDevice)) {
      cudaFree(d_c);
      *err = "DF-AO K: out of memory for the FP64 plan";
      return GBJK_OOM;
    }
    // the fitting coefficients (a pre-fitted tensor is its own
    // coefficients), then their dense expansion
    if (!d_Vinv)
      cudaMemcpyAsync(d_c, d_B, (size_t)nnz * 8, cudaMemcpyDeviceToDevice, st);
    for (int t0 = 0; d_Vinv && t0 < nfit; t0 += (1 << 20)) {
      const int n = std::min(1 << 20, nfit - t0);
      k_gemm_fp64<false><<<n, 256, 0, st>>>(d_groups, d_tiles + t0, 1.0);
      (*launches)++;
    }
    gbjk_status s = expand(st, L, d_c, d_cd, launches, err);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(d_c);
    if (s) return s;
    if (e != cudaSuccess) {
      *err = std::string("DF-AO K fitting: ") + cudaGetErrorString(e);
      return GBJK_CUDA_ERROR;
    }
    return GBJK_OK;
  }

  // --- split plan: dense Bfit digits (once), P digits, half transform,
  // exchange over upper tiles ----------------------------------------------
  gbjk_status plan_split(cudaStream_t st, const Layout& L, SplitState& sp, int64_t* launches,
                         std::string* err) {
    if (sp.nbatch != 1) {
      *err = "DF-AO K: the split path needs the whole auxiliary range (no auxiliary batching)";
      return GBJK_INVALID_ARG;
    }
    const int nbf = L.nbf, naux = L.naux, nblk = L.nblk;
    kdim = (long long)naux * nbf;
    const size_t big = (size_t)nbf * naux * nbf;
    p_nrb = cdiv_(nbf, kTileN) * (kTileN / 32);
    std::vector<long long> p_off(nblk);
    long long ptot = 0;
    for (int I = 0; I < nblk; ++I) {
      p_off[I] = ptot;
      ptot += (long long)p_nrb * sp.nkt[I] * kSlices * kImage;
    }
    r_nrb = std::max(cdiv_(nbf, kTileM) * (kTileM / 32), cdiv_(nbf, kTileN) * (kTileN / 32));
    // exchange tiles: a staircase over the upper triangle (column tiles of
    // row tile r0 start at r0), fewer than on the grid
    std::vector<std::pair<int, int>> ktiles;
    for (int r0 = 0; r0 < nbf; r0 += kTileM)
      for (int c0 = r0; c0 < nbf; c0 += kTileN) ktiles.push_back({r0, c0});
    for (const auto& t : ktiles) r_nrb = std::max(r_nrb, cdiv_(t.second + kTileN, 32));
    const int ntile = (int)ktiles.size();
    r_nkt = cdiv_(kdim, kTileK);
    const long long rdig = (long long)r_nrb * r_nkt * kSlices * kImage;
    const int ks = sp.choose_ksplit(r_nkt, ntile);
    const int kt_per = cdiv_(r_nkt, ks);
    ksplit = cdiv_(r_nkt, kt_per);
    if (alloc(&d_Pg, (size_t)L.ncols_total * nbf) || alloc(&d_cbar, big) ||
        alloc(&d_Kpart, (size_t)ksplit * nbf * nbf) || alloc(&d_Pdig, (size_t)ptot) ||
        alloc(&d_Cbdig, (size_t)rdig) || alloc(&d_Bdig, (size_t)rdig) ||
        alloc(&d_eP, (size_t)nblk * p_nrb * 32) || alloc(&d_eBd, (size_t)r_nrb * 32) ||
        alloc(&d_eCb, (size_t)r_nrb * 32) ||
        cudaMemsetAsync(d_Pdig, 0, (size_t)ptot * 2, st) ||
        cudaMemsetAsync(d_Cbdig, 0, (size_t)rdig * 2, st) ||
        cudaMemsetAsync(d_Bdig, 0, (size_t)rdig * 2, st) ||
        cudaMemsetAsync(d_eP, 0, (size_t)nblk * p_nrb * 32 * 4, st) ||
        cudaMemsetAsync(d_eBd, 0, (size_t)r_nrb * 32 * 4, st) ||
        cudaMemsetAsync(d_eCb, 0, (size_t)r_nrb * 32 * 4, st)) {
      *err = "DF-AO K: out of device memory for the split path";
      return GBJK_OOM;
    }
    // jobs: P rows per panel, the half-transformed rows M, and (once) the
    // dense Bfit rows N
    std::vector<SplitJob> jobs;
    j_p0 = 0;
    p_maxthr = 0;
    for (int I = 0; I < nblk; ++I) {
      SplitJob j;
      j.src = d_Pg + (long long)(*L.cmoff)[I] * nbf;
      j.rs = 1;
      j.cs = nbf;
      j.row0 = 0;
      j.nrows = nbf;
      j.ncols = (*L.panelK)[I];
      j.e = d_eP + (long long)I * p_nrb * 32;
      j.e_biased = 0;
      j.nrb = p_nrb;
      j.nkt = sp.nkt[I];
      j.dst = d_Pdig + p_off[I];
      jobs.push_back(j);
      p_maxthr = std::max(p_maxthr, (nbf / 8 + 2) * sp.nkt[I] * 32);
    }
    j_cb = (int)jobs.size();
    {
      SplitJob j;
      j.src = d_cbar;
      j.rs = kdim;
      j.cs = 1;
      j.row0 = 0;
      j.nrows = nbf;
      j.ncols = kdim;
      j.e = (int*)d_eCb;
      j.e_biased = 0;
      j.nrb = r_nrb;
      j.nkt = r_nkt;
      j.dst = d_Cbdig;
      jobs.push_back(j);
    }
    const int j_bd = (int)jobs.size();
    {
      SplitJob j = jobs[j_cb];
      j.src = d_cbar;  // the dense Bfit is staged in the cbar buffer once
      j.e = d_eBd;
      j.dst = d_Bdig;
      jobs.push_back(j);
    }
    // items
    std::vector<SplitItem> items;
    auto base = []() {
      SplitItem w;
      w.emax = nullptr;
      w.emax_row0 = 0;
      w.emax_div = 1;
      w.out2 = nullptr;
      w.c0 = 0;
      w.ncol1 = 1 << 30;
      return w;
    };
    i_ht0 = 0;
    for (int I = 0; I < nblk; ++I) {
      // A rows (m, Y) at m * sp.apitch + Y (SplitItem::apitch)
      const long long rows = (long long)(*L.bsize)[I] * sp.apitch;
      for (int mt = 0; mt < cdiv_(rows, kTileM); ++mt)
        for (int nt = 0; nt < cdiv_(nbf, kTileN); ++nt) {
          SplitItem w = base();
          w.a = sp.d_Aslices + sp.a_off[I];
          w.a_nrb = sp.a_nrb[I];
          w.a_rb0 = mt * (kTileM / 32);
          w.apitch = sp.apitch;
          w.arow0 = mt * kTileM;
          w.ay_valid = naux;
          w.b = d_Pdig + p_off[I];
          w.b_nrb = p_nrb;
          w.b_rb0 = nt * (kTileN / 32);
          w.kt0 = 0;
          w.nkt = sp.nkt[I];
          w.ea = sp.d_eA + sp.eA_off[I] + (long long)mt * kTileM;
          w.eb = d_eP + (long long)I * p_nrb * 32 + (long long)nt * kTileN;
          w.out = d_cbar + ((long long)(*L.boff)[I] * naux + (long long)mt * kTileM) * nbf +
                  (long long)nt * kTileN;
          w.ldr = nbf;
          w.m_valid = (int)std::min<long long>(kTileM, rows - (long long)mt * kTileM);
          w.n_valid = std::min(kTileN, nbf - nt * kTileN);
          // row (m, Y) of panel I is row M = boff[I] + m of cbar
          w.emax = d_eCb + (*L.boff)[I];
          w.emax_row0 = mt * kTileM;
          w.emax_div = naux;
          items.push_back(w);
        }
    }
    i_htn = (int)items.size() - i_ht0;
    i_k0 = (int)items.size();
    for (int k = 0; k < ksplit; ++k) {
      const int kt0 = k * kt_per, n_kt = std::min(kt_per, r_nkt - kt0);
      for (const auto& t : ktiles) {
          const int r0 = t.first, c0 = t.second;
          SplitItem w = base();
          w.a = d_Cbdig;
          w.a_nrb = r_nrb;
          w.a_rb0 = r0 / 32;
          w.b = d_Bdig;
          w.b_nrb = r_nrb;
          w.b_rb0 = c0 / 32;
          w.kt0 = kt0;
          w.nkt = n_kt;
          w.ea = (const int*)d_eCb + r0;
          w.eb = d_eBd + c0;
          w.out = d_Kpart + (long long)k * nbf * nbf + (long long)r0 * nbf + c0;
          w.ldr = nbf;
          w.m_valid = std::min(kTileM, nbf - r0);
          w.n_valid = std::min(kTileN, nbf - c0);
          items.push_back(w);
        }
    }
    i_kn = (int)items.size() - i_k0;
    if (alloc(&d_items, items.size()) || alloc(&d_jobs, jobs.size()) ||
        cudaMemcpy(d_items, items.data(), items.size() * sizeof(SplitItem),
                   cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_jobs, jobs.data(), jobs.size() * sizeof(SplitJob), cudaMemcpyHostToDevice)) {
      *err = "DF-AO K: out of memory for the work lists";
      return GBJK_OOM;
    }
    // once: the dense Bfit (staged in the cbar buffer), its row exponents
    // and digits
    gbjk_status s;
    if ((s = expand(st, L, sp.Bfit, d_cbar, launches, err))) return s;
    k_row_maxexp<<<dim3(cdiv_((long long)nbf * 32, 256), 1), 256, 0, st>>>(d_jobs + j_bd);
    const long long thr = (long long)(nbf / 8 + 2) * r_nkt * 32;
    k_split_tiles<<<dim3(cdiv_(thr, 256), 1), 256, 0, st>>>(d_jobs + j_bd);
    *launches += 2;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      *err = std::string("DF-AO K split preparation: ") + cudaGetErrorString(e);
      return GBJK_CUDA_ERROR;
    }
    return GBJK_OK;
  }

  gbjk_status prepare(cudaStream_t st, int prec, const Layout& L, const double* d_B,
                      const double* d_Vinv, SplitState& sp, int64_t* launches, std::string* err) {
    if (ready && precision == prec) return GBJK_OK;
    release();
    gbjk_status s = prec == GBJK_SPLIT_BF16 ? plan_split(st, L, sp, launches, err)
                                            : plan_fp64(st, L, d_B, d_Vinv, launches, err);
    if (s) {
      release();
      return s;
    }
    precision = prec;
    ready = true;
    return GBJK_OK;
  }

  // One exchange build from the density dP (nbf x nbf, device) into dK.
  gbjk_status run(cudaStream_t st, const Layout& L, const double* dP, double* dK, SplitState& sp,
                  int64_t* launches, std::string* err) {
    const int nbf = L.nbf;
    const long long nn = (long long)nbf * nbf;
    k_gather_cols<<<cdiv_((long long)L.ncols_total * nbf, 256), 256, 0, st>>>(
        dP, nbf, L.d_colmap, L.ncols_total, d_Pg);
    (*launches)++;
    if (precision == GBJK_SPLIT_BF16) {
      gbjk_status s;
      k_row_maxexp<<<dim3(cdiv_((long long)nbf * 32, 256), L.nblk), 256, 0, st>>>(d_jobs + j_p0);
      k_split_tiles<<<dim3(cdiv_(p_maxthr, 256), L.nblk), 256, 0, st>>>(d_jobs + j_p0);
      *launches += 2;
      if (cudaMemsetAsync(d_eCb, 0, (size_t)r_nrb * 32 * 4, st) != cudaSuccess) {
        *err = "DF-AO K: memset failed";
        return GBJK_CUDA_ERROR;
      }
      if ((s = sp.launch_gemm(st, d_items + i_ht0, i_htn, launches, err))) return s;
      k_exp_unbias<<<cdiv_((long long)r_nrb * 32, 256), 256, 0, st>>>((int*)d_eCb, r_nrb * 32);
      const long long thr = (long long)(nbf / 8 + 2) * r_nkt * 32;
      k_split_tiles<<<dim3(cdiv_(thr, 256), 1), 256, 0, st>>>(d_jobs + j_cb);
      *launches += 2;
      if ((s = sp.launch_gemm(st, d_items + i_k0, i_kn, launches, err))) return s;
      k_splitk_reduce<<<cdiv_(nn, 256), 256, 0, st>>>(d_Kpart, ksplit, nbf, -1.0, 1, dK);
      (*launches)++;
    } else {
      for (int t0 = 0; t0 < ht_n; t0 += (1 << 20)) {
        const int n = std::min(1 << 20, ht_n - t0);
        k_gemm_fp64<false><<<n, 256, 0, st>>>(d_groups, d_tiles + ht_0 + t0, 1.0);
        (*launches)++;
      }
      for (int t0 = 0; t0 < k_n; t0 += (1 << 20)) {
        const int n = std::min(1 << 20, k_n - t0);
        k_gemm_fp64<true><<<n, 256, 0, st>>>(d_groups, d_tiles + k_0 + t0, 1.0);
        (*launches)++;
      }
      k_splitk_reduce<<<cdiv_(nn, 256), 256, 0, st>>>(d_Kpart, ksplit, nbf, -1.0, 0, dK);
      (*launches)++;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      *err = std::string("DF-AO K launch: ") + cudaGetErrorString(e);
      return GBJK_CUDA_ERROR;
    }
    return GBJK_OK;
  }
};

}  // namespace gbjk
