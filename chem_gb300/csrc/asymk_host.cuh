// Non-symmetric DF-LMO exchange: megalochem's fock::DFLMO_K with
// set_sym(false) (src/fock/jkdf.cpp:1093-1323), the exchange that the ADC
// matrix-vector products request with different left and right
// coefficients (set_coeff_left_alpha / set_coeff_right_alpha,
// src/adc/adc_mvp_aoriadc2.cpp:182-220):
//
//   HTu(X,m,i) = sum_n (X|mn) u(n,i)          ("Xmn, ni -> Xmi")
//   HTv(X,m,i) = sum_n (X|mn) vt(i,n)         ("Xmn, in -> Xmi")
//   K(m,n)     = -sum_{X,i} HTu(X,m,i) [V^-1 HTv](X,n,i)
//
// FP64 path: the reference route (grouped half transforms, V^-1 fit of the
// v side, one non-symmetric split-K GEMM; bitwise equal to the oracle).
// Split path, Cholesky route on the prefitted tensor Bfit = L^-1 B:
// K = -(Bfit u)(Bfit v)^T over k = (Y, i), both half transforms as split
// GEMMs, then the exchange over all tiles, split over k.
#pragma once
#include <algorithm>
#include <string>
#include <vector>

#include "kernels_fp64.cuh"
#include "split_gemm.cuh"
#include "split_host.cuh"

namespace gbjk {

struct AsymKState {
  size_t bytes = 0;
  int precision = -1, nocc = 0, hld = 0, ksplit = 1;
  bool ready = false;
  double *d_U = nullptr, *d_V = nullptr, *d_Ug = nullptr, *d_Vg = nullptr;
  double *d_Hu = nullptr, *d_Hv = nullptr, *d_Hvf = nullptr, *d_Kpart = nullptr;
  // FP64 plan
  GemmGroup* d_groups = nullptr;
  GemmTile* d_tiles = nullptr;
  int ht_0 = 0, ht_n = 0, fit_0 = 0, fit_n = 0, k_0 = 0, k_n = 0;
  // split plan
  uint16_t *d_Cdig = nullptr, *d_Hdig = nullptr;
  int* d_eC = nullptr;
  unsigned int* d_eH = nullptr;
  SplitItem* d_items = nullptr;
  SplitJob* d_jobs = nullptr;
  int i_ht0 = 0, i_htn = 0, i_k0 = 0, i_kn = 0, j_h0 = 0;
  int c_nrb = 0, h_nrb = 0, h_nkt = 0, c_maxthr = 0;
  long long cdig_side = 0, hdig_side = 0;

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
    for (double** p : {&d_U, &d_V, &d_Ug, &d_Vg, &d_Hu, &d_Hv, &d_Hvf, &d_Kpart}) free_(p);
    free_(&d_groups);
    free_(&d_tiles);
    free_(&d_Cdig);
    free_(&d_Hdig);
    free_(&d_eC);
    free_(&d_eH);
    free_(&d_items);
    free_(&d_jobs);
    bytes = 0;
    precision = -1;
    nocc = 0;
    ready = false;
  }
  static int cdiv_(long long a, long long b) { return (int)((a + b - 1) / b); }

  struct Layout {
    int nbf, naux, nblk, ncols_total;
    const std::vector<int>*bsize, *boff, *panelK, *cmoff;
    const std::vector<long long>* panel_off;
  };

  gbjk_status plan(int prec, int nocc_, const Layout& L, const double* d_B, const double* d_Vinv,
                   SplitState& sp, std::string* err) {
    release();
    nocc = nocc_;
    // the split epilogue stores FP64 pairs (even stride); the FP64 path keeps
    // the unpadded k = (X, i) order of the oracle
    hld = prec == GBJK_SPLIT_BF16 ? nocc + (nocc & 1) : nocc;
    const size_t nbf = L.nbf, naux = L.naux;
    const size_t hsz = nbf * naux * hld;
    if (alloc(&d_U, nbf * nocc) || alloc(&d_V, nbf * nocc) ||
        alloc(&d_Ug, (size_t)L.ncols_total * nocc) || alloc(&d_Vg, (size_t)L.ncols_total * nocc) ||
        alloc(&d_Hu, hsz) || alloc(&d_Hv, hsz) || cudaMemset(d_Hu, 0, hsz * 8) ||
        cudaMemset(d_Hv, 0, hsz * 8)) {
      *err = "non-symmetric DF-LMO K: out of device memory";
      return GBJK_OOM;
    }
    gbjk_status s = prec == GBJK_SPLIT_BF16 ? plan_split(L, sp, err) : plan_fp64(L, d_B, d_Vinv, err);
    if (s) {
      release();
      return s;
    }
    precision = prec;
    ready = true;
    return GBJK_OK;
  }

  gbjk_status plan_fp64(const Layout& L, const double* d_B, const double* d_Vinv,
                        std::string* err) {
    const size_t nbf = L.nbf, naux = L.naux;
    const long long kdim = (long long)naux * hld;
    long long kc = kdim;
    gbjk_k_split_plan(L.nbf, L.naux, hld, &ksplit, &kc);
    if (alloc(&d_Hvf, nbf * naux * hld) || alloc(&d_Kpart, (size_t)ksplit * nbf * nbf)) {
      *err = "non-symmetric DF-LMO K: out of device memory";
      return GBJK_OOM;
    }
    std::vector<GemmGroup> groups;
    std::vector<GemmTile> tiles;
    auto add = [&](int group, int M, int N, int k0, int k1, long long coff) {
      for (int mt = 0; mt < cdiv_(M, 64); ++mt)
        for (int nt = 0; nt < cdiv_(N, 64); ++nt) tiles.push_back({group, mt, nt, k0, k1, coff});
    };
    ht_0 = 0;
    for (int side = 0; side < 2; ++side)
      for (int I = 0; I < L.nblk; ++I) {
        GemmGroup g;
        g.A = d_B + (*L.panel_off)[I];
        g.B = (side ? d_Vg : d_Ug) + (long long)(*L.cmoff)[I] * nocc;
        g.C = (side ? d_Hv : d_Hu) + (long long)(*L.boff)[I] * naux * hld;
        g.M = (*L.bsize)[I] * (int)naux;
        g.N = nocc;
        g.K = (*L.panelK)[I];
        g.lda = g.K;
        g.ldb = nocc;
        g.ldc = hld;
        g.flags = 0;
        if (g.K == 0) continue;
        add((int)groups.size(), g.M, g.N, 0, g.K, 0);
        groups.push_back(g);
      }
    ht_n = (int)tiles.size() - ht_0;
    fit_0 = (int)tiles.size();
    for (size_t mu = 0; mu < nbf; ++mu) {
      GemmGroup g;
      g.A = d_Vinv;
      g.B = d_Hv + mu * naux * hld;
      g.C = d_Hvf + mu * naux * hld;
      g.M = (int)naux;
      g.N = hld;
      g.K = (int)naux;
      g.lda = (int)naux;
      g.ldb = hld;
      g.ldc = hld;
      g.flags = 0;
      add((int)groups.size(), g.M, g.N, 0, g.K, 0);
      groups.push_back(g);
    }
    fit_n = (int)tiles.size() - fit_0;
    k_0 = (int)tiles.size();
    {
      GemmGroup g;
      g.A = d_Hu;
      g.B = d_Hvf;
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
      *err = "non-symmetric DF-LMO K: out of memory for the plan";
      return GBJK_OOM;
    }
    return GBJK_OK;
  }

  gbjk_status plan_split(const Layout& L, SplitState& sp, std::string* err) {
    if (sp.nbatch != 1) {
      *err = "non-symmetric DF-LMO K: the split path needs the whole auxiliary range";
      return GBJK_INVALID_ARG;
    }
    const int nbf = L.nbf, naux = L.naux, nblk = L.nblk;
    c_nrb = cdiv_(nocc, kTileN) * (kTileN / 32);
    std::vector<long long> c_off(nblk);
    long long ctot = 0;
    for (int I = 0; I < nblk; ++I) {
      c_off[I] = ctot;
      ctot += (long long)c_nrb * sp.nkt[I] * kSlices * kImage;
    }
    cdig_side = ctot;
    h_nrb = std::max(cdiv_(nbf, kTileM) * (kTileM / 32), cdiv_(nbf, kTileN) * (kTileN / 32));
    h_nkt = cdiv_((long long)naux * hld, kTileK);
    hdig_side = (long long)h_nrb * h_nkt * kSlices * kImage;
    const int ntile = cdiv_(nbf, kTileM) * cdiv_(nbf, kTileN);
    const int ks = sp.choose_ksplit(h_nkt, ntile);
    const int kt_per = cdiv_(h_nkt, ks);
    ksplit = cdiv_(h_nkt, kt_per);
    if (alloc(&d_Cdig, (size_t)2 * ctot) || alloc(&d_Hdig, (size_t)2 * hdig_side) ||
        alloc(&d_eC, (size_t)2 * nblk * c_nrb * 32) || alloc(&d_eH, (size_t)2 * h_nrb * 32) ||
        alloc(&d_Kpart, (size_t)ksplit * nbf * nbf) ||
        cudaMemset(d_Cdig, 0, (size_t)2 * ctot * 2) ||
        cudaMemset(d_Hdig, 0, (size_t)2 * hdig_side * 2) ||
        cudaMemset(d_eC, 0, (size_t)2 * nblk * c_nrb * 32 * 4)) {
      *err = "non-symmetric DF-LMO K: out of device memory for the split path";
      return GBJK_OOM;
    }
    std::vector<SplitJob> jobs;
    std::vector<SplitItem> items;
    c_maxthr = 0;
    for (int side = 0; side < 2; ++side)
      for (int I = 0; I < nblk; ++I) {
        SplitJob j;
        j.src = (side ? d_Vg : d_Ug) + (long long)(*L.cmoff)[I] * nocc;
        j.rs = 1;
        j.cs = nocc;
        j.row0 = 0;
        j.nrows = nocc;
        j.ncols = (*L.panelK)[I];
        j.e = d_eC + ((long long)side * nblk + I) * c_nrb * 32;
        j.e_biased = 0;
        j.nrb = c_nrb;
        j.nkt = sp.nkt[I];
        j.dst = d_Cdig + side * cdig_side + c_off[I];
        jobs.push_back(j);
        c_maxthr = std::max(c_maxthr, (nocc / 8 + 2) * sp.nkt[I] * 32);
      }
    j_h0 = (int)jobs.size();
    for (int side = 0; side < 2; ++side) {
      SplitJob j;
      j.src = side ? d_Hv : d_Hu;
      j.rs = (long long)naux * hld;
      j.cs = 1;
      j.row0 = 0;
      j.nrows = nbf;
      j.ncols = (long long)naux * hld;
      j.e = (int*)d_eH + (long long)side * h_nrb * 32;
      j.e_biased = 0;
      j.nrb = h_nrb;
      j.nkt = h_nkt;
      j.dst = d_Hdig + side * hdig_side;
      jobs.push_back(j);
    }
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
    // both sides' tiles of one A row tile are adjacent: its digits come
    // from HBM once and from L2 for the other side
    i_ht0 = 0;
    for (int I = 0; I < nblk; ++I) {
      // A rows (m, Y) at m * sp.apitch + Y (SplitItem::apitch)
      const long long rows = (long long)(*L.bsize)[I] * sp.apitch;
      for (int mt = 0; mt < cdiv_(rows, kTileM); ++mt)
        for (int side = 0; side < 2; ++side)
          for (int nt = 0; nt < cdiv_(nocc, kTileN); ++nt) {
            SplitItem w = base();
            w.a = sp.d_Aslices + sp.a_off[I];
            w.a_nrb = sp.a_nrb[I];
            w.a_rb0 = mt * (kTileM / 32);
            w.apitch = sp.apitch;
            w.arow0 = mt * kTileM;
            w.ay_valid = naux;
            w.b = d_Cdig + side * cdig_side + c_off[I];
            w.b_nrb = c_nrb;
            w.b_rb0 = nt * (kTileN / 32);
            w.kt0 = 0;
            w.nkt = sp.nkt[I];
            w.ea = sp.d_eA + sp.eA_off[I] + (long long)mt * kTileM;
            w.eb = d_eC + ((long long)side * nblk + I) * c_nrb * 32 + (long long)nt * kTileN;
            w.out = (side ? d_Hv : d_Hu) +
                    ((long long)(*L.boff)[I] * naux + (long long)mt * kTileM) * hld +
                    (long long)nt * kTileN;
            w.ldr = hld;
            w.m_valid = (int)std::min<long long>(kTileM, rows - (long long)mt * kTileM);
            w.n_valid = std::min(kTileN, nocc - nt * kTileN);
            w.emax = d_eH + (long long)side * h_nrb * 32 + (*L.boff)[I];
            w.emax_row0 = mt * kTileM;
            w.emax_div = naux;
            items.push_back(w);
          }
    }
    i_htn = (int)items.size() - i_ht0;
    i_k0 = (int)items.size();
    for (int k = 0; k < ksplit; ++k) {
      const int kt0 = k * kt_per, n_kt = std::min(kt_per, h_nkt - kt0);
      for (int mt = 0; mt < cdiv_(nbf, kTileM); ++mt)
        for (int nt = 0; nt < cdiv_(nbf, kTileN); ++nt) {
          SplitItem w = base();
          w.a = d_Hdig;
          w.a_nrb = h_nrb;
          w.a_rb0 = mt * (kTileM / 32);
          w.b = d_Hdig + hdig_side;
          w.b_nrb = h_nrb;
          w.b_rb0 = nt * (kTileN / 32);
          w.kt0 = kt0;
          w.nkt = n_kt;
          w.ea = (const int*)d_eH + (long long)mt * kTileM;
          w.eb = (const int*)d_eH + (long long)h_nrb * 32 + (long long)nt * kTileN;
          w.out = d_Kpart + (long long)k * nbf * nbf + (long long)mt * kTileM * nbf +
                  (long long)nt * kTileN;
          w.ldr = nbf;
          w.m_valid = std::min(kTileM, nbf - mt * kTileM);
          w.n_valid = std::min(kTileN, nbf - nt * kTileN);
          items.push_back(w);
        }
    }
    i_kn = (int)items.size() - i_k0;
    if (alloc(&d_items, items.size()) || alloc(&d_jobs, jobs.size()) ||
        cudaMemcpy(d_items, items.data(), items.size() * sizeof(SplitItem),
                   cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_jobs, jobs.data(), jobs.size() * sizeof(SplitJob), cudaMemcpyHostToDevice)) {
      *err = "non-symmetric DF-LMO K: out of memory for the work lists";
      return GBJK_OOM;
    }
    return GBJK_OK;
  }

  // K from u (nbf x nocc) and v (nbf x nocc, the transpose of the
  // reference's vt), both already in d_U / d_V.
  gbjk_status run(cudaStream_t st, int nbf, int naux, int nblk, int ncols_total,
                  const int* d_colmap, double* dK, SplitState& sp, int64_t* launches,
                  std::string* err) {
    const long long nn = (long long)nbf * nbf;
    const long long gtot = (long long)ncols_total * nocc;
    k_gather_cols<<<cdiv_(gtot, 256), 256, 0, st>>>(d_U, nocc, d_colmap, ncols_total, d_Ug);
    k_gather_cols<<<cdiv_(gtot, 256), 256, 0, st>>>(d_V, nocc, d_colmap, ncols_total, d_Vg);
    *launches += 2;
    if (precision == GBJK_SPLIT_BF16) {
      gbjk_status s;
      k_row_maxexp<<<dim3(cdiv_((long long)nocc * 32, 256), 2 * nblk), 256, 0, st>>>(d_jobs);
      k_split_tiles<<<dim3(cdiv_(c_maxthr, 256), 2 * nblk), 256, 0, st>>>(d_jobs);
      *launches += 2;
      if (cudaMemsetAsync(d_eH, 0, (size_t)2 * h_nrb * 32 * 4, st) != cudaSuccess) {
        *err = "non-symmetric DF-LMO K: memset failed";
        return GBJK_CUDA_ERROR;
      }
      if ((s = sp.launch_gemm(st, d_items + i_ht0, i_htn, launches, err))) return s;
      k_exp_unbias<<<cdiv_((long long)2 * h_nrb * 32, 256), 256, 0, st>>>((int*)d_eH,
                                                                          2 * h_nrb * 32);
      const long long thr = (long long)(nbf / 8 + 2) * h_nkt * 32;
      k_split_tiles<<<dim3(cdiv_(thr, 256), 2), 256, 0, st>>>(d_jobs + j_h0);
      *launches += 2;
      if ((s = sp.launch_gemm(st, d_items + i_k0, i_kn, launches, err))) return s;
    } else {
      auto gemm = [&](int t0, int n, bool transB) {
        for (int o = 0; o < n; o += (1 << 20)) {
          const int c = std::min(1 << 20, n - o);
          if (transB)
            k_gemm_fp64<true><<<c, 256, 0, st>>>(d_groups, d_tiles + t0 + o, 1.0);
          else
            k_gemm_fp64<false><<<c, 256, 0, st>>>(d_groups, d_tiles + t0 + o, 1.0);
          (*launches)++;
        }
      };
      gemm(ht_0, ht_n, false);
      gemm(fit_0, fit_n, false);
      gemm(k_0, k_n, true);
    }
    k_splitk_reduce<<<cdiv_(nn, 256), 256, 0, st>>>(d_Kpart, ksplit, nbf, -1.0, 0, dK);
    (*launches)++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      *err = std::string("non-symmetric DF-LMO K launch: ") + cudaGetErrorString(e);
      return GBJK_CUDA_ERROR;
    }
    return GBJK_OK;
  }
};

}  // namespace gbjk
