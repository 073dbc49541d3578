// Host side of the SOS-AO-MP2 Laplace batch: megalochem's ll_full Z builder
// (src/mp/z_full.cpp:427-620) for every quadrature point of the Laplace
// loop (src/mp/mp_compute.cpp:232-382) in one pass, on the prefitted tensor
// Bfit = L^-1 B that the J/K engine keeps resident.
//
// Per point t (occupied factor Lo_t, nbf x r_t; virtual factor Lv_t,
// nbf x rv_t; both zero-padded to the common strides hld, vld):
//   T1   H_t[n][X][i] = sum_m Bfit(X|nm) Lo_t[m][i]      ("mi, Xmn -> Xin")
//   T2   W_t[X][i][a] = sum_n H_t[n][X][i] Lv_t[n][a]    ("Na, XiN -> Xia")
//   Z    Z_t[X][Y]    = sum_{i,a} W_t[X][i][a] W_t[Y][i][a]
//   e_t  = sum_{X,Y} Z_t[X][Y]^2 = tr(Z V^-1 Z V^-1) of the unfitted Z
// Each of T1, T2 and Z is one launch over all points (a grouped FP64 GEMM,
// or the split-precision tensor-core GEMM of split_gemm.cuh); the energy is
// an ordered FP64 reduction.  Split path per build:
//   gather Lo rows per panel -> their digits -> T1 (A digits of Bfit are the
//   J/K engine's) -> column exponents of H -> H digits (rows (X,i), k = n)
//   and Lv digits -> T2 (epilogue: per-X exponent maxima of W) -> W digits
//   -> Z upper tiles, split over k -> ordered reduce -> row sums -> e_t.
#pragma once
#include <algorithm>
#include <string>
#include <vector>

#include "kernels_fp64.cuh"
#include "kernels_mp2.cuh"
#include "split_gemm.cuh"
#include "split_host.cuh"

namespace gbjk {

struct Mp2State {
  enum { kT1 = 0, kT2, kZ, kOps, kNumPh };
  size_t bytes = 0;
  int npts = 0, hld = 0, vld = 0, precision = -1;
  long long nrho = 0, kw = 0;  // rows (X, i) of T2; k length of Z (hld * vld)
  std::vector<int> ro, rv;
  bool ready = false, have_result = false;
  // inputs and intermediates (every point at a fixed stride)
  double *d_Lo = nullptr, *d_Lv = nullptr, *d_Cg = nullptr;
  double *d_H = nullptr, *d_W = nullptr, *d_Z = nullptr, *d_rsq = nullptr, *d_E = nullptr;
  long long cg_stride = 0, h_stride = 0, w_stride = 0;
  // FP64 plan
  GemmGroup* d_groups = nullptr;
  GemmTile* d_tiles = nullptr;
  int t1_0 = 0, t1_n = 0, t2_0 = 0, t2_n = 0, z_0 = 0, z_n = 0;
  // split plan
  uint16_t *d_Cdig = nullptr, *d_Hdig = nullptr, *d_Lvdig = nullptr, *d_Wdig = nullptr;
  int *d_eC = nullptr, *d_eH = nullptr, *d_eLv = nullptr;
  unsigned int* d_eW = nullptr;
  double* d_Zpart = nullptr;
  SplitItem* d_items = nullptr;
  SplitJob* d_jobs = nullptr;
  int i1_0 = 0, i1_n = 0, i2_0 = 0, i2_n = 0, iz_0 = 0, iz_n = 0;
  int jc_0 = 0, jlv_0 = 0, jh_0 = 0, jw_0 = 0;
  int c_nrb = 0, h_nrb = 0, h_nkt = 0, lv_nrb = 0, w_nrb = 0, w_nkt = 0, ksplit = 1;
  long long cdig_stride = 0, hdig_stride = 0, lvdig_stride = 0, wdig_stride = 0;
  int c_maxthr = 0;
  // profiling
  bool profile = false;
  double ms[kNumPh] = {};
  int64_t nl[kNumPh] = {};
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;

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
    free_(&d_Lo);
    free_(&d_Lv);
    free_(&d_Cg);
    free_(&d_H);
    free_(&d_W);
    free_(&d_Z);
    free_(&d_rsq);
    free_(&d_E);
    free_(&d_groups);
    free_(&d_tiles);
    free_(&d_Cdig);
    free_(&d_Hdig);
    free_(&d_Lvdig);
    free_(&d_Wdig);
    free_(&d_eC);
    free_(&d_eH);
    free_(&d_eLv);
    free_(&d_eW);
    free_(&d_Zpart);
    free_(&d_items);
    free_(&d_jobs);
    resolve();
    bytes = 0;
    npts = 0;
    precision = -1;
    ready = have_result = false;
  }

  // --- profiling ------------------------------------------------------------
  struct Scope {
    Mp2State* s;
    int ph;
    cudaStream_t st;
    cudaEvent_t a = nullptr, b = nullptr;
    Scope(Mp2State* s_, int p, cudaStream_t st_) : s(s_), ph(p), st(st_) {
      if (s->profile) {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, st);
      }
      s->nl[ph]++;
    }
    ~Scope() {
      if (s->profile) {
        cudaEventRecord(b, st);
        s->pending.push_back({ph, {a, b}});
      }
    }
  };
  void resolve() {
    for (auto& pe : pending) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, pe.second.first, pe.second.second) == cudaSuccess)
        ms[pe.first] += t;
      cudaEventDestroy(pe.second.first);
      cudaEventDestroy(pe.second.second);
    }
    pending.clear();
  }
  void reset_profile() {
    resolve();
    for (int i = 0; i < kNumPh; ++i) {
      ms[i] = 0;
      nl[i] = 0;
    }
  }
  int profile_read(int idx, const char** name, double* out_ms, int64_t* launches) {
    static const char* names[kNumPh] = {"mp2_t1", "mp2_t2", "mp2_z", "mp2_ops"};
    if (idx < 0 || idx >= kNumPh) return 0;
    resolve();
    if (name) *name = names[idx];
    if (out_ms) *out_ms = ms[idx];
    if (launches) *launches = nl[idx];
    return 1;
  }

  static int cdiv_(long long a, long long b) { return (int)((a + b - 1) / b); }

  // --- plan -------------------------------------------------------------------
  // Layout arguments are the J/K engine's (host copies); `sp` holds the
  // prefitted tensor and, for the split path, its A-operand digits.
  gbjk_status plan(cudaStream_t st, int prec, int npts_, const int* ro_, const int* rv_, int nbf,
                   int naux, int nblk, int ncols_total, const std::vector<int>& bsize,
                   const std::vector<int>& boff, const std::vector<int>& panelK,
                   const std::vector<int>& cmoff, const std::vector<long long>& panel_off,
                   SplitState& sp, std::string* err) {
    release();
    npts = npts_;
    ro.assign(ro_, ro_ + npts);
    rv.assign(rv_, rv_ + npts);
    int mo = 1, mv = 1;
    for (int t = 0; t < npts; ++t) {
      mo = std::max(mo, ro[t]);
      mv = std::max(mv, rv[t]);
    }
    hld = mo + (mo & 1);  // even strides: 16-byte aligned FP64 pairs
    vld = mv + (mv & 1);
    nrho = (long long)naux * hld;
    kw = (long long)hld * vld;
    cg_stride = (long long)ncols_total * hld;
    h_stride = (long long)nbf * nrho;
    w_stride = (long long)naux * kw;
    const size_t nn = (size_t)naux * naux;
    if (alloc(&d_Lo, (size_t)npts * nbf * hld) || alloc(&d_Lv, (size_t)npts * nbf * vld) ||
        alloc(&d_Cg, (size_t)npts * cg_stride) || alloc(&d_H, (size_t)npts * h_stride) ||
        alloc(&d_W, (size_t)npts * w_stride) || alloc(&d_Z, (size_t)npts * nn) ||
        alloc(&d_rsq, (size_t)npts * naux) || alloc(&d_E, (size_t)npts) ||
        cudaMemsetAsync(d_H, 0, (size_t)npts * h_stride * 8, st) ||
        cudaMemsetAsync(d_W, 0, (size_t)npts * w_stride * 8, st)) {
      release();
      *err = "MP2 batch: out of device memory for the transforms";
      return GBJK_OOM;
    }
    precision = prec;
    gbjk_status s = prec == GBJK_SPLIT_BF16
                        ? plan_split(st, nbf, naux, nblk, bsize, boff, panelK, cmoff, sp, err)
                        : plan_fp64(nbf, naux, nblk, bsize, boff, panelK, cmoff, panel_off,
                                    sp.Bfit, err);
    if (s) {
      release();
      return s;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) {
      release();
      *err = "MP2 batch: plan upload failed";
      return GBJK_CUDA_ERROR;
    }
    ready = true;
    return GBJK_OK;
  }

  gbjk_status plan_fp64(int nbf, int naux, int nblk, const std::vector<int>& bsize,
                        const std::vector<int>& boff, const std::vector<int>& panelK,
                        const std::vector<int>& cmoff, const std::vector<long long>& panel_off,
                        const double* Bfit, std::string* err) {
    std::vector<GemmGroup> groups;
    std::vector<GemmTile> tiles;
    auto add = [&](int group, int M, int N, int K, bool upper) {
      for (int mt = 0; mt < cdiv_(M, 64); ++mt)
        for (int nt = 0; nt < cdiv_(N, 64); ++nt) {
          if (upper && nt < mt) continue;
          tiles.push_back({group, mt, nt, 0, K, 0});
        }
    };
    t1_0 = 0;
    for (int t = 0; t < npts; ++t)
      for (int I = 0; I < nblk; ++I) {
        if (panelK[I] == 0) continue;
        GemmGroup g;
        g.A = Bfit + panel_off[I];
        g.B = d_Cg + t * cg_stride + (long long)cmoff[I] * hld;
        g.C = d_H + t * h_stride + (long long)boff[I] * naux * hld;
        g.M = bsize[I] * naux;
        g.N = hld;
        g.K = panelK[I];
        g.lda = panelK[I];
        g.ldb = hld;
        g.ldc = hld;
        g.flags = 0;
        add((int)groups.size(), g.M, g.N, g.K, false);
        groups.push_back(g);
      }
    t1_n = (int)tiles.size();
    t2_0 = (int)tiles.size();
    for (int t = 0; t < npts; ++t) {
      GemmGroup g;
      g.A = d_H + t * h_stride;  // K x M (n, rho): transposed operand
      g.B = d_Lv + (long long)t * nbf * vld;
      g.C = d_W + t * w_stride;
      g.M = (int)nrho;
      g.N = vld;
      g.K = nbf;
      g.lda = (int)nrho;
      g.ldb = vld;
      g.ldc = vld;
      g.flags = 0;
      add((int)groups.size(), g.M, g.N, g.K, false);
      groups.push_back(g);
    }
    t2_n = (int)tiles.size() - t2_0;
    z_0 = (int)tiles.size();
    for (int t = 0; t < npts; ++t) {
      GemmGroup g;
      g.A = d_W + t * w_stride;
      g.B = g.A;
      g.C = d_Z + (long long)t * naux * naux;
      g.M = naux;
      g.N = naux;
      g.K = (int)kw;
      g.lda = (int)kw;
      g.ldb = (int)kw;
      g.ldc = naux;
      g.flags = kTransB;
      add((int)groups.size(), g.M, g.N, g.K, true);
      groups.push_back(g);
    }
    z_n = (int)tiles.size() - z_0;
    if (alloc(&d_groups, groups.size()) || alloc(&d_tiles, tiles.size()) ||
        cudaMemcpy(d_groups, groups.data(), groups.size() * sizeof(GemmGroup),
                   cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_tiles, tiles.data(), tiles.size() * sizeof(GemmTile),
                   cudaMemcpyHostToDevice)) {
      *err = "MP2 batch: out of memory for the FP64 plan";
      return GBJK_OOM;
    }
    return GBJK_OK;
  }

  gbjk_status plan_split(cudaStream_t st, int nbf, int naux, int nblk,
                         const std::vector<int>& bsize, const std::vector<int>& boff,
                         const std::vector<int>& panelK, const std::vector<int>& cmoff,
                         SplitState& sp, std::string* err) {
    if (sp.nbatch != 1) {
      *err = "MP2 batch: the split path needs the whole auxiliary range (no auxiliary batching)";
      return GBJK_INVALID_ARG;
    }
    // digit buffers
    c_nrb = cdiv_(hld, kTileN) * (kTileN / 32);
    std::vector<long long> cdig_off(nblk);
    cdig_stride = 0;
    for (int I = 0; I < nblk; ++I) {
      cdig_off[I] = cdig_stride;
      cdig_stride += (long long)c_nrb * sp.nkt[I] * kSlices * kImage;
    }
    h_nrb = cdiv_(nrho, kTileM) * (kTileM / 32);
    h_nkt = cdiv_(nbf, kTileK);
    hdig_stride = (long long)h_nrb * h_nkt * kSlices * kImage;
    lv_nrb = cdiv_(vld, kTileN) * (kTileN / 32);
    lvdig_stride = (long long)lv_nrb * h_nkt * kSlices * kImage;
    w_nrb = std::max(cdiv_(naux, kTileM) * (kTileM / 32), cdiv_(naux, kTileN) * (kTileN / 32));
    // Z tiles: a staircase over the upper triangle (column tiles of row
    // tile r0 start at r0), fewer than on the grid
    std::vector<std::pair<int, int>> ztiles;
    for (int r0 = 0; r0 < naux; r0 += kTileM)
      for (int c0 = r0; c0 < naux; c0 += kTileN) ztiles.push_back({r0, c0});
    for (const auto& zt : ztiles) w_nrb = std::max(w_nrb, cdiv_(zt.second + kTileN, 32));
    const int ntile = (int)ztiles.size();
    w_nkt = cdiv_(kw, kTileK);
    wdig_stride = (long long)w_nrb * w_nkt * kSlices * kImage;
    const int ks = sp.choose_ksplit(w_nkt, ntile * npts);
    const int kt_per = cdiv_(w_nkt, ks);
    ksplit = cdiv_(w_nkt, kt_per);
    const size_t nn = (size_t)naux * naux;
    if (alloc(&d_Cdig, (size_t)npts * cdig_stride) || alloc(&d_Hdig, (size_t)npts * hdig_stride) ||
        alloc(&d_Lvdig, (size_t)npts * lvdig_stride) ||
        alloc(&d_Wdig, (size_t)npts * wdig_stride) ||
        alloc(&d_eC, (size_t)npts * nblk * c_nrb * 32) ||
        alloc(&d_eH, (size_t)npts * h_nrb * 32) || alloc(&d_eLv, (size_t)npts * lv_nrb * 32) ||
        alloc(&d_eW, (size_t)npts * w_nrb * 32) ||
        alloc(&d_Zpart, (size_t)ksplit * npts * nn) ||
        cudaMemsetAsync(d_Cdig, 0, (size_t)npts * cdig_stride * 2, st) ||
        cudaMemsetAsync(d_Hdig, 0, (size_t)npts * hdig_stride * 2, st) ||
        cudaMemsetAsync(d_Lvdig, 0, (size_t)npts * lvdig_stride * 2, st) ||
        cudaMemsetAsync(d_Wdig, 0, (size_t)npts * wdig_stride * 2, st) ||
        cudaMemsetAsync(d_eC, 0, (size_t)npts * nblk * c_nrb * 32 * 4, st) ||
        cudaMemsetAsync(d_eH, 0, (size_t)npts * h_nrb * 32 * 4, st) ||
        cudaMemsetAsync(d_eLv, 0, (size_t)npts * lv_nrb * 32 * 4, st)) {
      *err = "MP2 batch: out of device memory for the operand digits";
      return GBJK_OOM;
    }
    // jobs
    std::vector<SplitJob> jobs;
    jc_0 = 0;
    c_maxthr = 0;
    for (int t = 0; t < npts; ++t)
      for (int I = 0; I < nblk; ++I) {
        SplitJob j;
        j.src = d_Cg + t * cg_stride + (long long)cmoff[I] * hld;
        j.rs = 1;
        j.cs = hld;
        j.row0 = 0;
        j.nrows = ro[t];
        j.ncols = panelK[I];
        j.e = d_eC + ((long long)t * nblk + I) * c_nrb * 32;
        j.e_biased = 0;
        j.nrb = c_nrb;
        j.nkt = sp.nkt[I];
        j.dst = d_Cdig + t * cdig_stride + cdig_off[I];
        jobs.push_back(j);
        c_maxthr = std::max(c_maxthr, (ro[t] / 8 + 2) * sp.nkt[I] * 32);
      }
    jlv_0 = (int)jobs.size();
    for (int t = 0; t < npts; ++t) {
      SplitJob j;
      j.src = d_Lv + (long long)t * nbf * vld;
      j.rs = 1;
      j.cs = vld;
      j.row0 = 0;
      j.nrows = rv[t];
      j.ncols = nbf;
      j.e = d_eLv + (long long)t * lv_nrb * 32;
      j.e_biased = 0;
      j.nrb = lv_nrb;
      j.nkt = h_nkt;
      j.dst = d_Lvdig + t * lvdig_stride;
      jobs.push_back(j);
    }
    jh_0 = (int)jobs.size();
    for (int t = 0; t < npts; ++t) {
      SplitJob j;
      j.src = d_H + t * h_stride;  // row rho = (X, i), column n at stride nrho
      j.rs = 1;
      j.cs = nrho;
      j.row0 = 0;
      j.nrows = (int)nrho;
      j.ncols = nbf;
      j.e = d_eH + (long long)t * h_nrb * 32;
      j.e_biased = 0;
      j.nrb = h_nrb;
      j.nkt = h_nkt;
      j.dst = d_Hdig + t * hdig_stride;
      jobs.push_back(j);
    }
    jw_0 = (int)jobs.size();
    for (int t = 0; t < npts; ++t) {
      SplitJob j;
      j.src = d_W + t * w_stride;
      j.rs = kw;
      j.cs = 1;
      j.row0 = 0;
      j.nrows = naux;
      j.ncols = kw;
      j.e = (int*)d_eW + (long long)t * w_nrb * 32;
      j.e_biased = 0;
      j.nrb = w_nrb;
      j.nkt = w_nkt;
      j.dst = d_Wdig + t * wdig_stride;
      jobs.push_back(j);
    }
    // items
    std::vector<SplitItem> items;
    auto base_item = []() {
      SplitItem w;
      w.emax = nullptr;
      w.emax_row0 = 0;
      w.emax_div = 1;
      w.out2 = nullptr;
      w.c0 = 0;
      w.ncol1 = 1 << 30;
      return w;
    };
    // T1 items: the points' tiles of one A row tile are adjacent in the list
    // (and so run at the same time on different SMs), so the L^-1 B digit
    // tile is read from HBM once for all points and then served from L2
    i1_0 = 0;
    for (int I = 0; I < nblk; ++I) {
      // A rows (m, Y) at m * sp.apitch + Y (SplitItem::apitch)
      const long long rows = (long long)bsize[I] * sp.apitch;
      for (int mt = 0; mt < cdiv_(rows, kTileM); ++mt)
        for (int t = 0; t < npts; ++t)
          for (int nt = 0; nt < cdiv_(ro[t], kTileN); ++nt) {
            SplitItem w = base_item();
            w.a = sp.d_Aslices + sp.a_off[I];
            w.a_nrb = sp.a_nrb[I];
            w.a_rb0 = mt * (kTileM / 32);
            w.apitch = sp.apitch;
            w.arow0 = mt * kTileM;
            w.ay_valid = naux;
            w.b = d_Cdig + t * cdig_stride + cdig_off[I];
            w.b_nrb = c_nrb;
            w.b_rb0 = nt * (kTileN / 32);
            w.kt0 = 0;
            w.nkt = sp.nkt[I];
            w.ea = sp.d_eA + sp.eA_off[I] + (long long)mt * kTileM;
            w.eb = d_eC + ((long long)t * nblk + I) * c_nrb * 32 + (long long)nt * kTileN;
            w.out = d_H + t * h_stride + ((long long)boff[I] * naux + (long long)mt * kTileM) * hld +
                    (long long)nt * kTileN;
            w.ldr = hld;
            w.m_valid = (int)std::min<long long>(kTileM, rows - (long long)mt * kTileM);
            w.n_valid = std::min(kTileN, ro[t] - nt * kTileN);
            items.push_back(w);
          }
    }
    i1_n = (int)items.size();
    i2_0 = (int)items.size();
    for (int t = 0; t < npts; ++t)
      for (int mt = 0; mt < cdiv_(nrho, kTileM); ++mt)
        for (int nt = 0; nt < cdiv_(rv[t], kTileN); ++nt) {
          SplitItem w = base_item();
          w.a = d_Hdig + t * hdig_stride;
          w.a_nrb = h_nrb;
          w.a_rb0 = mt * (kTileM / 32);
          w.b = d_Lvdig + t * lvdig_stride;
          w.b_nrb = lv_nrb;
          w.b_rb0 = nt * (kTileN / 32);
          w.kt0 = 0;
          w.nkt = h_nkt;
          w.ea = d_eH + (long long)t * h_nrb * 32 + (long long)mt * kTileM;
          w.eb = d_eLv + (long long)t * lv_nrb * 32 + (long long)nt * kTileN;
          w.out = d_W + t * w_stride + (long long)mt * kTileM * vld + (long long)nt * kTileN;
          w.ldr = vld;
          w.m_valid = (int)std::min<long long>(kTileM, nrho - (long long)mt * kTileM);
          w.n_valid = std::min(kTileN, rv[t] - nt * kTileN);
          // row rho = X * hld + i of W belongs to auxiliary row X
          w.emax = d_eW + (long long)t * w_nrb * 32;
          w.emax_row0 = mt * kTileM;
          w.emax_div = hld;
          items.push_back(w);
        }
    i2_n = (int)items.size() - i2_0;
    iz_0 = (int)items.size();
    for (int k = 0; k < ksplit; ++k) {
      const int kt0 = k * kt_per, n_kt = std::min(kt_per, w_nkt - kt0);
      for (int t = 0; t < npts; ++t)
        for (const auto& zt : ztiles) {
            const int r0 = zt.first, c0 = zt.second;
            SplitItem w = base_item();
            w.a = d_Wdig + t * wdig_stride;
            w.a_nrb = w_nrb;
            w.a_rb0 = r0 / 32;
            w.b = w.a;
            w.b_nrb = w_nrb;
            w.b_rb0 = c0 / 32;
            w.kt0 = kt0;
            w.nkt = n_kt;
            const int* eW = (const int*)d_eW + (long long)t * w_nrb * 32;
            w.ea = eW + r0;
            w.eb = eW + c0;
            w.out = d_Zpart + ((long long)k * npts + t) * nn + (long long)r0 * naux + c0;
            w.ldr = naux;
            w.m_valid = std::min(kTileM, naux - r0);
            w.n_valid = std::min(kTileN, naux - c0);
            items.push_back(w);
          }
    }
    iz_n = (int)items.size() - iz_0;
    if (alloc(&d_items, items.size()) || alloc(&d_jobs, jobs.size()) ||
        cudaMemcpy(d_items, items.data(), items.size() * sizeof(SplitItem),
                   cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_jobs, jobs.data(), jobs.size() * sizeof(SplitJob), cudaMemcpyHostToDevice)) {
      *err = "MP2 batch: out of memory for the work lists";
      return GBJK_OOM;
    }
    return GBJK_OK;
  }

  // Upload the padded factors (host arrays nbf x ro[t] and nbf x rv[t]),
  // ordered on the stream after any evaluation still in flight.
  gbjk_status upload(cudaStream_t st, int nbf, const double* const* Lo, const double* const* Lv,
                     std::string* err) {
    std::vector<double> lo((size_t)npts * nbf * hld, 0.0), lv((size_t)npts * nbf * vld, 0.0);
    for (int t = 0; t < npts; ++t)
      for (int m = 0; m < nbf; ++m) {
        std::copy(Lo[t] + (size_t)m * ro[t], Lo[t] + (size_t)(m + 1) * ro[t],
                  lo.begin() + ((size_t)t * nbf + m) * hld);
        std::copy(Lv[t] + (size_t)m * rv[t], Lv[t] + (size_t)(m + 1) * rv[t],
                  lv.begin() + ((size_t)t * nbf + m) * vld);
      }
    if (cudaMemcpyAsync(d_Lo, lo.data(), lo.size() * 8, cudaMemcpyHostToDevice, st) ||
        cudaMemcpyAsync(d_Lv, lv.data(), lv.size() * 8, cudaMemcpyHostToDevice, st) ||
        cudaStreamSynchronize(st)) {
      *err = "MP2 batch: factor upload failed";
      return GBJK_CUDA_ERROR;
    }
    have_result = false;
    return GBJK_OK;
  }

  // --- one evaluation of every point ------------------------------------------
  gbjk_status run(cudaStream_t st, int nbf, int naux, int nblk, int ncols_total,
                  const int* d_colmap, SplitState& sp, int64_t* launches, std::string* err) {
    const long long nn = (long long)naux * naux;
    {
      Scope sc(this, kOps, st);
      k_mp2_gather<<<dim3(cdiv_((long long)ncols_total * hld, 256), npts), 256, 0, st>>>(
          d_Lo, (long long)nbf * hld, hld, d_colmap, ncols_total, d_Cg, cg_stride);
      (*launches)++;
    }
    if (precision == GBJK_SPLIT_BF16) {
      gbjk_status s;
      {
        Scope sc(this, kOps, st);
        const int maxrows = std::max(*std::max_element(ro.begin(), ro.end()),
                                     *std::max_element(rv.begin(), rv.end()));
        k_row_maxexp<<<dim3(cdiv_((long long)maxrows * 32, 256), npts * nblk + npts), 256, 0, st>>>(
            d_jobs + jc_0);
        k_split_tiles<<<dim3(cdiv_(c_maxthr, 256), npts * nblk), 256, 0, st>>>(d_jobs + jc_0);
        const long long lvthr = (long long)(vld / 8 + 2) * h_nkt * 32;
        k_split_tiles<<<dim3(cdiv_(lvthr, 256), npts), 256, 0, st>>>(d_jobs + jlv_0);
        *launches += 3;
      }
      {
        Scope sc(this, kT1, st);
        if ((s = sp.launch_gemm(st, d_items + i1_0, i1_n, launches, err))) return s;
      }
      {
        Scope sc(this, kOps, st);
        k_mp2_colmax_exp<<<dim3(cdiv_(nrho, 256), npts), 256, 0, st>>>(
            d_H, h_stride, nbf, nrho, d_eH, (long long)h_nrb * 32);
        const long long hthr = (nrho / 8 + 2) * (long long)h_nkt * 32;
        k_split_tiles<<<dim3(cdiv_(hthr, 256), npts), 256, 0, st>>>(d_jobs + jh_0);
        *launches += 2;
        if (cudaMemsetAsync(d_eW, 0, (size_t)npts * w_nrb * 32 * 4, st) != cudaSuccess) {
          *err = "MP2 batch: memset failed";
          return GBJK_CUDA_ERROR;
        }
      }
      {
        Scope sc(this, kT2, st);
        if ((s = sp.launch_gemm(st, d_items + i2_0, i2_n, launches, err))) return s;
      }
      {
        Scope sc(this, kOps, st);
        k_exp_unbias<<<cdiv_((long long)npts * w_nrb * 32, 256), 256, 0, st>>>(
            (int*)d_eW, npts * w_nrb * 32);
        const long long wthr = (long long)(naux / 8 + 2) * w_nkt * 32;
        k_split_tiles<<<dim3(cdiv_(wthr, 256), npts), 256, 0, st>>>(d_jobs + jw_0);
        *launches += 2;
      }
      {
        Scope sc(this, kZ, st);
        if ((s = sp.launch_gemm(st, d_items + iz_0, iz_n, launches, err))) return s;
      }
      {
        Scope sc(this, kOps, st);
        k_mp2_z_reduce<<<dim3(cdiv_(nn, 256), npts), 256, 0, st>>>(d_Zpart, ksplit, npts, naux,
                                                                   d_Z);
        (*launches)++;
      }
    } else {
      auto gemm = [&](int ph, int tile0, int ntiles, int kind) {
        Scope sc(this, ph, st);
        for (int t0 = 0; t0 < ntiles; t0 += (1 << 20)) {
          const int n = std::min(1 << 20, ntiles - t0);
          if (kind == 0)
            k_gemm_fp64<false><<<n, 256, 0, st>>>(d_groups, d_tiles + tile0 + t0, 1.0);
          else if (kind == 1)
            k_gemm_fp64<false, true><<<n, 256, 0, st>>>(d_groups, d_tiles + tile0 + t0, 1.0);
          else
            k_gemm_fp64<true><<<n, 256, 0, st>>>(d_groups, d_tiles + tile0 + t0, 1.0);
          (*launches)++;
        }
      };
      gemm(kT1, t1_0, t1_n, 0);
      gemm(kT2, t2_0, t2_n, 1);
      gemm(kZ, z_0, z_n, 2);
      Scope sc(this, kOps, st);
      k_mp2_z_mirror<<<dim3(cdiv_(nn, 256), npts), 256, 0, st>>>(d_Z, naux);
      (*launches)++;
    }
    {
      Scope sc(this, kOps, st);
      k_mp2_rowsq<<<dim3(cdiv_((long long)naux * 32, 256), npts), 256, 0, st>>>(d_Z, naux, d_rsq);
      k_mp2_energy<<<cdiv_(npts, 32), 32, 0, st>>>(d_rsq, naux, npts, d_E);
      *launches += 2;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      *err = std::string("MP2 batch launch: ") + cudaGetErrorString(e);
      return GBJK_CUDA_ERROR;
    }
    have_result = true;
    return GBJK_OK;
  }
};

}  // namespace gbjk
