// Host side of the split-precision K path: operand preparation and launch
// plans.
//
// Once per tensor upload:
//   Bfit = L^-1 B per panel row block (FP64 grouped GEMM, temporary), its row
//   exponents and slice images (the A operands of the half transform).
// Per nocc: buffers and the two work lists (half transform, exchange).
// Per build (stream-ordered, no host sync):
//   C digits (B operand of every panel) -> split GEMM Hfit = Bfit C (FP64,
//   row exponents by atomicMax) -> H digits -> split GEMM
//   Kpart = Hfit Hfit^T (upper tiles, split-K) -> ordered reduce
//   K = -sum Kpart.
// With hfuse the half-transform epilogue cuts the digits of Hfit itself
// (one exponent per AO function and group of 32 auxiliary indices) and the
// exchange is the segmented variant that applies those exponents.
// The A operand rows (m, y) of panel I sit at m * pad32(batch) + y, so that
// every 32-row block is one AO function and one auxiliary group.
// With the fit folded into the tensor, DF-MO and DF-LMO compute the same
// K = -(L^-1 B C)^T (L^-1 B C).
#pragma once
#include <algorithm>
#include <string>
#include <vector>

#include "kernels_fp64.cuh"
#include "split_gemm.cuh"

namespace gbjk {

struct SplitState {
  size_t bytes = 0;
  uint64_t frees = 0;  // buffers freed so far (a captured build using them is stale)
  int nbf = 0, naux = 0, nblk = 0;
  std::vector<int> bsize, boff, panelK, cmoff;
  std::vector<long long> panel_off;
  bool b_ready = false;
  int nocc = -1;
  // A operands and the prefitted tensor L^-1 B (FP64).  With `fitted` the
  // uploaded tensor already is L^-1 B and Bfit aliases it.
  bool fitted = false;
  bool bfit_owned = false;
  double* Bfit = nullptr;
  // compact copy of Bfit for the mixed-path J (k_encode_f32i16: FP32 hi and
  // a 16-bit remainder per element, 6 bytes; rows padded to a multiple of 8,
  // panels at d_cpo[I]), unbatched only
  float* d_Bhi = nullptr;
  uint16_t* d_Blo = nullptr;
  long long* d_cpo = nullptr;
  // the context's device copies of the panel layout (not owned)
  const long long* dd_panel_off = nullptr;
  const int *dd_blk_of = nullptr, *dd_boff = nullptr, *dd_panelK = nullptr;
  uint16_t* d_Aslices = nullptr;
  // auxiliary batching: xb auxiliary rows per batch (nbatch > 1 streams the
  // half transform and the exchange batch by batch; A digits per batch)
  int xb_req = 0, xb = 0, nbatch = 1;
  // A-row pitch of the full batch: pad32(xb) (pad32(naux) unbatched)
  int apitch = 0;
  // fused digit cut of H in the half transform (requested; in effect for
  // the per-nocc buffers).  Off by default: on GB300 the fused half
  // transform and segmented exchange together take longer than the FP64 H
  // round trip and digit pass they replace.
  bool hfuse = false, hfuse_eff = false;
  SplitJob* d_bjobs = nullptr;  // A-digit jobs, nbatch * nbf (one per (batch, mu))
  int bjob_maxthr = 0;
  std::vector<long long> a_off, eA_off;
  std::vector<int> a_nrb, nkt;
  int* d_eA = nullptr;
  // per build
  uint16_t* d_Cslices = nullptr;
  std::vector<long long> c_off;
  int c_nrb = 0;
  int* d_eC = nullptr;
  double* d_H = nullptr;
  uint16_t* d_Hslices = nullptr;
  int h_nrb = 0, h_nkt = 0, hld = 0;
  int* d_eH = nullptr;
  int* d_eHs = nullptr;  // fused: exponents [mu][auxiliary group], es_ld per row
  int es_ld = 0;
  double* d_Kpart = nullptr;
  double* d_dpart = nullptr;  // J partials [mu][Y] from the density columns
  double* d_dt = nullptr;     // L^-1 g
  int ksplit = 1;
  int maxb = 0;
  SplitItem* d_items = nullptr;
  int ht_nitems = 0, k_nitems = 0;
  SplitJob* d_jobs = nullptr;  // [0,nblk): C rows, [nblk,2nblk): P rows, [2nblk]: H
  int c_maxthreads = 0, c_maxrows = 0;
  long long h_threads = 0;
  int* d_err = nullptr;
  const double* d_Cg = nullptr;
  int nsm = 148;
  bool profile = false;
  // set by the caller for one build: event recorded right after the half
  // transform (the fork point of the J column sums), and the number of SMs
  // the exchange GEMM leaves free (0: all SMs)
  cudaEvent_t ev_ht = nullptr;
  int k_grid = 0;
  // requested exchange k parts (0 = choose_ksplit) and the number in effect
  int ks_req = 0, ks_eff = 0;
  // test hook (gbjk_test_split_stall): the producer stops at this work item
  // of every split GEMM launch (-1: never), and the waits' time limit
  int stop_item = -1;
  unsigned long long spin_ns = kSpinNs;
  double ms[4] = {0, 0, 0, 0};
  int64_t nl[4] = {0, 0, 0, 0};
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;

  void set_dev_layout(const long long* po, const int* blk_of, const int* bo, const int* pk) {
    dd_panel_off = po;
    dd_blk_of = blk_of;
    dd_boff = bo;
    dd_panelK = pk;
  }
  void init(int nbf_, int naux_, int nblk_, const std::vector<int>& bs,
            const std::vector<int>& bo, const std::vector<int>& pk, const std::vector<int>& cmo,
            const std::vector<long long>& po) {
    nbf = nbf_;
    naux = naux_;
    nblk = nblk_;
    bsize = bs;
    boff = bo;
    panelK = pk;
    cmoff = cmo;
    panel_off = po;
  }
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
    if (*p) {
      cudaFree(*p);
      frees++;
    }
    *p = nullptr;
  }
  void release_build() {
    free_(&d_Cslices);
    free_(&d_eC);
    free_(&d_H);
    free_(&d_Hslices);
    free_(&d_eH);
    free_(&d_eHs);
    free_(&d_Kpart);
    free_(&d_dpart);
    free_(&d_dt);
    free_(&d_items);
    free_(&d_jobs);
    plans.clear();
    nocc = -1;
  }
  void release() {
    release_build();
    if (bfit_owned) free_(&Bfit);
    Bfit = nullptr;
    bfit_owned = false;
    free_(&d_Bhi);
    free_(&d_Blo);
    free_(&d_cpo);
    free_(&d_Aslices);
    free_(&d_bjobs);
    free_(&d_eA);
    free_(&d_err);
    for (auto& pe : pending) {
      cudaEventDestroy(pe.second.first);
      cudaEventDestroy(pe.second.second);
    }
    pending.clear();
    b_ready = false;
    bytes = 0;
  }
  void invalidate_b() { release(); }
  void reset_profile() {
    resolve();
    for (int i = 0; i < 4; ++i) {
      ms[i] = 0;
      nl[i] = 0;
    }
  }
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
  int profile_read(int idx, const char** name, double* out_ms, int64_t* launches) {
    static const char* names[4] = {"split_gemm_ht", "split_gemm_k", "split_digits", "prefit"};
    if (idx < 0 || idx >= 4) return 0;
    resolve();
    if (name) *name = names[idx];
    if (out_ms) *out_ms = ms[idx];
    if (launches) *launches = nl[idx];
    return 1;
  }
  struct Scope {
    SplitState* s;
    int ph;
    cudaStream_t st;
    cudaEvent_t a = nullptr, b = nullptr;
    Scope(SplitState* s_, int p, cudaStream_t st_) : s(s_), ph(p), st(st_) {
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

  static int cdiv_(long long a, long long b) { return (int)((a + b - 1) / b); }
  // H rows hold the half transform in groups of 32 auxiliary indices (the
  // column-pair-outermost layout of SplitItem::perm_rs), so a batch of xbc
  // auxiliary rows spans pad32(xbc) * hld columns of H
  static int pad32(int x) { return (x + 31) & ~31; }

  // variant: 0 plain, 1 half transform with digit output, 2 segmented exchange
  bool attr_v[3] = {false, false, false};
  template <bool kH, bool kS>
  gbjk_status launch_gemm_v(cudaStream_t st, SplitItem* items, int n, int64_t* launches,
                            std::string* err, int leave_sms) {
    if (n == 0) return GBJK_OK;
    const int v = kH ? 1 : (kS ? 2 : 0);
    if (!attr_v[v]) {
      if (cudaFuncSetAttribute(k_split_gemm<kH, kS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               kSmemBytes) != cudaSuccess) {
        *err = "cannot reserve shared memory for the split GEMM";
        return GBJK_CUDA_ERROR;
      }
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      attr_v[v] = true;
    }
    const int grid = std::min(n, std::max(1, nsm - leave_sms));
    k_split_gemm<kH, kS><<<grid, kThreads, kSmemBytes, st>>>(items, n, d_err, stop_item, spin_ns);
    (*launches)++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      *err = std::string("split GEMM launch: ") + cudaGetErrorString(e);
      return GBJK_CUDA_ERROR;
    }
    return GBJK_OK;
  }
  gbjk_status launch_gemm(cudaStream_t st, SplitItem* items, int n, int64_t* launches,
                          std::string* err, int leave_sms = 0) {
    return launch_gemm_v<false, false>(st, items, n, launches, err, leave_sms);
  }

  // --- once per tensor: prefit and A-operand digits -----------------------
  gbjk_status prepare_b(cudaStream_t st, const double* d_B, const double* d_Linv,
                        int64_t* launches, std::string* err) {
    const long long nnz = panel_off.back() + (long long)bsize.back() * naux * panelK.back();
    if (alloc(&d_err, 1) != cudaSuccess || cudaMemsetAsync(d_err, 0, sizeof(int), st) != cudaSuccess) {
      *err = "split path: cannot allocate the error flag";
      return GBJK_OOM;
    }
    // batches of a multiple of 32 auxiliary rows, so that only the last
    // (shorter) batch has unused slots in its last 32-index group of H
    xb = (xb_req > 0 && xb_req < naux) ? std::max(32, xb_req & ~31) : naux;
    if (xb > naux) xb = naux;
    nbatch = (naux + xb - 1) / xb;
    apitch = pad32(xb);
    double* d_Bfit = nullptr;
    if (fitted) {
      d_Bfit = const_cast<double*>(d_B);
      bfit_owned = false;
    } else {
      if (alloc(&d_Bfit, (size_t)nnz) != cudaSuccess) {
        *err = "split path: out of memory for the prefitted tensor";
        return GBJK_OOM;
      }
      bfit_owned = true;
      // Bfit_I[m] = L^-1 B_I[m]  (naux x K_I per AO function m)
      std::vector<GemmGroup> groups;
      std::vector<GemmTile> tiles;
      for (int I = 0; I < nblk; ++I) {
        const int K = panelK[I];
        if (K == 0) continue;
        for (int m = 0; m < bsize[I]; ++m) {
          GemmGroup g;
          const long long off = panel_off[I] + (long long)m * naux * K;
          g.A = d_Linv;
          g.B = d_B + off;
          g.C = d_Bfit + off;
          g.M = naux;
          g.N = K;
          g.K = naux;
          g.lda = naux;
          g.ldb = K;
          g.ldc = K;
          g.flags = kLowerA;
          for (int mt = 0; mt < cdiv_(naux, 64); ++mt)
            for (int nt = 0; nt < cdiv_(K, 64); ++nt)
              tiles.push_back({(int)groups.size(), mt, nt, 0, naux, 0});
          groups.push_back(g);
        }
      }
      GemmGroup* dg = nullptr;
      GemmTile* dt = nullptr;
      if (alloc(&dg, groups.size()) != cudaSuccess || alloc(&dt, tiles.size()) != cudaSuccess) {
        free_(&dg);
        free_(&d_Bfit);
        *err = "split path: out of memory for the prefit plan";
        return GBJK_OOM;
      }
      cudaMemcpy(dg, groups.data(), groups.size() * sizeof(GemmGroup), cudaMemcpyHostToDevice);
      cudaMemcpy(dt, tiles.data(), tiles.size() * sizeof(GemmTile), cudaMemcpyHostToDevice);
      {
        Scope sc(this, 3, st);
        // the grid limit is 2^31-1 blocks; launch in slices of 1M tiles
        for (size_t t0 = 0; t0 < tiles.size(); t0 += (1u << 20)) {
          const int n = (int)std::min<size_t>(1u << 20, tiles.size() - t0);
          k_gemm_fp64<false><<<n, 256, 0, st>>>(dg, dt + t0, 1.0);
          (*launches)++;
        }
      }
      cudaStreamSynchronize(st);
      cudaFree(dg);
      cudaFree(dt);
    }
    Bfit = d_Bfit;
    if (nbatch == 1) {
      // the mixed-mode J reads L^-1 B once per build: a 6-byte copy
      std::vector<long long> cpo(nblk);
      long long ncomp = 0;
      for (int I = 0; I < nblk; ++I) {
        cpo[I] = ncomp;
        ncomp += (long long)bsize[I] * naux * ((panelK[I] + 7) & ~7);
      }
      if (alloc(&d_Bhi, (size_t)ncomp) != cudaSuccess ||
          alloc(&d_Blo, (size_t)ncomp) != cudaSuccess || alloc(&d_cpo, (size_t)nblk) != cudaSuccess ||
          cudaMemcpy(d_cpo, cpo.data(), nblk * sizeof(long long), cudaMemcpyHostToDevice) !=
              cudaSuccess) {
        *err = "split path: out of memory for the compact J tensor";
        return GBJK_OOM;
      }
      Scope sc(this, 3, st);
      k_encode_f32i16<<<dim3(naux, nbf), 128, 0, st>>>(d_Bfit, dd_panel_off, d_cpo, dd_blk_of,
                                                      dd_boff, dd_panelK, naux, d_Bhi, d_Blo);
      (*launches)++;
    }
    // A operands: rows (m, y) of panel I, y < xb (all auxiliary rows when
    // not batched), at m * pad32(batch) + y; columns k
    a_off.assign(nblk, 0);
    eA_off.assign(nblk, 0);
    a_nrb.assign(nblk, 0);
    nkt.assign(nblk, 0);
    long long atot = 0, etot = 0;
    for (int I = 0; I < nblk; ++I) {
      const long long rows = (long long)bsize[I] * apitch;
      a_nrb[I] = cdiv_(rows, kTileM) * (kTileM / 32);
      nkt[I] = std::max(1, cdiv_(panelK[I], kTileK));
      a_off[I] = atot;
      eA_off[I] = etot;
      atot += (long long)a_nrb[I] * nkt[I] * kSlices * kImage;
      etot += (long long)a_nrb[I] * 32;
    }
    if (alloc(&d_Aslices, (size_t)atot) != cudaSuccess || alloc(&d_eA, (size_t)etot) != cudaSuccess ||
        cudaMemsetAsync(d_Aslices, 0, (size_t)atot * 2, st) != cudaSuccess ||
        cudaMemsetAsync(d_eA, 0, (size_t)etot * 4, st) != cudaSuccess) {
      *err = "split path: out of memory for the operand digits";
      return GBJK_OOM;
    }
    if (nbatch == 1) {
      // one job per AO function: its naux rows (m, y) at m * apitch + y
      std::vector<SplitJob> jobs(nbf);
      long long maxthr = 0;
      for (int I = 0; I < nblk; ++I)
        for (int m = 0; m < bsize[I]; ++m) {
          SplitJob& j = jobs[boff[I] + m];
          j.src = d_Bfit + panel_off[I] + (long long)m * naux * panelK[I];
          j.rs = panelK[I];
          j.cs = 1;
          j.row0 = m * apitch;
          j.nrows = naux;
          j.ncols = panelK[I];
          j.e = d_eA + eA_off[I];
          j.e_biased = 0;
          j.nrb = a_nrb[I];
          j.nkt = nkt[I];
          j.dst = d_Aslices + a_off[I];
          maxthr = std::max(maxthr, (long long)(naux / 8 + 2) * j.nkt * 32);
        }
      SplitJob* dj = nullptr;
      if (alloc(&dj, jobs.size()) != cudaSuccess) {
        *err = "split path: out of memory";
        return GBJK_OOM;
      }
      cudaMemcpy(dj, jobs.data(), jobs.size() * sizeof(SplitJob), cudaMemcpyHostToDevice);
      {
        Scope sc(this, 2, st);
        k_row_maxexp<<<dim3(cdiv_((long long)naux * 32, 256), nbf), 256, 0, st>>>(dj);
        k_split_tiles<<<dim3(cdiv_(maxthr, 256), nbf), 256, 0, st>>>(dj);
        *launches += 2;
      }
      cudaStreamSynchronize(st);
      cudaFree(dj);
    } else {
      // one job per (batch, AO function): rows (m, y) of its panel
      std::vector<SplitJob> jobs((size_t)nbatch * nbf);
      bjob_maxthr = 0;
      for (int b = 0; b < nbatch; ++b) {
        const int Y0 = b * xb, xbc = std::min(xb, naux - Y0);
        for (int I = 0; I < nblk; ++I)
          for (int m = 0; m < bsize[I]; ++m) {
            SplitJob& j = jobs[(size_t)b * nbf + boff[I] + m];
            j.src = d_Bfit + panel_off[I] + ((long long)m * naux + Y0) * panelK[I];
            j.rs = panelK[I];
            j.cs = 1;
            j.row0 = m * pad32(xbc);
            j.nrows = xbc;
            j.ncols = panelK[I];
            j.e = d_eA + eA_off[I];
            j.e_biased = 0;
            j.nrb = a_nrb[I];
            j.nkt = nkt[I];
            j.dst = d_Aslices + a_off[I];
            bjob_maxthr = std::max(bjob_maxthr, (xbc / 8 + 2) * nkt[I] * 32);
          }
      }
      if (alloc(&d_bjobs, jobs.size()) != cudaSuccess) {
        *err = "split path: out of memory for the batch jobs";
        return GBJK_OOM;
      }
      cudaMemcpy(d_bjobs, jobs.data(), jobs.size() * sizeof(SplitJob), cudaMemcpyHostToDevice);
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      *err = std::string("split path preparation: ") + cudaGetErrorString(e);
      return GBJK_CUDA_ERROR;
    }
    b_ready = true;
    return GBJK_OK;
  }

  // --- per nocc: buffers and work lists ------------------------------------
  // One plan per distinct auxiliary batch size (the last batch may be
  // shorter): item ranges of the half transform and of the exchange.
  struct BatchPlan {
    int xbc, ht0, nht, k0, nk, ksplit, hjob;
  };
  std::vector<BatchPlan> plans;

  // parts of the exchange's k range: requested, or by the wave model below;
  // never fewer than an item's int64 headroom allows (<= 8192 k per item)
  int exchange_ksplit(int nkt_total, int ntile) const {
    if (ks_req > 0) return std::max(cdiv_(nkt_total, 256), std::min(ks_req, nkt_total));
    return choose_ksplit(nkt_total, ntile);
  }
  int choose_ksplit(int nkt_total, int ntile) const {
    const int ks_min = cdiv_(nkt_total, 256);  // int64 headroom: <= 8192 k per item
    double best = 1e300;
    int pick = ks_min;
    for (int ks = ks_min; ks <= std::max(ks_min, 4 * nsm); ++ks) {
      const int per = cdiv_(nkt_total, ks);
      if (per < 8 && ks > ks_min) break;
      const long long waves = ((long long)ntile * ks + nsm - 1) / nsm;
      const double t = (double)waves * (per + 2.0);  // +2: per-item overhead in k-tiles
      if (t < best) {
        best = t;
        pick = ks;
      }
    }
    return pick;
  }

  gbjk_status prepare_nocc(cudaStream_t st, int nocc_, std::string* err) {
    release_build();
    const bool jfused = nbatch == 1;  // density rows ride along only unbatched
    maxb = 0;
    for (int I = 0; I < nblk; ++I) maxb = std::max(maxb, bsize[I]);
    // B operand rows of panel I: nocc orbitals, then b_I density rows
    const int ntn = cdiv_(nocc_ + (jfused ? maxb : 0), kTileN);
    c_nrb = ntn * (kTileN / 32);
    c_off.assign(nblk, 0);
    long long ctot = 0;
    for (int I = 0; I < nblk; ++I) {
      c_off[I] = ctot;
      ctot += (long long)c_nrb * nkt[I] * kSlices * kImage;
    }
    hld = nocc_ + (nocc_ & 1);  // even row stride: 16-byte aligned pairs
    hfuse_eff = hfuse;
    const bool fuse = hfuse_eff;
    es_ld = apitch / 32;  // auxiliary groups of a full batch
    const long long hk = (long long)pad32(xb) * hld;
    // exchange k-tiles of a batch: fused, one per (auxiliary group, orbital);
    // unfused, the FP64 H row of pad32(xbc) * hld values in 32-value tiles
    auto xk_nkt = [&](int xbc) {
      return fuse ? (pad32(xbc) / 32) * nocc_ : cdiv_((long long)pad32(xbc) * hld, kTileK);
    };
    h_nkt = xk_nkt(xb);
    h_nrb = std::max(cdiv_(nbf, kTileM) * (kTileM / 32), cdiv_(nbf, kTileN) * (kTileN / 32));
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // exchange output tiles: a staircase over the upper triangle, the
    // column tiles of row tile r0 starting at column r0 (32-row operand
    // blocks allow any multiple of 32); every (m, c >= m) lies in the row
    // tile of m.  nbf 490: 15 tiles of 128 x 96 instead of 17 on the grid.
    std::vector<std::pair<int, int>> ktiles;
    for (int r0 = 0; r0 < nbf; r0 += kTileM)
      for (int c0 = r0; c0 < nbf; c0 += kTileN) ktiles.push_back({r0, c0});
    const int ntile = (int)ktiles.size();
    for (const auto& t : ktiles) h_nrb = std::max(h_nrb, cdiv_(t.second + kTileN, 32));
    std::vector<int> sizes = {xb};
    const int xlast = naux - (nbatch - 1) * xb;
    if (xlast != xb) sizes.push_back(xlast);
    ksplit = 1;
    for (int xbc : sizes) ksplit = std::max(ksplit, exchange_ksplit(xk_nkt(xbc), ntile));
    const size_t nH = fuse ? 1 : (size_t)nbf * hk;
    const size_t nEs = fuse ? (size_t)h_nrb * 32 * es_ld : 1;
    if (alloc(&d_Cslices, (size_t)ctot) != cudaSuccess ||
        alloc(&d_eC, (size_t)nblk * c_nrb * 32) != cudaSuccess ||
        alloc(&d_H, nH) != cudaSuccess ||
        alloc(&d_Hslices, (size_t)h_nrb * h_nkt * kSlices * kImage) != cudaSuccess ||
        alloc(&d_eH, (size_t)h_nrb * 32) != cudaSuccess ||
        alloc(&d_eHs, nEs) != cudaSuccess ||
        alloc(&d_Kpart, (size_t)ksplit * nbf * nbf) != cudaSuccess ||
        alloc(&d_dpart, jfused ? (size_t)nbf * naux : 1) != cudaSuccess ||
        alloc(&d_dt, (size_t)naux) != cudaSuccess ||
        cudaMemsetAsync(d_Cslices, 0, (size_t)ctot * 2, st) != cudaSuccess ||
        cudaMemsetAsync(d_eC, 0, (size_t)nblk * c_nrb * 32 * 4, st) != cudaSuccess ||
        cudaMemsetAsync(d_H, 0, nH * 8, st) != cudaSuccess ||
        cudaMemsetAsync(d_Hslices, 0, (size_t)h_nrb * h_nkt * kSlices * kImage * 2, st) !=
            cudaSuccess) {
      release_build();
      *err = "split path: out of memory for the per-build buffers";
      return GBJK_OOM;
    }
    // group exponents of rows that no half transform writes (beyond nbf,
    // panels without columns) stay "all zero"
    k_fill_int<<<(int)std::min<size_t>(cdiv_((long long)nEs, 256), 4 * nsm), 256, 0, st>>>(
        d_eHs, (long long)nEs, -2000);
    std::vector<SplitItem> items;
    std::vector<SplitJob> jobs(2 * nblk);
    plans.clear();
    for (size_t pi = 0; pi < sizes.size(); ++pi) {
      const int xbc = sizes[pi];
      BatchPlan pl;
      pl.xbc = xbc;
      // half transform: Hfit rows (m, y) of panel I, columns i (+ density);
      // A rows at m * pad32(xbc) + y
      pl.ht0 = (int)items.size();
      for (int I = 0; I < nblk; ++I) {
        const long long rows = (long long)bsize[I] * pad32(xbc);
        const int ncolI = nocc_ + (jfused ? bsize[I] : 0);
        for (int mt = 0; mt < cdiv_(rows, kTileM); ++mt)
          for (int nt = 0; nt < cdiv_(ncolI, kTileN); ++nt) {
            SplitItem w;
            w.a = d_Aslices + a_off[I];
            w.a_nrb = a_nrb[I];
            w.a_rb0 = mt * (kTileM / 32);
            w.b = d_Cslices + c_off[I];
            w.b_nrb = c_nrb;
            w.b_rb0 = nt * (kTileN / 32);
            w.kt0 = 0;
            w.nkt = nkt[I];
            w.ea = d_eA + eA_off[I] + (long long)mt * kTileM;
            w.eb = d_eC + (long long)I * c_nrb * 32 + (long long)nt * kTileN;
            w.apitch = pad32(xbc);
            w.arow0 = mt * kTileM;
            w.ay_valid = xbc;
            if (fuse) {
              // digits of H rows boff[I] + m, k-tile (y / 32) * nocc + i
              w.out = nullptr;
              w.ldr = 0;
              w.hdig = d_Hslices;
              w.h_nrb = h_nrb;
              w.hrow0 = boff[I];
              w.eseg = d_eHs;
              w.es_ld = es_ld;
              w.seg_nkt = nocc_;
            } else {
              // column-pair-outermost layout: each epilogue store is one
              // contiguous 512-byte run (SplitItem::perm_rs)
              w.out = d_H + (long long)boff[I] * pad32(xbc) * hld + (long long)nt * kTileN * 32;
              w.ldr = hld;
              w.perm_rs = (long long)pad32(xbc) * hld;
              w.perm_div = xbc;
            }
            w.m_valid = (int)std::min<long long>(kTileM, rows - (long long)mt * kTileM);
            w.n_valid = std::min(kTileN, ncolI - nt * kTileN);
            // row (m, y) of panel I belongs to H row mu = boff[I] + m
            w.emax = (unsigned int*)d_eH + boff[I];
            w.emax_row0 = mt * kTileM;
            w.emax_div = xbc;
            // density column m' = col - nocc: g-partial of row (m, Y) if m' == m
            w.out2 = jfused ? d_dpart + (long long)boff[I] * naux : nullptr;
            w.c0 = nt * kTileN;
            w.ncol1 = nocc_;
            items.push_back(w);
          }
      }
      pl.nht = (int)items.size() - pl.ht0;
      // exchange: upper tiles, split over k
      const int nk_b = xk_nkt(xbc);
      const int ksb = exchange_ksplit(nk_b, ntile);
      const int kt_per = cdiv_(nk_b, ksb);
      pl.ksplit = cdiv_(nk_b, kt_per);
      pl.k0 = (int)items.size();
      for (int ks = 0; ks < pl.ksplit; ++ks) {
        const int kt0 = ks * kt_per;
        const int n_kt = std::min(kt_per, nk_b - kt0);
        for (const auto& t : ktiles) {
            const int r0 = t.first, c0 = t.second;
            SplitItem w;
            w.a = d_Hslices;
            w.a_nrb = h_nrb;
            w.a_rb0 = r0 / 32;
            w.b = d_Hslices;
            w.b_nrb = h_nrb;
            w.b_rb0 = c0 / 32;
            w.kt0 = kt0;
            w.nkt = n_kt;
            w.ea = d_eH + r0;
            w.eb = d_eH + c0;
            w.out = d_Kpart + (long long)ks * nbf * nbf + (long long)r0 * nbf + c0;
            w.ldr = nbf;
            w.m_valid = std::min(kTileM, nbf - r0);
            w.n_valid = std::min(kTileN, nbf - c0);
            w.emax = nullptr;
            w.emax_row0 = 0;
            w.emax_div = 1;
            w.out2 = nullptr;
            w.c0 = 0;
            w.ncol1 = 1 << 30;
            if (fuse) {
              // segment g = auxiliary group: nocc k-tiles with the
              // exponents of (row, g)
              w.seg_nkt = nocc_;
              w.esa = d_eHs + (long long)r0 * es_ld;
              w.esb = d_eHs + (long long)c0 * es_ld;
              w.es_ld = es_ld;
            }
            items.push_back(w);
          }
      }
      pl.nk = (int)items.size() - pl.k0;
      // digits of the half-transformed batch (exponents from the epilogue)
      SplitJob hj;
      hj.src = d_H;
      hj.rs = (long long)pad32(xbc) * hld;
      hj.cs = 1;
      hj.row0 = 0;
      hj.nrows = nbf;
      hj.ncols = (long long)pad32(xbc) * hld;
      hj.e = d_eH;
      hj.e_biased = 0;
      hj.nrb = h_nrb;
      hj.nkt = nk_b;
      hj.dst = d_Hslices;
      pl.hjob = (int)jobs.size();
      jobs.push_back(hj);
      plans.push_back(pl);
    }
    ht_nitems = plans[0].nht;
    ks_eff = plans[0].ksplit;
    k_nitems = plans[0].nk;
    c_maxthreads = 0;
    c_maxrows = std::max(nocc_, maxb);
    for (int I = 0; I < nblk; ++I) {
      SplitJob& pj = jobs[nblk + I];  // density rows: Pg panel rows (none when batched)
      pj.src = nullptr;               // set per build
      pj.rs = panelK[I];
      pj.cs = 1;
      pj.row0 = nocc_;
      pj.nrows = jfused ? bsize[I] : 0;
      pj.ncols = panelK[I];
      pj.e = d_eC + (long long)I * c_nrb * 32;
      pj.e_biased = 0;
      pj.nrb = c_nrb;
      pj.nkt = nkt[I];
      pj.dst = d_Cslices + c_off[I];
      SplitJob& j = jobs[I];
      j.src = nullptr;  // set per build (Cg pointer owned by the context)
      j.rs = 1;
      j.cs = nocc_;
      j.row0 = 0;
      j.nrows = nocc_;
      j.ncols = panelK[I];
      j.e = d_eC + (long long)I * c_nrb * 32;
      j.e_biased = 0;
      j.nrb = c_nrb;
      j.nkt = nkt[I];
      j.dst = d_Cslices + c_off[I];
      c_maxthreads = std::max(c_maxthreads, ((nocc_ + maxb) / 8 + 2) * nkt[I] * 32);
    }
    if (alloc(&d_items, items.size()) != cudaSuccess || alloc(&d_jobs, jobs.size()) != cudaSuccess) {
      release_build();
      *err = "split path: out of memory for the work lists";
      return GBJK_OOM;
    }
    cudaMemcpy(d_items, items.data(), items.size() * sizeof(SplitItem), cudaMemcpyHostToDevice);
    host_jobs = jobs;
    jobs_cg = jobs_pg = nullptr;
    nocc = nocc_;
    return GBJK_OK;
  }
  std::vector<SplitJob> host_jobs;
  const double* jobs_cg = nullptr;
  const double* jobs_pg = nullptr;

  gbjk_status prepare(cudaStream_t st, const double* d_B, const double* d_Linv,
                      const double* d_Cg_, const double* d_Pg, const std::vector<long long>& pg_off,
                      int nocc_, int64_t* launches, std::string* err) {
    gbjk_status s;
    if (!b_ready && (s = prepare_b(st, d_B, d_Linv, launches, err))) return s;
    if (nocc != nocc_ && (s = prepare_nocc(st, nocc_, err))) return s;
    if (jobs_cg != d_Cg_ || jobs_pg != d_Pg) {
      for (int I = 0; I < nblk; ++I) {
        host_jobs[I].src = d_Cg_ + (long long)cmoff[I] * nocc_;
        host_jobs[nblk + I].src = d_Pg + pg_off[I];
      }
      jobs_cg = d_Cg_;
      jobs_pg = d_Pg;
      if (cudaMemcpy(d_jobs, host_jobs.data(), host_jobs.size() * sizeof(SplitJob),
                     cudaMemcpyHostToDevice) != cudaSuccess) {
        *err = "split path: job upload failed";
        return GBJK_CUDA_ERROR;
      }
    }
    return GBJK_OK;
  }

  bool fused_j() const { return nbatch == 1; }

  // --- per build ------------------------------------------------------------
  gbjk_status run_k(cudaStream_t st, double* dK, int64_t* launches, std::string* err) {
    gbjk_status s;
    // the flag a timed-out wait sets is per build: cleared at its start
    if (cudaMemsetAsync(d_err, 0, sizeof(int), st) != cudaSuccess) {
      *err = "split path: memset failed";
      return GBJK_CUDA_ERROR;
    }
    {
      Scope sc(this, 2, st);
      k_row_maxexp<<<dim3(cdiv_((long long)c_maxrows * 32, 256), 2 * nblk), 256, 0, st>>>(d_jobs);
      k_split_tiles<<<dim3(cdiv_((long long)c_maxthreads, 256), 2 * nblk), 256, 0, st>>>(d_jobs);
      *launches += 2;
    }
    for (int b = 0; b < nbatch; ++b) {
      const BatchPlan& pl = plans[(b == nbatch - 1 && plans.size() > 1) ? 1 : 0];
      if (nbatch > 1) {
        Scope sc(this, 2, st);
        const SplitJob* bj = d_bjobs + (size_t)b * nbf;
        k_row_maxexp<<<dim3(cdiv_((long long)pl.xbc * 32, 256), nbf), 256, 0, st>>>(bj);
        k_split_tiles<<<dim3(cdiv_((long long)bjob_maxthr, 256), nbf), 256, 0, st>>>(bj);
        *launches += 2;
      }
      if (nbatch > 1 && !hfuse_eff && pad32(pl.xbc) != pl.xbc) {
        // the last batch's H layout reuses slots the full batches wrote:
        // clear its unused auxiliary slots
        Scope sc(this, 2, st);
        const long long per = (long long)nbf * (hld / 2) * (32 - (pl.xbc & 31));
        k_zero_hpad<<<(int)std::min<long long>(cdiv_(per, 256), 4LL * nsm), 256, 0, st>>>(
            d_H, nbf, (long long)pad32(pl.xbc) * hld, (long long)(pl.xbc & ~31) * hld,
            pl.xbc & 31, hld / 2);
        (*launches)++;
      }
      {
        Scope sc(this, 0, st);
        // H row exponents are atomically maximised by the half-transform epilogue
        if (cudaMemsetAsync(d_eH, 0, (size_t)h_nrb * 32 * sizeof(int), st) != cudaSuccess) {
          *err = "split path: memset failed";
          return GBJK_CUDA_ERROR;
        }
        if (hfuse_eff)
          s = launch_gemm_v<true, false>(st, d_items + pl.ht0, pl.nht, launches, err, 0);
        else
          s = launch_gemm(st, d_items + pl.ht0, pl.nht, launches, err);
        if (s) return s;
      }
      if (ev_ht && nbatch == 1 && cudaEventRecord(ev_ht, st) != cudaSuccess) {
        *err = "split path: event record failed";
        return GBJK_CUDA_ERROR;
      }
      {
        Scope sc(this, 2, st);
        k_exp_unbias<<<cdiv_((long long)h_nrb * 32, 256), 256, 0, st>>>(d_eH, h_nrb * 32);
        (*launches)++;
        if (!hfuse_eff) {
          const long long hthr =
              (long long)(nbf / 8 + 2) * cdiv_((long long)pad32(pl.xbc) * hld, kTileK) * 32;
          k_split_tiles<<<dim3(cdiv_(hthr, 256), 1), 256, 0, st>>>(d_jobs + pl.hjob);
          (*launches)++;
        }
      }
      {
        Scope sc(this, 1, st);
        if (hfuse_eff)
          s = launch_gemm_v<false, true>(st, d_items + pl.k0, pl.nk, launches, err, k_grid);
        else
          s = launch_gemm(st, d_items + pl.k0, pl.nk, launches, err, k_grid);
        if (s) return s;
      }
      k_splitk_reduce_acc<<<cdiv_((long long)nbf * nbf, 256), 256, 0, st>>>(
          d_Kpart, pl.ksplit, nbf, -1.0, 1, b > 0 ? 1 : 0, dK);
      (*launches)++;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      *err = std::string("split path launch: ") + cudaGetErrorString(e);
      return GBJK_CUDA_ERROR;
    }
    return GBJK_OK;
  }

  // clear the timed-out-wait flag at the start of a computation (stream order)
  gbjk_status clear_error(cudaStream_t st) {
    if (d_err && cudaMemsetAsync(d_err, 0, sizeof(int), st) != cudaSuccess) return GBJK_CUDA_ERROR;
    return GBJK_OK;
  }
  // error code recorded by a timed-out wait inside the split GEMM (0 = none)
  int read_error() {
    int h = 0;
    if (d_err) cudaMemcpy(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    return h;
  }
};

}  // namespace gbjk
