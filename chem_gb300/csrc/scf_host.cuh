// SCF iteration on the device: the loop body of megalochem's closed-shell
// SCF (hf::hfmod, src/hf/hfscf.cpp:386-459) around the J/K build, as two
// CUDA graphs per iteration on the context's stream.
//
//   graph A ("build"), from the occupied coefficients C (nbf x nocc):
//     P_tot = 2 C C^T                                     (FP64 GEMM)
//     J, K  = the context's Fock build at P_tot, C
//     F     = H + J + K                   (form_fock, hfscf.cpp:228-276)
//     E_el  = sum P (H + F), P = P_tot / 2          (energy, :278-296)
//     U     = F P_tot S,  e = (U - U^T) / 2 = F P S - S P F
//                                               (error matrix, :298-324)
//     rms   = sqrt(sum e^2 / nbf^2)
//     F, e -> slot s of the DIIS ring (s from a device word), then the
//     overlaps <e, e_j> with every ring slot (DIIS B-matrix row,
//     src/math/solvers/diis.hpp:43-234)
//   graph B ("extrapolate"), from DIIS coefficients c_j (device words):
//     Fbar = sum_j c_j F_j,  Fo = X Fbar X        (X symmetric, S^-1/2)
//
// The host solves the small DIIS system and diagonalises Fo (FP64), as the
// reference does.  Every reduction goes through per-block partials summed in
// a fixed order, so results are deterministic.  Inputs of an iteration (C,
// the ring slot, the coefficients) are copied into fixed device buffers
// before a graph is launched; the graphs are captured once and recaptured
// when the engine's buffers or settings change.
#pragma once
#include <vector>

#include "kernels_fp64.cuh"

namespace gbjk {

constexpr int kScfBlocks = 256;  // partial sums per reduction
constexpr int kScfMaxDiis = 16;

// F = H + J + K; partial[b] = sum over the block's elements of
// Pt (H + F) (grid-stride, kScfBlocks blocks x 256 threads)
__global__ void k_scf_fock(const double* __restrict__ H, const double* __restrict__ J,
                           const double* __restrict__ K, const double* __restrict__ Pt,
                           double* __restrict__ F, long long n2, double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n2;
       i += (long long)gridDim.x * blockDim.x) {
    const double f = H[i] + J[i] + K[i];
    F[i] = f;
    s = fma(Pt[i], H[i] + f, s);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// e = (U - U^T) / 2 into ering[slot]; F into fring[slot]; partial sums of
// e^2.  Grid-stride over the n x n elements.
__global__ void k_scf_err(const double* __restrict__ U, const double* __restrict__ F, int n,
                          const int* __restrict__ slot, double* __restrict__ fring,
                          double* __restrict__ ering, double* __restrict__ part) {
  __shared__ double red[256];
  const long long n2 = (long long)n * n;
  double* e = ering + (long long)(*slot) * n2;
  double* fs = fring + (long long)(*slot) * n2;
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n2;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / n, c = i - r * n;
    const double v = 0.5 * (U[i] - U[c * n + r]);
    e[i] = v;
    fs[i] = F[i];
    s = fma(v, v, s);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// part[j][b] = partial of <e_slot, e_j> for every ring slot j (grid
// (kScfBlocks, nslots))
__global__ void k_scf_dots(const double* __restrict__ ering, long long n2,
                           const int* __restrict__ slot, double* __restrict__ part) {
  __shared__ double red[256];
  const double* e = ering + (long long)(*slot) * n2;
  const double* ej = ering + (long long)blockIdx.y * n2;
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n2;
       i += (long long)gridDim.x * blockDim.x)
    s = fma(e[i], ej[i], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(long long)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// scal[0] = 0.5 * sum part_E, scal[1] = sqrt(sum part_e2 / n^2),
// scal[2 + j] = sum part_dots[j]; one warp per output, fixed order
__global__ void k_scf_finish(const double* __restrict__ partE, const double* __restrict__ partR,
                             const double* __restrict__ partD, int nslots, int n,
                             double* __restrict__ scal) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (w >= 2 + nslots) return;
  const double* p = w == 0 ? partE : (w == 1 ? partR : partD + (long long)(w - 2) * kScfBlocks);
  double s = 0.0;
  for (int b = lane; b < kScfBlocks; b += 32) s += p[b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    if (w == 0)
      scal[0] = 0.5 * s;
    else if (w == 1)
      scal[1] = sqrt(s / ((double)n * n));
    else
      scal[w] = s;
  }
}

// Fbar = sum_j coef[j] F_j over the ring slots (in slot order)
__global__ void k_scf_combine(const double* __restrict__ fring, const double* __restrict__ coef,
                              int nslots, long long n2, double* __restrict__ Fbar) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n2;
       i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < nslots; ++j) s = fma(coef[j], fring[(long long)j * n2 + i], s);
    Fbar[i] = s;
  }
}

struct ScfState {
  bool ready = false;
  int nbf = 0, nocc = 0, nslots = 0;
  size_t bytes = 0;
  double *dH = nullptr, *dS = nullptr, *dX = nullptr, *dC = nullptr, *dPt = nullptr,
         *dJ = nullptr, *dK = nullptr, *dF = nullptr, *dT = nullptr, *dU = nullptr,
         *dFring = nullptr, *dEring = nullptr, *dFbar = nullptr, *dW = nullptr, *dFo = nullptr,
         *dpart = nullptr, *dscal = nullptr, *dcoef = nullptr;
  int* dslot = nullptr;
  GemmGroup* dgroups = nullptr;
  GemmTile* dtiles = nullptr;
  int t_pc = 0, n_pc = 0, t_ps = 0, n_ps = 0, t_fu = 0, n_fu = 0, t_xw = 0, n_xw = 0, t_wx = 0,
      n_wx = 0;
  // captured graphs and the engine epoch they were captured at
  cudaGraphExec_t gA = nullptr, gB = nullptr;
  cudaGraph_t grA = nullptr, grB = nullptr;
  uint64_t epA = ~0ull;
  int kmethodA = -1;
  int64_t launchesA = 0, launchesB = 0;

  template <class T>
  cudaError_t alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess)
      bytes += std::max<size_t>(n, 1) * sizeof(T);
    else
      cudaGetLastError();
    return e;
  }
  void drop_graphs() {
    if (gA) cudaGraphExecDestroy(gA);
    if (grA) cudaGraphDestroy(grA);
    if (gB) cudaGraphExecDestroy(gB);
    if (grB) cudaGraphDestroy(grB);
    gA = gB = nullptr;
    grA = grB = nullptr;
    epA = ~0ull;
  }
  void release() {
    drop_graphs();
    double** ps[] = {&dH, &dS, &dX, &dC, &dPt, &dJ, &dK, &dF, &dT, &dU, &dFring, &dEring,
                     &dFbar, &dW, &dFo, &dpart, &dscal, &dcoef};
    for (double** p : ps) {
      if (*p) cudaFree(*p);
      *p = nullptr;
    }
    if (dslot) cudaFree(dslot);
    if (dgroups) cudaFree(dgroups);
    if (dtiles) cudaFree(dtiles);
    dslot = nullptr;
    dgroups = nullptr;
    dtiles = nullptr;
    ready = false;
    bytes = 0;
  }

  static int cd(long long a, long long b) { return (int)((a + b - 1) / b); }
  static void tiles_for(std::vector<GemmTile>& t, int g, int M, int N, int K) {
    for (int mt = 0; mt < cd(M, 64); ++mt)
      for (int nt = 0; nt < cd(N, 64); ++nt) t.push_back({g, mt, nt, 0, K, 0});
  }

  // buffers and GEMM plans; H, S, X: host nbf x nbf
  gbjk_status begin(cudaStream_t st, int n, int no, int nd, const double* H, const double* S,
                    const double* X, std::string* err) {
    release();
    nbf = n;
    nocc = no;
    nslots = nd;
    const size_t n2 = (size_t)n * n;
    if (alloc(&dH, n2) || alloc(&dS, n2) || alloc(&dX, n2) || alloc(&dC, (size_t)n * no) ||
        alloc(&dPt, n2) || alloc(&dJ, n2) || alloc(&dK, n2) || alloc(&dF, n2) ||
        alloc(&dT, n2) || alloc(&dU, n2) || alloc(&dFring, n2 * nd) || alloc(&dEring, n2 * nd) ||
        alloc(&dFbar, n2) || alloc(&dW, n2) || alloc(&dFo, n2) ||
        alloc(&dpart, (size_t)(2 + nd) * kScfBlocks) || alloc(&dscal, (size_t)(2 + nd)) ||
        alloc(&dcoef, (size_t)nd) || alloc(&dslot, 1)) {
      release();
      *err = "SCF: out of device memory";
      return GBJK_OOM;
    }
    cudaMemcpy(dH, H, n2 * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dS, S, n2 * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dX, X, n2 * 8, cudaMemcpyHostToDevice);
    cudaMemsetAsync(dFring, 0, n2 * nd * 8, st);
    cudaMemsetAsync(dEring, 0, n2 * nd * 8, st);
    // GEMM groups: 0 Pt = 2 C C^T, 1 T = Pt S, 2 U = F T, 3 W = X Fbar, 4 Fo = W X
    std::vector<GemmGroup> g(5);
    g[0] = {dC, dC, dPt, n, n, no, no, no, n, kTransB};
    g[1] = {dPt, dS, dT, n, n, n, n, n, n, 0};
    g[2] = {dF, dT, dU, n, n, n, n, n, n, 0};
    g[3] = {dX, dFbar, dW, n, n, n, n, n, n, 0};
    g[4] = {dW, dX, dFo, n, n, n, n, n, n, 0};
    std::vector<GemmTile> t;
    t_pc = (int)t.size();
    tiles_for(t, 0, n, n, no);
    n_pc = (int)t.size() - t_pc;
    t_ps = (int)t.size();
    tiles_for(t, 1, n, n, n);
    n_ps = (int)t.size() - t_ps;
    t_fu = (int)t.size();
    tiles_for(t, 2, n, n, n);
    n_fu = (int)t.size() - t_fu;
    t_xw = (int)t.size();
    tiles_for(t, 3, n, n, n);
    n_xw = (int)t.size() - t_xw;
    t_wx = (int)t.size();
    tiles_for(t, 4, n, n, n);
    n_wx = (int)t.size() - t_wx;
    if (alloc(&dgroups, g.size()) || alloc(&dtiles, t.size())) {
      release();
      *err = "SCF: out of device memory";
      return GBJK_OOM;
    }
    cudaMemcpy(dgroups, g.data(), g.size() * sizeof(GemmGroup), cudaMemcpyHostToDevice);
    cudaMemcpy(dtiles, t.data(), t.size() * sizeof(GemmTile), cudaMemcpyHostToDevice);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
      release();
      *err = "SCF: set-up failed";
      return GBJK_CUDA_ERROR;
    }
    ready = true;
    return GBJK_OK;
  }

  void gemm(cudaStream_t st, int t0, int nt, bool transB, double alpha) {
    if (transB)
      k_gemm_fp64<true><<<nt, 256, 0, st>>>(dgroups, dtiles + t0, alpha);
    else
      k_gemm_fp64<false><<<nt, 256, 0, st>>>(dgroups, dtiles + t0, alpha);
  }
  // the part of graph A before the Fock build
  int64_t launch_pre(cudaStream_t st) {
    gemm(st, t_pc, n_pc, true, 2.0);
    return 1;
  }
  // the part of graph A after the Fock build
  int64_t launch_post(cudaStream_t st) {
    const long long n2 = (long long)nbf * nbf;
    k_scf_fock<<<kScfBlocks, 256, 0, st>>>(dH, dJ, dK, dPt, dF, n2, dpart);
    gemm(st, t_ps, n_ps, false, 1.0);
    gemm(st, t_fu, n_fu, false, 1.0);
    k_scf_err<<<kScfBlocks, 256, 0, st>>>(dU, dF, nbf, dslot, dFring, dEring,
                                          dpart + kScfBlocks);
    k_scf_dots<<<dim3(kScfBlocks, nslots), 256, 0, st>>>(dEring, n2, dslot,
                                                         dpart + 2 * kScfBlocks);
    k_scf_finish<<<1, 32 * (2 + nslots), 0, st>>>(dpart, dpart + kScfBlocks,
                                                  dpart + 2 * kScfBlocks, nslots, nbf, dscal);
    return 6;
  }
  int64_t launch_extrapolate(cudaStream_t st) {
    const long long n2 = (long long)nbf * nbf;
    k_scf_combine<<<kScfBlocks, 256, 0, st>>>(dFring, dcoef, nslots, n2, dFbar);
    gemm(st, t_xw, n_xw, false, 1.0);
    gemm(st, t_wx, n_wx, false, 1.0);
    return 3;
  }
};

}  // namespace gbjk
