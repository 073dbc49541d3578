/* gbjk — GB300 engine for the density-fitted J/K (Fock) build.
 *
 * Drop-in replacement for the block-sparse contractions megalochem's DF J/K
 * builders issue through DBCSR.  Each entry point stands in for a reference
 * interface:
 *
 *   gbjk_create          fock::create_j()/create_k() ... .build() + init()
 *                        (src/fock/jkbuilder.hpp:621-841,
 *                         src/fock/jkcommon.cpp:18-57)
 *   gbjk_upload_b        the aoloader registry entry key::dfit_coul_xbb /
 *                        eri3c2e_batched handed to the builders
 *                        (src/fock/jkbuilder.hpp:639-680,
 *                         src/ints/aoloader.cpp:287-398)
 *   gbjk_upload_metric   key::coul_xx_inv / key::coul_xx_invsqrt
 *                        (src/ints/aoloader.cpp:164-183)
 *   gbjk_compute_j       fock::DF_J::compute_J  (src/fock/jkdf.cpp:69-190)
 *   gbjk_compute_k       fock::DFMO_K::compute_K (src/fock/jkdf.cpp:221-462),
 *                        fock::DFLMO_K::compute_K (src/fock/jkdf.cpp:890-1091)
 *   gbjk_compute_jk      hf::hfmod::form_fock's J + K calls
 *                        (src/hf/hfscf.cpp:241-259)
 *   gbjk_set_precision   no counterpart (precision selection of this engine)
 *   gbjk_last_error      the what() of the std::runtime_error megalochem
 *                        throws (src/fock/jkbuilder.hpp:58)
 *
 * Conventions: dense row-major FP64 nbf x nbf matrices (P, J, K) and
 * nbf x nocc coefficient matrices at the boundary; block-sparse inside.
 * Host-pointer calls copy in, compute and copy out before returning; *_dev
 * variants take device pointers and are ordered on the context's stream.
 * A context belongs to one host thread and one CUDA device.
 */
#ifndef GBJK_H
#define GBJK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GBJK_OK = 0,
  GBJK_INVALID_ARG = 1,
  GBJK_OOM = 2,
  GBJK_CUDA_ERROR = 3,
  GBJK_TIMEOUT = 4,
  GBJK_NOT_CONVERGED = 5,
  GBJK_NOT_READY = 6
} gbjk_status;

typedef enum { GBJK_FP64 = 0, GBJK_SPLIT_BF16 = 1 } gbjk_precision;

/* K builder, by the reference's kmethod strings (src/fock/jkbuilder.hpp:37-60) */
typedef enum { GBJK_K_DFMO = 0, GBJK_K_DFLMO = 1, GBJK_K_DFAO = 2 } gbjk_kmethod;

/* Route of the FP64 J's metric step.  GBJK_J_VINV multiplies by the
 * explicit inverse V^-1 = L^-T L^-1, as fock::DF_J does
 * (src/fock/jkdf.cpp:137-141).  GBJK_J_CHOLESKY applies L^-1 and then
 * L^-T; for an ill-conditioned Coulomb metric (cond ~1e7 for C20H42 /
 * cc-pVDZ-jkfit) it is several orders of magnitude more accurate.  The mixed
 * path always uses the Cholesky route. */
typedef enum { GBJK_J_VINV = 0, GBJK_J_CHOLESKY = 1 } gbjk_jmode;

typedef struct gbjk_ctx gbjk_ctx;

/* Atom-block panel layout of the 3-center tensor (X|mu nu):
 * AO block I has blk_size[I] functions; panel I is the dense FP64 array
 * [blk_size[I]][naux][panel_K[I]] and colmap lists, panel after panel, the
 * AO index of each of its panel_K[I] columns.  Panels are stored back to
 * back in block order. */
typedef struct gbjk_desc {
  int nbf;
  int naux;
  int nblk;
  const int* blk_size;  /* nblk */
  const int* panel_K;   /* nblk */
  const int* colmap;    /* sum_I panel_K[I] */
  double filter_eps;    /* result-block filter on J and K; 0 disables */
  int device;           /* CUDA device ordinal */
} gbjk_desc;

gbjk_status gbjk_create(gbjk_ctx** ctx, const gbjk_desc* desc);
void gbjk_destroy(gbjk_ctx* ctx);
const char* gbjk_last_error(const gbjk_ctx* ctx);

/* B: host FP64 panel array (sum_I blk_size[I]*naux*panel_K[I] doubles). */
gbjk_status gbjk_upload_b(gbjk_ctx* ctx, const double* B);
/* Linv: lower-triangular L^-1 with V = L L^T; Vinv = L^-T L^-1 (naux^2 each). */
gbjk_status gbjk_upload_metric(gbjk_ctx* ctx, const double* Linv, const double* Vinv);

/* precision: GBJK_FP64 or GBJK_SPLIT_BF16; nslices = BF16 slices per FP64
 * operand for the split path (ignored for FP64; 0 picks the default). */
gbjk_status gbjk_set_precision(gbjk_ctx* ctx, int precision, int nslices);

/* fitted != 0: the uploaded tensor already is L^-1 (X|mu nu) (pre-fitted);
 * no metric is used: J = B^T (B Ptot), K = -(B C)^T (B C).  Used by the
 * synthetic DF-K workload, whose tensor is treated as pre-fitted.
 * No counterpart in the reference. */
gbjk_status gbjk_set_fitted(gbjk_ctx* ctx, int fitted);
/* FP64 path, tensor not pre-fitted: build K (DF-MO or DF-LMO) with the
 * occupied orbitals in batches of `cols` (0 = all at once), each batch's
 * half transform, fit and exchange in turn, so that the half-transformed
 * tensor exists for one batch only; the batch sums are added into K in
 * order.  As megalochem batches the occupied index (occ_nbatches,
 * src/fock/jkdf.cpp:254-268). */
gbjk_status gbjk_set_occ_batch(gbjk_ctx* ctx, int cols);
/* Process the auxiliary index in batches of `rows` (0 = all at once;
 * rounded down to a multiple of 32, at least 32).  Split path: streaming
 * the half transform and the exchange batch by batch so that the
 * half-transformed tensor never exists in full.  No counterpart in the
 * reference (it batches over X with DBCSR, src/fock/jkdf.cpp:412-422).
 * FP64 path with a pre-fitted tensor (gbjk_set_fitted): the half transform
 * and exchange of each batch in turn, the batch sums added into K in
 * order. */
gbjk_status gbjk_set_aux_batch(gbjk_ctx* ctx, int rows);
/* Fill the panel array on the device with the seeded synthetic tensor
 * (Y, mu, nu) = N(0,1)[seed, min(mu,nu), max(mu,nu), Y] exp(-|I-J|/(2 decay)),
 * symmetric in (mu, nu); gbjk_download_b copies the panels to the host.
 * No counterpart in the reference. */
gbjk_status gbjk_upload_b_synthetic(gbjk_ctx* ctx, unsigned long long seed, double decay);
gbjk_status gbjk_download_b(gbjk_ctx* ctx, double* B);

/* Shells of a basis, normalised as the host engine uses them (the output of
 * gbints_basis_shells): per shell l, primitive count, first basis function,
 * centre (3 doubles); exponents and contraction coefficients concatenated. */
typedef struct gbjk_shells {
  int nshell;
  const int* l;
  const int* nprim;
  const int* bf_off;
  const double* centers;
  const double* alpha;
  const double* coef;
} gbjk_shells;
/* Compute the 3-center tensor on the device straight into the panel layout
 * (replaces the host calc_ints 3c2e pass, src/ints/integrals.cpp:250-370,
 * and gbjk_upload_b): AO block pairs pair_I[p] <= pair_J[p] with their
 * panel columns col_IJ / col_JI, keep[p * nablk + A] the kept auxiliary
 * blocks, blk_shell_off / ablk_shell_off the shell ranges of the AO and
 * auxiliary blocks, sph the cartesian -> spherical tables of l = 0..3
 * (gbints_sph_coeffs, concatenated).  AO shells up to d, auxiliary shells up
 * to f.  No counterpart in the reference (its integrals run on the host). */
gbjk_status gbjk_upload_b_eri3c(gbjk_ctx* ctx, const gbjk_shells* ao, const gbjk_shells* aux,
                                const double* sph, const int* blk_shell_off, int nablk,
                                const int* ablk_shell_off, int npairs, const int* pair_I,
                                const int* pair_J, const unsigned char* keep, const int* col_IJ,
                                const int* col_JI);

/* Test hook for failure detection: item >= 0 makes every split-precision
 * GEMM launch of the context stop issuing operand copies at work item
 * `item`, with each pipeline wait bounded by wait_ms (1..2000) instead of
 * 2 s.  The waiting threads give up, every CTA waits for its own copies
 * and MMAs, and the build reports GBJK_TIMEOUT; the context stays usable.
 * item < 0 restores normal operation.  No counterpart in the reference. */
gbjk_status gbjk_test_split_stall(gbjk_ctx* ctx, int item, double wait_ms);

/* Mixed-precision build: after the half transform the J column sums
 * (HBM-bound) run on a second stream of the context beside the digit pass
 * and the exchange GEMM (tensor-bound), which leaves `sms` SMs to them;
 * 0 (default) gives the exchange every SM and the J blocks fill the
 * registers and shared memory its CTAs leave free; -1 runs the phases in
 * order on one stream.  Results are the same bits either way.  No
 * counterpart in the reference. */
gbjk_status gbjk_set_overlap(gbjk_ctx* ctx, int sms);
int gbjk_get_overlap(const gbjk_ctx* ctx);

/* Mixed-precision exchange: 1 cuts the digit slices of the half transform
 * H = (L^-1 B) C in the half-transform epilogue, with one exponent per AO
 * function and group of 32 auxiliary indices, and the exchange GEMM applies
 * those exponents per k segment; 0 (default) writes H in FP64 and cuts its
 * digits in a separate pass with one exponent per AO function.  Both stay
 * within the split path's accuracy bound; their results differ in the last
 * bits.  No counterpart in the reference. */
gbjk_status gbjk_set_split_fuse(gbjk_ctx* ctx, int on);
int gbjk_get_split_fuse(const gbjk_ctx* ctx);

/* jmode: GBJK_J_VINV (default, the reference route) or GBJK_J_CHOLESKY.
 * No counterpart in the reference. */
gbjk_status gbjk_set_jmode(gbjk_ctx* ctx, int jmode);

/* J_{mu nu} = sum_X (X|mu nu) [V^-1 g]_X, g_X = sum (X|mu nu) Ptot_{mu nu}. */
gbjk_status gbjk_compute_j(gbjk_ctx* ctx, const double* Ptot, double* J);
/* K_{mu nu} = -sum_{X,i} Bfit_{X mu i} Bfit_{X nu i}, Cocc is nbf x nocc. */
gbjk_status gbjk_compute_k(gbjk_ctx* ctx, int kmethod, const double* Cocc, int nocc, double* K);
/* DF-AO K (fock::DFAO_K, src/fock/jkdf.cpp:464-648, with the fitting
 * coefficients of ints::dfitting, src/ints/fitting.cpp:44-161):
 *   K_{MN} = -sum_{X,S} c_{XNS} cbar_{XMS},  cbar = (X|MN) P_{NS},
 *   c = V^-1 (Y|NS),
 * from the alpha density P (nbf x nbf, the builder's set_density_alpha).
 * The FP64 path follows that route (c fitted once per tensor, kept dense
 * over S); the split path uses the Cholesky route,
 *   K = -sum_{Y,S} [L^-1 B]_{YNS} [L^-1 cbar]_{YMS}.
 * Host and device-pointer (stream-ordered) forms. */
gbjk_status gbjk_compute_k_ao(gbjk_ctx* ctx, const double* P, double* K);
gbjk_status gbjk_compute_k_ao_dev(gbjk_ctx* ctx, const double* dP, double* dK);
/* Non-symmetric DF-LMO K (fock::DFLMO_K with set_sym(false),
 * src/fock/jkdf.cpp:1093-1323; the exchange of the ADC matrix-vector
 * products, set_coeff_left_alpha / set_coeff_right_alpha):
 *   K_{mn} = -sum_{X,i} [(X|m.) U]_{Xmi} [V^-1 (X|n.) Vt^T]_{Xni},
 * U: nbf x nocc (left), Vt: nocc x nbf (right, as the reference's v_mb).
 * The split path uses the Cholesky route of the metric. */
gbjk_status gbjk_compute_k_lmo_asym(gbjk_ctx* ctx, const double* U, const double* Vt, int nocc,
                                    double* K);
/* One Fock build: J from Ptot and K from Cocc in one call.  The first call
 * for a given (kmethod, nocc, J and/or K) runs the launches directly and
 * captures them as a CUDA graph on the context's own device buffers; later
 * calls with the same shape copy the inputs in, replay that graph and copy
 * J and K out.  Host buffers from gbjk_host_alloc (pinned) are copied by DMA
 * without staging; any other host memory works too. */
gbjk_status gbjk_compute_jk(gbjk_ctx* ctx, int kmethod, const double* Ptot, const double* Cocc,
                            int nocc, double* J, double* K);
/* Page-locked host memory for the inputs and outputs of the host-buffer
 * calls (cudaHostAlloc, portable).  NULL on failure.  No counterpart in the
 * reference, whose matrices live in host memory owned by DBCSR. */
void* gbjk_host_alloc(size_t bytes);
void gbjk_host_free(void* p);

/* Device-pointer variants, ordered on the context's stream (no host sync). */
gbjk_status gbjk_compute_jk_dev(gbjk_ctx* ctx, int kmethod, const double* dPtot,
                                const double* dCocc, int nocc, double* dJ, double* dK);
gbjk_status gbjk_synchronize(gbjk_ctx* ctx);
/* Capture one device-pointer Fock build (same arguments as
 * gbjk_compute_jk_dev) as a CUDA graph on the context's stream, after one
 * ordinary build that prepares every plan; gbjk_launch_graph replays it
 * (same pointers, new contents).  A call that frees or replaces any engine
 * buffer (an upload, gbjk_set_fitted, gbjk_set_aux_batch, a build with
 * another nocc or precision) discards the captured build, and
 * gbjk_launch_graph then returns GBJK_NOT_READY.  No counterpart in the
 * reference. */
gbjk_status gbjk_capture_graph(gbjk_ctx* ctx, int kmethod, const double* dPtot,
                               const double* dCocc, int nocc, double* dJ, double* dK);
gbjk_status gbjk_launch_graph(gbjk_ctx* ctx);
/* The context's cudaStream_t, as void*. */
void* gbjk_stream(gbjk_ctx* ctx);

/* Summation plan of the exchange contraction K = -sum_t A_mu,t B_nu,t over
 * t < naux*nocc: the t range is cut into *ksplit chunks of *kchunk (the last
 * one shorter), each summed in order, and the chunk sums are added in order.
 * Needs no GPU; lets a checker reproduce the device's rounding exactly.
 * No counterpart in the reference (DBCSR does not specify its order). */
gbjk_status gbjk_k_split_plan(int nbf, int naux, int nocc, int* ksplit, long long* kchunk);

/* ---- SCF iteration on the device -----------------------------------------
 * The loop body of megalochem's closed-shell SCF (hf::hfmod::compute,
 * src/hf/hfscf.cpp:386-459) around this context's Fock build, as CUDA
 * graphs on the context's stream; the host keeps the DIIS solve and the
 * FP64 diagonalisation.
 * gbjk_scf_begin: core Hamiltonian H, overlap S and a symmetric
 *   orthogonaliser X (e.g. S^-1/2), host nbf x nbf; nocc; DIIS depth
 *   max_diis (1..16 ring slots for Fock and error matrices).
 * gbjk_scf_build: from the occupied coefficients Cocc (host nbf x nocc),
 *   P_tot = 2 C C^T, the J/K build (kmethod as gbjk_compute_jk),
 *   F = H + J + K (form_fock, :228-276), E_el = sum P (H + F) (:278-296),
 *   e = F P S - S P F (:298-324) and its RMS; F and e go into ring slot
 *   `slot`; out[0] = E_el, out[1] = RMS, out[2 + j] = <e, e_j> for every
 *   slot j (the DIIS B-matrix row, src/math/solvers/diis.hpp:43-234).  The
 *   first call (and any after the engine's buffers or settings change)
 *   launches directly, then records the sequence as a graph for the next.
 * gbjk_scf_extrapolate: Fbar = sum_j coef[j] F_j (coef: max_diis values,
 *   0 for unused slots) and Fo = X Fbar X into host nbf x nbf.
 * gbjk_scf_read: F of a slot and J, K of the last build to host (any NULL).
 * gbjk_scf_end: frees the SCF buffers. */
gbjk_status gbjk_scf_begin(gbjk_ctx* ctx, const double* H, const double* S, const double* X,
                           int nocc, int max_diis);
gbjk_status gbjk_scf_build(gbjk_ctx* ctx, int kmethod, const double* Cocc, int slot,
                           double* out);
gbjk_status gbjk_scf_extrapolate(gbjk_ctx* ctx, const double* coef, double* Fo);
gbjk_status gbjk_scf_read(gbjk_ctx* ctx, int slot, double* F, double* J, double* K);
gbjk_status gbjk_scf_end(gbjk_ctx* ctx);

/* ---- Launch configuration and autotuning ----------------------------------
 * The choices a Fock build's launches depend on.  0 in a field selects the
 * engine's built-in rule for it.
 *   fp64_ht_tn    FP64 half transform and fit: 1 (one thread per output,
 *                 16 x 16 tiles), 16, 32 or 64 (64-row tiles of that width)
 *   fp64_k_tile   FP64 exchange: 1 (one thread per output) or 64
 *   fp64_kchunk   FP64 exchange: k per split-K part (rounded up to a
 *                 multiple of 16; the parts are summed in order)
 *   split_ksplit  split-precision exchange: parts of the k range (at least
 *                 the number an item's int64 headroom needs)
 *   overlap_sms   as gbjk_set_overlap
 * Every FP64 choice keeps each output an in-order fma chain over its k
 * part, so FP64 results depend on fp64_kchunk only, which
 * gbjk_tune_plan publishes for a checker.  No counterpart in the reference,
 * whose small-block GEMMs are DBCSR's (src/dbcsrx/dbcsr_tensor_ops.hpp:
 * 128-137). */
typedef struct gbjk_tunables {
  int fp64_ht_tn;
  int fp64_k_tile;
  long long fp64_kchunk;
  int split_ksplit;
  int overlap_sms;
} gbjk_tunables;

/* Effective FP64 choices for a problem size and requested tunables (the
 * built-in rules filled in, fp64_kchunk rounded and clamped); *ksplit is
 * the number of exchange parts.  Needs no GPU. */
gbjk_status gbjk_tune_plan(int nbf, int naux, int nocc, const gbjk_tunables* req,
                           gbjk_tunables* eff, int* ksplit);
/* Requested tunables of a context (takes effect at its next build). */
gbjk_status gbjk_set_tunables(gbjk_ctx* ctx, const gbjk_tunables* t);
/* The values in effect at the context's last build (requested or rule). */
gbjk_status gbjk_get_tunables(const gbjk_ctx* ctx, gbjk_tunables* t);
/* Problem signature of the context for precision, kmethod and nocc (the
 * autotuning cache key): writes at most len bytes into sig. */
gbjk_status gbjk_tune_signature(const gbjk_ctx* ctx, int kmethod, int nocc, char* sig,
                                size_t len);
/* Tuning cache: a text file, one line per tuned signature,
 *   <signature> <fp64_ht_tn> <fp64_k_tile> <fp64_kchunk> <split_ksplit> <overlap_sms>
 * the last line of a signature wins.  Lookup returns GBJK_NOT_READY when
 * the file or the signature is missing.  Need no GPU. */
gbjk_status gbjk_tune_cache_lookup(const char* path, const char* sig, gbjk_tunables* t);
gbjk_status gbjk_tune_cache_store(const char* path, const char* sig, const gbjk_tunables* t);
/* Autotune one Fock build (host P_tot and C_occ, the same arguments as
 * gbjk_compute_jk) at the context's precision.  With a cache_path whose
 * file holds this signature the recorded choice is adopted without
 * timing.  Otherwise candidates are timed one dimension at a time (each
 * with one warm-up build and `reps` timed builds, CUDA events on the
 * context's stream), starting from the built-in rules; a candidate replaces
 * the choice so far only when it is at least 0.5 % faster.  The choice is
 * appended to the cache when cache_path is given.  A JSON report of the candidates and times goes
 * to report (at most report_len bytes, may be NULL). */
gbjk_status gbjk_autotune(gbjk_ctx* ctx, int kmethod, const double* Ptot, const double* Cocc,
                          int nocc, int reps, const char* cache_path, char* report,
                          size_t report_len);

/* ---- SOS-AO-MP2 Laplace batch ------------------------------------------
 * Replaces the Z builder of megalochem's Laplace loop: mp::LL_FULL_Z
 * (src/mp/z_full.cpp:427-620, "mi, Xmn -> Xin", "Na, XiN -> Xia", then
 * "Xia, Yia -> XY"), driven by mpmod::compute (src/mp/mp_compute.cpp:232-382)
 * through zbuilder->set_occ_coeff / set_vir_coeff / compute / zmat
 * (src/mp/z_builder.hpp).  All quadrature points go in one call.
 *
 * Point t takes the occupied and virtual Cholesky factors of its
 * pseudo-densities, Lo[t] (nbf x rank_o[t]) and Lv[t] (nbf x rank_v[t]),
 * row-major host arrays (the reference's L_bu and L_br).  On the context's
 * resident tensor, fitted with the metric's Cholesky factor
 * ((X|mn)~ = L^-1 (X|mn), L L^T = V), it computes
 *   Z~_t(X,Y) = sum_{i,a} W_t(X,i,a) W_t(Y,i,a),
 *   W_t(X,i,a) = sum_{m,n} Lo_t(m,i) (X|mn)~ Lv_t(n,a),
 * i.e. Z~_t = L^-1 Z_t L^-T of the reference's Z_t, and the Laplace term
 *   e_t = sum_{X,Y} Z~_t(X,Y)^2 = tr(Z_t V^-1 Z_t V^-1)
 * which the reference forms as Ztilde = Z V^-1, e_t = Ztilde . Ztilde^T
 * (mp_compute.cpp:361-381).  The precision set by gbjk_set_precision
 * selects the FP64 grouped GEMMs or the split-precision tensor-core path.
 * The tensor must cover all auxiliary functions (no gbjk_set_aux_batch). */
gbjk_status gbjk_mp2_set_factors(gbjk_ctx* ctx, int npts, const int* rank_o,
                                 const double* const* Lo, const int* rank_v,
                                 const double* const* Lv);
/* Evaluate every point on the context's stream; results stay on the device. */
gbjk_status gbjk_mp2_compute_dev(gbjk_ctx* ctx);
/* Wait for the stream, then copy e_t (npts doubles) and, when Z is not NULL,
 * every Z~_t (npts x naux x naux, row-major) to host memory. */
gbjk_status gbjk_mp2_read(gbjk_ctx* ctx, double* energies, double* Z);
/* gbjk_mp2_set_factors + gbjk_mp2_compute_dev + gbjk_mp2_read. */
gbjk_status gbjk_mp2_laplace(gbjk_ctx* ctx, int npts, const int* rank_o, const double* const* Lo,
                             const int* rank_v, const double* const* Lv, double* energies,
                             double* Z);
/* Free the batch's device buffers (the engine's tensor stays resident). */
gbjk_status gbjk_mp2_release(gbjk_ctx* ctx);

/* DF-J for callers that cannot allocate device memory — for example code
 * embedded in a host framework that owns all GPU memory through its own
 * pool and forbids allocations of its own by the libraries it calls.
 * No counterpart in the reference; it is an addition of this engine.
 *
 * Computes the same J as gbjk_compute_j (same kernels, same summation order)
 * without a context: the caller passes the layout (desc: host arrays
 * blk_size and panel_K, read before the call returns; desc->colmap is
 * ignored), the panel column map d_colmap, the panels d_B, V^-1 d_Vinv and
 * P_tot d_Ptot in device memory, and receives J in d_J (device,
 * nbf x nbf), all ordered on `stream`.  It calls no cudaMalloc/cudaFree and
 * no allocating library routine: all scratch lives in one 16 MiB file-scope
 * device array that every GPU loading the library holds until exit.
 * Problems whose scratch (nbf*naux + sum_I blk_size[I]*panel_K[I] + 2*naux
 * doubles plus the layout arrays) exceeds 16 MiB, or with naux > 6144,
 * nbf > 65535 or more than 1024 atom blocks, are rejected with
 * GBJK_INVALID_ARG and a message in errbuf before anything is launched.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the array and it keeps the last call's contents: calls
 * whose work may overlap on the GPU race and corrupt each other's results,
 * so serialise them (one stream, or events between the streams). */
gbjk_status gbjk_compute_j_noalloc(const gbjk_desc* desc, const int* d_colmap, const double* d_B,
                                   const double* d_Vinv, const double* d_Ptot, double* d_J,
                                   void* stream, char* errbuf, size_t errlen);

/* Device memory held by the context, in bytes. */
size_t gbjk_device_bytes(const gbjk_ctx* ctx);
/* Kernels launched by this context since creation (for launch accounting). */
int64_t gbjk_kernel_launches(const gbjk_ctx* ctx);

/* Per-phase device time: enable != 0 starts recording CUDA events around
 * every launch on the context's stream (and clears the totals);
 * gbjk_profile_read(ctx, i, ...) returns 1 and the name, accumulated
 * milliseconds and launch count of phase i, or 0 past the last phase.
 * No counterpart in the reference (it times phases with util::mpi_time,
 * src/utils/mpi_time.hpp:12-120). */
gbjk_status gbjk_profile(gbjk_ctx* ctx, int enable);
int gbjk_profile_read(const gbjk_ctx* ctx, int idx, const char** name, double* ms,
                      int64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* GBJK_H */
