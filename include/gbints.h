/* Host integral engine for the DF Fock build (FP64, OpenMP).
 *
 * Replaces the libcint calls megalochem makes once per molecule; libcint is
 * an external dependency that megalochem does not vendor.  The functions map
 * onto the reference as follows:
 *   gbints_basis_create   ints::aofactory::impl setup + gto_normalize
 *                         (src/ints/aofactory.cpp:273-314, :558-583)
 *   gbints_one_electron   ao_overlap / ao_kinetic / ao_nuclear
 *                         (src/ints/aofactory.cpp, int1e_ovlp/kin/nuc_sph)
 *   gbints_coulomb_2c     ao_2c2e(coulomb)  (src/ints/aoloader.cpp:131)
 *   gbints_schwarz_pairs  calc_ints_schwarz_mn (src/ints/integrals.cpp:511-617)
 *   gbints_schwarz_aux    calc_ints_schwarz_x  (src/ints/integrals.cpp:619-689)
 *   gbints_eri3c_panels   calc_ints 3c2e into reserved blocks
 *                         (src/ints/integrals.cpp:250-370,
 *                          src/ints/aoloader.cpp:287-398)
 *   gbints_eri4c          int2e_sph (small systems; exact-J/K checks only)
 * All functions return 0 on success, 1 on an invalid argument, 2 when out of
 * host memory.  nthreads <= 0 uses the OpenMP default.
 */
#ifndef GBINTS_H
#define GBINTS_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbints_basis gbints_basis;

/* Shells s = 0..nshell-1: angular momentum l[s] (0..4), nprim[s] primitives,
 * centre centers[3s..3s+2] (bohr); alpha/coef hold the primitives of all
 * shells back to back, coef being the raw contraction coefficients. */
int gbints_basis_create(gbints_basis** out, int nshell, const int* l, const int* nprim,
                        const double* centers, const double* alpha, const double* coef);
void gbints_basis_destroy(gbints_basis* b);
int gbints_basis_nbf(const gbints_basis* b);
/* Normalised shell data (coefficients after gto_normalize) for a device
 * integral engine; no counterpart in the reference. */
int gbints_basis_shells(const gbints_basis* b, int* l, int* nprim, int* bf_off, double* centers,
                        double* alpha, double* coef);
/* Cartesian -> real-spherical table of shell l, (2l+1) x (l+1)(l+2)/2. */
int gbints_sph_coeffs(int l, double* out);

/* which: 0 overlap, 1 kinetic, 2 nuclear attraction (charges Z[natom], xyz
 * [natom*3] in bohr).  M is nbf x nbf row-major. */
int gbints_one_electron(const gbints_basis* b, int which, int natom, const double* Z,
                        const double* xyz, double* M, int nthreads);

/* Coulomb metric (X|Y), naux x naux row-major. */
int gbints_coulomb_2c(const gbints_basis* aux, double* M, int nthreads);

/* Full (mu nu|la si), nbf^4 row-major. */
int gbints_eri4c(const gbints_basis* b, double* out, int nthreads);

/* Shell-pair Schwarz factors (nshell x nshell) and auxiliary shell factors. */
int gbints_schwarz_pairs(const gbints_basis* b, double* Z, int nthreads);
int gbints_schwarz_aux(const gbints_basis* aux, double* z, int nthreads);

/* (X|mu nu) into the atom-block panel layout: panel I is a dense
 * [b_I][naux][K_I] FP64 array at B + panel_off[I]; block pair p = (pair_I[p],
 * pair_J[p]) with pair_I <= pair_J writes its b_J columns at col_IJ[p] of
 * panel I and its b_I columns at col_JI[p] of panel J.  keep[p*nablk + A] = 0
 * skips auxiliary block A for that pair (Schwarz-screened; left untouched, so
 * the caller zero-fills B).  blk_shell_off / ablk_shell_off give the shell
 * ranges of the AO / auxiliary atom blocks (nblk+1 / nablk+1 entries). */
int gbints_eri3c_panels(const gbints_basis* ao, const gbints_basis* aux, int nblk,
                        const int* blk_shell_off, int nablk, const int* ablk_shell_off,
                        int npairs, const int* pair_I, const int* pair_J,
                        const unsigned char* keep, const long long* panel_off,
                        const int* panel_K, const int* col_IJ, const int* col_JI, double* B,
                        int nthreads);

#ifdef __cplusplus
}
#endif

#endif /* GBINTS_H */
