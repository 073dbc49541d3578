// Host Gaussian-integral engine (McMurchie–Davidson) for the DF Fock build.
//
// Replaces the libcint calls megalochem makes once per molecule
// (src/ints/integrals.cpp:250-370 int3c2e_sph, :511-617 int2e_sph diagonal,
// :619-689 int2c2e_sph diagonal; src/ints/aofactory.cpp:558-583 function
// selection).  Conventions follow libcint as megalochem uses it:
//   * contracted shells normalised with the radial rule of
//     src/ints/aofactory.cpp:273-314 (gto_norm / gto_normalize);
//   * real spherical harmonics, orthonormal on the sphere; p shells ordered
//     (x, y, z), shells with l >= 2 ordered m = -l..l;
//   * 3-center integrals (X|mu nu) with X an auxiliary shell.
// Method: Hermite expansion coefficients E^{ij}_t and Hermite Coulomb
// integrals R_{tuv} (Helgaker, Jorgensen, Olsen, "Molecular
// Electronic-Structure Theory", ch. 9); Boys function by the series of
// eq. 9.8.12 with downward recursion 9.8.14 for small arguments and the
// asymptotic value with upward recursion for large ones.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace gbints {

constexpr int kMaxL = 4;          // largest shell angular momentum supported
constexpr int kMaxLTot = 12;  // largest total angular momentum of one integral class

struct Shell {
  int l = 0;
  double A[3] = {0, 0, 0};
  std::vector<double> alpha;  // primitive exponents
  std::vector<double> coef;   // contraction coefficients incl. primitive norms
  int bf_off = 0;             // first basis function of this shell
  int nsph() const { return 2 * l + 1; }
  int ncart() const { return (l + 1) * (l + 2) / 2; }
};

struct Basis {
  std::vector<Shell> shells;
  int nbf = 0;
  int max_l = 0;
};

// Boys function F_0..F_nmax at argument T.
void boys(int nmax, double T, double* F);

// Cartesian -> real-spherical transformation for shell l:
// sph[m][c] with m in output order and c in cartesian order
// (x^l, x^{l-1}y, x^{l-1}z, ..., z^l).
const std::vector<double>& sph_coeffs(int l);
void cart_exponents(int l, int c, int* ex);

// Hermite expansion coefficients for one primitive pair along one axis.
// E[i][j][t], i <= la, j <= lb, t <= i+j.  Stored flat with fixed strides.
struct Herm1D {
  static constexpr int S = kMaxL + 3;  // +2 for kinetic energy
  double e[S][S][2 * S];
};
void hermite_1d(int la, int lb, double p, double xpa, double xpb, double kab,
                Herm1D& E);

// Hermite Coulomb integrals R_{tuv}(alpha, X, Y, Z) for t+u+v <= L.
struct HermR {
  static constexpr int S = kMaxLTot + 1;
  double r[S][S][S];
};
void hermite_r(int L, double alpha, double X, double Y, double Z, HermR& R);

}  // namespace gbints
