// McMurchie–Davidson building blocks: Boys function, Hermite expansion
// coefficients, Hermite Coulomb integrals, cartesian->spherical transform.
#include "md_engine.hpp"

#include <cstring>
#include <mutex>
#include <utility>

namespace gbints {

// Boys function F_m(T) = int_0^1 t^{2m} exp(-T t^2) dt, m = 0..nmax.
// Small T: series F_n(T) = exp(-T) sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1))
// evaluated for n = nmax, then the downward recursion
// F_{m}(T) = (2T F_{m+1}(T) + exp(-T)) / (2m+1)  (all terms positive,
// so no cancellation).  Large T: F_0 = sqrt(pi/T) erf(sqrt T) / 2 and the
// upward recursion F_{m+1} = ((2m+1) F_m - exp(-T)) / (2T), which is stable
// there because exp(-T) is negligible against (2m+1) F_m.
namespace {
// Series form (also fills the interpolation grid below).
void boys_series(int nmax, double T, double* F) {
  if (T < 1e-15) {
    for (int m = 0; m <= nmax; ++m) F[m] = 1.0 / (2 * m + 1);
    return;
  }
  const double eT = std::exp(-T);
  if (T > 33.0 + nmax) {
    F[0] = 0.5 * std::sqrt(M_PI / T) * std::erf(std::sqrt(T));
    const double inv2T = 0.5 / T;
    for (int m = 0; m < nmax; ++m) F[m + 1] = ((2 * m + 1) * F[m] - eT) * inv2T;
    return;
  }
  double denom = 2 * nmax + 1;
  double term = 1.0 / denom;
  double sum = term;
  const double twoT = 2.0 * T;
  for (int k = 1; k < 400; ++k) {
    denom += 2.0;
    term *= twoT / denom;
    sum += term;
    if (term < 1e-17 * sum) break;
  }
  F[nmax] = eT * sum;
  for (int m = nmax - 1; m >= 0; --m) F[m] = (twoT * F[m + 1] + eT) / (2 * m + 1);
}

// F_m on the grid T_i = i h, m < kGridM, computed once by the series.  Since
// dF_m/dT = -F_{m+1}, the Taylor expansion about the nearest grid point,
//   F_m(T) = sum_{k<7} F_{m+k}(T_i) (T_i - T)^k / k!,  |T - T_i| <= h / 2,
// has a remainder below F_m (h/2)^7 / 7! = 1.2e-15 F_m for h = 1/20.
constexpr double kGridH = 0.05;
constexpr int kTaylor = 7;
constexpr int kGridM = kMaxLTot + kTaylor;
struct BoysGrid {
  int n;
  std::vector<double> f;  // [i][m]
  BoysGrid() {
    n = (int)((33.0 + kMaxLTot) / kGridH) + 2;
    f.resize((size_t)n * kGridM);
    for (int i = 0; i < n; ++i) boys_series(kGridM - 1, i * kGridH, &f[(size_t)i * kGridM]);
  }
};
const BoysGrid kGrid;
}  // namespace

void boys(int nmax, double T, double* F) {
  if (T > 33.0 + nmax) {
    boys_series(nmax, T, F);  // erf and upward recursion
    return;
  }
  const int i = (int)(T * (1.0 / kGridH) + 0.5);
  const double x = i * kGridH - T;
  const double* g = kGrid.f.data() + (size_t)i * kGridM;
  for (int m = 0; m <= nmax; ++m) {
    double s = g[m + kTaylor - 1];
    for (int k = kTaylor - 1; k >= 1; --k) s = g[m + k - 1] + (x / k) * s;
    F[m] = s;
  }
}

void cart_exponents(int l, int c, int* ex) {
  // order: for ix = l..0, iy = l-ix..0, iz = l-ix-iy
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

static double fact(int n) {
  double r = 1;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}
static double binom(int n, int k) {
  if (k < 0 || k > n) return 0;
  return fact(n) / (fact(k) * fact(n - k));
}

static int cart_index(int l, int ix, int iy, int iz) {
  (void)iz;
  // position of (ix,iy,iz) in the cartesian order above
  int idx = 0;
  for (int a = l; a > ix; --a) idx += l - a + 1;
  return idx + (l - ix - iy);
}

// Real solid harmonic S_lm (Helgaker et al. eq. 6.4.47-6.4.50), scaled by
// sqrt((2l+1)/(4 pi)) so that S_lm / r^l is orthonormal on the unit sphere.
static void solid_harmonic(int l, int m, std::vector<double>& row) {
  const int am = m < 0 ? -m : m;
  const int ncart = (l + 1) * (l + 2) / 2;
  row.assign(ncart, 0.0);
  const double Nlm = 1.0 / (std::pow(2.0, am) * fact(l)) *
                     std::sqrt(2.0 * fact(l + am) * fact(l - am) / (m == 0 ? 2.0 : 1.0));
  // v runs over v_m, v_m+1, ... with v_m = 0 (m>=0) or 1/2 (m<0); we loop over
  // twice v, i.e. 2v = 0,2,4,... or 1,3,5,...
  const int twovm = m < 0 ? 1 : 0;
  for (int t = 0; t <= (l - am) / 2; ++t)
    for (int u = 0; u <= t; ++u) {
      // v from v_m to floor(|m|/2 - v_m) + v_m
      const int vmax2 = 2 * ((am - twovm) / 2) + twovm;  // largest 2v
      for (int twov = twovm; twov <= vmax2; twov += 2) {
        const int sgn_exp = t + (twov - twovm) / 2;
        const double C = ((sgn_exp % 2) ? -1.0 : 1.0) * std::pow(0.25, t) * binom(l, t) *
                         binom(l - t, am + t) * binom(t, u) * binom(am, twov);
        const int ix = 2 * t + am - 2 * u - twov;
        const int iy = 2 * u + twov;
        const int iz = l - 2 * t - am;
        if (ix < 0 || iy < 0 || iz < 0) continue;
        row[cart_index(l, ix, iy, iz)] += Nlm * C;
      }
    }
  const double yn = std::sqrt((2 * l + 1) / (4.0 * M_PI));
  for (auto& v : row) v *= yn;
}

const std::vector<double>& sph_coeffs(int l) {
  static std::vector<double> table[kMaxL + 1];
  static std::once_flag once;
  std::call_once(once, [] {
    for (int L = 0; L <= kMaxL; ++L) {
      const int ncart = (L + 1) * (L + 2) / 2;
      std::vector<int> order;
      if (L == 1)
        order = {1, -1, 0};  // (x, y, z)
      else
        for (int m = -L; m <= L; ++m) order.push_back(m);
      table[L].assign((2 * L + 1) * ncart, 0.0);
      std::vector<double> row;
      for (int k = 0; k < 2 * L + 1; ++k) {
        solid_harmonic(L, order[k], row);
        for (int c = 0; c < ncart; ++c) table[L][k * ncart + c] = row[c];
      }
    }
  });
  return table[l];
}

// E^{ij}_t along one axis, for i <= la, j <= lb (McMurchie–Davidson
// recursions, Helgaker et al. eq. 9.5.6-9.5.7):
//   E^{00}_0 = K_ab
//   E^{i+1,j}_t = E^{ij}_{t-1}/(2p) + X_PA E^{ij}_t + (t+1) E^{ij}_{t+1}
//   E^{i,j+1}_t = E^{ij}_{t-1}/(2p) + X_PB E^{ij}_t + (t+1) E^{ij}_{t+1}
void hermite_1d(int la, int lb, double p, double xpa, double xpb, double kab,
                Herm1D& E) {
  const double oo2p = 0.5 / p;
  auto& e = E.e;
  for (int i = 0; i <= la; ++i)
    for (int j = 0; j <= lb; ++j)
      for (int t = 0; t < 2 * Herm1D::S; ++t) e[i][j][t] = 0.0;
  e[0][0][0] = kab;
  for (int i = 0; i < la; ++i)
    for (int t = 0; t <= i + 1; ++t) {
      double v = xpa * e[i][0][t] + (t + 1) * e[i][0][t + 1];
      if (t > 0) v += oo2p * e[i][0][t - 1];
      e[i + 1][0][t] = v;
    }
  for (int i = 0; i <= la; ++i)
    for (int j = 0; j < lb; ++j)
      for (int t = 0; t <= i + j + 1; ++t) {
        double v = xpb * e[i][j][t] + (t + 1) * e[i][j][t + 1];
        if (t > 0) v += oo2p * e[i][j][t - 1];
        e[i][j + 1][t] = v;
      }
}

// R_{tuv} = R^0_{tuv} from R^n_{000} = (-2 alpha)^n F_n(alpha R^2) and
//   R^{n}_{t+1,u,v} = t R^{n+1}_{t-1,u,v} + X R^{n+1}_{t,u,v}   (same in u, v)
// (Helgaker et al. eq. 9.9.18-9.9.20), built level by level from n = L down.
void hermite_r(int L, double alpha, double X, double Y, double Z, HermR& R) {
  double F[kMaxLTot + 1];
  boys(L, alpha * (X * X + Y * Y + Z * Z), F);
  static thread_local HermR prev;
  double fac = 1.0;
  double rn[kMaxLTot + 1];
  for (int n = 0; n <= L; ++n) {
    rn[n] = fac * F[n];
    fac *= -2.0 * alpha;
  }
  // level n holds totals t+u+v <= L-n; start with n = L (only 000).
  auto* cur = &R;
  auto* old = &prev;
  // choose buffer parity so that level 0 lands in R
  if (L % 2 == 1) std::swap(cur, old);
  cur->r[0][0][0] = rn[L];
  for (int n = L - 1; n >= 0; --n) {
    std::swap(cur, old);
    const int lt = L - n;
    for (int t = 0; t <= lt; ++t)
      for (int u = 0; u <= lt - t; ++u)
        for (int v = 0; v <= lt - t - u; ++v) {
          double val;
          if (t > 0) {
            val = X * old->r[t - 1][u][v];
            if (t > 1) val += (t - 1) * old->r[t - 2][u][v];
          } else if (u > 0) {
            val = Y * old->r[t][u - 1][v];
            if (u > 1) val += (u - 1) * old->r[t][u - 2][v];
          } else if (v > 0) {
            val = Z * old->r[t][u][v - 1];
            if (v > 1) val += (v - 1) * old->r[t][u][v - 2];
          } else {
            val = rn[n];
          }
          cur->r[t][u][v] = val;
        }
  }
}

}  // namespace gbints
