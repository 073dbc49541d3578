// C-ABI of the host integral engine.  Declared in include/gbints.h.
//
// Stands in for the libcint-based integral drivers megalochem runs once per
// molecule (src/ints/aofactory.cpp, src/ints/integrals.cpp).  Everything is
// FP64; the 3-center tensor is written straight into the atom-block panel
// layout that the device J/K engine keeps resident in HBM.
#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "md_engine.hpp"

using namespace gbints;

struct gbints_basis {
  Basis b;
};

namespace {

constexpr double kPi = 3.14159265358979323846;
// 2 pi^{5/2}
const double kTwoPi52 = 2.0 * std::pow(kPi, 2.5);
// primitive pairs whose |c_a c_b K_ab| falls below this are skipped
constexpr double kPrimCut = 1e-16;

double gaussian_int(int n, double a) {
  // int_0^inf r^n exp(-a r^2) dr   (src/ints/aofactory.cpp:278-282)
  const double n1 = (n + 1) * 0.5;
  return std::tgamma(n1) / (2.0 * std::pow(a, n1));
}

double gto_norm(int l, double a) { return 1.0 / std::sqrt(gaussian_int(2 * l + 2, 2 * a)); }

// Radial normalisation of a contracted shell (src/ints/aofactory.cpp:290-314).
std::vector<double> gto_normalize(int l, const std::vector<double>& es,
                                  const std::vector<double>& cs) {
  std::vector<double> c = cs;
  const size_t n = es.size();
  for (size_t i = 0; i < n; ++i) c[i] *= gto_norm(l, es[i]);
  double norm = 0.0;
  for (size_t p = 0; p < n; ++p)
    for (size_t q = 0; q < n; ++q) norm += c[p] * gaussian_int(2 * l + 2, es[p] + es[q]) * c[q];
  norm = 1.0 / std::sqrt(norm);
  for (auto& v : c) v *= norm;
  return c;
}

// One primitive pair of a shell pair: Gaussian product data and Hermite
// expansion tables for the three axes.
struct PrimPair {
  double p, P[3], coef;
  Herm1D E[3];
};

void make_primpair(const Shell& a, int ia, const Shell& b, int ib, int extra, PrimPair& pp) {
  const double al = a.alpha[ia], be = b.alpha[ib];
  const double p = al + be;
  pp.p = p;
  double ab2 = 0;
  for (int d = 0; d < 3; ++d) {
    pp.P[d] = (al * a.A[d] + be * b.A[d]) / p;
    const double dd = a.A[d] - b.A[d];
    ab2 += dd * dd;
  }
  const double kab = std::exp(-al * be / p * ab2);
  pp.coef = a.coef[ia] * b.coef[ib];
  for (int d = 0; d < 3; ++d)
    hermite_1d(a.l, b.l + extra, p, pp.P[d] - a.A[d], pp.P[d] - b.A[d], d == 0 ? kab : 1.0,
               pp.E[d]);
}

// Single-centre "pair": shell a times an s function with exponent 0.
void make_single(const Shell& a, int ia, PrimPair& pp) {
  pp.p = a.alpha[ia];
  for (int d = 0; d < 3; ++d) pp.P[d] = a.A[d];
  pp.coef = a.coef[ia];
  for (int d = 0; d < 3; ++d) hermite_1d(a.l, 0, pp.p, 0.0, 0.0, 1.0, pp.E[d]);
}

// Hermite expansion of the cartesian pair (ca of la, cb of lb) as a sparse
// list over (t,u,v): coefficient E^x_t E^y_u E^z_v.
struct HermTerm {
  int t, u, v;
  double c;
};

void herm_terms(const PrimPair& pp, int la, int ca, int lb, int cb, std::vector<HermTerm>& out) {
  int ea[3], eb[3];
  cart_exponents(la, ca, ea);
  cart_exponents(lb, cb, eb);
  out.clear();
  for (int t = 0; t <= ea[0] + eb[0]; ++t) {
    const double ex = pp.E[0].e[ea[0]][eb[0]][t];
    if (ex == 0.0) continue;
    for (int u = 0; u <= ea[1] + eb[1]; ++u) {
      const double ey = pp.E[1].e[ea[1]][eb[1]][u];
      if (ey == 0.0) continue;
      for (int v = 0; v <= ea[2] + eb[2]; ++v) {
        const double ez = pp.E[2].e[ea[2]][eb[2]][v];
        if (ez == 0.0) continue;
        out.push_back({t, u, v, ex * ey * ez});
      }
    }
  }
}

// Transform a cartesian block (na_c x nb_c [x rest]) to spherical on the
// first two indices: out[ma][mb][r] = sum sph_a[ma][ca] sph_b[mb][cb] in[ca][cb][r].
void cart2sph_2(int la, int lb, int nrest, const double* in, double* out) {
  const auto& sa = sph_coeffs(la);
  const auto& sb = sph_coeffs(lb);
  const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
  const int nsa = 2 * la + 1, nsb = 2 * lb + 1;
  std::vector<double> tmp((size_t)nsa * ncb * nrest, 0.0);
  for (int ma = 0; ma < nsa; ++ma)
    for (int ca = 0; ca < nca; ++ca) {
      const double f = sa[ma * nca + ca];
      if (f == 0.0) continue;
      const double* src = in + (size_t)ca * ncb * nrest;
      double* dst = tmp.data() + (size_t)ma * ncb * nrest;
      for (size_t k = 0; k < (size_t)ncb * nrest; ++k) dst[k] += f * src[k];
    }
  std::fill(out, out + (size_t)nsa * nsb * nrest, 0.0);
  for (int ma = 0; ma < nsa; ++ma)
    for (int mb = 0; mb < nsb; ++mb)
      for (int cb = 0; cb < ncb; ++cb) {
        const double f = sb[mb * ncb + cb];
        if (f == 0.0) continue;
        const double* src = tmp.data() + ((size_t)ma * ncb + cb) * nrest;
        double* dst = out + ((size_t)ma * nsb + mb) * nrest;
        for (int r = 0; r < nrest; ++r) dst[r] += f * src[r];
      }
}

// Two-electron Hermite contraction for one bra primitive pair and one ket
// primitive pair:  acc[bra_cart][ket_cart] += pref * sum_{tuv} E^bra_tuv
//   sum_{tau nu phi} (-1)^{tau+nu+phi} E^ket_{tau nu phi} R_{t+tau,u+nu,v+phi}.
void eri_prim(const PrimPair& bra, int la, int lb, const PrimPair& ket, int lc, int ld,
              double* acc, std::vector<HermTerm>& tb, std::vector<HermTerm>& tk,
              HermR& R) {
  const double p = bra.p, q = ket.p;
  const double alpha = p * q / (p + q);
  const double pref = kTwoPi52 / (p * q * std::sqrt(p + q)) * bra.coef * ket.coef;
  const int L = la + lb + lc + ld;
  hermite_r(L, alpha, bra.P[0] - ket.P[0], bra.P[1] - ket.P[1], bra.P[2] - ket.P[2], R);
  const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
  const int ncc = (lc + 1) * (lc + 2) / 2, ncd = (ld + 1) * (ld + 2) / 2;
  const int nket = ncc * ncd;
  // W[tuv][ket_cart] for all tuv with t+u+v <= la+lb
  const int Lb = la + lb;
  const int S = Lb + 1;
  std::vector<double> W((size_t)S * S * S * nket, 0.0);
  for (int cc = 0; cc < ncc; ++cc)
    for (int cd = 0; cd < ncd; ++cd) {
      herm_terms(ket, lc, cc, ld, cd, tk);
      const int kidx = cc * ncd + cd;
      for (int t = 0; t <= Lb; ++t)
        for (int u = 0; u <= Lb - t; ++u)
          for (int v = 0; v <= Lb - t - u; ++v) {
            double s = 0.0;
            for (const auto& h : tk) {
              const double sg = ((h.t + h.u + h.v) & 1) ? -1.0 : 1.0;
              s += sg * h.c * R.r[t + h.t][u + h.u][v + h.v];
            }
            W[(((size_t)t * S + u) * S + v) * nket + kidx] = s;
          }
    }
  for (int ca = 0; ca < nca; ++ca)
    for (int cb = 0; cb < ncb; ++cb) {
      herm_terms(bra, la, ca, lb, cb, tb);
      double* dst = acc + ((size_t)ca * ncb + cb) * nket;
      for (const auto& h : tb) {
        const double* w = W.data() + (((size_t)h.t * S + h.u) * S + h.v) * nket;
        const double f = pref * h.c;
        for (int k = 0; k < nket; ++k) dst[k] += f * w[k];
      }
    }
}

// Contracted (ab|cd) over shells, spherical output [a][b][c][d].
void shell_quartet(const Shell& a, const Shell& b, const Shell& c, const Shell& d,
                   std::vector<double>& out) {
  const int nca = a.ncart(), ncb = b.ncart(), ncc = c.ncart(), ncd = d.ncart();
  std::vector<double> acc((size_t)nca * ncb * ncc * ncd, 0.0);
  std::vector<HermTerm> tb, tk;
  static thread_local HermR R;
  PrimPair bra, ket;
  for (size_t ia = 0; ia < a.alpha.size(); ++ia)
    for (size_t ib = 0; ib < b.alpha.size(); ++ib) {
      make_primpair(a, ia, b, ib, 0, bra);
      if (std::fabs(bra.coef * bra.E[0].e[0][0][0]) < kPrimCut) continue;
      for (size_t ic = 0; ic < c.alpha.size(); ++ic)
        for (size_t id = 0; id < d.alpha.size(); ++id) {
          make_primpair(c, ic, d, id, 0, ket);
          if (std::fabs(ket.coef * ket.E[0].e[0][0][0]) < kPrimCut) continue;
          eri_prim(bra, a.l, b.l, ket, c.l, d.l, acc.data(), tb, tk, R);
        }
    }
  // transform bra, then ket
  const int nsa = a.nsph(), nsb = b.nsph(), nsc = c.nsph(), nsd = d.nsph();
  std::vector<double> t1((size_t)nsa * nsb * ncc * ncd);
  cart2sph_2(a.l, b.l, ncc * ncd, acc.data(), t1.data());
  // now transpose to [cd][ab] to reuse cart2sph_2 on the ket
  std::vector<double> t2((size_t)ncc * ncd * nsa * nsb);
  for (int i = 0; i < nsa * nsb; ++i)
    for (int k = 0; k < ncc * ncd; ++k) t2[(size_t)k * nsa * nsb + i] = t1[(size_t)i * ncc * ncd + k];
  std::vector<double> t3((size_t)nsc * nsd * nsa * nsb);
  cart2sph_2(c.l, d.l, nsa * nsb, t2.data(), t3.data());
  out.assign((size_t)nsa * nsb * nsc * nsd, 0.0);
  for (int k = 0; k < nsc * nsd; ++k)
    for (int i = 0; i < nsa * nsb; ++i) out[(size_t)i * nsc * nsd + k] = t3[(size_t)k * nsa * nsb + i];
}

// Contracted (a|c) 2-center Coulomb, spherical [a][c].
void shell_pair_2c(const Shell& a, const Shell& c, std::vector<double>& out) {
  const int nca = a.ncart(), ncc = c.ncart();
  std::vector<double> acc((size_t)nca * ncc, 0.0);
  std::vector<HermTerm> tb, tk;
  static thread_local HermR R;
  PrimPair bra, ket;
  for (size_t ia = 0; ia < a.alpha.size(); ++ia) {
    make_single(a, ia, bra);
    for (size_t ic = 0; ic < c.alpha.size(); ++ic) {
      make_single(c, ic, ket);
      eri_prim(bra, a.l, 0, ket, c.l, 0, acc.data(), tb, tk, R);
    }
  }
  // transform the two real indices only (the exponent-0 partners carry no
  // angular factor)
  const auto& sa = sph_coeffs(a.l);
  const auto& sc = sph_coeffs(c.l);
  out.assign((size_t)a.nsph() * c.nsph(), 0.0);
  for (int ma = 0; ma < a.nsph(); ++ma)
    for (int ca = 0; ca < nca; ++ca) {
      const double fa = sa[ma * nca + ca];
      if (fa == 0.0) continue;
      for (int mc = 0; mc < c.nsph(); ++mc) {
        double s = 0.0;
        for (int cc = 0; cc < ncc; ++cc) s += sc[mc * ncc + cc] * acc[(size_t)ca * ncc + cc];
        out[(size_t)ma * c.nsph() + mc] += fa * s;
      }
    }
}

// 3-center (X|ab) for one AO shell pair (a, b) against a list of auxiliary
// shells.  Output in cartesian a,b and spherical X:
//   acc[ca][cb][xoff(k) + mx]   for aux shell k of the list.
// Ket side of an auxiliary shell, per primitive and cartesian component:
// its single-centre Hermite terms with the sign (-1)^(t+u+v) of the Coulomb
// kernel folded into the coefficient (a product with +-1, so exact).  It
// depends on the auxiliary shell only, so it is built once per tensor rather
// than once per bra primitive pair.
struct KetTable {
  std::vector<std::vector<std::vector<HermTerm>>> terms;  // [prim][cc]
  std::vector<std::vector<std::vector<int>>> roff;        // flat R offsets of the terms
};

KetTable make_ket_table(const Shell& c) {
  KetTable t;
  t.terms.resize(c.alpha.size());
  t.roff.resize(c.alpha.size());
  PrimPair ket;
  for (size_t ic = 0; ic < c.alpha.size(); ++ic) {
    make_single(c, (int)ic, ket);
    t.terms[ic].resize(c.ncart());
    t.roff[ic].resize(c.ncart());
    for (int cc = 0; cc < c.ncart(); ++cc) {
      herm_terms(ket, c.l, cc, 0, 0, t.terms[ic][cc]);
      for (auto& h : t.terms[ic][cc]) {
        if ((h.t + h.u + h.v) & 1) h.c = -h.c;
        t.roff[ic][cc].push_back((h.t * HermR::S + h.u) * HermR::S + h.v);
      }
    }
  }
  return t;
}

struct Aux3c {
  const Shell* sh;
  int xoff;                    // offset of the shell's functions in the output row
  const KetTable* ket = nullptr;  // ket terms of the shell
};

void pair_vs_aux(const Shell& a, const Shell& b, const std::vector<Aux3c>& aux, int nxtot,
                 std::vector<double>& acc) {
  const int nca = a.ncart(), ncb = b.ncart();
  // the auxiliary index stays cartesian through the primitive loops and is
  // transformed to spherical once at the end (not once per primitive pair)
  int nxc = 0;
  for (const auto& ax : aux) nxc += ax.sh->ncart();
  std::vector<double> accc((size_t)nca * ncb * nxc, 0.0);
  static thread_local HermR R;
  PrimPair bra;
  const int Lb = a.l + b.l;
  const int S = Lb + 1;
  std::vector<double> W;
  std::vector<std::vector<HermTerm>> braterms(nca * ncb);
  for (size_t ia = 0; ia < a.alpha.size(); ++ia)
    for (size_t ib = 0; ib < b.alpha.size(); ++ib) {
      make_primpair(a, ia, b, ib, 0, bra);
      if (std::fabs(bra.coef * bra.E[0].e[0][0][0]) < kPrimCut) continue;
      for (int ca = 0; ca < nca; ++ca)
        for (int cb = 0; cb < ncb; ++cb) herm_terms(bra, a.l, ca, b.l, cb, braterms[ca * ncb + cb]);
      int xc = 0;
      for (const auto& ax : aux) {
        const Shell& c = *ax.sh;
        const int lc = c.l, ncc = c.ncart();
        // W[tuv][cc], cartesian auxiliary components
        W.assign((size_t)S * S * S * ncc, 0.0);
        for (size_t ic = 0; ic < c.alpha.size(); ++ic) {
          const double p = bra.p, q = c.alpha[ic];
          const double alpha = p * q / (p + q);
          const double pref = kTwoPi52 / (p * q * std::sqrt(p + q)) * bra.coef * c.coef[ic];
          hermite_r(Lb + lc, alpha, bra.P[0] - c.A[0], bra.P[1] - c.A[1], bra.P[2] - c.A[2], R);
          const double* R0 = &R.r[0][0][0];
          for (int cc = 0; cc < ncc; ++cc) {
            const std::vector<HermTerm>& tk = ax.ket->terms[ic][cc];
            const HermTerm* tb = tk.data();
            const int nt = (int)tk.size();
            const int* toff = ax.ket->roff[ic][cc].data();
            for (int t = 0; t <= Lb; ++t)
              for (int u = 0; u <= Lb - t; ++u)
                for (int v = 0; v <= Lb - t - u; ++v) {
                  double s = 0.0;
                  const double* Rb = R0 + (t * HermR::S + u) * HermR::S + v;
                  for (int q = 0; q < nt; ++q) s += tb[q].c * Rb[toff[q]];
                  W[(((size_t)t * S + u) * S + v) * ncc + cc] += pref * s;
                }
          }
        }
        for (int cab = 0; cab < nca * ncb; ++cab) {
          double* dst = accc.data() + (size_t)cab * nxc + xc;
          for (const auto& h : braterms[cab]) {
            const double* w = W.data() + (((size_t)h.t * S + h.u) * S + h.v) * ncc;
            for (int cc = 0; cc < ncc; ++cc) dst[cc] += h.c * w[cc];
          }
        }
        xc += ncc;
      }
    }
  // spherical auxiliary components: acc[cab][xoff + mc]
  acc.assign((size_t)nca * ncb * nxtot, 0.0);
  int xc = 0;
  for (const auto& ax : aux) {
    const Shell& c = *ax.sh;
    const int ncc = c.ncart(), nsc = c.nsph();
    const auto& sc = sph_coeffs(c.l);
    for (int cab = 0; cab < nca * ncb; ++cab) {
      const double* src = accc.data() + (size_t)cab * nxc + xc;
      double* dst = acc.data() + (size_t)cab * nxtot + ax.xoff;
      for (int mc = 0; mc < nsc; ++mc) {
        double v = 0.0;
        for (int cc = 0; cc < ncc; ++cc) v += sc[mc * ncc + cc] * src[cc];
        dst[mc] = v;
      }
    }
    xc += ncc;
  }
}

// One-electron integrals over a shell pair: which = 0 overlap, 1 kinetic,
// 2 nuclear attraction.  Spherical output [a][b].
void shell_pair_1e(const Shell& a, const Shell& b, int which, int natom, const double* Z,
                   const double* xyz, std::vector<double>& out) {
  const int nca = a.ncart(), ncb = b.ncart();
  std::vector<double> acc((size_t)nca * ncb, 0.0);
  PrimPair pp;
  static thread_local HermR R;
  for (size_t ia = 0; ia < a.alpha.size(); ++ia)
    for (size_t ib = 0; ib < b.alpha.size(); ++ib) {
      make_primpair(a, ia, b, ib, which == 1 ? 2 : 0, pp);
      const double p = pp.p;
      const double be = b.alpha[ib];
      const double sp = std::pow(kPi / p, 0.5);
      for (int ca = 0; ca < nca; ++ca)
        for (int cb = 0; cb < ncb; ++cb) {
          int ea[3], eb[3];
          cart_exponents(a.l, ca, ea);
          cart_exponents(b.l, cb, eb);
          double val = 0.0;
          if (which == 0 || which == 1) {
            double s1[3], t1[3];
            for (int d = 0; d < 3; ++d) {
              const auto& e = pp.E[d].e;
              const int i = ea[d], j = eb[d];
              s1[d] = e[i][j][0] * sp;
              if (which == 1) {
                double tk = -2.0 * be * be * e[i][j + 2][0] + be * (2 * j + 1) * e[i][j][0];
                if (j >= 2) tk -= 0.5 * j * (j - 1) * e[i][j - 2][0];
                t1[d] = tk * sp;
              }
            }
            if (which == 0)
              val = s1[0] * s1[1] * s1[2];
            else
              val = t1[0] * s1[1] * s1[2] + s1[0] * t1[1] * s1[2] + s1[0] * s1[1] * t1[2];
          } else {
            for (int C = 0; C < natom; ++C) {
              hermite_r(a.l + b.l, p, pp.P[0] - xyz[3 * C], pp.P[1] - xyz[3 * C + 1],
                        pp.P[2] - xyz[3 * C + 2], R);
              double s = 0.0;
              for (int t = 0; t <= ea[0] + eb[0]; ++t)
                for (int u = 0; u <= ea[1] + eb[1]; ++u)
                  for (int v = 0; v <= ea[2] + eb[2]; ++v)
                    s += pp.E[0].e[ea[0]][eb[0]][t] * pp.E[1].e[ea[1]][eb[1]][u] *
                         pp.E[2].e[ea[2]][eb[2]][v] * R.r[t][u][v];
              val -= Z[C] * 2.0 * kPi / p * s;
            }
          }
          acc[(size_t)ca * ncb + cb] += pp.coef * val;
        }
    }
  out.resize((size_t)a.nsph() * b.nsph());
  cart2sph_2(a.l, b.l, 1, acc.data(), out.data());
}

template <class F>
void for_shell_pairs(const Basis& B, bool sym, F&& f, int nthreads) {
  const int ns = (int)B.shells.size();
  std::vector<std::pair<int, int>> pairs;
  for (int i = 0; i < ns; ++i)
    for (int j = sym ? i : 0; j < ns; ++j) pairs.emplace_back(i, j);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (long k = 0; k < (long)pairs.size(); ++k) f(pairs[k].first, pairs[k].second);
}

int threads_or_default(int n) { return n > 0 ? n : omp_get_max_threads(); }

}  // namespace

extern "C" {

int gbints_basis_create(gbints_basis** out, int nshell, const int* l, const int* nprim,
                        const double* centers, const double* alpha, const double* coef) {
  if (!out || nshell <= 0) return 1;
  auto* bb = new (std::nothrow) gbints_basis;
  if (!bb) return 2;
  int off = 0, poff = 0;
  for (int s = 0; s < nshell; ++s) {
    if (l[s] < 0 || l[s] > kMaxL || nprim[s] <= 0) {
      delete bb;
      return 1;
    }
    Shell sh;
    sh.l = l[s];
    for (int d = 0; d < 3; ++d) sh.A[d] = centers[3 * s + d];
    std::vector<double> es(alpha + poff, alpha + poff + nprim[s]);
    std::vector<double> cs(coef + poff, coef + poff + nprim[s]);
    poff += nprim[s];
    sh.alpha = es;
    sh.coef = gto_normalize(sh.l, es, cs);
    sh.bf_off = off;
    off += sh.nsph();
    bb->b.max_l = std::max(bb->b.max_l, sh.l);
    bb->b.shells.push_back(std::move(sh));
  }
  bb->b.nbf = off;
  *out = bb;
  return 0;
}

void gbints_basis_destroy(gbints_basis* b) { delete b; }

// Normalised shell data as the engine uses it (contraction coefficients
// after gto_normalize); arrays sized by the caller: nshell entries of l,
// nprim and bf_off, 3 * nshell centres, sum(nprim) exponents and
// coefficients.
int gbints_basis_shells(const gbints_basis* b, int* l, int* nprim, int* bf_off, double* centers,
                        double* alpha, double* coef) {
  if (!b) return 1;
  int poff = 0;
  for (size_t s = 0; s < b->b.shells.size(); ++s) {
    const Shell& sh = b->b.shells[s];
    l[s] = sh.l;
    nprim[s] = (int)sh.alpha.size();
    bf_off[s] = sh.bf_off;
    for (int d = 0; d < 3; ++d) centers[3 * s + d] = sh.A[d];
    for (size_t i = 0; i < sh.alpha.size(); ++i) {
      alpha[poff + i] = sh.alpha[i];
      coef[poff + i] = sh.coef[i];
    }
    poff += (int)sh.alpha.size();
  }
  return 0;
}

// Cartesian -> real-spherical table of shell l: (2l+1) x (l+1)(l+2)/2,
// row-major, output order as the integral routines (p: x, y, z).
int gbints_sph_coeffs(int l, double* out) {
  if (l < 0 || l > kMaxL || !out) return 1;
  const auto& t = sph_coeffs(l);
  std::copy(t.begin(), t.end(), out);
  return 0;
}

int gbints_basis_nbf(const gbints_basis* b) { return b ? b->b.nbf : -1; }

int gbints_one_electron(const gbints_basis* bs, int which, int natom, const double* Z,
                        const double* xyz, double* M, int nthreads) {
  if (!bs || !M || which < 0 || which > 2) return 1;
  const Basis& B = bs->b;
  const int n = B.nbf;
  for_shell_pairs(
      B, true,
      [&](int i, int j) {
        const Shell &a = B.shells[i], &b = B.shells[j];
        std::vector<double> out;
        shell_pair_1e(a, b, which, natom, Z, xyz, out);
        for (int p = 0; p < a.nsph(); ++p)
          for (int q = 0; q < b.nsph(); ++q) {
            const double v = out[(size_t)p * b.nsph() + q];
            M[(size_t)(a.bf_off + p) * n + b.bf_off + q] = v;
            M[(size_t)(b.bf_off + q) * n + a.bf_off + p] = v;
          }
      },
      threads_or_default(nthreads));
  return 0;
}

int gbints_coulomb_2c(const gbints_basis* bs, double* M, int nthreads) {
  if (!bs || !M) return 1;
  const Basis& B = bs->b;
  const int n = B.nbf;
  for_shell_pairs(
      B, true,
      [&](int i, int j) {
        const Shell &a = B.shells[i], &c = B.shells[j];
        std::vector<double> out;
        shell_pair_2c(a, c, out);
        for (int p = 0; p < a.nsph(); ++p)
          for (int q = 0; q < c.nsph(); ++q) {
            const double v = out[(size_t)p * c.nsph() + q];
            M[(size_t)(a.bf_off + p) * n + c.bf_off + q] = v;
            M[(size_t)(c.bf_off + q) * n + a.bf_off + p] = v;
          }
      },
      threads_or_default(nthreads));
  return 0;
}

// Full 4-center tensor (mu nu|la si), row-major nbf^4.  Small systems only.
int gbints_eri4c(const gbints_basis* bs, double* out, int nthreads) {
  if (!bs || !out) return 1;
  const Basis& B = bs->b;
  const int ns = (int)B.shells.size();
  const size_t n = B.nbf;
  std::vector<std::array<int, 4>> quartets;
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b < ns; ++b)
      for (int c = 0; c < ns; ++c)
        for (int d = 0; d < ns; ++d) quartets.push_back({a, b, c, d});
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads_or_default(nthreads))
  for (long k = 0; k < (long)quartets.size(); ++k) {
    const auto& qq = quartets[k];
    const Shell &A = B.shells[qq[0]], &Bs = B.shells[qq[1]], &C = B.shells[qq[2]],
                &D = B.shells[qq[3]];
    std::vector<double> v;
    shell_quartet(A, Bs, C, D, v);
    for (int i = 0; i < A.nsph(); ++i)
      for (int j = 0; j < Bs.nsph(); ++j)
        for (int kk = 0; kk < C.nsph(); ++kk)
          for (int l = 0; l < D.nsph(); ++l)
            out[(((A.bf_off + i) * n + Bs.bf_off + j) * n + C.bf_off + kk) * n + D.bf_off + l] =
                v[((i * Bs.nsph() + j) * C.nsph() + kk) * D.nsph() + l];
  }
  return 0;
}

// Per-shell-pair Schwarz factor sqrt(sum_{i in a, j in b} |(ij|ij)|)
// (src/ints/integrals.cpp:511-617).  Z is nshell x nshell.
int gbints_schwarz_pairs(const gbints_basis* bs, double* Z, int nthreads) {
  if (!bs || !Z) return 1;
  const Basis& B = bs->b;
  const int ns = (int)B.shells.size();
  for_shell_pairs(
      B, true,
      [&](int i, int j) {
        const Shell &a = B.shells[i], &b = B.shells[j];
        std::vector<double> v;
        shell_quartet(a, b, a, b, v);
        const int na = a.nsph(), nb = b.nsph();
        double s = 0.0;
        for (int p = 0; p < na; ++p)
          for (int q = 0; q < nb; ++q) s += std::fabs(v[((p * nb + q) * na + p) * nb + q]);
        Z[(size_t)i * ns + j] = Z[(size_t)j * ns + i] = std::sqrt(s);
      },
      threads_or_default(nthreads));
  return 0;
}

// Per-shell auxiliary Schwarz factor sqrt(sum_{i in a} |(i|i)|)
// (src/ints/integrals.cpp:619-689).
int gbints_schwarz_aux(const gbints_basis* bs, double* z, int nthreads) {
  if (!bs || !z) return 1;
  const Basis& B = bs->b;
  const int ns = (int)B.shells.size();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads_or_default(nthreads))
  for (int i = 0; i < ns; ++i) {
    std::vector<double> v;
    shell_pair_2c(B.shells[i], B.shells[i], v);
    const int na = B.shells[i].nsph();
    double s = 0.0;
    for (int p = 0; p < na; ++p) s += std::fabs(v[(size_t)p * na + p]);
    z[i] = std::sqrt(s);
  }
  return 0;
}

// 3-center integrals (X|mu nu) written into the atom-block panel layout:
// panel I (AO block I) is a dense [b_I][naux][K_I] array at B + panel_off[I],
// K_I = sum of b_J over the blocks J kept with I; block pair p = (I, J),
// I <= J, puts its columns at col_IJ[p] of panel I and col_JI[p] of panel J.
// keep[p * nablk + A] = 0 leaves the (A, I, J) block at zero (screened).
int gbints_eri3c_panels(const gbints_basis* ao, const gbints_basis* aux, int nblk,
                        const int* blk_shell_off, int nablk, const int* ablk_shell_off,
                        int npairs, const int* pair_I, const int* pair_J,
                        const unsigned char* keep, const long long* panel_off,
                        const int* panel_K, const int* col_IJ, const int* col_JI, double* B,
                        int nthreads) {
  if (!ao || !aux || !B) return 1;
  const Basis& AO = ao->b;
  const Basis& AX = aux->b;
  const int naux = AX.nbf;
  for (int p = 0; p < npairs; ++p)
    if (pair_I[p] < 0 || pair_J[p] < pair_I[p] || pair_J[p] >= nblk) return 1;
  // work items: (pair, shell a in I, shell b in J) with a<=b when I==J
  struct Item {
    int p, a, b;
  };
  std::vector<Item> items;
  for (int p = 0; p < npairs; ++p) {
    const int I = pair_I[p], J = pair_J[p];
    for (int a = blk_shell_off[I]; a < blk_shell_off[I + 1]; ++a)
      for (int b = blk_shell_off[J]; b < blk_shell_off[J + 1]; ++b) {
        if (I == J && b < a) continue;
        items.push_back({p, a, b});
      }
  }
  std::vector<KetTable> kets(AX.shells.size());
  for (size_t s = 0; s < AX.shells.size(); ++s) kets[s] = make_ket_table(AX.shells[s]);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads_or_default(nthreads))
  for (long k = 0; k < (long)items.size(); ++k) {
    const Item it = items[k];
    const int I = pair_I[it.p], J = pair_J[it.p];
    const Shell& a = AO.shells[it.a];
    const Shell& b = AO.shells[it.b];
    std::vector<Aux3c> list;
    int nx = 0;
    for (int A = 0; A < nablk; ++A) {
      if (!keep[(size_t)it.p * nablk + A]) continue;
      for (int s = ablk_shell_off[A]; s < ablk_shell_off[A + 1]; ++s) {
        list.push_back({&AX.shells[s], nx, &kets[s]});
        nx += AX.shells[s].nsph();
      }
    }
    if (list.empty()) continue;
    std::vector<double> acc;
    pair_vs_aux(a, b, list, nx, acc);
    std::vector<double> sph((size_t)a.nsph() * b.nsph() * nx);
    cart2sph_2(a.l, b.l, nx, acc.data(), sph.data());
    const int I0 = AO.shells[blk_shell_off[I]].bf_off;
    const int J0 = AO.shells[blk_shell_off[J]].bf_off;
    const int KI = panel_K[I], KJ = panel_K[J];
    double* PI = B + panel_off[I];
    double* PJ = B + panel_off[J];
    for (const auto& ax : list) {
      const int X0 = ax.sh->bf_off;
      const int nsx = ax.sh->nsph();
      for (int ma = 0; ma < a.nsph(); ++ma)
        for (int mb = 0; mb < b.nsph(); ++mb) {
          const int mu = a.bf_off + ma - I0;  // local in I
          const int nu = b.bf_off + mb - J0;  // local in J
          const double* src = sph.data() + ((size_t)ma * b.nsph() + mb) * nx + ax.xoff;
          for (int x = 0; x < nsx; ++x) {
            const double v = src[x];
            const size_t X = X0 + x;
            PI[((size_t)mu * naux + X) * KI + col_IJ[it.p] + nu] = v;
            if (I != J)
              PJ[((size_t)nu * naux + X) * KJ + col_JI[it.p] + mu] = v;
            else if (it.a != it.b)
              PI[((size_t)nu * naux + X) * KI + col_IJ[it.p] + mu] = v;
          }
        }
    }
  }
  return 0;
}

}  // extern "C"
