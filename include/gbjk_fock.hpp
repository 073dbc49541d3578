// C++ J/K builders over the gbjk C ABI, with the shape of megalochem's
// fock::J / fock::K classes (src/fock/jkbuilder.hpp:62-210):
// set_density_alpha/beta, set_coeff_alpha/beta, set_sym, set_SAD, init(),
// compute_J()/compute_K(), get_J()/get_K_A()/get_K_B(), and the factories
// create_j()/create_k() keyed by the same method strings.  Matrices are
// dense row-major std::vector<double> (the reference passes DBCSR matrices,
// which its call sites convert to and from dense arrays).  Errors throw
// std::runtime_error carrying gbjk_last_error(), as the reference throws.
#pragma once
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbjk.h"

namespace gbjk_fock {

using matrix = std::shared_ptr<std::vector<double>>;

// Owns one gbjk context: the resident 3-center tensor and metric factors.
class engine {
 public:
  engine(const gbjk_desc& desc, const double* B, const double* Linv, const double* Vinv,
         int precision = GBJK_FP64, int nslices = 0)
      : nbf_(desc.nbf) {
    check(gbjk_create(&ctx_, &desc), "gbjk_create");
    check(gbjk_upload_b(ctx_, B), "gbjk_upload_b");
    check(gbjk_upload_metric(ctx_, Linv, Vinv), "gbjk_upload_metric");
    check(gbjk_set_precision(ctx_, precision, nslices), "gbjk_set_precision");
  }
  ~engine() { gbjk_destroy(ctx_); }
  engine(const engine&) = delete;
  engine& operator=(const engine&) = delete;

  gbjk_ctx* ctx() const { return ctx_; }
  int nbf() const { return nbf_; }
  void check(gbjk_status s, const char* what) const {
    if (s != GBJK_OK)
      throw std::runtime_error(std::string(what) + ": " + (ctx_ ? gbjk_last_error(ctx_) : ""));
  }

 private:
  gbjk_ctx* ctx_ = nullptr;
  int nbf_;
};

class JK_common {
 public:
  explicit JK_common(std::shared_ptr<engine> e) : eng_(std::move(e)) {}
  virtual ~JK_common() = default;
  void set_density_alpha(matrix p) { m_p_A = std::move(p); }
  void set_density_beta(matrix p) { m_p_B = std::move(p); }
  // coefficient matrices are nbf x nocc, row-major
  void set_coeff_alpha(matrix c, int nocc) { m_c_A = std::move(c); m_nocc_A = nocc; }
  void set_coeff_beta(matrix c, int nocc) { m_c_B = std::move(c); m_nocc_B = nocc; }
  void set_sym(bool sym) { m_sym = sym; }
  void set_SAD(bool sad, int rank) { m_SAD_iter = sad; m_SAD_rank = rank; }

 protected:
  std::shared_ptr<engine> eng_;
  matrix m_p_A, m_p_B, m_c_A, m_c_B;
  int m_nocc_A = 0, m_nocc_B = 0;
  bool m_sym = true, m_SAD_iter = false;
  int m_SAD_rank = 0;
};

class J : public JK_common {
 public:
  using JK_common::JK_common;
  virtual void init() = 0;
  virtual void compute_J() = 0;
  matrix get_J() { return m_J; }

 protected:
  matrix m_J;
};

class K : public JK_common {
 public:
  using JK_common::JK_common;
  virtual void init() = 0;
  virtual void compute_K() = 0;
  matrix get_K_A() { return m_K_A; }
  matrix get_K_B() { return m_K_B; }

 protected:
  matrix m_K_A, m_K_B;
};

// fock::DF_J (src/fock/jkdf.cpp:13-190): P_tot = 2 P_A (RHF) or P_A + P_B.
class DF_J : public J {
 public:
  using J::J;
  void init() override {
    m_J = std::make_shared<std::vector<double>>((size_t)eng_->nbf() * eng_->nbf());
  }
  void compute_J() override {
    if (!m_p_A) throw std::runtime_error("DF_J: density not set");
    const size_t n2 = (size_t)eng_->nbf() * eng_->nbf();
    std::vector<double> ptot(n2);
    for (size_t i = 0; i < n2; ++i)
      ptot[i] = m_p_B ? (*m_p_A)[i] + (*m_p_B)[i] : 2.0 * (*m_p_A)[i];
    eng_->check(gbjk_compute_j(eng_->ctx(), ptot.data(), m_J->data()), "DF_J::compute_J");
  }
};

// fock::DFMO_K / fock::DFLMO_K (src/fock/jkdf.cpp:192-462, :861-1091).
class DF_K : public K {
 public:
  DF_K(std::shared_ptr<engine> e, int kmethod) : K(std::move(e)), kmethod_(kmethod) {}
  void init() override {
    const size_t n2 = (size_t)eng_->nbf() * eng_->nbf();
    m_K_A = std::make_shared<std::vector<double>>(n2);
    if (m_c_B) m_K_B = std::make_shared<std::vector<double>>(n2);
  }
  void compute_K() override {
    if (!m_c_A) throw std::runtime_error("DF_K: coefficients not set");
    eng_->check(gbjk_compute_k(eng_->ctx(), kmethod_, m_c_A->data(), m_nocc_A, m_K_A->data()),
                "DF_K::compute_K");
    if (m_c_B) {
      if (!m_K_B) m_K_B = std::make_shared<std::vector<double>>(m_K_A->size());
      eng_->check(gbjk_compute_k(eng_->ctx(), kmethod_, m_c_B->data(), m_nocc_B, m_K_B->data()),
                  "DF_K::compute_K");
    }
  }

 private:
  int kmethod_;
};

// fock::DFLMO_K with set_sym(false) (src/fock/jkdf.cpp:1093-1323): left
// coefficients U (nbf x nocc) and right coefficients Vt (nocc x nbf), as
// the ADC matrix-vector products set them.
class DFLMO_K_asym : public K {
 public:
  using K::K;
  void set_coeff_left_alpha(matrix u, int nocc) { m_u_A = std::move(u); m_nocc_u = nocc; }
  void set_coeff_right_alpha(matrix vt) { m_vt_A = std::move(vt); }
  void init() override {
    m_K_A = std::make_shared<std::vector<double>>((size_t)eng_->nbf() * eng_->nbf());
  }
  void compute_K() override {
    if (!m_u_A || !m_vt_A) throw std::runtime_error("DFLMO_K: left/right coefficients not set");
    eng_->check(gbjk_compute_k_lmo_asym(eng_->ctx(), m_u_A->data(), m_vt_A->data(), m_nocc_u,
                                        m_K_A->data()),
                "DFLMO_K::compute_K");
  }

 private:
  matrix m_u_A, m_vt_A;
  int m_nocc_u = 0;
};

// fock::DFAO_K (src/fock/jkdf.cpp:464-648): K from the density with the
// fitting coefficients V^-1 (X|mn) (src/ints/fitting.cpp:44-161).
class DFAO_K : public K {
 public:
  using K::K;
  void init() override {
    const size_t n2 = (size_t)eng_->nbf() * eng_->nbf();
    m_K_A = std::make_shared<std::vector<double>>(n2);
    if (m_p_B) m_K_B = std::make_shared<std::vector<double>>(n2);
  }
  void compute_K() override {
    if (!m_p_A) throw std::runtime_error("DFAO_K: density not set");
    eng_->check(gbjk_compute_k_ao(eng_->ctx(), m_p_A->data(), m_K_A->data()), "DFAO_K::compute_K");
    if (m_p_B) {
      if (!m_K_B) m_K_B = std::make_shared<std::vector<double>>(m_K_A->size());
      eng_->check(gbjk_compute_k_ao(eng_->ctx(), m_p_B->data(), m_K_B->data()),
                  "DFAO_K::compute_K");
    }
  }
};

// mp::LL_FULL_Z (src/mp/z_full.cpp:427-620) for all Laplace points at once:
// set_occ_coeff / set_vir_coeff per point (nbf x rank, row-major), then
// compute(); energies() holds e_t = tr(Z_t V^-1 Z_t V^-1), zmat(t) the
// fitted Z~_t = L^-1 Z_t L^-T (naux x naux) when requested.
class LaplaceZ {
 public:
  LaplaceZ(std::shared_ptr<engine> e, int npts)
      : eng_(std::move(e)), lo_(npts), lv_(npts), ro_(npts, 0), rv_(npts, 0), e_(npts, 0.0) {}
  void set_occ_coeff(int t, matrix L, int rank) { lo_.at(t) = std::move(L); ro_.at(t) = rank; }
  void set_vir_coeff(int t, matrix L, int rank) { lv_.at(t) = std::move(L); rv_.at(t) = rank; }
  void compute(std::vector<double>* zmats = nullptr) {
    const int n = (int)lo_.size();
    std::vector<const double*> po(n), pv(n);
    for (int t = 0; t < n; ++t) {
      if (!lo_[t] || !lv_[t]) throw std::runtime_error("LaplaceZ: factor not set");
      po[t] = lo_[t]->data();
      pv[t] = lv_[t]->data();
    }
    eng_->check(gbjk_mp2_laplace(eng_->ctx(), n, ro_.data(), po.data(), rv_.data(), pv.data(),
                                 e_.data(), zmats ? zmats->data() : nullptr),
                "LaplaceZ::compute");
  }
  const std::vector<double>& energies() const { return e_; }

 private:
  std::shared_ptr<engine> eng_;
  std::vector<matrix> lo_, lv_;
  std::vector<int> ro_, rv_;
  std::vector<double> e_;
};

// fock::create_j / create_k (src/fock/jkbuilder.hpp:621-841).
inline std::shared_ptr<J> create_j(std::shared_ptr<engine> e, const std::string& method) {
  if (method == "dfao") return std::make_shared<DF_J>(std::move(e));
  throw std::runtime_error("Invalid jmethod");
}

inline std::shared_ptr<K> create_k(std::shared_ptr<engine> e, const std::string& method) {
  if (method == "dfmo") return std::make_shared<DF_K>(std::move(e), GBJK_K_DFMO);
  if (method == "dflmo") return std::make_shared<DF_K>(std::move(e), GBJK_K_DFLMO);
  // fock::DFMEM_K (src/fock/jkdf.cpp:650-859) is the DF-AO exchange with the
  // fit on the other factor, -(B^T V^-1 B P): the same builder serves it
  if (method == "dfao" || method == "dfmem") return std::make_shared<DFAO_K>(std::move(e));
  // fock::DFROBUST_K needs the PARI metric, which the reference requires
  // (src/fock/jkbuilder.hpp:598-603); this engine has the Coulomb metric only
  if (method == "dfrobust")
    throw std::runtime_error("Cannot use robust k for method other than PARI");
  throw std::runtime_error("Invalid kmethod");
}

}  // namespace gbjk_fock
