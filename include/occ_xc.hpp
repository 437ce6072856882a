// occ_xc.hpp -- C++ host interface over the C ABI (occ_xc.h), shaped like the
// XC part of OCC's occ::dft::DFT (include/occ/dft/dft.h:39, 83, 395, 590):
// construct from a method name and an AOBasis, call compute_vxc with mo.D,
// read exchange_correlation_energy().  Errors are thrown as exceptions, as
// OCC does.  Header-only; link libocc_xc.so.
//
//   occ_gb300::AOBasis basis(atoms, shells);   // shells normalised as OCC's
//   basis.set_pure(true);                      // gto::Shell after
//   occ_gb300::DFT dft("pbe", basis);          // incorporate_shell_norm
//   std::vector<double> V = dft.compute_vxc(D);           // D = mo.D, nbf x nbf
//   double exc = dft.exchange_correlation_energy();
#pragma once
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "occ_xc.h"

namespace occ_gb300 {

class Error : public std::runtime_error {
public:
  Error(const std::string &what, int code) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

private:
  int code_;
};

struct Atom { // occ::core::Atom: atomic number and position in Bohr
  int atomic_number;
  double x, y, z;
};

struct Shell { // occ::gto::Shell (one contraction), coefficients normalised
  int l;
  int atom; // index into the basis' atoms
  std::vector<double> exponents;
  std::vector<double> coefficients;
};

// Replaces Shell::incorporate_shell_norm (src/gto/shell.cpp:180-186).
inline void incorporate_shell_norm(Shell &s) {
  const int rc = occ_xc_normalize_shell(s.l, static_cast<int>(s.exponents.size()),
                                        s.exponents.data(), s.coefficients.data());
  if (rc != OCC_XC_OK)
    throw Error("occ_xc_normalize_shell failed", rc);
}

class AOBasis {
public:
  AOBasis(std::vector<Atom> atoms, std::vector<Shell> shells)
      : atoms_(std::move(atoms)), shells_(std::move(shells)) {}
  void set_pure(bool pure) { pure_ = pure; } // OCC's AOBasis is Cartesian until set_pure(true)
  bool is_pure() const { return pure_; }
  const std::vector<Atom> &atoms() const { return atoms_; }
  const std::vector<Shell> &shells() const { return shells_; }
  size_t nbf() const {
    size_t n = 0;
    for (const Shell &s : shells_)
      n += pure_ ? 2 * s.l + 1 : (s.l + 1) * (s.l + 2) / 2;
    return n;
  }

private:
  std::vector<Atom> atoms_;
  std::vector<Shell> shells_;
  bool pure_ = false;
};

// occ::io::GridSettings (include/occ/numint/grid_settings.h:81-95).
struct GridSettings {
  int max_angular_points = 302;
  int min_angular_points = 110;
  int radial_points = 50;
  double radial_precision = 1e-12;
  bool reduced_first_row_element_grid = true;
  bool treutler_alrichs_adjustment = true;
};

enum class Precision { FP64 = OCC_XC_FP64, Mixed = OCC_XC_MIXED };

namespace detail {
// One context per device for the life of the process.
inline occ_xc_context *context(int device) {
  static std::mutex mu;
  static std::map<int, occ_xc_context *> ctx;
  std::lock_guard<std::mutex> lock(mu);
  auto it = ctx.find(device);
  if (it != ctx.end())
    return it->second;
  occ_xc_context *c = nullptr;
  const int rc = occ_xc_context_create(device, &c);
  if (rc != OCC_XC_OK)
    throw Error("occ_xc_context_create failed on device " + std::to_string(device), rc);
  ctx[device] = c;
  return c;
}
} // namespace detail

class DFT {
public:
  // DFT(method, basis, grid_settings) (dft.h:39): grid, leaves and screening
  // are built here and kept on the GPU.
  DFT(const std::string &method, const AOBasis &basis, const GridSettings &grid = {},
      int device = 0)
      : ctx_(detail::context(device)), nbf_(basis.nbf()), natoms_(basis.atoms().size()) {
    std::vector<int> Z, l, atom, nprim;
    std::vector<double> xyz, exps, coefs;
    for (const Atom &a : basis.atoms()) {
      Z.push_back(a.atomic_number);
      xyz.insert(xyz.end(), {a.x, a.y, a.z});
    }
    for (const Shell &s : basis.shells()) {
      l.push_back(s.l);
      atom.push_back(s.atom);
      nprim.push_back(static_cast<int>(s.exponents.size()));
      exps.insert(exps.end(), s.exponents.begin(), s.exponents.end());
      coefs.insert(coefs.end(), s.coefficients.begin(), s.coefficients.end());
    }
    occ_xc_grid_settings g{grid.max_angular_points, grid.min_angular_points,
                           grid.radial_points, grid.radial_precision,
                           grid.reduced_first_row_element_grid ? 1 : 0,
                           grid.treutler_alrichs_adjustment ? 1 : 0, 1};
    occ_xc_molecule *m = nullptr;
    check(occ_xc_molecule_create(ctx_, static_cast<int>(Z.size()), Z.data(), xyz.data(),
                                 static_cast<int>(l.size()), l.data(), atom.data(), nprim.data(),
                                 exps.data(), coefs.data(), basis.is_pure() ? 1 : 0,
                                 method.c_str(), &g, nullptr, &m));
    mol_.reset(m);
  }

  // compute_vxc(mo) for a restricted wavefunction (dft.h:395-429): D = mo.D
  // (nbf x nbf, column-major), returns V_xc (nbf x nbf, column-major).
  // As OCC dispatches on mo.kind, the size of D decides: nbf x nbf is
  // restricted; 2 nbf x nbf (alpha block above beta, OCC's unrestricted
  // mo.D) is unrestricted and returns V_xc of the same shape.
  std::vector<double> compute_vxc(const std::vector<double> &D,
                                  Precision precision = Precision::Mixed) {
    if (D.size() == 2 * nbf_ * nbf_) {
      std::vector<double> V(2 * nbf_ * nbf_);
      double n2[2];
      check(occ_xc_compute_vxc_unrestricted(ctx_, mol_.get(), D.data(),
                                            static_cast<int>(precision), V.data(), &exc_, n2));
      nelec_ = n2[0] + n2[1];
      return V;
    }
    if (D.size() != nbf_ * nbf_)
      throw Error("density matrix must be nbf x nbf or 2 nbf x nbf", OCC_XC_ERR_ARG);
    std::vector<double> V(nbf_ * nbf_);
    check(occ_xc_compute_vxc(ctx_, mol_.get(), D.data(), static_cast<int>(precision), V.data(),
                             &exc_, &nelec_));
    return V;
  }

  // compute_xc_gradient(mo) (dft.h:599-749): dE_xc/dR with the grid held
  // fixed; 3 * natoms values, x, y, z per atom (the memory of OCC's
  // 3 x natoms Mat3N).  Also sets exchange_correlation_energy().
  // As compute_vxc, the size of D decides: nbf x nbf restricted, 2 nbf x nbf
  // (OCC's unrestricted mo.D) unrestricted.
  std::vector<double> compute_xc_gradient(const std::vector<double> &D,
                                          Precision precision = Precision::FP64) {
    std::vector<double> g(3 * natoms_);
    if (D.size() == 2 * nbf_ * nbf_) {
      check(occ_xc_compute_xc_gradient_unrestricted(ctx_, mol_.get(), D.data(),
                                                    static_cast<int>(precision), g.data(),
                                                    &exc_));
      return g;
    }
    if (D.size() != nbf_ * nbf_)
      throw Error("density matrix must be nbf x nbf or 2 nbf x nbf", OCC_XC_ERR_ARG);
    check(occ_xc_compute_xc_gradient(ctx_, mol_.get(), D.data(), static_cast<int>(precision),
                                     g.data(), &exc_));
    return g;
  }

  double exchange_correlation_energy() const { return exc_; } // dft.h:83
  double integrated_density() const { return nelec_; }
  size_t nbf() const { return nbf_; }

  // DFT::set_xc_screening_threshold (dft.h:590); rebuilds the screening.
  void set_xc_screening_threshold(double threshold) {
    occ_xc_build_settings b;
    occ_xc_default_build_settings(&b);
    b.xc_screening_threshold = threshold;
    check(occ_xc_molecule_set_build_settings(ctx_, mol_.get(), &b));
  }

private:
  struct Del {
    void operator()(occ_xc_molecule *m) const { occ_xc_molecule_destroy(m); }
  };
  void check(int rc) const {
    if (rc != OCC_XC_OK)
      throw Error(std::string("occ_xc: ") + occ_xc_last_error(ctx_), rc);
  }
  occ_xc_context *ctx_;
  std::unique_ptr<occ_xc_molecule, Del> mol_;
  size_t nbf_;
  size_t natoms_;
  double exc_ = 0.0, nelec_ = 0.0;
};

} // namespace occ_gb300
