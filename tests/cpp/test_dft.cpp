// C++ tests of the occ_gb300::DFT interface (include/occ_xc.hpp), written
// like the reference's Catch2 tests (tests/dft_tests.cpp).  The input -- a
// molecule, its basis, a density and the oracle's E_xc per method -- comes
// from tests/test_cpp_api.py in a plain text file (argv[1]).
#include <cmath>
#include <cstdio>
#include <fstream>
#include <functional>
#include <iostream>
#include <string>
#include <vector>

#include "occ_xc.hpp"

namespace {
int failures = 0;
std::vector<std::pair<std::string, std::function<void()>>> &cases() {
  static std::vector<std::pair<std::string, std::function<void()>>> c;
  return c;
}
struct Register {
  Register(const char *name, std::function<void()> f) { cases().emplace_back(name, f); }
};
#define TEST_CASE(name, fn) static Register reg_##fn(name, fn)
#define REQUIRE(cond)                                                                       \
  do {                                                                                      \
    if (!(cond)) {                                                                          \
      std::fprintf(stderr, "  REQUIRE failed: %s (line %d)\n", #cond, __LINE__);           \
      failures++;                                                                           \
    }                                                                                       \
  } while (0)

struct Input {
  occ_gb300::AOBasis basis{{}, {}};
  std::vector<double> D;
  std::vector<std::pair<std::string, double>> expected; // method, oracle E_xc
  std::vector<std::pair<std::string, std::vector<double>>> gradients; // method, oracle dE/dR
  double nelec = 0.0;
} in;

bool read_input(const char *path) {
  std::ifstream f(path);
  int natoms, nshells, pure;
  size_t nbf;
  if (!(f >> natoms))
    return false;
  std::vector<occ_gb300::Atom> atoms(natoms);
  for (auto &a : atoms)
    f >> a.atomic_number >> a.x >> a.y >> a.z;
  f >> nshells;
  std::vector<occ_gb300::Shell> shells(nshells);
  for (auto &s : shells) {
    int n;
    f >> s.l >> s.atom >> n;
    s.exponents.resize(n);
    s.coefficients.resize(n);
    for (int k = 0; k < n; k++)
      f >> s.exponents[k] >> s.coefficients[k];
    occ_gb300::incorporate_shell_norm(s);
  }
  f >> pure >> nbf >> in.nelec;
  in.basis = occ_gb300::AOBasis(atoms, shells);
  in.basis.set_pure(pure != 0);
  in.D.resize(nbf * nbf);
  for (double &x : in.D)
    f >> x;
  std::string m;
  while (f >> m) {
    if (m == "grad") { // grad <method> <3 natoms values>
      std::vector<double> g(3 * static_cast<size_t>(natoms));
      f >> m;
      for (double &x : g)
        f >> x;
      in.gradients.emplace_back(m, g);
      continue;
    }
    double e;
    f >> e;
    in.expected.emplace_back(m, e);
  }
  return static_cast<bool>(in.basis.nbf() == nbf);
}

double max_asym(const std::vector<double> &V, size_t n) {
  double m = 0.0;
  for (size_t i = 0; i < n; i++)
    for (size_t j = 0; j < n; j++)
      m = std::fmax(m, std::fabs(V[i * n + j] - V[j * n + i]));
  return m;
}

void compute_vxc_matches_oracle() {
  for (const auto &[method, e_ref] : in.expected) {
    occ_gb300::DFT dft(method, in.basis);
    auto V = dft.compute_vxc(in.D, occ_gb300::Precision::FP64);
    std::printf("  %-6s FP64  E_xc = %.12f  (oracle %.12f)  N = %.8f\n", method.c_str(),
                dft.exchange_correlation_energy(), e_ref, dft.integrated_density());
    REQUIRE(std::fabs(dft.exchange_correlation_energy() - e_ref) <= 1e-8);
    REQUIRE(std::fabs(dft.integrated_density() - in.nelec) <= 2e-5);
    REQUIRE(max_asym(V, dft.nbf()) <= 1e-12);
    auto Vm = dft.compute_vxc(in.D, occ_gb300::Precision::Mixed);
    std::printf("  %-6s mixed E_xc = %.12f\n", method.c_str(), dft.exchange_correlation_energy());
    REQUIRE(std::fabs(dft.exchange_correlation_energy() - e_ref) <= 1e-6);
    double dv = 0.0;
    for (size_t i = 0; i < V.size(); i++)
      dv = std::fmax(dv, std::fabs(V[i] - Vm[i]));
    REQUIRE(dv <= 1e-5);
  }
}
TEST_CASE("DFT::compute_vxc against the oracle, FP64 and mixed", compute_vxc_matches_oracle);

void xc_gradient_matches_oracle() {
  REQUIRE(!in.gradients.empty());
  for (const auto &[method, g_ref] : in.gradients) {
    occ_gb300::DFT dft(method, in.basis);
    auto g = dft.compute_xc_gradient(in.D);
    REQUIRE(g.size() == g_ref.size());
    double dg = 0.0;
    for (size_t i = 0; i < g.size() && i < g_ref.size(); i++)
      dg = std::fmax(dg, std::fabs(g[i] - g_ref[i]));
    std::printf("  %-6s dE_xc/dR  O = (%.8f, %.8f, %.8f)  max|d| = %.2e\n", method.c_str(), g[0],
                g[1], g[2], dg);
    REQUIRE(dg <= 1e-9);
  }
}
TEST_CASE("DFT::compute_xc_gradient against the oracle", xc_gradient_matches_oracle);

void screening_threshold() {
  occ_gb300::DFT dft("pbe", in.basis);
  dft.compute_vxc(in.D, occ_gb300::Precision::FP64);
  const double e0 = dft.exchange_correlation_energy();
  dft.set_xc_screening_threshold(1e-14);
  dft.compute_vxc(in.D, occ_gb300::Precision::FP64);
  REQUIRE(std::fabs(dft.exchange_correlation_energy() - e0) < 1e-8);
}
TEST_CASE("set_xc_screening_threshold: screened == dense within 1e-8", screening_threshold);

void errors_throw() {
  bool threw = false;
  try {
    occ_gb300::DFT dft("not-a-functional", in.basis);
  } catch (const occ_gb300::Error &e) {
    threw = e.code() == OCC_XC_ERR_METHOD;
  }
  REQUIRE(threw);
  threw = false;
  try {
    occ_gb300::DFT dft("lda", in.basis);
    dft.compute_vxc(std::vector<double>(3, 0.0));
  } catch (const occ_gb300::Error &e) {
    threw = e.code() == OCC_XC_ERR_ARG;
  }
  REQUIRE(threw);
}
TEST_CASE("errors are thrown as occ_gb300::Error", errors_throw);
} // namespace

int main(int argc, char **argv) {
  if (argc < 2 || !read_input(argv[1])) {
    std::fprintf(stderr, "usage: test_dft <input file>\n");
    return 2;
  }
  for (auto &[name, f] : cases()) {
    std::printf("TEST_CASE %s\n", name.c_str());
    const int before = failures;
    try {
      f();
    } catch (const std::exception &e) {
      std::fprintf(stderr, "  unexpected exception: %s\n", e.what());
      failures++;
    }
    std::printf("  %s\n", failures == before ? "passed" : "FAILED");
  }
  return failures == 0 ? 0 : 1;
}
