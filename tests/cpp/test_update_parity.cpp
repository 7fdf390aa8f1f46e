// C++ parity checks of the host interface include/swe_update.hpp (MODULE
// update / MODULE fct over the C ABI) against the FP64 oracle
// (oracle/swe_oracle.cpp, test infrastructure), on two cases: the unit-square
// dam break, and a wet/dry basin (a bump rising through the free surface).
// Every array must be equal bit for bit.  Prints "ok <check>" per check and
// exits 0 when all hold.  Built and run by tests/test_cpp_host.py.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "swe_update.hpp"

extern "C" {   // the oracle's entry points (same parameter record as swe_params)
void* orc_create(int np, int me, const int* jj, const double* rr);
void orc_destroy(void* h);
int orc_nnz(void* h);
void orc_get_matrices(void* h, int* ia, int* ja, double* mass, double* lumped, int* diag, double* cx, double* cy);
int orc_set_params(void* h, const swe_params* p);
void orc_set_bath(void* h, const double* bath);
int orc_compute_dij(void* h, const double* un, double* dij_out, double* dt_out);
int orc_euler(void* h, const double* un, double* unext, void* dump);
void orc_fct_positivity(void* h, const double* unext, const double* fmat, double* lij);
}

namespace {

int failures = 0;

template <typename T>
void same(const char* what, const std::vector<T>& a, const std::vector<T>& b) {
  if (a.size() != b.size()) { std::printf("FAIL %s: sizes %zu %zu\n", what, a.size(), b.size()); failures++; return; }
  for (size_t k = 0; k < a.size(); k++)
    if (std::memcmp(&a[k], &b[k], sizeof(T)) != 0) {
      std::printf("FAIL %s: first difference at %zu\n", what, k);
      failures++;
      return;
    }
  std::printf("ok %s\n", what);
}

struct Case {
  int np, me;
  std::vector<int> jj;
  std::vector<double> rr, bath, un;
};

// n x n lattice on [0,1]^2 (SW->NE diagonals), as in swe/mesh.py
Case lattice(int n) {
  Case c;
  c.np = n * n;
  c.me = 2 * (n - 1) * (n - 1);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      c.rr.push_back(i == n - 1 ? 1.0 : i * (1.0 / (n - 1)));
      c.rr.push_back(j == n - 1 ? 1.0 : j * (1.0 / (n - 1)));
    }
  for (int j = 0; j < n - 1; j++)
    for (int i = 0; i < n - 1; i++) {
      const int sw = i + n * j + 1, se = sw + 1, nw = sw + n, ne = sw + n + 1;
      const int t[6] = {sw, se, ne, sw, ne, nw};
      c.jj.insert(c.jj.end(), t, t + 6);
    }
  c.bath.assign(c.np, 0.0);
  c.un.assign(3 * (size_t)c.np, 0.0);
  return c;
}

void check_case(const char* name, const Case& c, const swe_params& p) {
  std::printf("case %s\n", name);
  swe::Update upd(c.np, c.me, c.jj.data(), c.rr.data(), c.bath.data(), p);
  void* o = orc_create(c.np, c.me, c.jj.data(), c.rr.data());
  orc_set_params(o, &p);
  orc_set_bath(o, c.bath.data());
  const int nnz = orc_nnz(o);
  std::vector<int> ia(c.np + 1), ja(nnz), diag(c.np);
  std::vector<double> mass(nnz), lumped(c.np);
  orc_get_matrices(o, ia.data(), ja.data(), mass.data(), lumped.data(), diag.data(), nullptr, nullptr);
  same("construct_matrices ia", upd.ia(), ia);
  same("construct_matrices ja", upd.ja(), ja);
  same("construct_matrices mass", upd.mass(), mass);
  same("construct_matrices lumped", upd.lumped(), lumped);
  same("construct_matrices diag", upd.diag(), diag);

  std::vector<double> dg(nnz), dr(nnz);
  double dt_g = upd.compute_dij(c.un.data(), dg.data()), dt_r = 0.0;
  orc_compute_dij(o, c.un.data(), dr.data(), &dt_r);
  same("compute_dij dij", dg, dr);
  same("compute_dij dt", std::vector<double>{dt_g}, std::vector<double>{dt_r});

  swe_params q = p;
  q.dt = dt_r;
  upd.set_inputs(q);
  orc_set_params(o, &q);
  std::vector<double> eg(c.un.size()), er(c.un.size());
  upd.euler(c.un.data(), eg.data());
  orc_euler(o, c.un.data(), er.data(), nullptr);
  same("euler unext", eg, er);

  std::vector<double> scaled(c.np), fmat(nnz), lg(nnz), lr(nnz);
  for (int i = 0; i < c.np; i++) scaled[i] = lumped[i] / dt_r * er[3 * (size_t)i];
  for (int k = 0; k < nnz; k++) fmat[k] = std::sin(0.37 * k) * 1e-3;   // an antisymmetry-free test matrix
  upd.fct_positivity(scaled.data(), fmat.data(), lg.data());
  orc_fct_positivity(o, scaled.data(), fmat.data(), lr.data());
  same("FCT_positivity lij", lg, lr);
  orc_destroy(o);
}

}  // namespace

int main() {
  swe_params p{};
  p.gravity = 9.81; p.cfl = 0.25; p.max_water_h = 1.0; p.htiny = 1e-4;
  p.type_test = 4; p.syst_size = 3; p.viscosity_type = SWE_VISC_FCT; p.viscous_type = 2;
  p.if_alpha_limit = 1; p.if_lumped = 1; p.if_roundoff_fix = 1; p.precision = SWE_PREC_FP64;
  try {
    Case dam = lattice(31);
    for (int v = 0; v < dam.np; v++) dam.un[3 * (size_t)v] = dam.rr[2 * (size_t)v] < 0.5 ? 1.0 : 0.1;
    check_case("dam break", dam, p);

    Case basin = lattice(31);                    // a bump rising through the surface: dry nodes
    for (int v = 0; v < basin.np; v++) {
      const double x = basin.rr[2 * (size_t)v] - 0.5, y = basin.rr[2 * (size_t)v + 1] - 0.5;
      basin.bath[v] = 0.6 * std::exp(-(x * x + y * y) / 0.02);
      const double h = 0.4 - basin.bath[v];
      basin.un[3 * (size_t)v] = h > 0 ? h : 0.0;
      basin.un[3 * (size_t)v + 1] = 0.05 * basin.un[3 * (size_t)v];
    }
    check_case("wet/dry basin", basin, p);
  } catch (const swe::Stop& e) {
    std::printf("FAIL stop: %s\n", e.what());
    return 2;
  }
  std::printf("%d failures\n", failures);
  return failures ? 1 : 0;
}
