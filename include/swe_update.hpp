// swe_update.hpp — C++ host side over the C ABI (swe_gpu.h), mirroring the
// reference's Fortran interface for the explicit step:
//
//   MODULE update  (SOURCES/update.f90:1-16)   construct_matrices, euler,
//                  compute_dij, and the public data lumped, diag, mass
//   MODULE fct     (SOURCES/fct.f90:1-5)       FCT_positivity
//   time loop      (SOURCES/main.f90:61-91)    COMPUTE_DT + SSP-RK3 + bdy,
//                                              run on the device by rk3
//
// Same names and argument meanings as the Fortran procedures; arrays are in
// the reference layout (un(S, np) column-major FP64, 1-based node and element
// numbers).  Where the reference STOPs (check_hmin, compute_lambda_vacc's
// Delta < 0) these calls throw swe::Stop carrying the C ABI status and
// message.  Header only: link libswe_gpu.so.
#ifndef SWE_UPDATE_HPP
#define SWE_UPDATE_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "swe_gpu.h"

namespace swe {

// The reference's WRITE + STOP, as an exception (status = SWE_ERR_*)
class Stop : public std::runtime_error {
 public:
  Stop(int status, const std::string& msg) : std::runtime_error(msg), status(status) {}
  int status;
};

class Update {
 public:
  // construct_matrices (update.f90:18-132) for the mesh jj(3, me) 1-based,
  // rr(2, np), with the bathymetry and the inputs record p
  Update(int np, int me, const int* jj, const double* rr, const double* bath, const swe_params& p)
      : np_(np), S_(p.syst_size) {
    check(swe_create(&ctx_, np, me, jj, rr, bath, &p), "construct_matrices");
    int n = 0;
    check(swe_sizes(ctx_, 0, &n, &nnz_), "construct_matrices");
    ia_.resize(np + 1);
    ja_.resize(nnz_);
    mass_.resize(nnz_);
    lumped_.resize(np);
    diag_.resize(np);
    check(swe_get_matrices(ctx_, 0, ia_.data(), ja_.data(), mass_.data(), lumped_.data(), diag_.data(), nullptr,
                           nullptr),
          "construct_matrices");
  }
  ~Update() { swe_destroy(ctx_); }
  Update(const Update&) = delete;
  Update& operator=(const Update&) = delete;

  // module data (CSR 1-based like mass%ia, mass%ja; diag 1-based positions)
  const std::vector<int>& ia() const { return ia_; }
  const std::vector<int>& ja() const { return ja_; }
  const std::vector<double>& mass() const { return mass_; }
  const std::vector<double>& lumped() const { return lumped_; }
  const std::vector<int>& diag() const { return diag_; }
  int np() const { return np_; }
  int nnz() const { return nnz_; }
  int syst_size() const { return S_; }

  // inputs%... after a change in the caller (dt, flags)
  void set_inputs(const swe_params& p) { check(swe_set_params(ctx_, 0, &p), "set_inputs"); }
  // bath(np) of boundary_conditions, after init
  void set_bath(const double* bath) { check(swe_set_bath(ctx_, 0, bath), "set_bath"); }
  // Dirichlet nodes js (1-based) of component comp (0 = h) with values
  void set_dirichlet(int comp, const std::vector<int>& js, const std::vector<double>& vals) {
    check(swe_set_dirichlet(ctx_, 0, comp, (int)js.size(), js.data(), vals.empty() ? nullptr : vals.data()),
          "set_dirichlet");
  }

  // euler(un, unext) (update.f90:134-289), dt = inputs%dt
  void euler(const double* un, double* unext) { check(swe_euler(ctx_, 0, un, unext), "euler"); }
  // compute_dij(un) (update.f90:291-326): dij%aa (nnz) and COMPUTE_DT's
  // dt = CFL / max |d_ii| / m_i (main.f90:166-174)
  double compute_dij(const double* un, double* dij_aa) {
    double dt = 0.0;
    check(swe_compute_dij(ctx_, 0, un, dij_aa, &dt), "compute_dij");
    return dt;
  }
  // FCT_positivity(unext, mat, lij) (fct.f90:5-42)
  void fct_positivity(const double* unext, const double* mat, double* lij) {
    check(swe_fct_positivity(ctx_, 0, unext, mat, lij), "FCT_positivity");
  }

  // the time loop on the device: un uploaded, DO WHILE(time < t_final) for at
  // most max_steps steps, un downloaded (one swe_rk3_steps_host call); returns
  // the steps taken
  int rk3(double* un, double& time, double t_final, int max_steps, double* dt_last = nullptr) {
    check(swe_set_time(ctx_, &time, &t_final), "set_time");
    double t = time, dt = 0.0;
    int done = 0;
    check(swe_rk3_steps_host(ctx_, un, un, max_steps, &t, &dt, &done), "time loop");
    time = t;
    if (dt_last) *dt_last = dt;
    return done;
  }
  double total_mass() {
    double m[2] = {0.0, 0.0};
    check(swe_mass(ctx_, m), "mass");
    return m[0];
  }

  swe_ctx* context() { return ctx_; }

 private:
  void check(int rc, const char* where) const {
    if (rc != SWE_OK) throw Stop(rc, std::string(where) + ": " + swe_last_error(ctx_));
  }
  swe_ctx* ctx_ = nullptr;
  int np_ = 0, S_ = 3, nnz_ = 0;
  std::vector<int> ia_, ja_, diag_;
  std::vector<double> mass_, lumped_;
};

}  // namespace swe

#endif  // SWE_UPDATE_HPP
