// FP64 stage kernels in the reference's evaluation order.
//
// One thread owns one mesh row and walks its entries in the reference CSR
// order, so every sum is formed in the same order as the Fortran loops.  This
// translation unit is compiled with -fmad=false (no FMA contraction) and uses
// IEEE sqrt/div: the result equals the FP64 CPU restatement bit for bit (the
// Manning friction's pow() aside).  It is the parity path and the "plain FP64
// GPU step" of the measurements.
//
// Per stage (SOURCES/update.f90 euler, :134-289, 'fct' + 'type2'):
//   k_node   : one_over_h, velocity, entropy E, alpha_i       (flux, alpha_limit)
//   k_low    : d_ij, mu_ij (alpha-limited), low-order state,   (compute_dij, compute_muij,
//              entropy residual res_i                           smb_2_roundoff, smb_2, maxmin)
//   k_fct    : f_ij, R^-_i                                      (compute_fct_matrix, FCT_positivity)
//   k_update : limited antidiffusion, RK combination, Dirichlet (apply_viscosity, main.f90:77-90)
// Per step: k_dt (COMPUTE_DT) and the time bookkeeping kernels.
#include "swe_kernels.hpp"

namespace swe {

struct NodeF64 {        // per-row arrays of the FP64 path
  double* ovh;
  double* v1;
  double* v2;
  double* ent;
  double* alpha;
  double* sqgh;         // sqrt(g |h|), the sql / sqr of compute_lambda_vacc
};

// ---------------------------------------------------------------------------
// k_node: flux() globals (SOURCES/condlim.f90:21-77, 79-90), the entropy
// E_i = 0.5 (g h^2 + v.q) of entropy_residual (update.f90:844-851) and the
// smoothness indicator alpha_i of alpha_limit (update.f90:758-781).
// ---------------------------------------------------------------------------
__global__ void k_node_f64(Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                           StateF64 u, NodeF64 nd) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= G.n_rows) return;
  int L = G.len[r];
  if (L == 0) return;
  int b = G.slice_inst[r >> 5];
  if (St[b].done) return;
  const InstConst& c = C[b];
  double h = u.h[r], qx = u.q1[r], qy = u.q2[r];
  double o = one_over_h(h, c.htiny);
  double v1 = qx * o;
  double v2 = (c.type_test == 13) ? qy * o * 0.0 : qy * o;
  nd.ovh[r] = o;
  nd.v1[r] = v1;
  nd.v2[r] = v2;
  nd.sqgh[r] = sqrt(c.g * tabs(h));
  double E = c.g * (h * h);
  E = E + v1 * qx;
  E = E + v2 * qy;
  nd.ent[r] = 0.5 * E;
  double alpha = 1.0;
  if (c.alpha_limit && !(h <= c.htiny)) {
    const int64_t base = entry_base(G, r);
    const int dp = G.dpos[r];
    double num = 0.0, denom = 0.0;
    for (int kk = 0; kk <= L; kk++) {          // reference order, diagonal at dp
      const int k = kk - (kk > dp ? 1 : 0);
      const double hj = (kk == dp) ? h : u.h[G.col[base + 32 * k]];
      num = num + hj - h;
      denom = denom + tabs(hj - h);
    }
    double a = (denom <= tabs(num)) ? 1.0 : tabs(num) / (denom);
    double a2 = a * a, a4 = a2 * a2;
    alpha = a4 * a4;
  }
  nd.alpha[r] = alpha;
}

// Source terms (SOURCES/update.f90:425-551) added to the undivided rk of one
// row.  velocity is the row's own (v1, v2).
__device__ __forceinline__ void source_f64(const InstConst& c, const InstState& st, double m, const double* ui,
                                           double v1, double v2, double* rk, double pt_sum_x, double pt_sum_y,
                                           double s_i) {
  const int S = c.S;
  if (c.type_test == 9 || c.type_test == 10) {
    const double gamma = 4.0 / 3.0, chi = 1.0;
    double fric = c.g * c.mannings * c.mannings;
    double hstar = pow(tmax(ui[0], c.htiny), gamma);
    double vel = fric * sqrt(v1 * v1 + v2 * v2);
    double hloc = chi * vel * st.dt;
    for (int k = 1; k < S; k++) rk[k] = rk[k] - m * ui[k] * vel * 2 / (hstar + tmax(hstar, hloc));
  } else if (c.type_test == 11) {
    const double kappa = 0.2;
    for (int k = 1; k < S; k++) rk[k] = rk[k] - m * kappa * ui[k];
  } else if (c.type_test == 12) {
    const double f = 2.0;
    for (int j = 3; j <= S; j++) {
      rk[S - 2] = rk[S - 2] + m * f * ui[S - 1];
      rk[S - 1] = rk[S - 1] - m * f * ui[S - 2];
    }
  } else if (c.type_test == 13) {
    rk[1] = pt_sum_x;   // already accumulated in entry order by the caller
    rk[2] = pt_sum_y;
    rk[3] = rk[3] + m * ui[4];
    rk[4] = rk[4] - m * s_i;
  }
}

// SGN pressure pTilde_n and source s_n (mSGN_RHS, update.f90:505-529)
__device__ __forceinline__ void sgn_node_f64(const InstConst& c, double m, double h, double heta,
                                             double* pTilde, double* s) {
  double lms = sqrt(m);
  double pc = c.lambda_sgn * c.g / (3.0 * lms);
  double x = heta / (h * h);
  double psi = 12.0 * (x - 1.0);
  double x3 = (x * x) * x, x4 = (x * x) * (x * x);
  *pTilde = pc * ((h * h) * h) * (2.0 + 4.0 * x3 - 6.0 * x4);
  double t = heta / h;
  *s = 3.0 * pc * (t * t) * psi;
}

// Viscosities seen by the row sums: the low-order (alpha-limited) d_ij, mu_ij,
// or the entropy-viscosity d^H = MIN(d, res_ij), mu^H = MIN(mu, res_ij) of
// update.f90:232-239 (applied to the diagonal too: res_ii = res_i).
struct LowVisc {
  const double* dL;
  const double* muL;
  double dii, muii;
  __device__ void get(bool isd, int64_t e, int, double& d, double& mu) const {
    d = isd ? dii : dL[e];
    mu = isd ? muii : muL[e];
  }
};
struct HighVisc {
  const double* dL;
  const double* muL;
  const double* res;
  double dii, muii, resi;
  __device__ void get(bool isd, int64_t e, int j, double& d, double& mu) const {
    const double rij = isd ? tmax(resi, resi) : tmax(resi, res[j]);
    d = tmin(isd ? dii : dL[e], 1.0 * rij);
    mu = tmin(isd ? muii : muL[e], 1.0 * rij);
  }
};

struct RowSums {
  double rk[5] = {0, 0, 0, 0, 0};    // smb_2_roundoff (htiny tests), with fix
  double rk2[5] = {0, 0, 0, 0, 0};   // smb_2 (h <= 0 tests)
  double rk1[5] = {0, 0, 0, 0, 0};   // smb_1 ('type1')
  double fix = 0.0;                   // fix_roundoff
  double emax = 0.0, emin = 0.0;      // maxmin of the entropy over the row
};

// One row of smb_2_roundoff (update.f90:554-624), smb_2 (:626-682) and smb_1
// (:366-423), each with its source terms (:425-551), over the row's entries
// in reference order with the diagonal at dp; the entropy max/min of maxmin
// (:924-935) on the way.  Undivided by the lumped mass.
template <class V>
__device__ __forceinline__ void smb_rows_f64(const Graph& G, const InstConst& c, const InstState& st, const StateF64& u,
                                             const NodeF64& nd, int64_t r, int64_t base, int L, int dp,
                                             const double* ui, double zi, double m, const V& visc, bool want_round,
                                             bool want_plain, bool want_t1, RowSums& o) {
  const int S = c.S;
  const double g = c.g, htiny = c.htiny;
  const double v1i = nd.v1[r], v2i = nd.v2[r];
  double* rk = o.rk;
  double* rk2 = o.rk2;
  double* rk1 = o.rk1;
  o.emax = nd.ent[r];
  o.emin = o.emax;
  for (int kk = 0; kk <= L; kk++) {
    const bool isd = (kk == dp);
    const int64_t e = base + 32 * (kk - (kk > dp ? 1 : 0));
    const int j = isd ? (int)r : G.col[e];
    double uj[5];
    uj[0] = u.h[j]; uj[1] = u.q1[j]; uj[2] = u.q2[j];
    if (S == 5) { uj[3] = u.q3[j]; uj[4] = u.q4[j]; }
    const double zj = G.bath[j];
    const double v1j = nd.v1[j], v2j = nd.v2[j];
    double d, mu;
    visc.get(isd, e, j, d, mu);
    const double cxe = isd ? G.cxii[r] : G.cx[e], cye = isd ? G.cyii[r] : G.cy[e];
    const double ej = nd.ent[j];
    o.emax = tmax(o.emax, ej);
    o.emin = tmin(o.emin, ej);
    const double zmax = tmax(zi, zj);
    const double Hij = tmax(0.0, ui[0] + zi - zmax);
    const double Hji = tmax(0.0, uj[0] + zj - zmax);
    // H*/h, formed once for the three rows (each tests h against its own bound)
    const double qij = (ui[0] <= 0.0) ? 0.0 : Hij / ui[0];
    const double qji = (uj[0] <= 0.0) ? 0.0 : Hji / uj[0];
    if (want_round) {   // smb_2_roundoff (htiny tests)
      const double ratij = (ui[0] <= htiny) ? 0.0 : (ui[0] > 0.0 ? qij : Hij / ui[0]);   // h > htiny >= 0: qij
      const double ratji = (uj[0] <= htiny) ? 0.0 : (uj[0] > 0.0 ? qji : Hji / uj[0]);
      double xx = 0.0;
      xx = xx - cxe * (v1j);
      xx = xx - cye * (v2j);
      if (isd) {
        o.fix = o.fix + xx;
      } else {
        o.fix = o.fix - mu + (d - mu) * (-ratij);
        rk[0] = rk[0] + (xx + mu) * uj[0] + tmax((d - mu) * Hji, 0.0);
      }
      for (int q = 1; q < S; q++) {
        double x2 = 0.0;
        x2 = x2 - cxe * (v1j * uj[q]);
        x2 = x2 - cye * (v2j * uj[q]);
        rk[q] = rk[q] + x2 + d * (uj[q] * ratji - ui[q] * ratij) + mu * (uj[q] * (1.0 - ratji) - ui[q] * (1.0 - ratij));
      }
      rk[1] = rk[1] - g * ui[0] * (uj[0] + zj - ui[0] - zi) * cxe;
      rk[2] = rk[2] - g * ui[0] * (uj[0] + zj - ui[0] - zi) * cye;
    }
    if (want_plain) {   // smb_2 (h <= 0 tests)
      const double ratij = qij;
      const double ratji = qji;
      for (int q = 0; q < S; q++) {
        double x2 = 0.0;
        x2 = x2 - cxe * (v1j * uj[q]);
        x2 = x2 - cye * (v2j * uj[q]);
        rk2[q] = rk2[q] + x2 + d * (uj[q] * ratji - ui[q] * ratij) + mu * (uj[q] * (1.0 - ratji) - ui[q] * (1.0 - ratij));
      }
      rk2[1] = rk2[1] - g * ui[0] * (uj[0] + zj - ui[0] - zi) * cxe;
      rk2[2] = rk2[2] - g * ui[0] * (uj[0] + zj - ui[0] - zi) * cye;
    }
    if (want_t1) {      // smb_1 (htiny tests, flux vv = velocity u_k)
      const double ratij = (ui[0] <= htiny) ? 0.0 : (ui[0] > 0.0 ? qij : Hij / ui[0]);   // h > htiny >= 0: qij
      const double ratji = (uj[0] <= htiny) ? 0.0 : (uj[0] > 0.0 ? qji : Hji / uj[0]);
      for (int q = 0; q < S; q++) {
        double xx = 0.0;
        xx = xx - cxe * ((v1j * uj[q]) * ratji + (v1i * ui[q]) * ratij);
        xx = xx - cye * ((v2j * uj[q]) * ratji + (v2i * ui[q]) * ratij);
        rk1[q] = rk1[q] + xx + d * (uj[q] * ratji - ui[q] * ratij);
      }
      rk1[1] = rk1[1] - 0.5 * g * (Hji * Hji - Hij * Hij) * cxe;
      rk1[2] = rk1[2] - 0.5 * g * (Hji * Hji - Hij * Hij) * cye;
    }
  }
  // source terms
  if (c.type_test == 13) {
    // mSGN_RHS adds -pTilde_j c_ij after the smb loops, entry by entry, onto
    // the momentum rows: redo that accumulation in entry order on top of rk.
    double s_i, p_i;
    sgn_node_f64(c, m, ui[0], ui[3], &p_i, &s_i);
    double ax = rk[1], ay = rk[2], bx = rk2[1], by = rk2[2], tx = rk1[1], ty = rk1[2];
    for (int kk = 0; kk <= L; kk++) {
      const bool isd = (kk == dp);
      const int64_t e = base + 32 * (kk - (kk > dp ? 1 : 0));
      const int j = isd ? (int)r : G.col[e];
      const double cxe = isd ? G.cxii[r] : G.cx[e], cye = isd ? G.cyii[r] : G.cy[e];
      double pj, sj;
      sgn_node_f64(c, G.lumped[j], u.h[j], u.q3[j], &pj, &sj);
      ax = ax - pj * cxe; ay = ay - pj * cye;
      bx = bx - pj * cxe; by = by - pj * cye;
      tx = tx - pj * cxe; ty = ty - pj * cye;
    }
    if (want_round) source_f64(c, st, m, ui, v1i, v2i, rk, ax, ay, s_i);
    if (want_plain) source_f64(c, st, m, ui, v1i, v2i, rk2, bx, by, s_i);
    if (want_t1) source_f64(c, st, m, ui, v1i, v2i, rk1, tx, ty, s_i);
  } else {
    if (want_round) source_f64(c, st, m, ui, v1i, v2i, rk, 0, 0, 0);
    if (want_plain) source_f64(c, st, m, ui, v1i, v2i, rk2, 0, 0, 0);
    if (want_t1) source_f64(c, st, m, ui, v1i, v2i, rk1, 0, 0, 0);
  }
}

// ---------------------------------------------------------------------------
// k_low: compute_dij + compute_muij + MAX + alpha_limit (update.f90:180-187,
// 291-364, 782-798), smb_2_roundoff (:554-624) -> low-order state
// (:202-210), smb_2 + entropy residual (:825-878).  Writes dL/muL per entry,
// uL per row, res per row, fix_roundoff-free low-order h.
// ---------------------------------------------------------------------------
__global__ void k_low_f64(Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                          StateF64 u, NodeF64 nd, double* __restrict__ dL, double* __restrict__ muL,
                          double* __restrict__ dLii, double* __restrict__ muLii, StateF64 uL,
                          double* __restrict__ res, const double* __restrict__ dij_in, unsigned* __restrict__ err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= G.n_rows) return;
  const int L = G.len[r];
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const InstState st = St[b];
  if (st.done) return;
  const InstConst& c = C[b];
  const int S = c.S;
  const double g = c.g, htiny = c.htiny, dt = st.dt;
  const LamConstF64<double> lk = lam_const_f64(g, sqrt(2.0));
  const int64_t base = entry_base(G, r);
  const int dp = G.dpos[r];
  double ui[5];
  ui[0] = u.h[r]; ui[1] = u.q1[r]; ui[2] = u.q2[r];
  if (S == 5) { ui[3] = u.q3[r]; ui[4] = u.q4[r]; }
  const double ovhi = nd.ovh[r], v1i = nd.v1[r], v2i = nd.v2[r], ai = nd.alpha[r];
  const double zi = G.bath[r], m = G.lumped[r];
  bool delta_bad = false;

  // pass 1: raw d_ij (lambda_max) and mu_ij, diagonals = -row sums (the
  // diagonal's own value, 0, adds nothing to the sums).  'galerkin' sets
  // every d_ij and mu_ij to 0 (update.f90:155-158).
  double sd = 0.0, sm = 0.0;
  for (int k = 0; k < (c.visc == VISC_GALERKIN ? 0 : L); k++) {
    const int64_t e = base + 32 * k;
    const int j = G.col[e];
    double d = 0.0, mu = 0.0;
    {
      const double cxe = G.cx[e], cye = G.cy[e];
      if (dij_in) {                            // stage 1: k_dt computed this d_ij on this state
        d = dij_in[e];
      } else {
        const double norm = G.cnorm[e], nx = G.cnx[e], ny = G.cny[e];   // sqrt(c.c), c/norm
        double lam;
        if (!lambda_vacc(ui[0], ui[1], ui[2], ovhi, nd.sqgh[r], u.h[j], u.q1[j], u.q2[j], nd.ovh[j], nd.sqgh[j], nx,
                         ny, g, htiny, lk,
                         &lam))
          delta_bad = true;
        d = norm * lam;
      }
      const double sl = cxe * v1i + cye * v2i;
      // compute_muij uses q*ovh of the raw state, equal to velocity except
      // for type 13 whose velocity(2) is zeroed: recompute from q there
      double sr;
      if (c.type_test == 13) {
        const double ulx = ui[1] * ovhi, uly = ui[2] * ovhi;
        const double ox = nd.ovh[j];
        const double urx = u.q1[j] * ox, ury = u.q2[j] * ox;
        const double sl2 = cxe * ulx + cye * uly;
        sr = cxe * urx + cye * ury;
        mu = tmax(tmax(-sl2, 0.0), tmax(sr, 0.0));
      } else {
        sr = cxe * nd.v1[j] + cye * nd.v2[j];
        mu = tmax(tmax(-sl, 0.0), tmax(sr, 0.0));
      }
    }
    dL[e] = d;
    muL[e] = mu;
    sd = sd + d;
    sm = sm + mu;
  }
  const double dii_raw = -sd, muii_raw = -sm;
  // pass 2: dij = MAX(dij, muij) on every entry, then alpha limiting with the
  // reference's diagonal re-summation (the mu sum includes the old mu_ii at
  // its place in the row)
  sd = 0.0; sm = 0.0;
  double dii = tmax(dii_raw, muii_raw), muii = muii_raw;
  if (c.alpha_limit) dii = 0.0;
  if (c.visc == VISC_GALERKIN) {
    for (int k = 0; k < L; k++) { dL[base + 32 * k] = 0.0; muL[base + 32 * k] = 0.0; }
    dii = 0.0; muii = 0.0;
  }
  for (int kk = 0; kk <= (c.visc == VISC_GALERKIN ? -1 : L); kk++) {
    if (kk == dp) {
      sd = sd + dii;
      sm = sm + muii;
      continue;
    }
    const int64_t e = base + 32 * (kk - (kk > dp ? 1 : 0));
    double mu = muL[e];
    double d = tmax(dL[e], mu);
    if (c.alpha_limit) {
      const double s = tmax(ai, nd.alpha[G.col[e]]);
      d = d * s;
      mu = mu * s;
    }
    sd = sd + d;
    sm = sm + mu;
    dL[e] = d;
    muL[e] = mu;
  }
  if (c.alpha_limit && c.visc != VISC_GALERKIN) {
    dii = -sd;
    muii = -sm;
  }
  dLii[r] = dii;
  muLii[r] = muii;

  // pass 3: smb_2_roundoff / smb_2 / smb_1 rows and maxmin of the entropy,
  // in reference order with the diagonal at dp
  const bool galerkin = c.visc == VISC_GALERKIN;
  const bool type1 = !galerkin && c.viscous_type == 1;
  const bool need_res = c.visc == VISC_ENTROPY || c.visc == VISC_FCT;
  RowSums rs;
  const LowVisc lv{dL, muL, dii, muii};
  smb_rows_f64(G, c, st, u, nd, r, base, L, dp, ui, zi, m, lv,
               !galerkin && !type1 && c.roundoff_fix,              // smb_2_roundoff: low order
               galerkin || need_res || (!type1 && !c.roundoff_fix), // smb_2: Galerkin, residual, plain type2
               type1, rs);
  const double* rk2 = rs.rk2;
  // divide_by_lumped (:801-808) and the low-order state (:202-215)
  double ul[5];
  if (type1) {
    for (int q = 0; q < S; q++) ul[q] = ui[q] + dt * (rs.rk1[q] / m);
  } else if (!galerkin && c.roundoff_fix) {
    ul[0] = ui[0] * (1 + dt * rs.fix / m) + dt * (rs.rk[0] / m);
    for (int q = 1; q < S; q++) ul[q] = ui[q] + dt * (rs.rk[q] / m);
  } else {
    ul[0] = tmax(ui[0] + dt * (rk2[0] / m), 0.0);
    for (int q = 1; q < S; q++) ul[q] = ui[q] + dt * (rk2[q] / m);
  }
  uL.h[r] = ul[0]; uL.q1[r] = ul[1]; uL.q2[r] = ul[2];
  if (S == 5) { uL.q3[r] = ul[3]; uL.q4[r] = ul[4]; }
  if (delta_bad) atomicOr(err, ERRB_DELTA);
  if (!need_res) return;
  const double emax = rs.emax, emin = rs.emin;
  double rk2m[5];
  for (int q = 0; q < S; q++) rk2m[q] = rk2[q] / m;
  // entropy residual (update.f90:838-868), rescale hoisted
  double un_[5];
  for (int q = 0; q < S; q++) un_[q] = ui[q] + dt * rk2m[q];
  const double on = one_over_h(un_[0], htiny);
  const double vn1 = un_[1] * on, vn2 = un_[2] * on;
  double En = g * (un_[0] * un_[0]);
  En = En + vn1 * un_[1];
  En = En + vn2 * un_[2];
  En = 0.5 * En;
  const double E = nd.ent[r];
  double Ep[5] = {0, 0, 0, 0, 0};
  Ep[0] = g * ui[0];
  Ep[0] = Ep[0] - 0.5 * (v1i * v1i);
  Ep[1] = v1i;
  Ep[0] = Ep[0] - 0.5 * (v2i * v2i);
  Ep[2] = v2i;
  double rsd = m * (En - E) / dt;
  for (int q = 0; q < S; q++) rsd = rsd - m * rk2m[q] * Ep[q];
  const double rescale = tabs(emax - emin) / 2 + c.rescale_floor;
  res[r] = tabs(rsd) / rescale;
}

// ---------------------------------------------------------------------------
// k_fct: d^H = MIN(dL, res_ij), mu^H likewise (update.f90:232-239), f_ij
// (compute_fct_matrix :721-748), check_hmin of the low-order state (:271) and
// R^-_i of FCT_positivity (SOURCES/fct.f90:15-30).
// ---------------------------------------------------------------------------
__global__ void k_fct_f64(Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                          StateF64 u, const double* __restrict__ dL, const double* __restrict__ muL,
                          StateF64 uL, const double* __restrict__ res, double* __restrict__ fct,
                          double* __restrict__ rminus, unsigned* __restrict__ err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= G.n_rows) return;
  const int L = G.len[r];
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const InstState st = St[b];
  if (st.done) return;
  const InstConst& c = C[b];
  if (c.visc != VISC_FCT) return;
  const int64_t base = entry_base(G, r);
  const double hi = u.h[r], zi = G.bath[r], resi = res[r];
  double P = -1.e-15;
  for (int k = 0; k < L; k++) {
    const int64_t e = base + 32 * k;
    const int j = G.col[e];
    const double rij = tmax(resi, res[j]);
    const double d0 = dL[e], m0 = muL[e];
    const double dH = tmin(d0, 1.0 * rij), mH = tmin(m0, 1.0 * rij);
    const double hj = u.h[j], zj = G.bath[j];
    const double zmax = tmax(zi, zj);
    const double Hij = tmax(0.0, hi + zi - zmax);
    const double Hji = tmax(0.0, hj + zj - zmax);
    const double ratij = (hi <= 0.0) ? 0.0 : Hij / hi;
    const double ratji = (hj <= 0.0) ? 0.0 : Hji / hj;
    const double f = (dH - d0) * (hj * ratji - hi * ratij) + (mH - m0) * (hj * (1.0 - ratji) - hi * (1.0 - ratij));
    fct[e] = f;
    if (f < 0.0) P = P + f;
  }
  const double hL = uL.h[r];
  if (hL < 0.0) atomicOr(err, ERRB_NEG_H);
  const double scaled = (G.lumped[r] / st.dt) * hL;
  const double Q = 0.0 - scaled;
  double R = tmin(Q / P, 1.0);
  if (scaled <= c.htiny) R = 0.0;
  rminus[r] = R;
}

// Component q of a state at row r (no local arrays of pointers: the row's
// values stay in registers).
__device__ __forceinline__ double comp_f64(const StateF64& s, int q, int64_t r) {
  switch (q) {
    case 0: return s.h[r];
    case 1: return s.q1[r];
    case 2: return s.q2[r];
    case 3: return s.q3[r];
    default: return s.q4[r];
  }
}
__device__ __forceinline__ void store_f64(const StateF64& s, int q, int64_t r, double v) {
  switch (q) {
    case 0: s.h[r] = v; break;
    case 1: s.q1[r] = v; break;
    case 2: s.q2[r] = v; break;
    case 3: s.q3[r] = v; break;
    default: s.q4[r] = v; break;
  }
}

// End of a stage for one row: check_hmin (when the mode has it), non-finite
// check, the SSP-RK combination and bdy of the time loop (main.f90:77-90)
// when rk_stage > 0, and the store.
__device__ __forceinline__ void finish_row_f64(const Graph& G, const InstConst& c, const InstState& st, int64_t r,
                                               int S, double (&un)[5], bool check_hmin, int rk_stage,
                                               const StateF64& u0, const StateF64& out, unsigned* err) {
  if (check_hmin && un[0] < 0.0) atomicOr(err, ERRB_NEG_H);
  if (!(un[0] == un[0]) || !(un[1] == un[1]) || !(un[2] == un[2])) atomicOr(err, ERRB_NAN);
  const unsigned msk = (rk_stage >= 1 && G.dir_mask) ? G.dir_mask[r] : 0u;
#pragma unroll
  for (int q = 0; q < 5; q++) {
    if (q >= S) break;
    double v = un[q];
    if (rk_stage == 2) v = (3 * comp_f64(u0, q, r) + v) / 4;
    else if (rk_stage == 3) v = (comp_f64(u0, q, r) + 2 * v) / 3;
    if (msk & (1u << q)) v = dirichlet_value(G, c, st, rk_stage, q, r);
    store_f64(out, q, r, v);
  }
}

// ---------------------------------------------------------------------------
// k_update: l_ij (fct.f90:31-41), (d^H-d^L) l_ij and (mu^H-mu^L) l_ij
// (update.f90:278-279), apply_viscosity (:684-718), unext = u^L + dt rk/m
// (:281-282), check_hmin (:285), then the SSP-RK combination and bdy of the
// time loop (main.f90:77-90) when rk_stage > 0.
//   rk_stage 0: out = unext                       (plain euler call)
//   rk_stage 1: out = unext, Dirichlet
//   rk_stage 2: out = (3 u0 + unext)/4, Dirichlet
//   rk_stage 3: out = (u0 + 2 unext)/3, Dirichlet
// ---------------------------------------------------------------------------
__global__ void k_update_f64(Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                             StateF64 u, const double* __restrict__ dL, const double* __restrict__ muL,
                             StateF64 uL, const double* __restrict__ res, const double* __restrict__ fct,
                             const double* __restrict__ rminus, StateF64 u0, StateF64 out, int rk_stage,
                             double* __restrict__ lij_out, unsigned* __restrict__ err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= G.n_rows) return;
  const int L = G.len[r];
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const InstState st = St[b];
  if (st.done) return;
  const InstConst& c = C[b];
  if (c.visc == VISC_ENTROPY) return;          // k_entropy_f64 writes these rows
  const bool fct_mode = c.visc == VISC_FCT;
  const int S = c.S;
  const int64_t base = entry_base(G, r);
  double ui[5];
  ui[0] = u.h[r]; ui[1] = u.q1[r]; ui[2] = u.q2[r];
  if (S == 5) { ui[3] = u.q3[r]; ui[4] = u.q4[r]; }
  const double zi = G.bath[r], resi = res[r], Ri = fct_mode ? rminus[r] : 0.0;
  double xx[5] = {0, 0, 0, 0, 0};
  for (int k = 0; k < (fct_mode ? L : 0); k++) {   // 'galerkin' / 'viscous': u^L is the result
    const int64_t e = base + 32 * k;
    const int j = G.col[e];
    const double f = fct[e];
    const double l = (f >= 0.0) ? rminus[j] : Ri;
    if (lij_out) lij_out[e] = l;
    const double rij = tmax(resi, res[j]);
    const double d0 = dL[e], m0 = muL[e];
    const double dd = (tmin(d0, 1.0 * rij) - d0) * l;
    const double dm = (tmin(m0, 1.0 * rij) - m0) * l;
    double uj[5];
    uj[0] = u.h[j]; uj[1] = u.q1[j]; uj[2] = u.q2[j];
    if (S == 5) { uj[3] = u.q3[j]; uj[4] = u.q4[j]; }
    const double zj = G.bath[j];
    const double zmax = tmax(zi, zj);
    const double Hij = tmax(0.0, ui[0] + zi - zmax);
    const double Hji = tmax(0.0, uj[0] + zj - zmax);
    const double ratij = (ui[0] <= 0.0) ? 0.0 : Hij / ui[0];
    const double ratji = (uj[0] <= 0.0) ? 0.0 : Hji / uj[0];
    for (int q = 0; q < S; q++)
      xx[q] = xx[q] + dd * (uj[q] * ratji - ui[q] * ratij) + dm * (uj[q] * (1.0 - ratji) - ui[q] * (1.0 - ratij));
  }
  const double m = G.lumped[r], dt = st.dt;
  double un[5] = {0, 0, 0, 0, 0};
  const double* ulp[5] = {uL.h, uL.q1, uL.q2, uL.q3, uL.q4};
  for (int q = 0; q < S; q++) un[q] = ulp[q][r] + dt * (xx[q] / m);
  // check_hmin follows 'fct' (update.f90:285); 'viscous' and 'galerkin' return
  // before it (:219-222, :155-176)
  finish_row_f64(G, c, st, r, S, un, fct_mode, rk_stage, u0, out, err);
}

// ---------------------------------------------------------------------------
// k_entropy: 'entropy_visc' (update.f90:225-262): the smb_2_roundoff (or
// smb_2) rows with d^H = MIN(d, res_ij), mu^H = MIN(mu, res_ij), the update
// u = u(1 + dt fix/m) + dt rk/m, check_hmin (:285), then the RK combination
// and bdy like k_update.
// ---------------------------------------------------------------------------
__global__ void k_entropy_f64(Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                              StateF64 u, NodeF64 nd, const double* __restrict__ dL, const double* __restrict__ muL,
                              const double* __restrict__ dLii, const double* __restrict__ muLii,
                              const double* __restrict__ res, StateF64 u0, StateF64 out, int rk_stage,
                              unsigned* __restrict__ err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= G.n_rows) return;
  const int L = G.len[r];
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const InstState st = St[b];
  if (st.done) return;
  const InstConst& c = C[b];
  if (c.visc != VISC_ENTROPY) return;
  const int S = c.S;
  const int64_t base = entry_base(G, r);
  const int dp = G.dpos[r];
  double ui[5];
  ui[0] = u.h[r]; ui[1] = u.q1[r]; ui[2] = u.q2[r];
  if (S == 5) { ui[3] = u.q3[r]; ui[4] = u.q4[r]; }
  const double zi = G.bath[r], m = G.lumped[r], dt = st.dt;
  const HighVisc hv{dL, muL, res, dLii[r], muLii[r], res[r]};
  RowSums rs;
  smb_rows_f64(G, c, st, u, nd, r, base, L, dp, ui, zi, m, hv, c.roundoff_fix != 0, c.roundoff_fix == 0, false, rs);
  double un[5] = {0, 0, 0, 0, 0};
  if (c.roundoff_fix) {
    un[0] = ui[0] * (1 + dt * rs.fix / m) + dt * (rs.rk[0] / m);
    for (int q = 1; q < S; q++) un[q] = ui[q] + dt * (rs.rk[q] / m);
  } else {
    un[0] = tmax(ui[0] + dt * (rs.rk2[0] / m), 0.0);
    for (int q = 1; q < S; q++) un[q] = ui[q] + dt * (rs.rk2[q] / m);
  }
  finish_row_f64(G, c, st, r, S, un, true, rk_stage, u0, out, err);
}

// ---------------------------------------------------------------------------
// k_dt: compute_dij (update.f90:291-326) diagonal and COMPUTE_DT's
// max |d_ii|/m_i (main.f90:166-174), per instance.  d_out (nullable)
// receives every d_ij.
// ---------------------------------------------------------------------------
__global__ void k_dt_f64(Graph G, const InstConst* __restrict__ C, InstState* __restrict__ St, StateF64 u,
                         const double* __restrict__ ovh, const double* __restrict__ sqgh, double* __restrict__ d_out,
                         double* __restrict__ dii_out, unsigned* __restrict__ err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double val = 0.0;
  int b = -1;
  if (r < G.n_rows && G.len[r] > 0) {
    b = G.slice_inst[r >> 5];
    if (!St[b].done) {
      const InstConst& c = C[b];
      const int L = G.len[r];
      const int64_t base = entry_base(G, r);
      const LamConstF64<double> lk = lam_const_f64(c.g, sqrt(2.0));
      const double hi = u.h[r], q1 = u.q1[r], q2 = u.q2[r];
      const double ovhi = ovh ? ovh[r] : one_over_h(hi, c.htiny);
      const double sqgi = sqgh ? sqgh[r] : sqrt(c.g * tabs(hi));
      double s = 0.0;
      bool bad = false;
      for (int k = 0; k < L; k++) {
        const int64_t e = base + 32 * k;
        double d = 0.0;
        {
          const int j = G.col[e];
          const double norm = G.cnorm[e];                                  // sqrt(c.c)
          const double hj = u.h[j];
          const double ovhj = ovh ? ovh[j] : one_over_h(hj, c.htiny);
          const double sqgj = sqgh ? sqgh[j] : sqrt(c.g * tabs(hj));
          double lam;
          if (!lambda_vacc(hi, q1, q2, ovhi, sqgi, hj, u.q1[j], u.q2[j], ovhj, sqgj, G.cnx[e], G.cny[e], c.g,
                           c.htiny, lk, &lam))
            bad = true;
          d = norm * lam;
        }
        if (d_out) d_out[e] = d;
        s = s + d;
      }
      if (dii_out) dii_out[r] = -s;
      val = tabs(-s) / G.lumped[r];
      if (bad) atomicOr(err, ERRB_DELTA);
    } else {
      b = -1;
    }
  }
  // warp-level max per instance: a warp covers one 32-row slice and a slice
  // never straddles two instances
  (void)b;
  const unsigned full = 0xffffffffu;
  for (int off = 16; off > 0; off >>= 1) val = fmax(val, __shfl_down_sync(full, val, off));
  const int64_t r0 = r & ~(int64_t)31;
  if ((threadIdx.x & 31) == 0 && r0 < G.n_rows) {
    const int bw = G.slice_inst[r0 >> 5];
    if (!St[bw].done && val > 0.0) atomicMax(&St[bw].maxd_bits, (unsigned long long)__double_as_longlong(val));
  }
}

// Start of a time step: DO WHILE(time < Tfinal) and dt = CFL/max (main.f90:61,
// 173), or the fixed dt = 2.5e-2 of the Malpasset case (type 9, main.f90:67-69)
__global__ void k_step_begin(const InstConst* __restrict__ C, InstState* __restrict__ St, int n_inst) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_inst) return;
  InstState& s = St[b];
  if (s.done) return;
  if (!(s.time < s.t_final)) { s.done = 1; return; }
  double mx = __longlong_as_double((long long)s.maxd_bits);
  inst_set_dt(s, C[b].type_test == 9 ? 2.5e-2 : C[b].cfl * 1 / mx);
  s.maxd_bits = 0ull;
}

// Start of a swe_rk3_steps call: step counters and the lambda_max maximum
// restart (the instances' time, dt and done flags carry over)
__global__ void k_reset_counters(InstState* __restrict__ St, int n_inst) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_inst) return;
  St[b].steps = 0;
  St[b].maxd_bits = 0ull;
}

// End of a time step: time = to + dt (main.f90:91)
__global__ void k_step_end(InstState* __restrict__ St, int n_inst) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_inst) return;
  InstState& s = St[b];
  if (s.done) return;
  s.time = s.time + s.dt;
  s.steps += 1;
}

// FCT_positivity as a stand-alone operator on one instance (fct.f90:5-42)
__global__ void k_fct_positivity_f64(Graph G, const InstConst* __restrict__ C, const double* __restrict__ unext,
                                     const double* __restrict__ mat, const double* __restrict__ matii,
                                     double* __restrict__ rtmp, double* __restrict__ lij, int pass) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= G.n_rows) return;
  const int L = G.len[r];
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const int64_t base = entry_base(G, r);
  if (pass == 0) {
    const int dp = G.dpos[r];
    double P = -1.e-15;
    for (int kk = 0; kk <= L; kk++) {         // reference order, diagonal at dp
      const double f = (kk == dp) ? matii[r] : mat[base + 32 * (kk - (kk > dp ? 1 : 0))];
      if (f < 0.0) P = P + f;
    }
    double R = tmin((0.0 - unext[r]) / P, 1.0);
    if (unext[r] <= C[b].htiny) R = 0.0;
    rtmp[r] = R;
  } else {
    for (int k = 0; k < L; k++) {
      const int64_t e = base + 32 * k;
      lij[e] = (mat[e] >= 0.0) ? rtmp[G.col[e]] : rtmp[r];
    }
  }
}

// FCT_generic (SOURCES/SAFE/fct.f90:3-43) as a stand-alone operator: the
// two-sided Zalesak limiter with local bounds maxn/minn.  Pass 0: P+-, Q+-,
// R+- per row (entries in reference order, the diagonal at dpos); pass 1:
// sum_j l_ij f_ij with l_ij = MIN(R+_i, R-_j) (f >= 0) or MIN(R-_i, R+_j), and
// u_i += x / dg_i.
__global__ void k_fct_generic_f64(Graph G, double* __restrict__ unext, const double* __restrict__ maxn,
                                  const double* __restrict__ minn, const double* __restrict__ dg,
                                  const double* __restrict__ mat, const double* __restrict__ matii,
                                  double* __restrict__ rplus, double* __restrict__ rminus, int pass) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= G.n_rows) return;
  const int L = G.len[r];
  if (L == 0) return;
  const int64_t base = entry_base(G, r);
  const int dp = G.dpos[r];
  if (pass == 0) {
    const double Qplus = dg[r] * (maxn[r] - unext[r]);
    const double Qminus = dg[r] * (minn[r] - unext[r]);
    double Pplus = 1.e-15, Pminus = -1.e-15;
    for (int kk = 0; kk <= L; kk++) {
      const double f = (kk == dp) ? matii[r] : mat[base + 32 * (kk - (kk > dp ? 1 : 0))];
      if (f >= 0.0) Pplus = Pplus + f;
      else Pminus = Pminus + f;
    }
    rplus[r] = tmin(Qplus / Pplus, 1.0);
    rminus[r] = tmin(Qminus / Pminus, 1.0);
  } else {
    double x = 0.0;
    for (int kk = 0; kk <= L; kk++) {
      const int64_t e = base + 32 * (kk - (kk > dp ? 1 : 0));
      const double f = (kk == dp) ? matii[r] : mat[e];
      const int64_t j = (kk == dp) ? r : (int64_t)G.col[e];
      const double l = (f >= 0.0) ? tmin(rplus[r], rminus[j]) : tmin(rminus[r], rplus[j]);
      x = x + l * f;
    }
    unext[r] = unext[r] + x / dg[r];
  }
}


// ----------------------------- launchers -----------------------------------
static inline unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

#define EV_BEGIN(k) if (kev) cudaEventRecord(kev->ev[2 * (k)], s)
#define EV_END(k) if (kev) cudaEventRecord(kev->ev[2 * (k) + 1], s)

void launch_node_f64(const StageArgs& a, cudaStream_t s) {
  NodeF64 nd{a.w.ovh, a.w.v1, a.w.v2, a.w.ent, a.w.alpha, a.w.sqgh};
  k_node_f64<<<nblk(a.G.n_rows, a.block), a.block, 0, s>>>(a.G, a.C, a.St, a.u, nd);
}

void launch_stage_f64(const StageArgs& a, cudaStream_t s, const KernelEvents* kev) {
  const int bs = a.block;
  NodeF64 nd{a.w.ovh, a.w.v1, a.w.v2, a.w.ent, a.w.alpha, a.w.sqgh};
  EV_BEGIN(1);
  if (!a.skip_node) k_node_f64<<<nblk(a.G.n_rows, bs), bs, 0, s>>>(a.G, a.C, a.St, a.u, nd);
  EV_END(1); EV_BEGIN(2);
  k_low_f64<<<nblk(a.G.n_rows, bs), bs, 0, s>>>(a.G, a.C, a.St, a.u, nd, a.w.dL, a.w.muL, a.w.dLii, a.w.muLii,
                                                a.w.uL, a.w.res, a.dij_in, a.err);
  EV_END(2); EV_BEGIN(3);
  k_fct_f64<<<nblk(a.G.n_rows, bs), bs, 0, s>>>(a.G, a.C, a.St, a.u, a.w.dL, a.w.muL, a.w.uL, a.w.res, a.w.fct,
                                                a.w.rminus, a.err);
  EV_END(3); EV_BEGIN(4);
  k_update_f64<<<nblk(a.G.n_rows, bs), bs, 0, s>>>(a.G, a.C, a.St, a.u, a.w.dL, a.w.muL, a.w.uL, a.w.res, a.w.fct,
                                                   a.w.rminus, a.u0, a.out, a.rk_stage, a.lij_out, a.err);
  if (a.entropy)
    k_entropy_f64<<<nblk(a.G.n_rows, bs), bs, 0, s>>>(a.G, a.C, a.St, a.u, nd, a.w.dL, a.w.muL, a.w.dLii, a.w.muLii,
                                                      a.w.res, a.u0, a.out, a.rk_stage, a.err);
  EV_END(4);
}

void launch_dt_f64(const Graph& G, const InstConst* C, InstState* St, const StateF64& u, double* d_out,
                   double* dii_out, unsigned* err, int block, cudaStream_t s, const WorkF64* node) {
  k_dt_f64<<<nblk(G.n_rows, block), block, 0, s>>>(G, C, St, u, node ? node->ovh : nullptr,
                                                   node ? node->sqgh : nullptr, d_out, dii_out, err);
}

void launch_step_begin(const InstConst* C, InstState* St, int n_inst, cudaStream_t s) {
  k_step_begin<<<nblk(n_inst, 128), 128, 0, s>>>(C, St, n_inst);
}

void launch_step_end(InstState* St, int n_inst, cudaStream_t s) {
  k_step_end<<<nblk(n_inst, 128), 128, 0, s>>>(St, n_inst);
}
void launch_reset_counters(InstState* St, int n_inst, cudaStream_t s) {
  k_reset_counters<<<nblk(n_inst, 128), 128, 0, s>>>(St, n_inst);
}

void launch_fct_positivity_f64(const Graph& G, const InstConst* C, const double* unext, const double* mat,
                               const double* matii, double* rtmp, double* lij, cudaStream_t s) {
  k_fct_positivity_f64<<<nblk(G.n_rows, 128), 128, 0, s>>>(G, C, unext, mat, matii, rtmp, lij, 0);
  k_fct_positivity_f64<<<nblk(G.n_rows, 128), 128, 0, s>>>(G, C, unext, mat, matii, rtmp, lij, 1);
}

void launch_fct_generic_f64(const Graph& G, double* unext, const double* maxn, const double* minn, const double* dg,
                            const double* mat, const double* matii, double* rplus, double* rminus, cudaStream_t s) {
  k_fct_generic_f64<<<nblk(G.n_rows, 128), 128, 0, s>>>(G, unext, maxn, minn, dg, mat, matii, rplus, rminus, 0);
  k_fct_generic_f64<<<nblk(G.n_rows, 128), 128, 0, s>>>(G, unext, maxn, minn, dg, mat, matii, rplus, rminus, 1);
}


}  // namespace swe
