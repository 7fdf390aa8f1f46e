// Device-side data layout and per-edge physics shared by the FP64 and the
// mixed-precision kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace swe {

// Error bits raised by kernels (never a trap); the host maps them to
// SWE_ERR_* after each launch sequence.
enum : unsigned { ERRB_NEG_H = 1u, ERRB_DELTA = 2u, ERRB_NAN = 4u };

// inputs%viscosity_type (the values of SWE_VISC_* in the C ABI header)
enum : int { VISC_GALERKIN = 0, VISC_VISCOUS = 1, VISC_ENTROPY = 2, VISC_FCT = 3 };

// Per-instance constants (one record per mesh of a batch).  The FP32 copies
// are rounded once on the host: the mixed kernels never convert per row
// (a float<->double conversion issues on GB300's narrow FP64 pipe).
struct InstConst {
  double g, htiny, cfl, mannings, lambda_sgn, max_water_h, rescale_floor;
  int type_test, S, visc, viscous_type, alpha_limit, roundoff_fix;
  float gf, htinyf, htiny_lo;      // htiny = htinyf + htiny_lo (double-float)
  float fricf;                     // g n^2 (friction)
  float lambda_sgnf, rescale_floorf;
};

// Per-instance time-loop state, device resident.
struct InstState {
  double dt, inv_dt, time, t_final;
  unsigned long long maxd_bits;   // max |d_ii|/m_i of the current step (double bits)
  int done, steps;
  float dtf, inv_dtf;             // FP32 copies of dt and inv_dt
};

__host__ __device__ inline void inst_set_dt(InstState& s, double dt) {
  s.dt = dt;
  s.inv_dt = dt > 0.0 ? 1.0 / dt : 0.0;
  s.dtf = (float)s.dt;
  s.inv_dtf = (float)s.inv_dt;
}

// The SELL-32 edge graph (see swe_setup.hpp).  Entry k of row r is at
// slice_ptr[r>>5] + 32*k + (r&31); entries are the off-diagonal CSR entries
// in reference order, the diagonal (c_ii) is stored per row and belongs
// between entries dpos-1 and dpos of the reference row.
struct Graph {
  int64_t n_rows;
  const int64_t* __restrict__ slice_ptr;
  const int* __restrict__ slice_inst;
  const int* __restrict__ col;
  const uint8_t* __restrict__ len;       // off-diagonal entries (0: padding row)
  const uint8_t* __restrict__ dpos;
  const double* __restrict__ cx;
  const double* __restrict__ cy;
  const double* __restrict__ cxii;
  const double* __restrict__ cyii;
  const float2* __restrict__ cf;          // mixed path, per entry: c_ij in FP32, (x, y) interleaved
  const float* __restrict__ cxiif;
  const float* __restrict__ cyiif;
  const double* __restrict__ cnorm;       // FP64 path, per entry: |c_ij| and c_ij/|c_ij|
  const double* __restrict__ cnx;         // (compute_dij's norm and normal, formed once)
  const double* __restrict__ cny;
  const double* __restrict__ lumped;
  const double* __restrict__ inv_lumped;
  const float* __restrict__ lumpedf;      // FP32 copies (mixed path)
  const float* __restrict__ inv_lumpedf;
  const double* __restrict__ bath;
  const float2* __restrict__ bathdf;     // mixed path: bathymetry as a double-float pair
  const uint8_t* __restrict__ dir_mask;   // bit k: component k is Dirichlet
  const double* __restrict__ dir_val;     // (S, n_rows) SoA, read where masked
  const uint8_t* __restrict__ dir_anal;   // bit k: component k's value is sol_anal(t) (or null)
  const double* __restrict__ rr_row;      // node coordinates (x, y) per row, where dir_anal is set
};

// sol_anal(k, rr, t) (SOURCES/condlim.f90:421-456, 751-791) of the analytic
// cases whose boundary data change with time, components 1-3 (h, qx, qy):
// type 5 (Thacker's planar oscillation, with the current reference's +htiny
// film) and type 13 (the SGN solitary wave).  The operations follow the
// reference's expressions in its order; cos, sin and cosh are CUDA's.
__device__ inline double sol_anal_dev(int type_test, int k, double x, double y, double t, double g, double htiny) {
  if (type_test == 5) {
    const double a = 1.0, h0 = 0.1, hL = 4.0, eta = 0.5;
    const double omega = sqrt(2 * g * h0) / a;
    const double dx = x - hL / 2.0, dy = y - hL / 2.0;
    const double bathi = -h0 * (1.0 - (dx * dx + dy * dy) / (a * a));
    const double v = (eta * h0 / (a * a)) * (2.0 * dx * cos(omega * t) + 2.0 * dy * sin(omega * t)) - bathi;
    const double base = v > 0.0 ? v : 0.0;
    if (k == 1) return base + htiny;
    if (k == 2) return -eta * omega * sin(omega * t) * base;
    return eta * omega * cos(omega * t) * base;
  }
  // type 13
  const double h1 = 10.0 / 100.0, h2 = 11.0 / 100.0, x0 = 2.75;
  const double D = sqrt(g * h2);
  const double z = sqrt((3.0 * (h2 - h1)) / (h2 * (h1 * h1)));
  const double arg = 1.0 / 2.0 * z * (x - x0 - D * t);
  const double se = 1.0 / cosh(arg);
  const double hv = h1 + (h2 - h1) * (se * se);
  const double ht = hv > 0.0 ? hv : 0.0;
  if (k == 1) return ht;
  if (k == 2) return ht * D - h1 * D;
  return ht * 0.0;
}

// Value bdy (main.f90:176-188) writes into component q of row r after RK
// stage rk_stage of the device loop: the fixed value, or sol_anal at the
// reference's bdy time of that stage (main.f90:78, 84, 90: to + dt, then
// (to + dt) + dt/2, then (to + dt/2) + dt).
__device__ inline double dirichlet_value(const Graph& G, const InstConst& c, const InstState& st, int rk_stage, int q,
                                         int64_t r) {
  if (G.dir_anal && ((G.dir_anal[r] >> q) & 1u)) {
    const double to = st.time, dt = st.dt;
    const double t = rk_stage == 1 ? to + dt : (rk_stage == 2 ? (to + dt) + dt / 2 : (to + dt / 2) + dt);
    return sol_anal_dev(c.type_test, q + 1, G.rr_row[2 * r], G.rr_row[2 * r + 1], t, c.g, c.htiny);
  }
  return G.dir_val[(int64_t)q * G.n_rows + r];
}

__device__ __forceinline__ int64_t entry_base(const Graph& G, int64_t r) {
  return G.slice_ptr[r >> 5] + (r & 31);
}

// FP32 shadow of an FP64 depth that keeps the sign of (h - htiny) and of h:
// the mixed kernels branch on h <= htiny and h <= 0 (SOURCES/update.f90:572-582,
// 644-655) with the shadow, so both branch decisions must match the FP64 depth.
__device__ __forceinline__ float shadow_depth(double h, double htiny) {
  float f = (float)h;
  const float ft = (float)htiny;
  if (h > htiny && !(f > ft)) f = nextafterf(ft, 3.4e38f);
  if (h > 0.0 && !(f > 0.0f)) f = 1.17549435e-38f;   // smallest normal (FTZ-safe)
  return f;
}

// ---- double-float arithmetic (value = x + y, two FP32 words, |y| <= ulp(x)/2)
// Knuth's two-sum and the FMA two-product, written with explicit roundings so
// that no contraction changes them.  About 48 significant bits; every
// operation issues on the FP32 pipes.
__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_float2(s, e);
}
__device__ __forceinline__ float2 df_from_double(double v) {
  const float hi = __double2float_rn(v);
  return make_float2(hi, __double2float_rn(v - (double)hi));
}
__device__ __forceinline__ double df_to_double(float2 a) { return (double)a.x + (double)a.y; }
__device__ __forceinline__ float2 df_add_f(float2 a, float b) {     // a + b
  const float2 t = two_sum(a.x, b);
  return two_sum(t.x, __fadd_rn(t.y, a.y));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {      // a + b
  const float2 t = two_sum(a.x, b.x);
  return two_sum(t.x, __fadd_rn(t.y, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 df_mul_f(float2 a, float b) {     // a * b
  const float p = __fmul_rn(a.x, b);
  const float e = __fmaf_rn(a.y, b, __fmaf_rn(a.x, b, -p));
  return two_sum(p, e);
}
__device__ __forceinline__ float2 df_scale(float2 a, float pow2) {  // a * 2^k, exact
  return make_float2(__fmul_rn(a.x, pow2), __fmul_rn(a.y, pow2));
}
__device__ __forceinline__ float2 df_div3(float2 a) {               // a / 3
  const float q1 = __fdiv_rn(a.x, 3.0f);
  const float r = __fadd_rn(__fmaf_rn(-3.0f, q1, a.x), a.y);      // a.x - 3 q1 is exact
  return two_sum(q1, __fdiv_rn(r, 3.0f));
}
// a > (hi + lo) for normalised pairs
__device__ __forceinline__ bool df_gt(float2 a, float hi, float lo) { return a.x > hi || (a.x == hi && a.y > lo); }

template <typename T> __device__ __forceinline__ T tmax(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T tmin(T a, T b) { return a < b ? a : b; }
template <typename T> __device__ __forceinline__ T tabs(T a) { return a < T(0) ? -a : a; }

// compute_one_over_h (SOURCES/condlim.f90:79-90): 2h/(h^2 + max(h,htiny)^2)
template <typename T> __device__ __forceinline__ T one_over_h(T h, T htiny) {
  T mh = tmax(h, htiny);
  return T(2) * h / (h * h + mh * mh);
}

// Per-call constants of compute_lambda_vacc, formed once per thread with the
// reference's own expressions (so every use sees the value the reference
// forms at that point).
template <typename T>
struct LamConstF64 {
  T x0;              // (2 sqrt2 - 1)^2
  T a, two_a;        // 1/(2 sqrt2), 2 a
  T sixteen_g;       // 16 g
  T two_sqrt_g;      // 2 sqrt(g)
  T sqrt_2_over_g;   // sqrt(2/g)
  T g_half;          // g/2
};
template <typename T>
__device__ __forceinline__ LamConstF64<T> lam_const_f64(T g, T sqrt2) {
  LamConstF64<T> k;
  const T t0 = T(2) * sqrt2 - T(1);
  k.x0 = t0 * t0;
  k.a = T(1) / (T(2) * sqrt2);
  k.two_a = T(2) * k.a;
  k.sixteen_g = T(16) * g;
  k.two_sqrt_g = T(2) * sqrt(g);
  k.sqrt_2_over_g = sqrt(T(2) / g);
  k.g_half = g / T(2);
  return k;
}

// phi (SOURCES/condlim.f90:960-981).  The node terms one_over_h(hl),
// one_over_h(hr) and sqrt(g hl), sqrt(g hr) are the nodes' per-node values
// (ovhl, ovhr; sqghl = sqrt(g |hl|) equals sqrt(g hl) for hl > 0, and is
// recomputed otherwise), so each is formed once per node instead of per
// entry and per call; one_over_h(h) and sqrt(g h) are formed once per call.
template <typename T>
__device__ __forceinline__ T phi_fn(T h, T ul, T hl, T ur, T hr, T g, T htiny, T ovhl, T ovhr, T sqghl, T sqghr,
                                    T g_half) {
  const bool shock_l = h > hl, shock_r = h > hr;
  const T ovh = (shock_l || shock_r) ? one_over_h(h, htiny) : T(0);
  const T sgh = (!shock_l || !shock_r) ? sqrt(g * h) : T(0);
  T fl, fr;
  if (shock_l) fl = (h - hl) * sqrt(g_half * (ovh + ovhl));
  else fl = T(2) * (sgh - (hl > T(0) ? sqghl : sqrt(g * hl)));
  if (shock_r) fr = (h - hr) * sqrt(g_half * (ovh + ovhr));
  else fr = T(2) * (sgh - (hr > T(0) ? sqghr : sqrt(g * hr)));
  return fl + fr + ur - ul;
}

// compute_lambda_vacc (SOURCES/condlim.f90:879-957) with the node values
// ovhl/ovhr (one_over_h) and sqghl/sqghr (sqrt(g |h|), the reference's
// sql/sqr) passed in; they equal what the reference forms bit for bit.
// Returns false where the reference STOPs (Delta < 0).
template <typename T>
__device__ __forceinline__ bool lambda_vacc(T hl, T qxl, T qyl, T ovhl, T sqghl, T hr, T qxr, T qyr, T ovhr, T sqghr,
                                            T nx, T ny, T g, T htiny, const LamConstF64<T>& k, T* lambda) {
  T vl = (qxl * nx + qyl * ny) * ovhl;
  T vr = (qxr * nx + qyr * ny) * ovhr;
  const T sql = sqghl, sqr = sqghr;
  T hmin, hmax;
  if (hl <= hr) { hmin = hl; hmax = hr; } else { hmin = hr; hmax = hl; }
  T ht;
  bool ok = true;
  T fh = phi_fn(k.x0 * hmin, vl, hl, vr, hr, g, htiny, ovhl, ovhr, sql, sqr, k.g_half);
  if (T(0) <= fh) {
    T s = tmax(vl - vr + T(2) * sql + T(2) * sqr, T(0));
    ht = tmin(k.x0 * hmin, s * s / k.sixteen_g);
  } else {
    fh = phi_fn(k.x0 * hmax, vl, hl, vr, hr, g, htiny, ovhl, ovhr, sql, sqr, k.g_half);
    T sqrmin = sqrt(hmin), sqrmax = sqrt(hmax);
    if (T(0) <= fh) {
      T c = -(hmin * k.a) - sqrmin * sqrmax + sqrmin * (vr - vl) / k.two_sqrt_g;
      T Delta = hmin - T(4) * k.a * c;
      if (Delta < T(0)) { ok = false; Delta = T(0); }
      T s = (-sqrmin + sqrt(Delta)) / k.two_a;
      ht = tmin(k.x0 * hmax, s * s);
    } else {
      ht = sqrmin * sqrmax * (T(1) + k.sqrt_2_over_g * (vl - vr) / (sqrmin + sqrmax));
    }
  }
  T lbdl = vl - sql * sqrt((T(1) + tmax((ht - hl) * ovhl / T(2), T(0))) * (T(1) + tmax((ht - hl) * ovhl, T(0))));
  T lbdr = vr + sqr * sqrt((T(1) + tmax((ht - hr) * ovhr / T(2), T(0))) * (T(1) + tmax((ht - hr) * ovhr, T(0))));
  *lambda = tmax(tabs(lbdl), tabs(lbdr));
  return ok;
}

}  // namespace swe
