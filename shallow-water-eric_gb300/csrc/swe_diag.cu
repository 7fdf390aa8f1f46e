// Diagnostics on the device-resident state: the quadrature norms of
// ns_anal_l1 / ns_anal_0 / ns_l1 (SFEMaNS/FEMSUB_OBJET/fem_tn.f90:1513-1553,
// 1679-1716) used by compute_errors (SOURCES/main.f90:198-263) and by the
// time-loop monitor of types 1, 2 and 10 (main.f90:94-99), without copying
// the state back to the host.
//
// One thread per element interpolates the field at the three Gauss points
// (the same expression as the reference, sum_n f(jj(n,m)) ww(n,l)) and adds
// |f - f_anal| rj and (f - f_anal)^2 rj; the sums are combined per warp in
// double-double and accumulated with atomics, so they equal the reference's
// sequential sums to rounding (order-independent to ~1e-16 relative).
#include "swe_kernels.hpp"

namespace swe {

struct DiagField {
  int field;            // 0..4 a component, kFieldH32 for h^(3/2)
  int precision;        // 0 FP64 state, 1 mixed state
  StateF64 a;
  StateMix m;
};

__device__ __forceinline__ double field_value(const DiagField& f, int64_t r) {
  double h, q = 0.0;
  if (f.precision == 0) {
    h = f.a.h[r];
    switch (f.field) {
      case 1: q = f.a.q1[r]; break;
      case 2: q = f.a.q2[r]; break;
      case 3: q = f.a.q3[r]; break;
      case 4: q = f.a.q4[r]; break;
      default: break;
    }
  } else {
    h = df_to_double(f.m.h[r]);
    const float4 v = f.m.nq[r];
    switch (f.field) {
      case 1: q = v.y; break;
      case 2: q = v.z; break;
      case 3: q = f.m.q3[r]; break;
      case 4: q = f.m.q4[r]; break;
      default: break;
    }
  }
  if (f.field == 0) return h;
  if (f.field == kFieldH32) return h * sqrt(h);
  return q;
}

__device__ __forceinline__ void dd_warp_sum(double& v, double& c) {
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_down_sync(0xffffffffu, v, off);
    const double oc = __shfl_down_sync(0xffffffffu, c, off);
    const double s = v + o;             // two-sum
    const double bb = s - v;
    const double e = (v - (s - bb)) + (o - bb);
    v = s;
    c = c + oc + e;
  }
}

// acc[0..1]: L1 sum (hi, lo); acc[2..3]: L2 sum of squares (hi, lo)
__global__ void k_norms(DiagField f, const int* __restrict__ jj, const double* __restrict__ rj, int me,
                        const int* __restrict__ row_of_node, const double* __restrict__ f_anal,
                        double* __restrict__ acc) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  double t1 = 0.0, t2 = 0.0;
  if (m < me) {
    const double one = 1, two = 2, three = 3, six = 6;
    const double xx[3] = {one / six, two / three, one / six};
    const double yy[3] = {one / six, one / six, two / three};
    double fn[3];
    for (int n = 0; n < 3; n++) fn[n] = field_value(f, row_of_node[jj[3 * m + n]]);
    for (int l = 0; l < 3; l++) {
      const double ww[3] = {one - xx[l] - yy[l], xx[l], yy[l]};
      double fl = 0.0;
      for (int n = 0; n < 3; n++) fl = fl + fn[n] * ww[n];
      const size_t idx = (size_t)m * 3 + l;
      const double d = fl - (f_anal ? f_anal[idx] : 0.0);
      t1 = t1 + fabs(d) * rj[idx];
      t2 = t2 + d * d * rj[idx];
    }
  }
  double c1 = 0.0, c2 = 0.0;
  dd_warp_sum(t1, c1);
  dd_warp_sum(t2, c2);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&acc[0], t1);
    atomicAdd(&acc[1], c1);
    atomicAdd(&acc[2], t2);
    atomicAdd(&acc[3], c2);
  }
}

void launch_norms(int field, int precision, const StateF64& a, const StateMix& mx, const int* jj, const double* rj,
                  int me, const int* row_of_node, const double* f_anal, double* acc, cudaStream_t s) {
  DiagField f{field, precision, a, mx};
  k_norms<<<(unsigned)((me + 255) / 256), 256, 0, s>>>(f, jj, rj, me, row_of_node, f_anal, acc);
}

}  // namespace swe
