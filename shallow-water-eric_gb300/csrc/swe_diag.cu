// Diagnostics on the device-resident state: the quadrature norms of
// ns_anal_l1 / ns_anal_0 / ns_l1 (SFEMaNS/FEMSUB_OBJET/fem_tn.f90:1513-1553,
// 1679-1716) used by compute_errors (SOURCES/main.f90:198-263) and by the
// time-loop monitor of types 1, 2 and 10 (main.f90:94-99), without copying
// the state back to the host.
//
// One thread per element interpolates the field at the three Gauss points
// (the same expression as the reference, sum_n f(jj(n,m)) ww(n,l)) and adds
// |f - f_anal| rj and (f - f_anal)^2 rj; the sums are combined per warp in
// double-double, and the warps' partial sums are added by one block in a
// fixed order: equal to the reference's sequential sums to rounding, and the
// same bits on every call.
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

__device__ __forceinline__ void dd_add(double& v, double& c, double o, double oc) {
  const double s = v + o;               // two-sum
  const double bb = s - v;
  const double e = (v - (s - bb)) + (o - bb);
  v = s;
  c = c + oc + e;
}

// part[4 w + 0..3], per warp w: L1 sum (hi, lo), L2 sum of squares (hi, lo)
__global__ void k_norms(DiagField f, const int* __restrict__ jj, const double* __restrict__ rj, int me,
                        const int* __restrict__ row_of_node, const double* __restrict__ f_anal,
                        double* __restrict__ part) {
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
    const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    part[4 * w + 0] = t1;
    part[4 * w + 1] = c1;
    part[4 * w + 2] = t2;
    part[4 * w + 3] = c2;
  }
}

// One block of kNormThreads: thread t adds the partials t, t + kNormThreads,
// ... in order, the warps combine by the fixed shuffle tree, thread 0 adds
// the warps in order into acc[0..3].
constexpr int kNormThreads = 256;

__global__ void __launch_bounds__(kNormThreads) k_norms_final(const double* __restrict__ part, int64_t nw,
                                                              double* __restrict__ acc) {
  double v1 = 0.0, c1 = 0.0, v2 = 0.0, c2 = 0.0;
  for (int64_t w = threadIdx.x; w < nw; w += kNormThreads) {
    dd_add(v1, c1, part[4 * w + 0], part[4 * w + 1]);
    dd_add(v2, c2, part[4 * w + 2], part[4 * w + 3]);
  }
  dd_warp_sum(v1, c1);
  dd_warp_sum(v2, c2);
  __shared__ double sw[kNormThreads / 32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { sw[warp][0] = v1; sw[warp][1] = c1; sw[warp][2] = v2; sw[warp][3] = c2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a1 = 0.0, b1 = 0.0, a2 = 0.0, b2 = 0.0;
    for (int k = 0; k < kNormThreads / 32; k++) { dd_add(a1, b1, sw[k][0], sw[k][1]); dd_add(a2, b2, sw[k][2], sw[k][3]); }
    acc[0] = a1; acc[1] = b1; acc[2] = a2; acc[3] = b2;
  }
}

int64_t norm_partials(int me) { return (int64_t)((me + 255) / 256) * (256 / 32); }

void launch_norms(int field, int precision, const StateF64& a, const StateMix& mx, const int* jj, const double* rj,
                  int me, const int* row_of_node, const double* f_anal, double* part, double* acc, cudaStream_t s) {
  DiagField f{field, precision, a, mx};
  k_norms<<<(unsigned)((me + 255) / 256), 256, 0, s>>>(f, jj, rj, me, row_of_node, f_anal, part);
  k_norms_final<<<1, kNormThreads, 0, s>>>(part, norm_partials(me), acc);
}

// ---- total mass sum_i m_i h_i per instance (main.f90:94-99 monitors it),
// added in a fixed order so that every call gives the same bits: one
// double-double partial per 32-row slice (a slice belongs to one instance),
// then one block per instance adds its slices like k_norms_final, with
// 1024 threads (an instance may hold 10^5 slices).
__global__ void k_mass_part(Graph G, const double* __restrict__ h64, const float2* __restrict__ hdf,
                            double* __restrict__ part) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double v = 0.0, c = 0.0;
  if (r < G.n_rows && G.len[r] > 0) v = G.lumped[r] * (h64 ? h64[r] : df_to_double(hdf[r]));
  dd_warp_sum(v, c);
  if ((threadIdx.x & 31) == 0 && r < G.n_rows) {
    part[2 * (r >> 5)] = v;
    part[2 * (r >> 5) + 1] = c;
  }
}

constexpr int kMassThreads = 1024;

__global__ void __launch_bounds__(kMassThreads) k_mass_final(const double* __restrict__ part,
                                                             const int64_t* __restrict__ inst_slice,
                                                             double* __restrict__ acc) {
  const int b = blockIdx.x;
  double v = 0.0, c = 0.0;
  for (int64_t w = inst_slice[b] + threadIdx.x; w < inst_slice[b + 1]; w += kMassThreads)
    dd_add(v, c, part[2 * w], part[2 * w + 1]);
  dd_warp_sum(v, c);
  __shared__ double sw[kMassThreads / 32][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { sw[warp][0] = v; sw[warp][1] = c; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, e = 0.0;
    for (int k = 0; k < kMassThreads / 32; k++) dd_add(a, e, sw[k][0], sw[k][1]);
    acc[2 * b] = a;
    acc[2 * b + 1] = e;
  }
}

void launch_mass(const Graph& G, int n_inst, const double* h64, const float2* hdf, const int64_t* inst_slice,
                 double* part, double* acc, cudaStream_t s) {
  k_mass_part<<<(unsigned)((G.n_rows + 255) / 256), 256, 0, s>>>(G, h64, hdf, part);
  k_mass_final<<<n_inst, kMassThreads, 0, s>>>(part, inst_slice, acc);
}

}  // namespace swe
