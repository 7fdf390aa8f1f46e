// Mixed-precision stage kernels: every per-edge and per-row operation issues
// on the FP32 pipes.
//
// Same sweep structure as the FP64 path (one thread per row, SELL-32 graph)
// with the flux, lambda_max, viscosity, entropy-residual and antidiffusion
// arithmetic in FP32 on FP32 data (q, the free surface eta, c_ij, d_ij,
// mu_ij and an FP32 shadow of h).  A warp-wide FP64 instruction, or a
// float<->double conversion, costs GB300 tens of SM cycles (FP64 runs at
// ~1/64 of the FP32 rate), and a design that kept the limiter sums and the
// per-row depth updates in FP64 measured its FP64 pipe 73-79% busy in the
// limiter and update sweeps.  The precision the scheme needs is kept without
// FP64:
//   * the depth h (state, low-order h^L, new depth, RK combination) is a
//     double-float pair hi + lo (about 48 significant bits), so the FP32
//     increments of a stage are never lost to the rounding of h;
//   * h^L = h + a (P - N - c_ii.v_i h) with a = dt/m_i, P >= 0 and
//     a N <= CFL h (SOURCES/update.f90:202-215): non-negative in any rounding;
//   * the limiter R^-_i = min(1, (1 - 2^-18) Q^-_i / P^-_i) (fct.f90:15-30) is
//     FP32; the 2^-18 margin (64 units in the last place) bounds the at most
//     ~12 roundings between the limiter and the depth update, so the limited
//     update cannot take more than h^L out of a node (see k_fct_mix);
//   * the reference's threshold tests (h <= htiny, h <= 0) use an FP32 shadow
//     of h that keeps both decisions exact, and m h^L/dt <= htiny is decided in
//     FP64 inside a 1e-5 band around htiny.
//
// Well-balancing.  Node data that neighbours gather is packed per node as
// float4 {h shadow, qx, qy, eta}: one 16-byte load (one L2 sector) per
// neighbour, with the free surface eta = h + z rounded once per node from
// the double-float depth and the double-float bathymetry.  A lake at rest
// then has bit-identical eta at every wet node, and every term of a row
// vanishes exactly there:
//   * the topography term g h_i (eta_j - eta_i) c_ij (update.f90:606-610);
//   * the bathymetry difference z_j - z_i = (eta_j - eta_i) + (h_i - h_j),
//     which is then h_i - h_j exactly (Sterbenz), so the hydrostatic depths
//     H*_ij = max(0, h_i - max(0, z_j - z_i)) and H*_ji are equal bit for bit;
//   * the mass rows in the difference form d (H*_ji - H*_ij) (the reference's
//     d (h_j rat_ji - h_i rat_ij), with h rat = H* written out).
//
// Reproducibility.  The file is built without FMA contraction (-fmad=false);
// every fused multiply-add is written out with __fmaf_rn.  Every launch
// variant (block size, entry batch, resident grid, shared-memory tile,
// register cap) and the lambda_max reuse of stage 1 therefore perform the
// same IEEE operations on the same values in the same order: all variants,
// and hence any autotuner choice, give bit-identical results.
#include "swe_kernels.hpp"

namespace swe {

__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Programmatic dependent launch: the stage kernels are launched so that a
// kernel's blocks may start while the previous kernel's last blocks still
// run.  Each kernel lets its dependents launch at once (pdl_trigger), may
// prefetch data no kernel writes (the graph), then waits in pdl_wait until
// the previous grid has completed and its writes are visible, before it
// reads anything a kernel produced or writes anything.  Completion is
// transitive (every kernel waits before it can exit), so outputs of any
// earlier kernel are visible after the wait.  Without the launch attribute
// both instructions do nothing.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" :::); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// c . v with an explicit rounding sequence.  The low-order mass flux
// (mu_ij - c.v_j) h_j is non-negative only if mu_ij >= c.v_j holds bit for
// bit, so c.v_j is formed once per entry with a fixed rounding.
__device__ __forceinline__ float dotc(float cx, float cy, float vx, float vy) {
  return __fmaf_rn(cx, vx, __fmul_rn(cy, vy));
}

__device__ __forceinline__ float ovh_f(float h, float htiny) {
  float mh = fmaxf(h, htiny);
  return fdiv(2.0f * h, __fmaf_rn(h, h, __fmul_rn(mh, mh)));
}

// FP32 shadow of a double-float depth that keeps the sign of (h - htiny) and
// of h (the mixed kernels branch on h <= htiny and h <= 0 with it).
__device__ __forceinline__ float shadow_df(float2 h, const InstConst& c) {
  float f = h.x;
  const bool above = df_gt(h, c.htinyf, c.htiny_lo);
  if (above && !(f > c.htinyf)) f = nextafterf(c.htinyf, 3.4e38f);
  if (!above && f > c.htinyf) f = c.htinyf;
  if (!(f > 0.0f) && (h.x > 0.0f || h.y > 0.0f)) f = 1.17549435e-38f;   // smallest normal (FTZ-safe)
  return f;
}

// Free surface eta = h + z of a node record, rounded once from the
// double-float depth and the double-float bathymetry.
__device__ __forceinline__ float eta_of(float2 h, float2 z) { return df_add(h, z).x; }

// Hydrostatic reconstruction H*_ij = max(0, h_i + z_i - max(z_i, z_j))
// (SOURCES/update.f90:569-570) in the algebraically equal, cancellation-free
// form max(0, h_i - max(0, dz)), dz = z_j - z_i.  In FP32 the reference form
// loses (h_i + z_i) - z_i to rounding at the scale of z, which for thin
// layers on high bathymetry is a large relative error in H*/h.  H*_ij = h_i
// exactly when dz <= 0 and never exceeds h_i.
struct Recon {
  float Hij, Hji;
};
__device__ __forceinline__ Recon recon(float hi, float hj, float dz) {
  Recon R;
  R.Hij = (dz <= 0.f) ? hi : fmaxf(0.f, __fsub_rn(hi, dz));
  R.Hji = (dz >= 0.f) ? hj : fmaxf(0.f, __fadd_rn(hj, dz));
  return R;
}
// rat_ij = H*_ij / h_i with the reference's h <= 0 test (0 there); 1 exactly
// downhill and never above 1.
__device__ __forceinline__ float rat_of(float H, float h, bool flat, float invh) {
  return (h > 0.f) ? (flat ? 1.f : fminf(__fmul_rn(H, invh), 1.f)) : 0.f;
}
__device__ __forceinline__ float inv_pos(float h) { return (h > 0.f) ? fdiv(1.0f, h) : 0.f; }
// z_j - z_i from the node records: (eta_j - eta_i) + (h_i - h_j)
__device__ __forceinline__ float dz_of(float deta, float hi, float hj) { return __fadd_rn(deta, __fsub_rn(hi, hj)); }

// antidiffusive h-flux f_ij of compute_fct_matrix (update.f90:744-745),
// dd (h_j rat_ji - h_i rat_ij) + dm (h_j (1 - rat_ji) - h_i (1 - rat_ij)) with
// h rat = H* written out, in explicit roundings: k_fct and k_update must see
// the same f, bit for bit.
__device__ __forceinline__ float fct_from(float dd, float dm, float hi, float hj, const Recon& R) {
  const float a = __fsub_rn(R.Hji, R.Hij);
  const float b = __fsub_rn(__fsub_rn(hj, R.Hji), __fsub_rn(hi, R.Hij));
  return __fadd_rn(__fmul_rn(dd, a), __fmul_rn(dm, b));
}

// ---- lambda_max of the two-rarefaction bound (condlim.f90:879-981) in FP32.
// Per-node inputs are formed once and reused: the normal velocities come from
// the c.v products that mu_ij needs anyway, sqrt(g h) of both states, and
// sqrt(h) = sqrt(g h) / sqrt(g).
struct LamK {
  float g, htiny, rsg;   // rsg = 1/sqrt(g)
};
__device__ __forceinline__ LamK lam_k(float g, float htiny) { return LamK{g, htiny, rsqrtf(g)}; }

// phi (condlim.f90:960-981); one_over_h(h) and sqrt(g h) are shared by the
// two sides
__device__ __forceinline__ float phi_f(float h, float vl, float hl, float vr, float hr, float ovhl, float ovhr,
                                       float sql, float sqr, const LamK& k) {
  const float ovh = ovh_f(h, k.htiny);
  const float hg = 0.5f * k.g;
  float fl, fr;
  if (h > hl && h > hr) {              // two shocks: the usual case at h = x0 h_min
    fl = (h - hl) * sqrtf(hg * (ovh + ovhl));
    fr = (h - hr) * sqrtf(hg * (ovh + ovhr));
  } else {
    const float sgh = sqrtf(k.g * h);
    fl = (h > hl) ? (h - hl) * sqrtf(hg * (ovh + ovhl)) : 2.f * (sgh - sql);
    fr = (h > hr) ? (h - hr) * sqrtf(hg * (ovh + ovhr)) : 2.f * (sgh - sqr);
  }
  return fl + fr + vr - vl;
}

// compute_lambda_vacc (condlim.f90:879-957).  vl, vr: normal velocities;
// ovh*: one_over_h of the states; sq*: sqrt(g |h|).  Returns false where the
// reference STOPs (Delta < 0), with a relative band of 1e-5 h_min for FP32
// rounding.
__device__ __forceinline__ bool lambda_f(float hl, float hr, float vl, float vr, float ovhl, float ovhr, float sql,
                                         float sqr, const LamK& k, float* lambda) {
  const float x0 = 3.34314575f;   // (2 sqrt(2) - 1)^2
  const bool lmin = hl <= hr;
  const float hmin = lmin ? hl : hr, hmax = lmin ? hr : hl;
  bool ok = true;
  float ht;
  float fh = phi_f(x0 * hmin, vl, hl, vr, hr, ovhl, ovhr, sql, sqr, k);
  if (0.f <= fh) {
    const float s = fmaxf(fma_(2.f, sqr, fma_(2.f, sql, vl - vr)), 0.f);
    ht = fminf(x0 * hmin, fdiv(s * s, 16.f * k.g));
  } else {
    fh = phi_f(x0 * hmax, vl, hl, vr, hr, ovhl, ovhr, sql, sqr, k);
    const float sqrmin = (lmin ? sql : sqr) * k.rsg, sqrmax = (lmin ? sqr : sql) * k.rsg;
    if (0.f <= fh) {
      const float a = 0.353553391f;   // 1 / (2 sqrt(2))
      const float cc = fma_(sqrmin * (vr - vl), 0.5f * k.rsg, -(hmin * a) - sqrmin * sqrmax);
      float Delta = fma_(-4.f * a, cc, hmin);
      if (Delta < 0.f) {
        if (Delta < -1e-5f * hmin) ok = false;
        Delta = 0.f;
      }
      const float s = (sqrtf(Delta) - sqrmin) * 1.41421356f;   // / (2a)
      ht = fminf(x0 * hmax, s * s);
    } else {
      ht = sqrmin * sqrmax * fma_(1.41421356f * k.rsg, fdiv(vl - vr, sqrmin + sqrmax), 1.f);
    }
  }
  const float tl = (ht - hl) * ovhl, tr = (ht - hr) * ovhr;
  const float lbdl = fma_(-sql, sqrtf((1.f + fmaxf(tl * 0.5f, 0.f)) * (1.f + fmaxf(tl, 0.f))), vl);
  const float lbdr = fma_(sqr, sqrtf((1.f + fmaxf(tr * 0.5f, 0.f)) * (1.f + fmaxf(tr, 0.f))), vr);
  *lambda = fmaxf(fabsf(lbdl), fabsf(lbdr));
  return ok;
}

// |c_ij| lambda_max for one entry: the same operations wherever it is formed
// (k_dt_mix for stage 1, k_low_mix otherwise), so stage 1's reuse is exact.
__device__ __forceinline__ bool dlam_f(float cxe, float cye, float cvi, float cvj, float hi, float hj, float ovhi,
                                       float ovhj, float sqi, float sqj, const LamK& k, float* dl) {
  const float n2 = fma_(cxe, cxe, cye * cye);
  const float inv = rsqrtf(n2);
  float lam;
  const bool ok = lambda_f(hi, hj, cvi * inv, cvj * inv, ovhi, ovhj, sqi, sqj, k, &lam);
  *dl = (n2 * inv) * lam;
  return ok;
}

// Entry loops are processed in batches of B entries: every global load of a
// batch is issued before any of them is used, so a thread keeps B loads in
// flight (the kernels are latency-bound otherwise); the tile variants read
// neighbours from shared memory at the point of use (no registers held for
// them).  Sums keep the entry order, so every batch size gives the same
// bits.  The autotuner picks B per kernel.

// Neighbour access of the entry loops: straight from HBM by column index
// (NbGlobal), or from the block's shared-memory copy of its tile and halo
// nodes by tile-local position (NbTile, rows of 3-component systems only).
// aux is the per-node scalar the loop needs besides the node record (alpha
// in k_low, the residual in k_fct and k_update); R is R^- (k_update).
// Entry k of a row is read at row_index(base)[32 k]: a per-row pointer and a
// 32-bit offset.  self(r) is the row's own position in nq / aux / R (the
// tile variants read their own rows from shared memory too), len(r) and
// base(r) its entry count and first entry (the tile variants read them from
// shared memory, staged with the tile).
struct NbGlobal {
  static constexpr bool kGlobal = true;
  const int* col;
  const float4* nq;
  const float* aux;
  const float* R;
  const double* R64;          // FP64 R^- (precision split), or null
  __device__ __forceinline__ const int* row_index(int64_t base) const { return col + base; }
  __device__ __forceinline__ int self(int64_t r) const { return (int)r; }
  __device__ __forceinline__ int len(const Graph& G, int64_t r) const { return G.len[r]; }
  __device__ __forceinline__ int64_t base(const Graph& G, int64_t r) const { return entry_base(G, r); }
};
struct NbTile {
  static constexpr bool kGlobal = false;
  const int16_t* loc;
  const float4* nq;
  const float* aux;
  const float* R;
  const double* R64;
  int64_t t0;
  const int64_t* sp;          // slice pointers of the tile's slices
  const uint8_t* ln;          // entry counts of the tile's rows
  __device__ __forceinline__ const int16_t* row_index(int64_t base) const { return loc + base; }
  __device__ __forceinline__ int self(int64_t r) const { return (int)(r - t0); }
  __device__ __forceinline__ int len(const Graph&, int64_t r) const { return ln[r - t0]; }
  __device__ __forceinline__ int64_t base(const Graph&, int64_t r) const { return sp[(r - t0) >> 5] + (r & 31); }
};

// Shared-memory tile of one block: node records, aux and R^- (and the FP64
// R^- of the precision split) of the tile's rows (positions 0 .. T-1) and of
// its halo rows (T .. T+nh-1), then the slice pointers and entry counts of
// the tile's rows.  Layout: nq | R64 (split only) | aux | R | sp | ln.
struct TileSmem {
  float4* nq;
  double* R64;
  float* aux;
  float* R;
  int64_t* sp;
  uint8_t* ln;
};
template <bool D>
__device__ __forceinline__ TileSmem tile_smem(void* base, int cap, int T) {
  float4* nq = reinterpret_cast<float4*>(base);
  double* r64 = reinterpret_cast<double*>(nq + cap);
  float* aux = reinterpret_cast<float*>(D ? (void*)(r64 + cap) : (void*)(nq + cap));
  float* R = aux + cap;
  int64_t* sp = reinterpret_cast<int64_t*>(R + cap);   // 24 or 32 bytes per position before it: 8-byte aligned
  return TileSmem{nq, D ? r64 : nullptr, aux, R, sp, reinterpret_cast<uint8_t*>(sp + T / 32)};
}

// Copy the tile's and the halo's node data into shared memory (coalesced for
// the tile rows, ascending gathers for the halo); returns the tile start.
template <bool AUX, bool RM, bool D = false>
__device__ __forceinline__ int64_t stage_tile(const Graph& G, const TileCtl& tc, const StateMix& u,
                                              const float* __restrict__ aux, const float* __restrict__ rminus,
                                              const TileSmem& sm, const double* __restrict__ rminus64 = nullptr) {
  const int T = tc.tile_rows;
  const int64_t t0 = (int64_t)blockIdx.x * T;
  const int h0 = tc.halo_ptr[blockIdx.x], nh = tc.halo_ptr[blockIdx.x + 1] - h0;
  for (int i = threadIdx.x; i < T + nh; i += blockDim.x) {
    const int64_t row = i < T ? t0 + i : (int64_t)tc.halo_rows[h0 + i - T];
    if (row < G.n_rows) {
      sm.nq[i] = u.nq[row];
      if (AUX) sm.aux[i] = aux[row];
      if (RM) sm.R[i] = rminus[row];
      if (RM && D) sm.R64[i] = rminus64[row];
      if (i < T) sm.ln[i] = G.len[row];
    }
    // slices of the tile that exist (the last tile may be partial)
    if (i < T / 32 && t0 + 32 * (int64_t)i < G.n_rows) sm.sp[i] = G.slice_ptr[(t0 >> 5) + i];
  }
  __syncthreads();
  return t0;
}

__device__ __forceinline__ int64_t tile_end(const Graph& G, const TileCtl& tc, int64_t t0) {
  return t0 + tc.tile_rows < G.n_rows ? t0 + tc.tile_rows : G.n_rows;
}

// L2 prefetch of a byte range with the TMA unit (cp.async.bulk.prefetch):
// no registers or shared memory are held while the data comes in.  The range
// is widened to the 16-byte granule the instruction requires; every array
// passed here starts 256-byte aligned and is a multiple of 16 bytes long
// (per-row and per-entry arrays of a multiple of 32 elements), so the
// widened range stays inside it.
__device__ __forceinline__ void prefetch_l2(const void* p, int64_t bytes) {
  if (bytes <= 0) return;
  const uint64_t a = reinterpret_cast<uint64_t>(p);
  const uint64_t lo = a & ~uint64_t(15), hi = (a + (uint64_t)bytes + 15) & ~uint64_t(15);
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((unsigned)(hi - lo)) : "memory");
}

// The tile's per-entry arrays are one contiguous range (its slices are
// consecutive): one thread of the block prefetches it into L2, with the
// per-row arrays the rows read after their entry loops, while the block
// stages its nodes.  e0/e1: the tile's first and one-past-last entry.
struct TilePrefetch {
  const void* ent[3];   // per-entry arrays
  int esz[3];           // their element sizes (0: unused)
  const void* row[6];   // per-row arrays
  int rsz[6];
};
__device__ __forceinline__ void tile_prefetch(const Graph& G, const TileCtl& tc, const TilePrefetch& pf) {
  if (threadIdx.x != 0) return;
  const int64_t t0 = (int64_t)blockIdx.x * tc.tile_rows;
  const int64_t t1 = tile_end(G, tc, t0);
  const int64_t e0 = G.slice_ptr[t0 >> 5], e1 = G.slice_ptr[(t1 + 31) >> 5];
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (pf.esz[k]) prefetch_l2(static_cast<const char*>(pf.ent[k]) + e0 * pf.esz[k], (e1 - e0) * pf.esz[k]);
#pragma unroll
  for (int k = 0; k < 6; k++)
    if (pf.rsz[k]) prefetch_l2(static_cast<const char*>(pf.row[k]) + t0 * pf.rsz[k], (t1 - t0) * pf.rsz[k]);
}

// alpha_i (SOURCES/update.f90:758-781) from the stencil sums of the FP32
// depth: |num| / denom, 1 where denom <= |num|, to the 8th power.
__device__ __forceinline__ float alpha_from(float num, float denom) {
  const float a = (denom <= fabsf(num)) ? 1.0f : fdiv(fabsf(num), denom);
  const float a2 = a * a, a4 = a2 * a2;
  return a4 * a4;
}

// k_node_mix: alpha_i from the FP32 depth.
template <int B, class Nb>
__device__ __forceinline__ void node_row(int64_t r, Graph G, const InstConst* __restrict__ C,
                                                  const InstState* __restrict__ St, StateMix u,
                                                  float* __restrict__ alpha_out, const Nb& nb) {
  const int L = nb.len(G, r);
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  if (St[b].done) return;
  const InstConst& c = C[b];
  const float* hs = reinterpret_cast<const float*>(nb.nq);
  const int me = nb.self(r);
  const float h = hs[4 * me];
  float alpha = 1.0f;
  if (c.alpha_limit && !(h <= c.htinyf)) {
    const auto ip = nb.row_index(nb.base(G, r));
    float num = 0.0f, denom = 0.0f;
    for (int k0 = 0; k0 < L; k0 += B) {
      int j[B];
#pragma unroll
      for (int q = 0; q < B; q++) j[q] = (k0 + q < L) ? (int)ip[32 * (k0 + q)] : me;
      float hj[B];
#pragma unroll
      for (int q = 0; q < B; q++) hj[q] = hs[4 * (int64_t)j[q]];
#pragma unroll
      for (int q = 0; q < B; q++)
        if (k0 + q < L) {
          num += hj[q] - h;
          denom += fabsf(hj[q] - h);
        }
    }
    alpha = alpha_from(num, denom);
  }
  alpha_out[r] = alpha;
}

template <int B>
__global__ void __launch_bounds__(256) k_node_mix(Graph G, const InstConst* __restrict__ C,
                                                  const InstState* __restrict__ St, StateMix u,
                                                  float* __restrict__ alpha_out) {
  pdl_trigger();
  pdl_wait();
  const NbGlobal nb{G.col, u.nq, nullptr, nullptr, nullptr};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.n_rows; r += (int64_t)gridDim.x * blockDim.x)
    node_row<B>(r, G, C, St, u, alpha_out, nb);
}

template <int B>
__global__ void __launch_bounds__(256) k_node_tile(Graph G, const InstConst* __restrict__ C,
                                                   const InstState* __restrict__ St, StateMix u,
                                                   float* __restrict__ alpha_out, TileCtl tc) {
  extern __shared__ float4 tile_mem[];
  pdl_trigger();
  tile_prefetch(G, tc, TilePrefetch{{tc.loc, nullptr, nullptr}, {2, 0, 0}, {}, {}});
  pdl_wait();
  const TileSmem sm = tile_smem<false>(tile_mem, tc.tile_rows + tc.halo_cap, tc.tile_rows);
  const int64_t t0 = stage_tile<false, false>(G, tc, u, nullptr, nullptr, sm);
  const int64_t t1 = tile_end(G, tc, t0);
  const NbTile nb{tc.loc, sm.nq, nullptr, nullptr, nullptr, t0, sm.sp, sm.ln};
  for (int64_t r = t0 + threadIdx.x; r < t1; r += blockDim.x) node_row<B>(r, G, C, St, u, alpha_out, nb);
}

struct NodeF {   // FP32 view of one node used by the edge loop
  float h, q1, q2, eta, ovh, v1, v2;
};

__device__ __forceinline__ NodeF node_from(const float4 a, float htiny) {
  NodeF n;
  n.h = a.x; n.q1 = a.y; n.q2 = a.z; n.eta = a.w;
  n.ovh = ovh_f(n.h, htiny);
  n.v1 = n.q1 * n.ovh;
  n.v2 = n.q2 * n.ovh;
  return n;
}

// 0.5 (g h^2 + v1 q1 + v2 q2): the entropy of the reference's entropy_residual
__device__ __forceinline__ float entropy_f(float g, float h, float v1, float q1, float v2, float q2) {
  return 0.5f * fma_(v2, q2, fma_(v1, q1, (g * h) * h));
}

__device__ __forceinline__ float sgn_pressure(float lambda_sgn, float g, float m, float h, float heta) {
  const float pc = fdiv(lambda_sgn * g, 3.0f * sqrtf(m));
  const float x = fdiv(heta, h * h);
  return pc * h * h * h * (2.f + 4.f * x * x * x - 6.f * x * x * x * x);   // mSGN_RHS pTilde (update.f90:522)
}

// k_low_mix: one pass over the row's entries computing d_ij (lambda_max),
// mu_ij, their alpha scaling, the low-order RHS (smb_2_roundoff), the
// Galerkin RHS (smb_2) and the entropy stencil max/min, then the low-order
// state and the entropy residual (SOURCES/update.f90:180-210, 291-364,
// 554-682, 750-799, 825-878).  Each neighbour is loaded once, and c.v_j is
// formed once and shared by mu_ij, lambda_max and the Galerkin flux.  The
// diagonal entry only enters through terms that vanish identically
// (u_i rat_ii - u_i rat_ii) and the Galerkin boundary term -c_ii.v_i.
//
// The smb_2_roundoff mass row h (1 + a fix) + a rk_1 is formed as
// h + a (P - N - c_ii.v_i h) with P = sum (mu - c.v_j) h_j + (d - mu) H*_ji
// (every term >= 0) and N = sum mu h_i + (d - mu) H*_ij [h_i > htiny]
// (N <= h_i sum d, so a N <= CFL h_i): the reference's fix h + rk_1 with
// rat_ij h_i = H*_ij.  At rest the two sums add equal terms in the same
// order, so P - N is exactly 0.
template <int B, bool LAMIN, int MINB, bool D, class Nb>
__device__ __forceinline__ void low_row(int64_t r, Graph G, const InstConst* __restrict__ C,
                                                       const InstState* __restrict__ St, StateMix u,
                                                       const float* __restrict__ alpha, float2* __restrict__ dmu,
                                                       WorkMix w, float* __restrict__ res, unsigned* __restrict__ err,
                                                       const Nb& nb) {
  const int L = nb.len(G, r);
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const InstState& st = St[b];
  if (st.done) return;
  const InstConst& c = C[b];
  const int S = Nb::kGlobal ? c.S : 3;         // tiles hold 3-component systems only
  const bool sgn = Nb::kGlobal && c.type_test == 13;
  const bool galerkin = c.visc == VISC_GALERKIN;   // every d_ij, mu_ij = 0 (update.f90:155-158)
  const float vis = galerkin ? 0.f : 1.f;
  const float g = c.gf, htiny = c.htinyf, dtf = st.dtf;
  const LamK lk = lam_k(g, htiny);
  // the low-order momenta: smb_2_roundoff's htiny tests, or smb_2's h <= 0
  // tests (rat = 0 already where h <= 0) when the step is not roundoff-fixed
  const bool roundoff = c.roundoff_fix && !galerkin;
  const float hthr = roundoff ? htiny : 0.f;
  const int64_t base = nb.base(G, r);
  const int me = nb.self(r);
  const auto ip = nb.row_index(base);
  const float2* cp = G.cf + base;
  const float* dlp = w.dlam + base;
  float2* dmp = dmu + base;
  const NodeF ni = node_from(nb.nq[me], htiny);
  const float sqi = sqrtf(g * fabsf(ni.h));
  const float v2i_flux = sgn ? 0.f : ni.v2;          // flux() zeroes velocity(2) for type 13
  const float ai = nb.aux[me];
  const float m = G.lumpedf[r];
  const float ghi = g * ni.h;
  const bool wet_i = !(ni.h <= hthr);
  float ui3 = 0.f, ui4 = 0.f;
  if (S == 5) { ui3 = u.q3[r]; ui4 = u.q4[r]; }
  const float invhi = inv_pos(ni.h);
  bool delta_bad = false;

  float P = 0.f, N = 0.f;                                          // smb_2_roundoff mass row
  float rk1 = 0.f, rk2_ = 0.f, rk3 = 0.f, rk4 = 0.f;               // smb_2_roundoff momenta
  float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f, g4 = 0.f;          // smb_2
  const float Ei = entropy_f(g, ni.h, ni.v1, ni.q1, v2i_flux, ni.q2);
  float emax = Ei, emin = Ei;
  float ptx = 0.f, pty = 0.f;
  // diagonal: Galerkin boundary term -c_ii.v_i (fix_roundoff / smb_2);
  // its viscous and topography terms vanish
  const float cxd = G.cxiif[r], cyd = G.cyiif[r];
  const float cvd = dotc(cxd, cyd, ni.v1, v2i_flux);
  g0 = -cvd * ni.h;
  rk1 = -cvd * ni.q1; rk2_ = -cvd * ni.q2;
  g1 = rk1; g2 = rk2_;
  if (S == 5) { rk3 = -cvd * ui3; rk4 = -cvd * ui4; g3 = rk3; g4 = rk4; }
  if (sgn) {
    const float pt = sgn_pressure(c.lambda_sgnf, g, m, ni.h, ui3);
    ptx = -pt * cxd;
    pty = -pt * cyd;
  }
  for (int k0 = 0; k0 < L; k0 += B) {
   int jb[B];
   float cxb[B], cyb[B], dlb[B];
#pragma unroll
   for (int q = 0; q < B; q++) {
     if (k0 + q < L) {
       const int off = 32 * (k0 + q);
       const float2 cc = cp[off];
       jb[q] = ip[off]; cxb[q] = cc.x; cyb[q] = cc.y;
       dlb[q] = LAMIN ? dlp[off] : 0.f;
     } else {
       jb[q] = me; cxb[q] = 0.f; cyb[q] = 0.f; dlb[q] = 0.f;
     }
   }
   float4 nqb[Nb::kGlobal ? B : 1];
   float alb[Nb::kGlobal ? B : 1];
   if constexpr (Nb::kGlobal) {
#pragma unroll
     for (int q = 0; q < B; q++) { nqb[q] = nb.nq[jb[q]]; alb[q] = nb.aux[jb[q]]; }
   }
#pragma unroll
   for (int q = 0; q < B; q++) {
    if (k0 + q >= L) break;
    const int off = 32 * (k0 + q);
    const float cxe = cxb[q], cye = cyb[q];
    const int j = jb[q];
    const NodeF nj = node_from(Nb::kGlobal ? nqb[q] : nb.nq[j], htiny);
    const float alj = Nb::kGlobal ? alb[q] : nb.aux[j];
    // --- viscosities: compute_dij, compute_muij, MAX, alpha_limit
    const float cvi = dotc(cxe, cye, ni.v1, ni.v2);                   // c.v_i (compute_muij)
    const float cvj = dotc(cxe, cye, nj.v1, nj.v2);                   // c.v_j
    float dlam;                                                       // |c_ij| lambda_max
    if (LAMIN) {
      dlam = dlb[q];                                                  // from k_dt_mix on this state
    } else if (!dlam_f(cxe, cye, cvi, cvj, ni.h, nj.h, ni.ovh, nj.ovh, sqi, sqrtf(g * fabsf(nj.h)), lk, &dlam)) {
      delta_bad = true;
    }
    float mu = fmaxf(fmaxf(-cvi, 0.f), fmaxf(cvj, 0.f));
    float d = fmaxf(dlam, mu);
    const float s = (c.alpha_limit ? fmaxf(ai, alj) : 1.f) * vis;
    d *= s;
    mu *= s;
    dmp[off] = make_float2(d, mu);
    // --- entropy stencil
    const float v2j_flux = sgn ? 0.f : nj.v2;
    const float Ej = entropy_f(g, nj.h, nj.v1, nj.q1, v2j_flux, nj.q2);
    emax = fmaxf(emax, Ej);
    emin = fminf(emin, Ej);
    // --- hydrostatic reconstruction from the free surface
    const float deta = __fsub_rn(nj.eta, ni.eta);
    const float dz = dz_of(deta, ni.h, nj.h);
    const Recon R = recon(ni.h, nj.h, dz);
    const float rij = rat_of(R.Hij, ni.h, dz <= 0.f, invhi);          // h <= 0 tests (smb_2)
    const float rji = rat_of(R.Hji, nj.h, dz >= 0.f, inv_pos(nj.h));
    const bool wet_j = !(nj.h <= hthr);
    const float rijt = wet_i ? rij : 0.f;                             // h <= htiny tests
    const float rjit = wet_j ? rji : 0.f;
    const float cvj_flux = sgn ? dotc(cxe, cye, nj.v1, 0.f) : cvj;   // c.velocity_j of flux()
    const float topo = ghi * deta;                                    // g h_i (eta_j - eta_i)
    const float dmu = d - mu;
    // --- smb_2_roundoff mass row: P - N
    P = fma_(dmu, R.Hji, fma_(mu - cvj_flux, nj.h, P));
    N = fma_(dmu, wet_i ? R.Hij : 0.f, fma_(mu, ni.h, N));
    // --- smb_2 mass row and the momenta of both RHS, written as
    // -c.v_j u_j + mu (u_j - u_i) + (d - mu) (u_j rat_ji - u_i rat_ij), which
    // equals d (u_j rat_ji - u_i rat_ij) + mu (u_j (1 - rat_ji) - u_i (1 - rat_ij))
    g0 = fma_(dmu, __fsub_rn(R.Hji, R.Hij), fma_(mu, nj.h - ni.h, fma_(-cvj_flux, nj.h, g0)));
    const float A1 = fma_(mu, nj.q1 - ni.q1, -cvj_flux * nj.q1);
    const float A2 = fma_(mu, nj.q2 - ni.q2, -cvj_flux * nj.q2);
    const float T1 = fma_(dmu, fma_(nj.q1, rji, -ni.q1 * rij), A1);
    const float T2 = fma_(dmu, fma_(nj.q2, rji, -ni.q2 * rij), A2);
    g1 = fma_(-topo, cxe, g1 + T1);
    g2 = fma_(-topo, cye, g2 + T2);
    if (rijt == rij && rjit == rji) {                                 // both wet: same terms
      rk1 += T1;
      rk2_ += T2;
    } else {
      rk1 += fma_(dmu, fma_(nj.q1, rjit, -ni.q1 * rijt), A1);
      rk2_ += fma_(dmu, fma_(nj.q2, rjit, -ni.q2 * rijt), A2);
    }
    rk1 = fma_(-topo, cxe, rk1);
    rk2_ = fma_(-topo, cye, rk2_);
    if (Nb::kGlobal && S == 5) {
      const float uj3 = u.q3[j], uj4 = u.q4[j];
      const float A3 = fma_(mu, uj3 - ui3, -cvj_flux * uj3);
      const float A4 = fma_(mu, uj4 - ui4, -cvj_flux * uj4);
      rk3 += fma_(dmu, fma_(uj3, rjit, -ui3 * rijt), A3);
      rk4 += fma_(dmu, fma_(uj4, rjit, -ui4 * rijt), A4);
      g3 += fma_(dmu, fma_(uj3, rji, -ui3 * rij), A3);
      g4 += fma_(dmu, fma_(uj4, rji, -ui4 * rij), A4);
      if (sgn) {
        const float pt = sgn_pressure(c.lambda_sgnf, g, G.lumpedf[j], nj.h, uj3);
        ptx = fma_(-pt, cxe, ptx);
        pty = fma_(-pt, cye, pty);
      }
    }
   }
  }
  // source terms (update.f90:425-551)
  if (c.type_test == 9 || c.type_test == 10) {
    const float hstar = __powf(fmaxf(ni.h, htiny), 4.0f / 3.0f);
    const float vel = c.fricf * sqrtf(fma_(ni.v1, ni.v1, ni.v2 * ni.v2));
    const float hloc = vel * dtf;
    const float coef = fdiv(m * vel * 2.f, hstar + fmaxf(hstar, hloc));
    rk1 = fma_(-coef, ni.q1, rk1); rk2_ = fma_(-coef, ni.q2, rk2_);
    g1 = fma_(-coef, ni.q1, g1); g2 = fma_(-coef, ni.q2, g2);
  } else if (c.type_test == 11) {
    const float k = m * 0.2f;
    rk1 = fma_(-k, ni.q1, rk1); rk2_ = fma_(-k, ni.q2, rk2_);
    g1 = fma_(-k, ni.q1, g1); g2 = fma_(-k, ni.q2, g2);
  } else if (c.type_test == 12) {
    const float a1 = m * 2.0f * ni.q2, a2 = m * 2.0f * ni.q1;
    rk1 += a1; rk2_ -= a2; g1 += a1; g2 -= a2;
  } else if (sgn) {
    const float pc = fdiv(c.lambda_sgnf * g, 3.0f * sqrtf(m));
    const float t = fdiv(ui3, ni.h);
    const float x = fdiv(ui3, ni.h * ni.h);
    const float s_i = 3.f * pc * t * t * 12.f * (x - 1.f);
    rk1 += ptx; rk2_ += pty; g1 += ptx; g2 += pty;
    rk3 = fma_(m, ui4, rk3); rk4 = fma_(-m, s_i, rk4);
    g3 = fma_(m, ui4, g3); g4 = fma_(-m, s_i, g4);
  }
  // low-order state: double-float depth plus an FP32 increment, or (precision
  // split) the FP64 update h + (dt/m) (P - N - c_ii.v_i h) of the FP32 sums
  const float invm = G.inv_lumpedf[r];
  const float a = dtf * invm;
  const float2 h = u.h[r];
  // ('entropy_visc' without the roundoff fix keeps h + dt rk unclipped: its
  // k_update adds the high-order correction before MAX(., 0))
  const bool clip = !(c.visc == VISC_ENTROPY);
  if (D) {
    const double hd = df_to_double(h), ad = st.dt * G.inv_lumped[r];
    double hL;
    if (roundoff) {
      hL = fma(ad, fma(-(double)cvd, (double)ni.h, (double)P - (double)N), hd);
    } else {
      hL = fma(ad, (double)g0, hd);
      if (clip && hL < 0.0) hL = 0.0;
    }
    w.hL64[r] = hL;
  } else {
    float2 hL;
    if (roundoff) {
      hL = df_add_f(h, a * fma_(-cvd, ni.h, P - N));   // h + a (fix h + rk_1), a N <= CFL h
    } else {                                            // smb_2 and MAX(h + dt rk, 0)
      hL = df_add_f(h, a * g0);
      if (clip && hL.x < 0.f) hL = make_float2(0.f, 0.f);
    }
    w.hL[r] = hL;
  }
  w.qL[r] = make_float2(fma_(dtf, rk1 * invm, ni.q1), fma_(dtf, rk2_ * invm, ni.q2));
  if (S == 5) { w.q3L[r] = fma_(dtf, rk3 * invm, ui3); w.q4L[r] = fma_(dtf, rk4 * invm, ui4); }
  // entropy residual (update.f90:838-868), rescale once per node
  const float un0 = fma_(dtf, g0 * invm, ni.h);
  const float un1 = fma_(dtf, g1 * invm, ni.q1);
  const float un2 = fma_(dtf, g2 * invm, ni.q2);
  const float on = ovh_f(un0, htiny);
  const float En = entropy_f(g, un0, un1 * on, un1, un2 * on, un2);
  const float Ep0 = fma_(-0.5f * v2i_flux, v2i_flux, fma_(-0.5f * ni.v1, ni.v1, g * ni.h));
  float rs = m * (En - Ei) * st.inv_dtf;
  rs -= fma_(g2, v2i_flux, fma_(g1, ni.v1, g0 * Ep0));
  const float rescale = fma_(0.5f, fabsf(emax - emin), c.rescale_floorf);
  res[r] = fdiv(fabsf(rs), rescale);
  if (delta_bad) atomicOr(err, ERRB_DELTA);
}

template <int B, bool LAMIN, int MINB, bool D>
__global__ void __launch_bounds__(256, MINB) k_low_mix(Graph G, const InstConst* __restrict__ C,
                                                       const InstState* __restrict__ St, StateMix u,
                                                       const float* __restrict__ alpha, float2* __restrict__ dmu,
                                                       WorkMix w, float* __restrict__ res, unsigned* __restrict__ err) {
  pdl_trigger();
  pdl_wait();
  const NbGlobal nb{G.col, u.nq, alpha, nullptr, nullptr};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.n_rows; r += (int64_t)gridDim.x * blockDim.x)
    low_row<B, LAMIN, MINB, D>(r, G, C, St, u, alpha, dmu, w, res, err, nb);
}

template <int B, bool LAMIN, int MINB, bool D>
__global__ void __launch_bounds__(256, MINB) k_low_tile(Graph G, const InstConst* __restrict__ C,
                                                        const InstState* __restrict__ St, StateMix u,
                                                        const float* __restrict__ alpha, float2* __restrict__ dmu,
                                                        WorkMix w, float* __restrict__ res, unsigned* __restrict__ err,
                                                        TileCtl tc) {
  extern __shared__ float4 tile_mem[];
  pdl_trigger();
  tile_prefetch(G, tc, TilePrefetch{{tc.loc, G.cf, nullptr}, {2, 8, 0},
                                    {G.lumpedf, G.inv_lumpedf, G.cxiif, G.cyiif, nullptr, nullptr}, {4, 4, 4, 4, 0, 0}});
  pdl_wait();
  tile_prefetch(G, tc, TilePrefetch{{w.dlam, nullptr, nullptr}, {LAMIN ? 4 : 0, 0, 0}, {u.h}, {8}});
  const TileSmem sm = tile_smem<false>(tile_mem, tc.tile_rows + tc.halo_cap, tc.tile_rows);
  const int64_t t0 = stage_tile<true, false>(G, tc, u, alpha, nullptr, sm);
  const int64_t t1 = tile_end(G, tc, t0);
  const NbTile nb{tc.loc, sm.nq, sm.aux, nullptr, nullptr, t0, sm.sp, sm.ln};
  for (int64_t r = t0 + threadIdx.x; r < t1; r += blockDim.x)
    low_row<B, LAMIN, MINB, D>(r, G, C, St, u, alpha, dmu, w, res, err, nb);
}

// 'viscous' with viscous_type 'type1' (update.f90:189-201, smb_1 :366-423):
// d_ij as in low_row (lambda_max, MAX with mu_ij, alpha scaling), then the
// RHS of smb_1 -- the centred flux -c.(v_j u_j rat_ji + v_i u_i rat_ij),
// d_ij (u_j rat_ji - u_i rat_ij) and the pressure term
// -g/2 (H*_ji^2 - H*_ij^2) c_ij, with the h <= htiny tests -- and the
// low-order state u + dt rk / m (no clipping, as the reference).  Rows of
// other instances of a batch run low_row.  3-component systems only.
template <bool D>
__device__ __forceinline__ void low_row_type1(int64_t r, const Graph& G, const InstConst& c, const InstState& st,
                                              const StateMix& u, const float* __restrict__ alpha,
                                              float2* __restrict__ dmu, const WorkMix& w, unsigned* __restrict__ err) {
  const NbGlobal nb{G.col, u.nq, alpha, nullptr, nullptr};
  const int L = nb.len(G, r);
  const float g = c.gf, htiny = c.htinyf, dtf = st.dtf;
  const LamK lk = lam_k(g, htiny);
  const int64_t base = nb.base(G, r);
  const int me = nb.self(r);
  const int* ip = nb.row_index(base);
  const float2* cp = G.cf + base;
  float2* dmp = dmu + base;
  const NodeF ni = node_from(nb.nq[me], htiny);
  const float sqi = sqrtf(g * fabsf(ni.h));
  const float ai = nb.aux[me];
  const float invhi = inv_pos(ni.h);
  const bool wet_i = !(ni.h <= htiny);
  // diagonal: the centred flux -c_ii.v_i u_i (rat_ii = 1 for h_i > htiny)
  const float cxd = G.cxiif[r], cyd = G.cyiif[r];
  const float cvd = dotc(cxd, cyd, ni.v1, ni.v2);
  const float rdd = wet_i ? 1.f : 0.f;
  float rk0 = -2.f * cvd * ni.h * rdd, rk1 = -2.f * cvd * ni.q1 * rdd, rk2 = -2.f * cvd * ni.q2 * rdd;
  bool delta_bad = false;
  for (int k = 0; k < L; k++) {
    const int off = 32 * k;
    const float2 cc = cp[off];
    const int j = ip[off];
    const NodeF nj = node_from(nb.nq[j], htiny);
    const float cxe = cc.x, cye = cc.y;
    const float cvi = dotc(cxe, cye, ni.v1, ni.v2), cvj = dotc(cxe, cye, nj.v1, nj.v2);
    float dlam;
    if (!dlam_f(cxe, cye, cvi, cvj, ni.h, nj.h, ni.ovh, nj.ovh, sqi, sqrtf(g * fabsf(nj.h)), lk, &dlam))
      delta_bad = true;
    float mu = fmaxf(fmaxf(-cvi, 0.f), fmaxf(cvj, 0.f));
    float d = fmaxf(dlam, mu);
    const float s = c.alpha_limit ? fmaxf(ai, nb.aux[j]) : 1.f;
    d *= s;
    mu *= s;
    dmp[off] = make_float2(d, mu);
    const float deta = __fsub_rn(nj.eta, ni.eta);
    const float dz = dz_of(deta, ni.h, nj.h);
    const Recon R = recon(ni.h, nj.h, dz);
    const float rij = wet_i ? rat_of(R.Hij, ni.h, dz <= 0.f, invhi) : 0.f;
    const float rji = !(nj.h <= htiny) ? rat_of(R.Hji, nj.h, dz >= 0.f, inv_pos(nj.h)) : 0.f;
    const float ai_ = cvi * rij, aj = cvj * rji;          // c.v_i rat_ij, c.v_j rat_ji
    rk0 += fma_(d, fma_(nj.h, rji, -ni.h * rij), -fma_(aj, nj.h, ai_ * ni.h));
    rk1 += fma_(d, fma_(nj.q1, rji, -ni.q1 * rij), -fma_(aj, nj.q1, ai_ * ni.q1));
    rk2 += fma_(d, fma_(nj.q2, rji, -ni.q2 * rij), -fma_(aj, nj.q2, ai_ * ni.q2));
    const float pr = 0.5f * g * fma_(R.Hji, R.Hji, -R.Hij * R.Hij);
    rk1 = fma_(-pr, cxe, rk1);
    rk2 = fma_(-pr, cye, rk2);
  }
  // source terms (update.f90:425-486)
  const float m = G.lumpedf[r];
  if (c.type_test == 9 || c.type_test == 10) {
    const float hstar = __powf(fmaxf(ni.h, htiny), 4.0f / 3.0f);
    const float vel = c.fricf * sqrtf(fma_(ni.v1, ni.v1, ni.v2 * ni.v2));
    const float coef = fdiv(m * vel * 2.f, hstar + fmaxf(hstar, vel * dtf));
    rk1 = fma_(-coef, ni.q1, rk1); rk2 = fma_(-coef, ni.q2, rk2);
  } else if (c.type_test == 11) {
    rk1 = fma_(-m * 0.2f, ni.q1, rk1); rk2 = fma_(-m * 0.2f, ni.q2, rk2);
  } else if (c.type_test == 12) {
    rk1 += m * 2.0f * ni.q2; rk2 -= m * 2.0f * ni.q1;
  }
  const float invm = G.inv_lumpedf[r];
  if (D) w.hL64[r] = fma(st.dt * G.inv_lumped[r], (double)rk0, df_to_double(u.h[r]));
  else w.hL[r] = df_add_f(u.h[r], (dtf * invm) * rk0);
  w.qL[r] = make_float2(fma_(dtf, rk1 * invm, ni.q1), fma_(dtf, rk2 * invm, ni.q2));
  if (delta_bad) atomicOr(err, ERRB_DELTA);
}

template <bool D>
__global__ void __launch_bounds__(256) k_low_type1(Graph G, const InstConst* __restrict__ C,
                                                   const InstState* __restrict__ St, StateMix u,
                                                   const float* __restrict__ alpha, float2* __restrict__ dmu, WorkMix w,
                                                   float* __restrict__ res, unsigned* __restrict__ err) {
  pdl_trigger();
  pdl_wait();
  const NbGlobal nb{G.col, u.nq, alpha, nullptr, nullptr};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.n_rows; r += (int64_t)gridDim.x * blockDim.x) {
    if (G.len[r] == 0) continue;
    const int b = G.slice_inst[r >> 5];
    if (St[b].done) continue;
    const InstConst& c = C[b];
    if (c.viscous_type == 1 && c.visc == VISC_VISCOUS) low_row_type1<D>(r, G, c, St[b], u, alpha, dmu, w, err);
    else low_row<1, false, 3, D>(r, G, C, St, u, alpha, dmu, w, res, err, nb);
  }
}

// Limiter margin: (1 - 2^-18) Q^-.  Between the limiter and the depth update
// the negative part of sum_j l_ij f_ij passes through at most ~12 FP32
// roundings (h^L to FP32, m and dt and their reciprocals, two products here,
// the quotient, R P, the row sum and dt/m times it in k_update_mix), each at
// most 2^-24 relative, so (1 - 2^-18)(1 + 2^-24)^12 < 1 and the update never
// removes more than h^L from a node.
constexpr float kLimiterShrink = 1.0f - 3.814697265625e-6f;

// f_ij with the high-order viscosities MIN(d, res_ij), MIN(mu, res_ij)
// (update.f90:233-239, 721-748) for one entry; k_fct and k_update share it.
__device__ __forceinline__ float fct_entry(float d0, float m0, float rij, float hi, float hj, const Recon& R) {
  return fct_from(fminf(d0, rij) - d0, fminf(m0, rij) - m0, hi, hj, R);
}

// k_fct_mix: f_ij and the limiter R^-_i (fct.f90:15-30): P^- = sum f^- - 1e-15,
// Q^- = -m h^L/dt, R^- = min(Q^-/P^-, 1), 0 where m h^L/dt <= htiny.
template <int B, bool D, class Nb>
__device__ __forceinline__ void fct_row(int64_t r, Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St, StateMix u,
                          const float2* __restrict__ dmu, WorkMix w, const float* __restrict__ res,
                          unsigned* __restrict__ err, const Nb& nb) {
  const int L = nb.len(G, r);
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const InstState& st = St[b];
  if (st.done) return;
  const InstConst& c = C[b];
  if (c.visc != VISC_FCT) return;
  const int64_t base = nb.base(G, r);
  const int me = nb.self(r);
  const auto ip = nb.row_index(base);
  const float2* dmp = dmu + base;
  const float4 ni = nb.nq[me];
  const float hi = ni.x, etai = ni.w, resi = nb.aux[me];
  float neg = 0.f;                       // f_ii = 0 adds nothing
  for (int k0 = 0; k0 < L; k0 += B) {
    int jb[B];
    float d0b[B], m0b[B];
#pragma unroll
    for (int q = 0; q < B; q++) {
      if (k0 + q < L) {
        const int off = 32 * (k0 + q);
        jb[q] = ip[off]; const float2 v = dmp[off]; d0b[q] = v.x; m0b[q] = v.y;
      } else {
        jb[q] = me; d0b[q] = 0.f; m0b[q] = 0.f;
      }
    }
    float4 njb[Nb::kGlobal ? B : 1];
    float rsb[Nb::kGlobal ? B : 1];
    if constexpr (Nb::kGlobal) {
#pragma unroll
      for (int q = 0; q < B; q++) { njb[q] = nb.nq[jb[q]]; rsb[q] = nb.aux[jb[q]]; }
    }
#pragma unroll
    for (int q = 0; q < B; q++) {
      if (k0 + q >= L) break;
      const float4 nj = Nb::kGlobal ? njb[q] : nb.nq[jb[q]];
      const float rsj = Nb::kGlobal ? rsb[q] : nb.aux[jb[q]];
      const Recon R = recon(hi, nj.x, dz_of(__fsub_rn(nj.w, etai), hi, nj.x));
      const float f = fct_entry(d0b[q], m0b[q], fmaxf(resi, rsj), hi, nj.x, R);
      if (f < 0.f) neg = __fadd_rn(neg, f);
    }
  }
  if (D) {   // precision split: Q^-, P^-, R^- and the dry test in FP64, as the reference
    const double hL = w.hL64[r];
    if (hL < 0.0) atomicOr(err, ERRB_NEG_H);
    const double scaled = (G.lumped[r] / st.dt) * hL;                           // (lumped/dt) h^L
    double R = 0.0;
    if (!(scaled <= c.htiny)) {
      const double Pm = -1.e-15 + (double)neg;
      R = fmin((0.0 - scaled) / Pm, 1.0);
    }
    w.rminus64[r] = R;
    w.rminus[r] = (float)R;
    return;
  }
  const float2 hL = w.hL[r];
  if (hL.x < 0.f) atomicOr(err, ERRB_NEG_H);
  const float scaled = __fmul_rn(__fmul_rn(hL.x, G.lumpedf[r]), st.inv_dtf);   // m h^L / dt
  bool dry = scaled <= c.htinyf;
  if (fabsf(scaled - c.htinyf) <= 1e-5f * c.htinyf)                           // decide in FP64 near htiny
    dry = G.lumped[r] * st.inv_dt * df_to_double(hL) <= c.htiny;
  float R = 0.f;
  if (!dry) {
    const float mP = __fsub_rn(1.e-15f, neg);                                  // -P^- > 0
    const float Q = __fmul_rn(scaled, kLimiterShrink);                         // -Q^- >= 0
    R = (Q >= mP) ? 1.f : __fdiv_rn(Q, mP);
  }
  w.rminus[r] = R;
}

template <int B, bool D>
__global__ void __launch_bounds__(256) k_fct_mix(Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                                                 StateMix u, const float2* __restrict__ dmu, WorkMix w,
                                                 const float* __restrict__ res, unsigned* __restrict__ err) {
  pdl_trigger();
  pdl_wait();
  const NbGlobal nb{G.col, u.nq, res, nullptr, nullptr};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.n_rows; r += (int64_t)gridDim.x * blockDim.x)
    fct_row<B, D>(r, G, C, St, u, dmu, w, res, err, nb);
}

template <int B, bool D>
__global__ void __launch_bounds__(256) k_fct_tile(Graph G, const InstConst* __restrict__ C,
                                                  const InstState* __restrict__ St, StateMix u,
                                                  const float2* __restrict__ dmu, WorkMix w,
                                                  const float* __restrict__ res, unsigned* __restrict__ err, TileCtl tc) {
  extern __shared__ float4 tile_mem[];
  pdl_trigger();
  tile_prefetch(G, tc, TilePrefetch{{tc.loc, nullptr, nullptr}, {2, 0, 0}, {G.lumpedf}, {4}});
  pdl_wait();
  tile_prefetch(G, tc, TilePrefetch{{dmu, nullptr, nullptr}, {8, 0, 0},
                                    {D ? (const void*)w.hL64 : (const void*)w.hL}, {8}});
  const TileSmem sm = tile_smem<false>(tile_mem, tc.tile_rows + tc.halo_cap, tc.tile_rows);
  const int64_t t0 = stage_tile<true, false>(G, tc, u, res, nullptr, sm);
  const int64_t t1 = tile_end(G, tc, t0);
  const NbTile nb{tc.loc, sm.nq, sm.aux, nullptr, nullptr, t0, sm.sp, sm.ln};
  for (int64_t r = t0 + threadIdx.x; r < t1; r += blockDim.x) fct_row<B, D>(r, G, C, St, u, dmu, w, res, err, nb);
}

// End of a stage for one row: non-finite check, the SSP-RK combination and
// bdy of the time loop (main.f90:77-90) when rk_stage > 0, and the store of
// the double-float depth and the node record with its free surface.
__device__ __forceinline__ void finish_mix(const Graph& G, const InstConst& c, const InstState& st, int64_t r, int S,
                                           float2 hn, float q1, float q2, float q3, float q4, int rk_stage,
                                           const StateMix& u0, const StateMix& out, unsigned* err) {
  if (!(hn.x == hn.x) || !(q1 == q1) || !(q2 == q2)) atomicOr(err, ERRB_NAN);
  if (rk_stage >= 2) {
    const float4 a0 = u0.nq[r];
    const float2 h0 = u0.h[r];
    if (rk_stage == 2) {
      hn = df_scale(df_add(df_mul_f(h0, 3.f), hn), 0.25f);
      q1 = fma_(3.f, a0.y, q1) * 0.25f;
      q2 = fma_(3.f, a0.z, q2) * 0.25f;
      if (S == 5) { q3 = fma_(3.f, u0.q3[r], q3) * 0.25f; q4 = fma_(3.f, u0.q4[r], q4) * 0.25f; }
    } else {
      hn = df_div3(df_add(h0, df_scale(hn, 2.f)));
      q1 = fma_(2.f, q1, a0.y) * (1.f / 3.f);
      q2 = fma_(2.f, q2, a0.z) * (1.f / 3.f);
      if (S == 5) { q3 = fma_(2.f, q3, u0.q3[r]) * (1.f / 3.f); q4 = fma_(2.f, q4, u0.q4[r]) * (1.f / 3.f); }
    }
  }
  if (rk_stage >= 1 && G.dir_mask) {
    const unsigned msk = G.dir_mask[r];
    if (msk) {
      if (msk & 1u) hn = df_from_double(dirichlet_value(G, c, st, rk_stage, 0, r));
      if (msk & 2u) q1 = (float)dirichlet_value(G, c, st, rk_stage, 1, r);
      if (msk & 4u) q2 = (float)dirichlet_value(G, c, st, rk_stage, 2, r);
      if (S == 5 && (msk & 8u)) q3 = (float)G.dir_val[3 * G.n_rows + r];
      if (S == 5 && (msk & 16u)) q4 = (float)G.dir_val[4 * G.n_rows + r];
    }
  }
  out.h[r] = hn;
  out.nq[r] = make_float4(shadow_df(hn, c), q1, q2, eta_of(hn, G.bathdf[r]));
  if (S == 5) { out.q3[r] = q3; out.q4[r] = q4; }
}

// k_update_mix: limited antidiffusion (update.f90:276-282, apply_viscosity
// :684-718), RK combination and Dirichlet data (main.f90:77-90).  The h-row
// sum is R^-_i P_i plus sum_{f_ij >= 0} R^-_j f_ij, with P_i = sum_{f_ij < 0}
// f_ij formed in the entry order of k_fct_mix (the same value, bit for bit,
// as the one the limiter saw).
//
// 'entropy_visc' (update.f90:241-269) recomputes the RHS with the
// high-order viscosities d^H = MIN(d, res_ij), mu^H = MIN(mu, res_ij).  That
// RHS is linear in (d, mu), so u^H = u^L + (dt/m) sum_j [dm (u_j - u_i) +
// (dd - dm) (u_j rat_ji - u_i rat_ij)] with dd = d^H - d, dm = mu^H - mu:
// this kernel's antidiffusion with every l_ij = 1, and the rats of the RHS
// the stage uses (smb_2_roundoff: the htiny tests, the mass row testing
// only h_i; smb_2: the h <= 0 tests, then MAX(h, 0)).
template <int B, bool D, class Nb>
__device__ __forceinline__ void update_row(int64_t r, Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                             StateMix u, const float2* __restrict__ dmu, WorkMix w,
                             const float* __restrict__ res, StateMix u0, StateMix out, int rk_stage,
                             unsigned* __restrict__ err, const Nb& nb) {
  const int L = nb.len(G, r);
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const InstState& st = St[b];
  if (st.done) return;
  const InstConst& c = C[b];
  const int S = Nb::kGlobal ? c.S : 3;
  const int me = nb.self(r);
  const float4 ni = nb.nq[me];
  const bool ent = c.visc == VISC_ENTROPY;
  if (c.visc != VISC_FCT && !ent) {             // 'galerkin' / 'viscous': u^L is the result
    const float2 qL = w.qL[r];
    finish_mix(G, c, st, r, S, D ? df_from_double(w.hL64[r]) : w.hL[r], qL.x, qL.y, S == 5 ? w.q3L[r] : 0.f,
               S == 5 ? w.q4L[r] : 0.f, rk_stage, u0, out, err);
    return;
  }
  const int64_t base = nb.base(G, r);
  const auto ip = nb.row_index(base);
  const float2* dmp = dmu + base;
  const float hi = ni.x, etai = ni.w, resi = nb.aux[me];
  const float invhi = inv_pos(hi);
  const float Ri = ent ? 1.f : nb.R[me];
  // entropy_visc with the roundoff fix: smb_2_roundoff's h <= htiny tests
  const float hthr = (ent && c.roundoff_fix) ? c.htinyf : 0.f;
  const bool wet_i = !(hi <= hthr);
  float ui3 = 0.f, ui4 = 0.f;
  if (S == 5) { ui3 = u.q3[r]; ui4 = u.q4[r]; }
  float neg = 0.f, pos = 0.f;            // sum_{f < 0} f_ij, sum_{f >= 0} R_j f_ij
  double pos64 = 0.0;                    // precision split: sum_{f >= 0} R_j f_ij in FP64
  float x1 = 0.f, x2 = 0.f, x3 = 0.f, x4 = 0.f;
  for (int k0 = 0; k0 < L; k0 += B) {    // the diagonal's terms vanish: u_i rat_ii - u_i rat_ii = 0
   int jb[B];
   float d0b[B], m0b[B];
#pragma unroll
   for (int q = 0; q < B; q++) {
     if (k0 + q < L) {
       const int off = 32 * (k0 + q);
       jb[q] = ip[off]; const float2 v = dmp[off]; d0b[q] = v.x; m0b[q] = v.y;
     } else {
       jb[q] = me; d0b[q] = 0.f; m0b[q] = 0.f;
     }
   }
   float4 njb[Nb::kGlobal ? B : 1];
   float rsb[Nb::kGlobal ? B : 1], Rjb[Nb::kGlobal ? B : 1];
   if constexpr (Nb::kGlobal) {
#pragma unroll
     for (int q = 0; q < B; q++) { njb[q] = nb.nq[jb[q]]; rsb[q] = nb.aux[jb[q]]; Rjb[q] = ent ? 1.f : nb.R[jb[q]]; }
   }
#pragma unroll
   for (int q = 0; q < B; q++) {
    if (k0 + q >= L) break;
    const float4 nj = Nb::kGlobal ? njb[q] : nb.nq[jb[q]];
    const float d0 = d0b[q], m0 = m0b[q];
    const float rij = fmaxf(resi, Nb::kGlobal ? rsb[q] : nb.aux[jb[q]]);
    const float ddr = fminf(d0, rij) - d0, dmr = fminf(m0, rij) - m0;
    const float dz = dz_of(__fsub_rn(nj.w, etai), hi, nj.x);
    Recon R = recon(hi, nj.x, dz);
    float rij_ = rat_of(R.Hij, hi, dz <= 0.f, invhi);
    float rji_ = rat_of(R.Hji, nj.x, dz >= 0.f, inv_pos(nj.x));
    if (ent) {           // the rats and the mass row's H*_ij of the stage's RHS
      if (!wet_i) { rij_ = 0.f; R.Hij = 0.f; }
      if (nj.x <= hthr) rji_ = 0.f;
    }
    const float f = fct_from(ddr, dmr, hi, nj.x, R);
    float lf = Ri;
    if (f >= 0.f) {
      lf = ent ? 1.f : (Nb::kGlobal ? Rjb[q] : nb.R[jb[q]]);
      if (D && !ent) pos64 = fma(nb.R64[jb[q]], (double)f, pos64);
      else pos = __fmaf_rn(lf, f, pos);
    } else {
      neg = __fadd_rn(neg, f);
    }
    // l (dd (u_j rat_ji - u_i rat_ij) + dm (u_j (1 - rat_ji) - u_i (1 - rat_ij)))
    // = l (dm (u_j - u_i) + (dd - dm) (u_j rat_ji - u_i rat_ij))
    const float dm = dmr * lf, dx = (ddr - dmr) * lf;
    x1 = fma_(dx, fma_(nj.y, rji_, -ni.y * rij_), fma_(dm, nj.y - ni.y, x1));
    x2 = fma_(dx, fma_(nj.z, rji_, -ni.z * rij_), fma_(dm, nj.z - ni.z, x2));
    if constexpr (Nb::kGlobal) {
      if (S == 5) {
        const int j = jb[q];
        const float uj3 = u.q3[j], uj4 = u.q4[j];
        x3 = fma_(dx, fma_(uj3, rji_, -ui3 * rij_), fma_(dm, uj3 - ui3, x3));
        x4 = fma_(dx, fma_(uj4, rji_, -ui4 * rij_), fma_(dm, uj4 - ui4, x4));
      }
    }
   }
  }
  const float invm = G.inv_lumpedf[r], dtf = st.dtf;
  float2 hn;
  if (D) {       // u^L + dt/m sum l_ij f_ij for the depth, in FP64
    const double sh = ent ? (double)__fadd_rn(neg, pos) : fma(nb.R64[me], (double)neg, pos64);
    double h64 = fma(st.dt * G.inv_lumped[r], sh, w.hL64[r]);
    if (ent && !c.roundoff_fix && h64 < 0.0) h64 = 0.0;       // smb_2: MAX(h + dt rk, 0)
    hn = df_from_double(h64);
  } else {
    const float sh = __fadd_rn(__fmul_rn(Ri, neg), pos);
    hn = df_add_f(w.hL[r], __fmul_rn(__fmul_rn(dtf, invm), sh));
    if (ent && !c.roundoff_fix && hn.x < 0.f) hn = make_float2(0.f, 0.f);
  }
  const float2 qL = w.qL[r];
  const float q1 = fma_(dtf, x1 * invm, qL.x);
  const float q2 = fma_(dtf, x2 * invm, qL.y);
  float q3 = 0.f, q4 = 0.f;
  if (S == 5) { q3 = fma_(dtf, x3 * invm, w.q3L[r]); q4 = fma_(dtf, x4 * invm, w.q4L[r]); }
  if (hn.x < 0.f) atomicOr(err, ERRB_NEG_H);   // check_hmin (update.f90:285)
  finish_mix(G, c, st, r, S, hn, q1, q2, q3, q4, rk_stage, u0, out, err);
}

template <int B, bool D>
__global__ void __launch_bounds__(256) k_update_mix(Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                                                    StateMix u, const float2* __restrict__ dmu, WorkMix w,
                                                    const float* __restrict__ res, StateMix u0, StateMix out,
                                                    int rk_stage, unsigned* __restrict__ err) {
  pdl_trigger();
  pdl_wait();
  const NbGlobal nb{G.col, u.nq, res, w.rminus, w.rminus64};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.n_rows; r += (int64_t)gridDim.x * blockDim.x)
    update_row<B, D>(r, G, C, St, u, dmu, w, res, u0, out, rk_stage, err, nb);
}

template <int B, bool D>
__global__ void __launch_bounds__(256) k_update_tile(Graph G, const InstConst* __restrict__ C,
                                                     const InstState* __restrict__ St, StateMix u,
                                                     const float2* __restrict__ dmu, WorkMix w,
                                                     const float* __restrict__ res, StateMix u0, StateMix out,
                                                     int rk_stage, unsigned* __restrict__ err, TileCtl tc) {
  extern __shared__ float4 tile_mem[];
  pdl_trigger();
  tile_prefetch(G, tc, TilePrefetch{{tc.loc, nullptr, nullptr}, {2, 0, 0}, {G.inv_lumpedf, G.bathdf}, {4, 8}});
  pdl_wait();
  tile_prefetch(G, tc, TilePrefetch{{dmu, nullptr, nullptr}, {8, 0, 0},
                                    {w.hL, w.qL, rk_stage >= 2 ? (const void*)u0.nq : nullptr,
                                     rk_stage >= 2 ? (const void*)u0.h : nullptr},
                                    {8, 8, rk_stage >= 2 ? 16 : 0, rk_stage >= 2 ? 8 : 0}});
  const TileSmem sm = tile_smem<D>(tile_mem, tc.tile_rows + tc.halo_cap, tc.tile_rows);
  const int64_t t0 = stage_tile<true, true, D>(G, tc, u, res, w.rminus, sm, w.rminus64);
  const int64_t t1 = tile_end(G, tc, t0);
  const NbTile nb{tc.loc, sm.nq, sm.aux, sm.R, sm.R64, t0, sm.sp, sm.ln};
  for (int64_t r = t0 + threadIdx.x; r < t1; r += blockDim.x)
    update_row<B, D>(r, G, C, St, u, dmu, w, res, u0, out, rk_stage, err, nb);
}

// One row of k_dt_mix: FP32 lambda_max, |d_ii| / m_i (main.f90:166-174; 0 for
// padding and finished rows).  It walks the neighbours of the state that
// stage 1 starts from, so it also stores |c_ij| lambda_max per entry (dlam,
// reused by stage 1's k_low_mix) and alpha_i (alpha_out, stage 1's
// k_node_mix), when those are non-null.
template <int B, class Nb>
__device__ __forceinline__ float dt_row(int64_t r, const Graph& G, const InstConst* __restrict__ C,
                                        const InstState* __restrict__ St, const StateMix& u, float* __restrict__ dlam,
                                        float* __restrict__ alpha_out, unsigned* __restrict__ err, const Nb& nb) {
  if (r >= G.n_rows || nb.len(G, r) == 0) return 0.f;
  const int b = G.slice_inst[r >> 5];
  if (St[b].done) return 0.f;
  const InstConst& c = C[b];
  const float g = c.gf, htiny = c.htinyf;
  const LamK lk = lam_k(g, htiny);
  const int L = nb.len(G, r);
  const int64_t base = nb.base(G, r);
  const int me = nb.self(r);
  const auto ip = nb.row_index(base);
  const float2* cp = G.cf + base;
  const NodeF ni = node_from(nb.nq[me], htiny);
  const float sqi = sqrtf(g * fabsf(ni.h));
  float s = 0.f;
  float num = 0.f, denom = 0.f;          // alpha_limit stencil (as k_node_mix)
  bool bad = false;
  for (int k0 = 0; k0 < L; k0 += B) {
    int jb[B];
    float cxb[B], cyb[B];
#pragma unroll
    for (int q = 0; q < B; q++) {
      if (k0 + q < L) {
        const int off = 32 * (k0 + q);
        const float2 cc = cp[off];
        jb[q] = ip[off]; cxb[q] = cc.x; cyb[q] = cc.y;
      } else {
        jb[q] = me; cxb[q] = 1.f; cyb[q] = 0.f;
      }
    }
    float4 njb[B];
#pragma unroll
    for (int q = 0; q < B; q++) njb[q] = nb.nq[jb[q]];
#pragma unroll
    for (int q = 0; q < B; q++) {
      if (k0 + q >= L) break;
      const NodeF nj = node_from(njb[q], htiny);
      const float cxe = cxb[q], cye = cyb[q];
      float dl;
      if (!dlam_f(cxe, cye, dotc(cxe, cye, ni.v1, ni.v2), dotc(cxe, cye, nj.v1, nj.v2), ni.h, nj.h, ni.ovh, nj.ovh,
                  sqi, sqrtf(g * fabsf(nj.h)), lk, &dl))
        bad = true;
      if (dlam) dlam[base + 32 * (k0 + q)] = dl;
      s += dl;
      num += nj.h - ni.h;
      denom += fabsf(nj.h - ni.h);
    }
  }
  if (alpha_out) alpha_out[r] = (c.alpha_limit && !(ni.h <= c.htinyf)) ? alpha_from(num, denom) : 1.0f;
  if (bad) atomicOr(err, ERRB_DELTA);
  return s * G.inv_lumpedf[r];
}

// Warp max of |d_ii| / m_i into the instance's maximum (the 32 rows of a warp
// are one slice, so one instance).  A maximum does not depend on the order.
__device__ __forceinline__ void dt_reduce(float val, int64_t r, const Graph& G, InstState* __restrict__ St) {
  for (int off = 16; off > 0; off >>= 1) val = fmaxf(val, __shfl_down_sync(0xffffffffu, val, off));
  const int64_t r0 = r & ~(int64_t)31;
  if ((threadIdx.x & 31) == 0 && r0 < G.n_rows) {
    const int bw = G.slice_inst[r0 >> 5];
    if (!St[bw].done && val > 0.f)
      atomicMax(&St[bw].maxd_bits, (unsigned long long)__double_as_longlong((double)val));
  }
}

// k_dt_mix: FP32 lambda_max, max |d_ii|/m_i per instance (main.f90:166-174).
template <int B>
__global__ void __launch_bounds__(256) k_dt_mix(Graph G, const InstConst* __restrict__ C, InstState* __restrict__ St, StateMix u,
                         float* __restrict__ dlam, float* __restrict__ alpha_out, unsigned* __restrict__ err) {
  pdl_trigger();
  pdl_wait();
  // grid-stride over block-sized row ranges: every lane of a warp runs the
  // same iterations (the warp reduction needs all 32)
  const NbGlobal nb{G.col, u.nq, nullptr, nullptr, nullptr};
  for (int64_t rb = blockIdx.x * (int64_t)blockDim.x; rb < G.n_rows; rb += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = rb + threadIdx.x;
    dt_reduce(dt_row<B>(r, G, C, St, u, dlam, alpha_out, err, nb), r, G, St);
  }
}

template <int B>
__global__ void __launch_bounds__(256) k_dt_tile(Graph G, const InstConst* __restrict__ C, InstState* __restrict__ St,
                                                 StateMix u, float* __restrict__ dlam, float* __restrict__ alpha_out,
                                                 unsigned* __restrict__ err, TileCtl tc) {
  extern __shared__ float4 tile_mem[];
  pdl_trigger();
  tile_prefetch(G, tc, TilePrefetch{{tc.loc, G.cf, nullptr}, {2, 8, 0}, {G.inv_lumpedf}, {4}});
  pdl_wait();
  const TileSmem sm = tile_smem<false>(tile_mem, tc.tile_rows + tc.halo_cap, tc.tile_rows);
  const int64_t t0 = stage_tile<false, false>(G, tc, u, nullptr, nullptr, sm);
  const NbTile nb{tc.loc, sm.nq, nullptr, nullptr, nullptr, t0, sm.sp, sm.ln};
  // tile_rows is a multiple of 32: every lane of a warp runs the same iterations
  for (int64_t rb = t0; rb < t0 + tc.tile_rows; rb += blockDim.x) {
    const int64_t r = rb + threadIdx.x;
    if (rb - t0 + (int64_t)threadIdx.x - (threadIdx.x & 31) >= tc.tile_rows) break;   // warp past the tile
    dt_reduce(dt_row<B>(r, G, C, St, u, dlam, alpha_out, err, nb), r, G, St);
  }
}

// Free surface of the packed node records after a bathymetry change
__global__ void k_refresh_eta(Graph G, StateMix u) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= G.n_rows) return;
  u.nq[r].w = eta_of(u.h[r], G.bathdf[r]);
}

static inline unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// Launch of a stage kernel with programmatic stream serialization (the
// kernels wait for their predecessor themselves, pdl_wait); SWE_PDL=0 makes
// it an ordinary launch.
static bool pdl_enabled() {
  static const int on = [] {
    const char* e = getenv("SWE_PDL");
    return (e && e[0] == '0') ? 0 : 1;
  }();
  return on != 0;
}
template <typename... KArgs, typename... Args>
static void launch_k(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// Grid of a row kernel: one thread per row (mode 0), or a resident grid of
// mode x (blocks per SM at full occupancy) x SMs whose threads stride over
// the rows (the kernels loop), which keeps every warp slot busy instead of
// paying a block launch per 64-256 rows.
template <typename K>
static unsigned row_grid(K kern, int64_t n, int block, int mode) {
  const unsigned full = nblk(n, block);
  if (mode <= 0) return full;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0) != cudaSuccess || per_sm <= 0) {
    cudaGetLastError();
    return full;
  }
  const unsigned g = (unsigned)(per_sm * sms * mode);
  return g < full ? g : full;
}

#define EV_BEGIN(k) if (kev) cudaEventRecord(kev->ev[2 * (k)], s)
#define EV_END(k) if (kev) cudaEventRecord(kev->ev[2 * (k) + 1], s)

#define SWE_DISPATCH_B(b, KERNEL, N, BS, MODE, ...)                                              \
  switch (b) {                                                                                  \
    case 8: launch_k(KERNEL<8>, row_grid(KERNEL<8>, N, BS, MODE), BS, 0, s, __VA_ARGS__); break;      \
    case 4: launch_k(KERNEL<4>, row_grid(KERNEL<4>, N, BS, MODE), BS, 0, s, __VA_ARGS__); break;      \
    case 2: launch_k(KERNEL<2>, row_grid(KERNEL<2>, N, BS, MODE), BS, 0, s, __VA_ARGS__); break;      \
    default: launch_k(KERNEL<1>, row_grid(KERNEL<1>, N, BS, MODE), BS, 0, s, __VA_ARGS__); break;     \
  }
// the same for kernels with a second template argument D
#define SWE_DISPATCH_BD(b, KERNEL, D, N, BS, MODE, ...)                                                         \
  switch (b) {                                                                                                 \
    case 8: launch_k(KERNEL<8, D>, row_grid(KERNEL<8, D>, N, BS, MODE), BS, 0, s, __VA_ARGS__); break;         \
    case 4: launch_k(KERNEL<4, D>, row_grid(KERNEL<4, D>, N, BS, MODE), BS, 0, s, __VA_ARGS__); break;         \
    case 2: launch_k(KERNEL<2, D>, row_grid(KERNEL<2, D>, N, BS, MODE), BS, 0, s, __VA_ARGS__); break;         \
    default: launch_k(KERNEL<1, D>, row_grid(KERNEL<1, D>, N, BS, MODE), BS, 0, s, __VA_ARGS__); break;        \
  }

// Tile variants: one block per tile, shared memory for the tile's and the
// halo's node records, residuals and R^- (24 B per row; 32 B with the FP64
// R^- of the precision split)
size_t tile_smem_bytes(const TileCtl& tc, bool d) {
  const size_t cap = tc.tile_rows + tc.halo_cap;
  return cap * (d ? 32 : 24) + (size_t)tc.tile_rows / 32 * 8 + tc.tile_rows;
}
#define SWE_DISPATCH_TILE(b, KERNEL, BS, TC, NROWS, ...)                                                \
  do {                                                                                                \
    const TileCtl& tc_ = (TC);                                                                        \
    const unsigned g_ = (unsigned)(((NROWS) + tc_.tile_rows - 1) / tc_.tile_rows);                    \
    const size_t sm_ = tile_smem_bytes(tc_);                                                          \
    switch (b) {                                                                                      \
      case 8: launch_k(KERNEL<8>, g_, BS, sm_, s, __VA_ARGS__); break;                                \
      case 4: launch_k(KERNEL<4>, g_, BS, sm_, s, __VA_ARGS__); break;                                \
      case 2: launch_k(KERNEL<2>, g_, BS, sm_, s, __VA_ARGS__); break;                                \
      default: launch_k(KERNEL<1>, g_, BS, sm_, s, __VA_ARGS__); break;                               \
    }                                                                                                 \
  } while (0)
#define SWE_DISPATCH_TILE_D(b, KERNEL, BS, TC, NROWS, D, SMEM, ...)                                     \
  do {                                                                                                \
    const TileCtl& tc_ = (TC);                                                                        \
    const unsigned g_ = (unsigned)(((NROWS) + tc_.tile_rows - 1) / tc_.tile_rows);                    \
    const size_t sm_ = (SMEM);                                                                        \
    switch (b) {                                                                                      \
      case 8: launch_k(KERNEL<8, D>, g_, BS, sm_, s, __VA_ARGS__); break;                             \
      case 4: launch_k(KERNEL<4, D>, g_, BS, sm_, s, __VA_ARGS__); break;                             \
      case 2: launch_k(KERNEL<2, D>, g_, BS, sm_, s, __VA_ARGS__); break;                             \
      default: launch_k(KERNEL<1, D>, g_, BS, sm_, s, __VA_ARGS__); break;                            \
    }                                                                                                 \
  } while (0)

// k_low variants: entry batch 1 or 2, lambda_max computed or taken from
// k_dt_mix (stage 1), registers capped at 85, 64 or 51 (3, 4 or 5 resident
// blocks of 256 threads per SM; the compiler would take ~106 with no cap)
template <bool LAMIN, bool D>
static void launch_low(const StageArgsMix& a, int batch, int cap, int mode, int block, bool tiled, cudaStream_t s) {
  if (tiled && a.tiles) {
    const TileCtl& tc = *a.tiles;
    const unsigned g = (unsigned)((a.G.n_rows + tc.tile_rows - 1) / tc.tile_rows);
    const size_t sm = tile_smem_bytes(tc);
#define SWE_LOWT(BB, MB) \
    launch_k(k_low_tile<BB, LAMIN, MB, D>, g, block, sm, s, a.G, a.C, a.St, a.u, a.w.alpha, a.w.dmu, a.w, a.w.res, \
             a.err, tc)
    if (batch >= 2) { if (cap == 2) SWE_LOWT(2, 5); else if (cap) SWE_LOWT(2, 4); else SWE_LOWT(2, 3); }
    else { if (cap == 2) SWE_LOWT(1, 5); else if (cap) SWE_LOWT(1, 4); else SWE_LOWT(1, 3); }
#undef SWE_LOWT
    return;
  }
#define SWE_LOW(BB, MB)                                                                                  \
  launch_k(k_low_mix<BB, LAMIN, MB, D>, row_grid(k_low_mix<BB, LAMIN, MB, D>, a.G.n_rows, block, mode), block, 0, s, \
           a.G, a.C, a.St, a.u, a.w.alpha, a.w.dmu, a.w, a.w.res, a.err)
  if (batch >= 2) { if (cap == 2) SWE_LOW(2, 5); else if (cap) SWE_LOW(2, 4); else SWE_LOW(2, 3); }
  else { if (cap == 2) SWE_LOW(1, 5); else if (cap) SWE_LOW(1, 4); else SWE_LOW(1, 3); }
#undef SWE_LOW
}

bool kind_has_tiles(int kind) { return kind >= 0 && kind <= 4; }

template <bool D>
static void launch_kernel_mix_d(int kind, const StageArgsMix& a, const KernelTune& t, cudaStream_t s) {
  const int64_t n = a.G.n_rows;
  switch (kind) {
    case 1: if (t.tiled[1] && a.tiles) {
              SWE_DISPATCH_TILE(t.batch[1], k_node_tile, t.block[1], *a.tiles, n, a.G, a.C, a.St, a.u, a.w.alpha, *a.tiles);
            } else {
              SWE_DISPATCH_B(t.batch[1], k_node_mix, n, t.block[1], t.grid[1], a.G, a.C, a.St, a.u, a.w.alpha)
            }
            break;
    case 2: if (a.type1)                       // some instance runs 'viscous' with 'type1'
              launch_k(k_low_type1<D>, nblk(n, 128), 128, 0, s, a.G, a.C, a.St, a.u, a.w.alpha, a.w.dmu, a.w, a.w.res,
                       a.err);
            else if (a.rk_stage == 1 && a.w.dlam)   // stage 1 follows k_dt_mix on the same state
              launch_low<true, D>(a, t.batch[2], t.cap_low, t.grid[2], t.block[2], t.tiled[2], s);
            else
              launch_low<false, D>(a, t.batch[2], t.cap_low, t.grid[2], t.block[2], t.tiled[2], s);
            break;
    case 3: if (t.tiled[3] && a.tiles) {
              SWE_DISPATCH_TILE_D(t.batch[3], k_fct_tile, t.block[3], *a.tiles, n, D, tile_smem_bytes(*a.tiles), a.G, a.C, a.St, a.u, a.w.dmu, a.w,
                                  a.w.res, a.err, *a.tiles);
            } else {
              SWE_DISPATCH_BD(t.batch[3], k_fct_mix, D, n, t.block[3], t.grid[3], a.G, a.C, a.St, a.u, a.w.dmu, a.w,
                              a.w.res, a.err)
            }
            break;
    case 4: if (t.tiled[4] && a.tiles) {
              SWE_DISPATCH_TILE_D(t.batch[4], k_update_tile, t.block[4], *a.tiles, n, D, tile_smem_bytes(*a.tiles, D), a.G, a.C, a.St, a.u,
                                  a.w.dmu, a.w, a.w.res, a.u0, a.out, a.rk_stage, a.err, *a.tiles);
            } else {
              SWE_DISPATCH_BD(t.batch[4], k_update_mix, D, n, t.block[4], t.grid[4], a.G, a.C, a.St, a.u, a.w.dmu,
                              a.w, a.w.res, a.u0, a.out, a.rk_stage, a.err)
            }
            break;
    default: break;
  }
}

void launch_kernel_mix(int kind, const StageArgsMix& a, const KernelTune& t, cudaStream_t s) {
  if (a.f64) launch_kernel_mix_d<true>(kind, a, t, s);
  else launch_kernel_mix_d<false>(kind, a, t, s);
}

void launch_stage_mix(const StageArgsMix& a, cudaStream_t s, const KernelEvents* kev, const KernelTune& t) {
  for (int kind = 1; kind <= 4; kind++) {
    EV_BEGIN(kind);
    // stage 1 follows k_dt_mix on the same state, which already stored alpha
    if (!(kind == 1 && a.rk_stage == 1 && a.w.dlam)) launch_kernel_mix(kind, a, t, s);
    EV_END(kind);
  }
}

void launch_dt_mix(const Graph& G, const InstConst* C, InstState* St, const StateMix& u, float* dlam, float* alpha,
                   unsigned* err, const KernelTune& t, const TileCtl* tiles, cudaStream_t s) {
  if (t.tiled[0] && tiles) {
    SWE_DISPATCH_TILE(t.batch[0], k_dt_tile, t.block[0], *tiles, G.n_rows, G, C, St, u, dlam, alpha, err, *tiles);
  } else {
    SWE_DISPATCH_B(t.batch[0], k_dt_mix, G.n_rows, t.block[0], t.grid[0], G, C, St, u, dlam, alpha, err)
  }
}

void launch_refresh_eta(const Graph& G, StateMix u, cudaStream_t s) {
  k_refresh_eta<<<nblk(G.n_rows, 256), 256, 0, s>>>(G, u);
}

}  // namespace swe
