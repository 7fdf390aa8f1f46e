// Mixed-precision stage kernels: every per-edge and per-row operation issues
// on the FP32 pipes.
//
// Same sweep structure as the FP64 path (one thread per row, SELL-32 graph)
// with the flux, lambda_max, viscosity, entropy-residual and antidiffusion
// arithmetic in FP32 on FP32 data (q, z, c_ij, d_ij, mu_ij and an FP32 shadow
// of h).  A warp-wide FP64 instruction, or a float<->double conversion, costs
// GB300 tens of SM cycles (FP64 runs at ~1/64 of the FP32 rate), and a design
// that kept the limiter sums and the per-row depth updates in FP64 measured
// its FP64 pipe 73-79% busy in the limiter and update sweeps.  The precision
// the scheme needs is kept without FP64:
//   * the depth h (state, low-order h^L, new depth, RK combination) is a
//     double-float pair hi + lo (about 48 significant bits), so the FP32
//     increments of a stage are never lost to the rounding of h;
//   * h^L = h + a (fix h + rk_1) with a = dt/m_i: non-negative in any
//     rounding, because a |fix| <= CFL < 1 and rk_1 >= 0 (SOURCES/update.f90:
//     202-215);
//   * the limiter R^-_i = min(1, (1 - 2^-18) Q^-_i / P^-_i) (fct.f90:15-30) is
//     FP32; the 2^-18 margin (64 units in the last place) bounds the at most
//     ~12 roundings between the limiter and the depth update, so the limited
//     update cannot take more than h^L out of a node (see k_fct_mix);
//   * the reference's threshold tests (h <= htiny, h <= 0) use an FP32 shadow
//     of h that keeps both decisions exact, and m h^L/dt <= htiny is decided in
//     FP64 inside a 1e-5 band around htiny.
//
// Node data that neighbours gather is packed per node as float4
// {h shadow, qx, qy, z}: one 16-byte load (one L2 sector) per neighbour.
#include "swe_kernels.hpp"

namespace swe {

__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }

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

// Hydrostatic reconstruction H*_ij = max(0, h_i + z_i - max(z_i, z_j))
// (SOURCES/update.f90:569-570) in the algebraically equal, cancellation-free
// form max(0, h_i - max(0, z_j - z_i)).  In FP32 the reference form loses
// (h_i + z_i) - z_i to rounding at the scale of z, which for thin layers on
// high bathymetry is a large relative error in H*/h.  rat = H*/h is 1
// exactly when z_j <= z_i and never exceeds 1.
struct Recon {
  float Hij, Hji, rij, rji;   // rij, rji: H*/h with the h <= 0 tests
};
__device__ __forceinline__ Recon recon(float hi, float hj, float dz, float invhi, float invhj) {
  Recon R;
  R.Hij = (dz <= 0.f) ? hi : fmaxf(0.f, hi - dz);
  R.Hji = (dz >= 0.f) ? hj : fmaxf(0.f, hj + dz);
  R.rij = (hi > 0.f) ? ((dz <= 0.f) ? 1.f : fminf(__fmul_rn(R.Hij, invhi), 1.f)) : 0.f;
  R.rji = (hj > 0.f) ? ((dz >= 0.f) ? 1.f : fminf(__fmul_rn(R.Hji, invhj), 1.f)) : 0.f;
  return R;
}
__device__ __forceinline__ float inv_pos(float h) { return (h > 0.f) ? fdiv(1.0f, h) : 0.f; }

// antidiffusive h-flux f_ij of compute_fct_matrix (update.f90:744-745) with
// explicit roundings: k_fct and k_update must see the same f, bit for bit.
__device__ __forceinline__ float fct_from(float dd, float dm, float hi, float hj, const Recon& R) {
  const float a = __fsub_rn(__fmul_rn(hj, R.rji), __fmul_rn(hi, R.rij));
  const float b = __fsub_rn(__fmul_rn(hj, __fsub_rn(1.f, R.rji)), __fmul_rn(hi, __fsub_rn(1.f, R.rij)));
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
  float fl, fr;
  if (h > hl && h > hr) {              // two shocks: the usual case at h = x0 h_min
    fl = (h - hl) * sqrtf(0.5f * k.g * (ovh + ovhl));
    fr = (h - hr) * sqrtf(0.5f * k.g * (ovh + ovhr));
  } else {
    const float sgh = sqrtf(k.g * h);
    fl = (h > hl) ? (h - hl) * sqrtf(0.5f * k.g * (ovh + ovhl)) : 2.f * (sgh - sql);
    fr = (h > hr) ? (h - hr) * sqrtf(0.5f * k.g * (ovh + ovhr)) : 2.f * (sgh - sqr);
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
    const float s = fmaxf(vl - vr + 2.f * sql + 2.f * sqr, 0.f);
    ht = fminf(x0 * hmin, fdiv(s * s, 16.f * k.g));
  } else {
    fh = phi_f(x0 * hmax, vl, hl, vr, hr, ovhl, ovhr, sql, sqr, k);
    const float sqrmin = (lmin ? sql : sqr) * k.rsg, sqrmax = (lmin ? sqr : sql) * k.rsg;
    if (0.f <= fh) {
      const float a = 0.353553391f;   // 1 / (2 sqrt(2))
      const float cc = -(hmin * a) - sqrmin * sqrmax + sqrmin * (vr - vl) * (0.5f * k.rsg);
      float Delta = hmin - 4.f * a * cc;
      if (Delta < 0.f) {
        if (Delta < -1e-5f * hmin) ok = false;
        Delta = 0.f;
      }
      const float s = (sqrtf(Delta) - sqrmin) * 1.41421356f;   // / (2a)
      ht = fminf(x0 * hmax, s * s);
    } else {
      ht = sqrmin * sqrmax * (1.f + 1.41421356f * k.rsg * fdiv(vl - vr, sqrmin + sqrmax));
    }
  }
  const float lbdl = vl - sql * sqrtf((1.f + fmaxf((ht - hl) * ovhl * 0.5f, 0.f)) * (1.f + fmaxf((ht - hl) * ovhl, 0.f)));
  const float lbdr = vr + sqr * sqrtf((1.f + fmaxf((ht - hr) * ovhr * 0.5f, 0.f)) * (1.f + fmaxf((ht - hr) * ovhr, 0.f)));
  *lambda = fmaxf(fabsf(lbdl), fabsf(lbdr));
  return ok;
}

// Entry loops are processed in batches of B entries: every load of a batch is
// issued before any of them is used, so a thread keeps B gathers in flight
// (the kernels are latency-bound otherwise).  Sums keep the entry order; the
// instantiations may contract FMAs differently, so batch sizes agree to FP32
// rounding.  The autotuner picks B per kernel.

// Neighbour access of the entry loops: straight from HBM by column index
// (NbGlobal), or from the block's shared-memory copy of its tile and halo
// nodes by tile-local position (NbTile, rows of 3-component systems only).
// aux is the per-node scalar the loop needs besides the node record (alpha
// in k_low, the residual in k_fct and k_update); R is R^- (k_update).
struct NbGlobal {
  static constexpr bool kGlobal = true;
  const int* col;
  const float4* nq;
  const float* aux;
  const float* R;
  __device__ __forceinline__ int index(int64_t e) const { return col[e]; }
  __device__ __forceinline__ int self(int64_t r) const { return (int)r; }
};
struct NbTile {
  static constexpr bool kGlobal = false;
  const int16_t* loc;
  const float4* nq;
  const float* aux;
  const float* R;
  int64_t t0;
  __device__ __forceinline__ int index(int64_t e) const { return loc[e]; }
  __device__ __forceinline__ int self(int64_t r) const { return (int)(r - t0); }
};

// Shared-memory tile of one block: node records, aux and R^- of the tile's
// rows (positions 0 .. T-1) and of its halo rows (T .. T+nh-1).
struct TileSmem {
  float4* nq;
  float* aux;
  float* R;
};
__device__ __forceinline__ TileSmem tile_smem(void* base, int cap) {
  float4* nq = reinterpret_cast<float4*>(base);
  float* aux = reinterpret_cast<float*>(nq + cap);
  return TileSmem{nq, aux, aux + cap};
}

// Copy the tile's and the halo's node data into shared memory (coalesced for
// the tile rows, ascending gathers for the halo); returns the tile start.
template <bool AUX, bool RM>
__device__ __forceinline__ int64_t stage_tile(const Graph& G, const TileCtl& tc, const StateMix& u,
                                              const float* __restrict__ aux, const float* __restrict__ rminus,
                                              const TileSmem& sm) {
  const int T = tc.tile_rows;
  const int64_t t0 = (int64_t)blockIdx.x * T;
  const int h0 = tc.halo_ptr[blockIdx.x], nh = tc.halo_ptr[blockIdx.x + 1] - h0;
  for (int i = threadIdx.x; i < T + nh; i += blockDim.x) {
    const int64_t row = i < T ? t0 + i : (int64_t)tc.halo_rows[h0 + i - T];
    if (row < G.n_rows) {
      sm.nq[i] = u.nq[row];
      if (AUX) sm.aux[i] = aux[row];
      if (RM) sm.R[i] = rminus[row];
    }
  }
  __syncthreads();
  return t0;
}

__device__ __forceinline__ int64_t tile_end(const Graph& G, const TileCtl& tc, int64_t t0) {
  return t0 + tc.tile_rows < G.n_rows ? t0 + tc.tile_rows : G.n_rows;
}

// k_node_mix: alpha_i (SOURCES/update.f90:758-781) from the FP32 depth.
template <int B, class Nb>
__device__ __forceinline__ void node_row(int64_t r, Graph G, const InstConst* __restrict__ C,
                                                  const InstState* __restrict__ St, StateMix u,
                                                  float* __restrict__ alpha_out, const Nb& nb) {
  const int L = G.len[r];
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  if (St[b].done) return;
  const InstConst& c = C[b];
  const float* hs = reinterpret_cast<const float*>(nb.nq);
  const float h = reinterpret_cast<const float*>(u.nq)[4 * r];
  float alpha = 1.0f;
  if (c.alpha_limit && !(h <= c.htinyf)) {
    const int64_t base = entry_base(G, r);
    float num = 0.0f, denom = 0.0f;
    for (int k0 = 0; k0 < L; k0 += B) {
      int j[B];
#pragma unroll
      for (int q = 0; q < B; q++) j[q] = (k0 + q < L) ? nb.index(base + 32 * (k0 + q)) : nb.self(r);
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
    const float a = (denom <= fabsf(num)) ? 1.0f : fdiv(fabsf(num), denom);
    const float a2 = a * a, a4 = a2 * a2;
    alpha = a4 * a4;
  }
  alpha_out[r] = alpha;
}

template <int B>
__global__ void __launch_bounds__(256) k_node_mix(Graph G, const InstConst* __restrict__ C,
                                                  const InstState* __restrict__ St, StateMix u,
                                                  float* __restrict__ alpha_out) {
  const NbGlobal nb{G.col, u.nq, nullptr, nullptr};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.n_rows; r += (int64_t)gridDim.x * blockDim.x)
    node_row<B>(r, G, C, St, u, alpha_out, nb);
}

template <int B>
__global__ void __launch_bounds__(256) k_node_tile(Graph G, const InstConst* __restrict__ C,
                                                   const InstState* __restrict__ St, StateMix u,
                                                   float* __restrict__ alpha_out, TileCtl tc) {
  extern __shared__ float4 tile_mem[];
  const TileSmem sm = tile_smem(tile_mem, tc.tile_rows + tc.halo_cap);
  const int64_t t0 = stage_tile<false, false>(G, tc, u, nullptr, nullptr, sm);
  const int64_t t1 = tile_end(G, tc, t0);
  const NbTile nb{tc.loc, sm.nq, nullptr, nullptr, t0};
  for (int64_t r = t0 + threadIdx.x; r < t1; r += blockDim.x) node_row<B>(r, G, C, St, u, alpha_out, nb);
}

struct NodeF {   // FP32 view of one node used by the edge loop
  float h, q1, q2, z, ovh, v1, v2;
};

__device__ __forceinline__ NodeF node_from(const float4 a, float htiny) {
  NodeF n;
  n.h = a.x; n.q1 = a.y; n.q2 = a.z; n.z = a.w;
  n.ovh = ovh_f(n.h, htiny);
  n.v1 = n.q1 * n.ovh;
  n.v2 = n.q2 * n.ovh;
  return n;
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
template <int B, bool LAMIN, int MINB, class Nb>
__device__ __forceinline__ void low_row(int64_t r, Graph G, const InstConst* __restrict__ C,
                                                       const InstState* __restrict__ St, StateMix u,
                                                       const float* __restrict__ alpha, float2* __restrict__ dmu,
                                                       WorkMix w, float* __restrict__ res, unsigned* __restrict__ err,
                                                       const Nb& nb) {
  const int L = G.len[r];
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
  const int64_t base = entry_base(G, r);
  const NodeF ni = node_from(u.nq[r], htiny);
  const float sqi = sqrtf(g * fabsf(ni.h));
  const float v2i_flux = sgn ? 0.f : ni.v2;          // flux() zeroes velocity(2) for type 13
  const float ai = alpha[r];
  const float m = G.lumpedf[r];
  float ui3 = 0.f, ui4 = 0.f;
  if (S == 5) { ui3 = u.q3[r]; ui4 = u.q4[r]; }
  const float invhi = inv_pos(ni.h);
  bool delta_bad = false;

  float fix = 0.f, rk0 = 0.f;
  float rk1 = 0.f, rk2_ = 0.f, rk3 = 0.f, rk4 = 0.f;               // smb_2_roundoff momenta
  float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f, g4 = 0.f;          // smb_2
  const float Ei = 0.5f * (g * ni.h * ni.h + ni.v1 * ni.q1 + v2i_flux * ni.q2);
  float emax = Ei, emin = Ei;
  float ptx = 0.f, pty = 0.f;
  {
    // diagonal: Galerkin boundary term -c_ii.v_i (fix_roundoff / smb_2);
    // its viscous and topography terms vanish
    const float cxe = G.cxiif[r], cye = G.cyiif[r];
    const float cvi = dotc(cxe, cye, ni.v1, v2i_flux);
    fix -= cvi;
    g0 -= cvi * ni.h;
    rk1 -= cvi * ni.q1; rk2_ -= cvi * ni.q2;
    g1 -= cvi * ni.q1; g2 -= cvi * ni.q2;
    if (S == 5) { rk3 -= cvi * ui3; rk4 -= cvi * ui4; g3 -= cvi * ui3; g4 -= cvi * ui4; }
    if (sgn) {
      const float pt = sgn_pressure(c.lambda_sgnf, g, m, ni.h, ui3);
      ptx -= pt * cxe;
      pty -= pt * cye;
    }
  }
  for (int k0 = 0; k0 < L; k0 += B) {
   int jb[B];
   float cxb[B], cyb[B], dlb[B];
#pragma unroll
   for (int q = 0; q < B; q++) {
     if (k0 + q < L) {
       const int64_t e = base + 32 * (k0 + q);
       jb[q] = nb.index(e); cxb[q] = G.cxf[e]; cyb[q] = G.cyf[e];
       dlb[q] = LAMIN ? w.dlam[e] : 0.f;
     } else {
       jb[q] = nb.self(r); cxb[q] = 0.f; cyb[q] = 0.f; dlb[q] = 0.f;
     }
   }
   float4 nqb[B];
   float alb[B];
#pragma unroll
   for (int q = 0; q < B; q++) { nqb[q] = nb.nq[jb[q]]; alb[q] = nb.aux[jb[q]]; }
#pragma unroll
   for (int q = 0; q < B; q++) {
    if (k0 + q >= L) break;
    const int64_t e = base + 32 * (k0 + q);
    const float cxe = cxb[q], cye = cyb[q];
    const int j = jb[q];
    const NodeF nj = node_from(nqb[q], htiny);
    // --- viscosities: compute_dij, compute_muij, MAX, alpha_limit
    const float cvi = dotc(cxe, cye, ni.v1, ni.v2);                   // c.v_i (compute_muij)
    const float cvj = dotc(cxe, cye, nj.v1, nj.v2);                   // c.v_j
    float dlam;                                                       // |c_ij| lambda_max
    if (LAMIN) {
      dlam = dlb[q];                                                  // from k_dt_mix on this state
    } else {
      const float n2 = cxe * cxe + cye * cye;
      const float inv = rsqrtf(n2);
      float lam;
      if (!lambda_f(ni.h, nj.h, cvi * inv, cvj * inv, ni.ovh, nj.ovh, sqi, sqrtf(g * fabsf(nj.h)), lk, &lam))
        delta_bad = true;
      dlam = (n2 * inv) * lam;
    }
    float mu = fmaxf(fmaxf(-cvi, 0.f), fmaxf(cvj, 0.f));
    float d = fmaxf(dlam, mu);
    const float s = (c.alpha_limit ? fmaxf(ai, alb[q]) : 1.f) * vis;
    d *= s;
    mu *= s;
    dmu[e] = make_float2(d, mu);
    // --- entropy stencil
    const float v2j_flux = sgn ? 0.f : nj.v2;
    const float Ej = 0.5f * (g * nj.h * nj.h + nj.v1 * nj.q1 + v2j_flux * nj.q2);
    emax = fmaxf(emax, Ej);
    emin = fminf(emin, Ej);
    // --- hydrostatic reconstruction
    const float dz = nj.z - ni.z;
    const Recon R = recon(ni.h, nj.h, dz, invhi, inv_pos(nj.h));
    const float rij = R.rij, rji = R.rji;                             // h <= 0 tests (smb_2)
    const float rijt = (ni.h <= hthr) ? 0.f : rij;                    // h <= htiny tests
    const float rjit = (nj.h <= hthr) ? 0.f : rji;
    const float cvj_flux = sgn ? dotc(cxe, cye, nj.v1, 0.f) : cvj;   // c.velocity_j of flux()
    const float topo = g * ni.h * ((nj.h - ni.h) + dz);               // g h_i (eta_j - eta_i)
    // --- smb_2_roundoff mass row (fix_roundoff, rk_1), in the reference's
    // form: its sign properties give h^L >= 0
    const float dmu = d - mu;
    fix += -mu - dmu * rijt;
    rk0 += (mu - cvj_flux) * nj.h + fmaxf(dmu * R.Hji, 0.f);
    // --- smb_2 mass row and the momenta of both RHS, written as
    // -c.v_j u_j + mu (u_j - u_i) + (d - mu) (u_j rat_ji - u_i rat_ij), which
    // equals d (u_j rat_ji - u_i rat_ij) + mu (u_j (1 - rat_ji) - u_i (1 - rat_ij))
    g0 += -cvj_flux * nj.h + mu * (nj.h - ni.h) + dmu * (nj.h * rji - ni.h * rij);
    const float A1 = mu * (nj.q1 - ni.q1) - cvj_flux * nj.q1;
    const float A2 = mu * (nj.q2 - ni.q2) - cvj_flux * nj.q2;
    const float T1 = A1 + dmu * (nj.q1 * rji - ni.q1 * rij);
    const float T2 = A2 + dmu * (nj.q2 * rji - ni.q2 * rij);
    g1 += T1;
    g2 += T2;
    if (rijt == rij && rjit == rji) {                                 // both wet: same terms
      rk1 += T1;
      rk2_ += T2;
    } else {
      rk1 += A1 + dmu * (nj.q1 * rjit - ni.q1 * rijt);
      rk2_ += A2 + dmu * (nj.q2 * rjit - ni.q2 * rijt);
    }
    rk1 -= topo * cxe; rk2_ -= topo * cye;
    g1 -= topo * cxe; g2 -= topo * cye;
    if (Nb::kGlobal && S == 5) {
      const float uj3 = u.q3[j], uj4 = u.q4[j];
      const float A3 = mu * (uj3 - ui3) - cvj_flux * uj3;
      const float A4 = mu * (uj4 - ui4) - cvj_flux * uj4;
      rk3 += A3 + dmu * (uj3 * rjit - ui3 * rijt);
      rk4 += A4 + dmu * (uj4 * rjit - ui4 * rijt);
      g3 += A3 + dmu * (uj3 * rji - ui3 * rij);
      g4 += A4 + dmu * (uj4 * rji - ui4 * rij);
      if (sgn) {
        const float pt = sgn_pressure(c.lambda_sgnf, g, G.lumpedf[j], nj.h, uj3);
        ptx -= pt * cxe;
        pty -= pt * cye;
      }
    }
   }
  }
  // source terms (update.f90:425-551)
  if (c.type_test == 9 || c.type_test == 10) {
    const float hstar = __powf(fmaxf(ni.h, htiny), 4.0f / 3.0f);
    const float vel = c.fricf * sqrtf(ni.v1 * ni.v1 + ni.v2 * ni.v2);
    const float hloc = vel * dtf;
    const float coef = fdiv(m * vel * 2.f, hstar + fmaxf(hstar, hloc));
    rk1 -= coef * ni.q1; rk2_ -= coef * ni.q2;
    g1 -= coef * ni.q1; g2 -= coef * ni.q2;
  } else if (c.type_test == 11) {
    rk1 -= m * 0.2f * ni.q1; rk2_ -= m * 0.2f * ni.q2;
    g1 -= m * 0.2f * ni.q1; g2 -= m * 0.2f * ni.q2;
  } else if (c.type_test == 12) {
    const float a1 = m * 2.0f * ni.q2, a2 = m * 2.0f * ni.q1;
    rk1 += a1; rk2_ -= a2; g1 += a1; g2 -= a2;
  } else if (sgn) {
    const float pc = fdiv(c.lambda_sgnf * g, 3.0f * sqrtf(m));
    const float t = fdiv(ui3, ni.h);
    const float x = fdiv(ui3, ni.h * ni.h);
    const float s_i = 3.f * pc * t * t * 12.f * (x - 1.f);
    rk1 += ptx; rk2_ += pty; g1 += ptx; g2 += pty;
    rk3 += m * ui4; rk4 -= m * s_i;
    g3 += m * ui4; g4 -= m * s_i;
  }
  // low-order state: double-float depth plus an FP32 increment
  const float invm = G.inv_lumpedf[r];
  const float a = dtf * invm;
  const float2 h = u.h[r];
  float2 hL;
  if (roundoff) {
    hL = df_add_f(h, a * __fmaf_rn(fix, ni.h, rk0));   // h + a (fix h + rk_1), a |fix| <= CFL
  } else {                                             // smb_2 and MAX(h + dt rk, 0)
    hL = df_add_f(h, a * g0);
    if (hL.x < 0.f) hL = make_float2(0.f, 0.f);
  }
  w.hL[r] = hL;
  w.qL[r] = make_float2(ni.q1 + dtf * (rk1 * invm), ni.q2 + dtf * (rk2_ * invm));
  if (S == 5) { w.q3L[r] = ui3 + dtf * (rk3 * invm); w.q4L[r] = ui4 + dtf * (rk4 * invm); }
  // entropy residual (update.f90:838-868), rescale once per node
  const float un0 = ni.h + dtf * (g0 * invm);
  const float un1 = ni.q1 + dtf * (g1 * invm);
  const float un2 = ni.q2 + dtf * (g2 * invm);
  const float on = ovh_f(un0, htiny);
  const float En = 0.5f * (g * un0 * un0 + (un1 * on) * un1 + (un2 * on) * un2);
  const float Ep0 = g * ni.h - 0.5f * (ni.v1 * ni.v1) - 0.5f * (v2i_flux * v2i_flux);
  float rs = m * (En - Ei) * st.inv_dtf;
  rs -= g0 * Ep0 + g1 * ni.v1 + g2 * v2i_flux;
  const float rescale = 0.5f * fabsf(emax - emin) + c.rescale_floorf;
  res[r] = fdiv(fabsf(rs), rescale);
  if (delta_bad) atomicOr(err, ERRB_DELTA);
}

template <int B, bool LAMIN, int MINB>
__global__ void __launch_bounds__(256, MINB) k_low_mix(Graph G, const InstConst* __restrict__ C,
                                                       const InstState* __restrict__ St, StateMix u,
                                                       const float* __restrict__ alpha, float2* __restrict__ dmu,
                                                       WorkMix w, float* __restrict__ res, unsigned* __restrict__ err) {
  const NbGlobal nb{G.col, u.nq, alpha, nullptr};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.n_rows; r += (int64_t)gridDim.x * blockDim.x)
    low_row<B, LAMIN, MINB>(r, G, C, St, u, alpha, dmu, w, res, err, nb);
}

template <int B, bool LAMIN, int MINB>
__global__ void __launch_bounds__(256, MINB) k_low_tile(Graph G, const InstConst* __restrict__ C,
                                                        const InstState* __restrict__ St, StateMix u,
                                                        const float* __restrict__ alpha, float2* __restrict__ dmu,
                                                        WorkMix w, float* __restrict__ res, unsigned* __restrict__ err,
                                                        TileCtl tc) {
  extern __shared__ float4 tile_mem[];
  const TileSmem sm = tile_smem(tile_mem, tc.tile_rows + tc.halo_cap);
  const int64_t t0 = stage_tile<true, false>(G, tc, u, alpha, nullptr, sm);
  const int64_t t1 = tile_end(G, tc, t0);
  const NbTile nb{tc.loc, sm.nq, sm.aux, nullptr, t0};
  for (int64_t r = t0 + threadIdx.x; r < t1; r += blockDim.x)
    low_row<B, LAMIN, MINB>(r, G, C, St, u, alpha, dmu, w, res, err, nb);
}

// Limiter margin: (1 - 2^-18) Q^-.  Between the limiter and the depth update
// the negative part of sum_j l_ij f_ij passes through at most ~12 FP32
// roundings (h^L to FP32, m and dt and their reciprocals, two products here,
// the quotient, R P, the row sum and dt/m times it in k_update_mix), each at
// most 2^-24 relative, so (1 - 2^-18)(1 + 2^-24)^12 < 1 and the update never
// removes more than h^L from a node.
constexpr float kLimiterShrink = 1.0f - 3.814697265625e-6f;

// k_fct_mix: f_ij and the limiter R^-_i (fct.f90:15-30): P^- = sum f^- - 1e-15,
// Q^- = -m h^L/dt, R^- = min(Q^-/P^-, 1), 0 where m h^L/dt <= htiny.  Also
// stores R^-_i P_i (the limited negative part of the h-row, reused by the
// update).
template <int B, class Nb>
__device__ __forceinline__ void fct_row(int64_t r, Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St, StateMix u,
                          const float2* __restrict__ dmu, WorkMix w, const float* __restrict__ res,
                          unsigned* __restrict__ err, const Nb& nb) {
  const int L = G.len[r];
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const InstState& st = St[b];
  if (st.done) return;
  const InstConst& c = C[b];
  if (c.visc != VISC_FCT) return;
  const int64_t base = entry_base(G, r);
  const float4 ni = u.nq[r];
  const float hi = ni.x, zi = ni.w, resi = res[r];
  const float invhi = inv_pos(hi);
  float neg = 0.f;                       // f_ii = 0 adds nothing
  for (int k0 = 0; k0 < L; k0 += B) {
    int jb[B];
    float d0b[B], m0b[B];
#pragma unroll
    for (int q = 0; q < B; q++) {
      if (k0 + q < L) {
        const int64_t e = base + 32 * (k0 + q);
        jb[q] = nb.index(e); const float2 v = dmu[e]; d0b[q] = v.x; m0b[q] = v.y;
      } else {
        jb[q] = nb.self(r); d0b[q] = 0.f; m0b[q] = 0.f;
      }
    }
    float4 njb[B];
    float rsb[B];
#pragma unroll
    for (int q = 0; q < B; q++) { njb[q] = nb.nq[jb[q]]; rsb[q] = nb.aux[jb[q]]; }
#pragma unroll
    for (int q = 0; q < B; q++) {
      if (k0 + q >= L) break;
      const float d0 = d0b[q], m0 = m0b[q], rij = fmaxf(resi, rsb[q]);
      const float4 nj = njb[q];
      const Recon R = recon(hi, nj.x, nj.w - zi, invhi, inv_pos(nj.x));
      const float f = fct_from(fminf(d0, rij) - d0, fminf(m0, rij) - m0, hi, nj.x, R);
      if (f < 0.f) neg = __fadd_rn(neg, f);
    }
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
  w.rneg[r] = __fmul_rn(R, neg);
}

template <int B>
__global__ void __launch_bounds__(256) k_fct_mix(Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                                                 StateMix u, const float2* __restrict__ dmu, WorkMix w,
                                                 const float* __restrict__ res, unsigned* __restrict__ err) {
  const NbGlobal nb{G.col, u.nq, res, nullptr};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.n_rows; r += (int64_t)gridDim.x * blockDim.x)
    fct_row<B>(r, G, C, St, u, dmu, w, res, err, nb);
}

template <int B>
__global__ void __launch_bounds__(256) k_fct_tile(Graph G, const InstConst* __restrict__ C,
                                                  const InstState* __restrict__ St, StateMix u,
                                                  const float2* __restrict__ dmu, WorkMix w,
                                                  const float* __restrict__ res, unsigned* __restrict__ err, TileCtl tc) {
  extern __shared__ float4 tile_mem[];
  const TileSmem sm = tile_smem(tile_mem, tc.tile_rows + tc.halo_cap);
  const int64_t t0 = stage_tile<true, false>(G, tc, u, res, nullptr, sm);
  const int64_t t1 = tile_end(G, tc, t0);
  const NbTile nb{tc.loc, sm.nq, sm.aux, nullptr, t0};
  for (int64_t r = t0 + threadIdx.x; r < t1; r += blockDim.x) fct_row<B>(r, G, C, St, u, dmu, w, res, err, nb);
}

// End of a stage for one row: non-finite check, the SSP-RK combination and
// bdy of the time loop (main.f90:77-90) when rk_stage > 0, and the store.
__device__ __forceinline__ void finish_mix(const Graph& G, const InstConst& c, int64_t r, int S, float2 hn, float q1,
                                           float q2, float q3, float q4, float zi, int rk_stage, const StateMix& u0,
                                           const StateMix& out, unsigned* err) {
  if (!(hn.x == hn.x) || !(q1 == q1) || !(q2 == q2)) atomicOr(err, ERRB_NAN);
  if (rk_stage >= 2) {
    const float4 a0 = u0.nq[r];
    const float2 h0 = u0.h[r];
    if (rk_stage == 2) {
      hn = df_scale(df_add(df_mul_f(h0, 3.f), hn), 0.25f);
      q1 = (3.f * a0.y + q1) * 0.25f;
      q2 = (3.f * a0.z + q2) * 0.25f;
      if (S == 5) { q3 = (3.f * u0.q3[r] + q3) * 0.25f; q4 = (3.f * u0.q4[r] + q4) * 0.25f; }
    } else {
      hn = df_div3(df_add(h0, df_scale(hn, 2.f)));
      q1 = (a0.y + 2.f * q1) * (1.f / 3.f);
      q2 = (a0.z + 2.f * q2) * (1.f / 3.f);
      if (S == 5) { q3 = (u0.q3[r] + 2.f * q3) * (1.f / 3.f); q4 = (u0.q4[r] + 2.f * q4) * (1.f / 3.f); }
    }
  }
  if (rk_stage >= 1 && G.dir_mask) {
    const unsigned msk = G.dir_mask[r];
    if (msk) {
      if (msk & 1u) hn = df_from_double(G.dir_val[r]);
      if (msk & 2u) q1 = (float)G.dir_val[G.n_rows + r];
      if (msk & 4u) q2 = (float)G.dir_val[2 * G.n_rows + r];
      if (S == 5 && (msk & 8u)) q3 = (float)G.dir_val[3 * G.n_rows + r];
      if (S == 5 && (msk & 16u)) q4 = (float)G.dir_val[4 * G.n_rows + r];
    }
  }
  out.h[r] = hn;
  out.nq[r] = make_float4(shadow_df(hn, c), q1, q2, zi);
  if (S == 5) { out.q3[r] = q3; out.q4[r] = q4; }
}

// k_update_mix: limited antidiffusion (update.f90:276-282, apply_viscosity
// :684-718), RK combination and Dirichlet data (main.f90:77-90).  The h-row
// sum is R^-_i P_i (from k_fct_mix) plus sum_{f_ij >= 0} R^-_j f_ij.
template <int B, class Nb>
__device__ __forceinline__ void update_row(int64_t r, Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                             StateMix u, const float2* __restrict__ dmu, WorkMix w,
                             const float* __restrict__ res, StateMix u0, StateMix out, int rk_stage,
                             unsigned* __restrict__ err, const Nb& nb) {
  const int L = G.len[r];
  if (L == 0) return;
  const int b = G.slice_inst[r >> 5];
  const InstState& st = St[b];
  if (st.done) return;
  const InstConst& c = C[b];
  const int S = Nb::kGlobal ? c.S : 3;
  const float4 ni = u.nq[r];
  if (c.visc != VISC_FCT) {                     // 'galerkin' / 'viscous': u^L is the result
    const float2 qL = w.qL[r];
    finish_mix(G, c, r, S, w.hL[r], qL.x, qL.y, S == 5 ? w.q3L[r] : 0.f, S == 5 ? w.q4L[r] : 0.f, ni.w, rk_stage,
               u0, out, err);
    return;
  }
  const int64_t base = entry_base(G, r);
  const float hi = ni.x, zi = ni.w, resi = res[r];
  const float invhi = inv_pos(hi);
  const float Ri = w.rminus[r];
  float ui3 = 0.f, ui4 = 0.f;
  if (S == 5) { ui3 = u.q3[r]; ui4 = u.q4[r]; }
  float pos = 0.f;                       // sum_{f >= 0} R_j f_ij
  float x1 = 0.f, x2 = 0.f, x3 = 0.f, x4 = 0.f;
  for (int k0 = 0; k0 < L; k0 += B) {    // the diagonal's terms vanish: u_i rat_ii - u_i rat_ii = 0
   int jb[B];
   float d0b[B], m0b[B];
#pragma unroll
   for (int q = 0; q < B; q++) {
     if (k0 + q < L) {
       const int64_t e = base + 32 * (k0 + q);
       jb[q] = nb.index(e); const float2 v = dmu[e]; d0b[q] = v.x; m0b[q] = v.y;
     } else {
       jb[q] = nb.self(r); d0b[q] = 0.f; m0b[q] = 0.f;
     }
   }
   float4 njb[B];
   float rsb[B], Rjb[B];
#pragma unroll
   for (int q = 0; q < B; q++) { njb[q] = nb.nq[jb[q]]; rsb[q] = nb.aux[jb[q]]; Rjb[q] = nb.R[jb[q]]; }
#pragma unroll
   for (int q = 0; q < B; q++) {
    if (k0 + q >= L) break;
    const float4 nj = njb[q];
    const float d0 = d0b[q], m0 = m0b[q];
    const float rij = fmaxf(resi, rsb[q]);
    const float ddr = fminf(d0, rij) - d0, dmr = fminf(m0, rij) - m0;
    const Recon R = recon(hi, nj.x, nj.w - zi, invhi, inv_pos(nj.x));
    const float f = fct_from(ddr, dmr, hi, nj.x, R);
    float lf = Ri;
    if (f >= 0.f) { lf = Rjb[q]; pos = __fmaf_rn(lf, f, pos); }
    // l (dd (u_j rat_ji - u_i rat_ij) + dm (u_j (1 - rat_ji) - u_i (1 - rat_ij)))
    // = l (dm (u_j - u_i) + (dd - dm) (u_j rat_ji - u_i rat_ij))
    const float dm = dmr * lf, dx = (ddr - dmr) * lf;
    x1 += dm * (nj.y - ni.y) + dx * (nj.y * R.rji - ni.y * R.rij);
    x2 += dm * (nj.z - ni.z) + dx * (nj.z * R.rji - ni.z * R.rij);
    if constexpr (Nb::kGlobal) {
      if (S == 5) {
        const int j = jb[q];
        const float uj3 = u.q3[j], uj4 = u.q4[j];
        x3 += dm * (uj3 - ui3) + dx * (uj3 * R.rji - ui3 * R.rij);
        x4 += dm * (uj4 - ui4) + dx * (uj4 * R.rji - ui4 * R.rij);
      }
    }
   }
  }
  const float invm = G.inv_lumpedf[r], dtf = st.dtf;
  const float sh = __fadd_rn(w.rneg[r], pos);
  const float2 hn = df_add_f(w.hL[r], __fmul_rn(__fmul_rn(dtf, invm), sh));
  const float2 qL = w.qL[r];
  const float q1 = qL.x + dtf * (x1 * invm);
  const float q2 = qL.y + dtf * (x2 * invm);
  float q3 = 0.f, q4 = 0.f;
  if (S == 5) { q3 = w.q3L[r] + dtf * (x3 * invm); q4 = w.q4L[r] + dtf * (x4 * invm); }
  if (hn.x < 0.f) atomicOr(err, ERRB_NEG_H);   // check_hmin (update.f90:285)
  finish_mix(G, c, r, S, hn, q1, q2, q3, q4, zi, rk_stage, u0, out, err);
}

template <int B>
__global__ void __launch_bounds__(256) k_update_mix(Graph G, const InstConst* __restrict__ C, const InstState* __restrict__ St,
                                                    StateMix u, const float2* __restrict__ dmu, WorkMix w,
                                                    const float* __restrict__ res, StateMix u0, StateMix out,
                                                    int rk_stage, unsigned* __restrict__ err) {
  const NbGlobal nb{G.col, u.nq, res, w.rminus};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.n_rows; r += (int64_t)gridDim.x * blockDim.x)
    update_row<B>(r, G, C, St, u, dmu, w, res, u0, out, rk_stage, err, nb);
}

template <int B>
__global__ void __launch_bounds__(256) k_update_tile(Graph G, const InstConst* __restrict__ C,
                                                     const InstState* __restrict__ St, StateMix u,
                                                     const float2* __restrict__ dmu, WorkMix w,
                                                     const float* __restrict__ res, StateMix u0, StateMix out,
                                                     int rk_stage, unsigned* __restrict__ err, TileCtl tc) {
  extern __shared__ float4 tile_mem[];
  const TileSmem sm = tile_smem(tile_mem, tc.tile_rows + tc.halo_cap);
  const int64_t t0 = stage_tile<true, true>(G, tc, u, res, w.rminus, sm);
  const int64_t t1 = tile_end(G, tc, t0);
  const NbTile nb{tc.loc, sm.nq, sm.aux, sm.R, t0};
  for (int64_t r = t0 + threadIdx.x; r < t1; r += blockDim.x)
    update_row<B>(r, G, C, St, u, dmu, w, res, u0, out, rk_stage, err, nb);
}

// k_dt_mix: FP32 lambda_max, max |d_ii|/m_i per instance (main.f90:166-174).
// It walks the neighbours of the state that stage 1 starts from, so it also
// stores |c_ij| lambda_max per entry (dlam, reused by stage 1's k_low_mix)
// and alpha_i (alpha_out, stage 1's k_node_mix), when those are non-null.
// One row of k_dt_mix; returns |d_ii| / m_i (0 for padding and finished rows).
template <int B, class Nb>
__device__ __forceinline__ float dt_row(int64_t r, const Graph& G, const InstConst* __restrict__ C,
                                        const InstState* __restrict__ St, const StateMix& u, float* __restrict__ dlam,
                                        float* __restrict__ alpha_out, unsigned* __restrict__ err, const Nb& nb) {
  if (r >= G.n_rows || G.len[r] == 0) return 0.f;
  const int b = G.slice_inst[r >> 5];
  if (St[b].done) return 0.f;
  const InstConst& c = C[b];
  const float g = c.gf, htiny = c.htinyf;
  const LamK lk = lam_k(g, htiny);
  const int L = G.len[r];
  const int64_t base = entry_base(G, r);
  const NodeF ni = node_from(u.nq[r], htiny);
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
        const int64_t e = base + 32 * (k0 + q);
        jb[q] = nb.index(e); cxb[q] = G.cxf[e]; cyb[q] = G.cyf[e];
      } else {
        jb[q] = nb.self(r); cxb[q] = 1.f; cyb[q] = 0.f;
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
      const float n2 = cxe * cxe + cye * cye;
      const float inv = rsqrtf(n2);
      float lam;
      if (!lambda_f(ni.h, nj.h, dotc(cxe, cye, ni.v1, ni.v2) * inv, dotc(cxe, cye, nj.v1, nj.v2) * inv, ni.ovh,
                    nj.ovh, sqi, sqrtf(g * fabsf(nj.h)), lk, &lam))
        bad = true;
      const float dl = (n2 * inv) * lam;
      if (dlam) dlam[base + 32 * (k0 + q)] = dl;
      s += dl;
      num += nj.h - ni.h;
      denom += fabsf(nj.h - ni.h);
    }
  }
  if (alpha_out) {
    float alpha = 1.0f;
    if (c.alpha_limit && !(ni.h <= c.htinyf)) {
      const float a = (denom <= fabsf(num)) ? 1.0f : fdiv(fabsf(num), denom);
      const float a2 = a * a, a4 = a2 * a2;
      alpha = a4 * a4;
    }
    alpha_out[r] = alpha;
  }
  if (bad) atomicOr(err, ERRB_DELTA);
  return s * G.inv_lumpedf[r];
}

// Warp max of |d_ii| / m_i into the instance's maximum (the 32 rows of a warp
// are one slice, so one instance).
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
// It walks the neighbours of the state that stage 1 starts from, so it also
// stores |c_ij| lambda_max per entry (dlam, reused by stage 1's k_low_mix)
// and alpha_i (alpha_out, stage 1's k_node_mix), when those are non-null.
template <int B>
__global__ void __launch_bounds__(256) k_dt_mix(Graph G, const InstConst* __restrict__ C, InstState* __restrict__ St, StateMix u,
                         float* __restrict__ dlam, float* __restrict__ alpha_out, unsigned* __restrict__ err) {
  // grid-stride over block-sized row ranges: every lane of a warp runs the
  // same iterations (the warp reduction needs all 32)
  const NbGlobal nb{G.col, u.nq, nullptr, nullptr};
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
  const TileSmem sm = tile_smem(tile_mem, tc.tile_rows + tc.halo_cap);
  const int64_t t0 = stage_tile<false, false>(G, tc, u, nullptr, nullptr, sm);
  const NbTile nb{tc.loc, sm.nq, nullptr, nullptr, t0};
  // tile_rows is a multiple of 32: every lane of a warp runs the same iterations
  for (int64_t rb = t0; rb < t0 + tc.tile_rows; rb += blockDim.x) {
    const int64_t r = rb + threadIdx.x;
    if (rb - t0 + (int64_t)threadIdx.x - (threadIdx.x & 31) >= tc.tile_rows) break;   // warp past the tile
    dt_reduce(dt_row<B>(r, G, C, St, u, dlam, alpha_out, err, nb), r, G, St);
  }
}

// Copy the bathymetry into the packed node records after a bathymetry change
__global__ void k_refresh_z(Graph G, StateMix u) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= G.n_rows) return;
  u.nq[r].w = G.bathf[r];
}

// Total mass sum m_i h_i per instance from the double-float depth, combined
// in double-double per warp (atomics on two words per instance).
__global__ void k_mass_mix(Graph G, const float2* __restrict__ h, double* __restrict__ acc) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double v = 0.0;
  int b = -1;
  if (r < G.n_rows && G.len[r] > 0) { b = G.slice_inst[r >> 5]; v = G.lumped[r] * df_to_double(h[r]); }
  double cmp = 0.0;
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_down_sync(0xffffffffu, v, off);
    const double oc = __shfl_down_sync(0xffffffffu, cmp, off);
    const double s = v + o;              // two-sum
    const double bb = s - v;
    const double e = (v - (s - bb)) + (o - bb);
    v = s;
    cmp = cmp + oc + e;
  }
  const int b0 = __shfl_sync(0xffffffffu, b, 0);
  if ((threadIdx.x & 31) == 0 && b0 >= 0) {
    atomicAdd(&acc[2 * b0], v);
    atomicAdd(&acc[2 * b0 + 1], cmp);
  }
}

static inline unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

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
    case 8: KERNEL<8><<<row_grid(KERNEL<8>, N, BS, MODE), BS, 0, s>>>(__VA_ARGS__); break;      \
    case 4: KERNEL<4><<<row_grid(KERNEL<4>, N, BS, MODE), BS, 0, s>>>(__VA_ARGS__); break;      \
    case 2: KERNEL<2><<<row_grid(KERNEL<2>, N, BS, MODE), BS, 0, s>>>(__VA_ARGS__); break;      \
    default: KERNEL<1><<<row_grid(KERNEL<1>, N, BS, MODE), BS, 0, s>>>(__VA_ARGS__); break;     \
  }

// Tile variants: one block per tile, shared memory for the tile's and the
// halo's node records, residuals and R^- (24 B per row)
inline size_t tile_smem_bytes(const TileCtl& tc) { return (size_t)(tc.tile_rows + tc.halo_cap) * 24; }
#define SWE_DISPATCH_TILE(b, KERNEL, BS, TC, NROWS, ...)                                                \
  do {                                                                                                \
    const TileCtl& tc_ = (TC);                                                                        \
    const unsigned g_ = (unsigned)(((NROWS) + tc_.tile_rows - 1) / tc_.tile_rows);                    \
    const size_t sm_ = tile_smem_bytes(tc_);                                                          \
    switch (b) {                                                                                      \
      case 8: KERNEL<8><<<g_, BS, sm_, s>>>(__VA_ARGS__); break;                                      \
      case 4: KERNEL<4><<<g_, BS, sm_, s>>>(__VA_ARGS__); break;                                      \
      case 2: KERNEL<2><<<g_, BS, sm_, s>>>(__VA_ARGS__); break;                                      \
      default: KERNEL<1><<<g_, BS, sm_, s>>>(__VA_ARGS__); break;                                     \
    }                                                                                                 \
  } while (0)

// k_low variants: entry batch 1 or 2, lambda_max computed or taken from
// k_dt_mix (stage 1), registers capped at 85, 64 or 51 (3, 4 or 5 resident
// blocks of 256 threads per SM; the compiler would take ~106 with no cap)
template <bool LAMIN>
static void launch_low(const StageArgsMix& a, int batch, int cap, int mode, int block, bool tiled, cudaStream_t s) {
  if (tiled && a.tiles) {
    const TileCtl& tc = *a.tiles;
    const unsigned g = (unsigned)((a.G.n_rows + tc.tile_rows - 1) / tc.tile_rows);
    const size_t sm = tile_smem_bytes(tc);
#define SWE_LOWT(BB, MB) \
    k_low_tile<BB, LAMIN, MB><<<g, block, sm, s>>>(a.G, a.C, a.St, a.u, a.w.alpha, a.w.dmu, a.w, a.w.res, a.err, tc)
    if (batch >= 2) { if (cap == 2) SWE_LOWT(2, 5); else if (cap) SWE_LOWT(2, 4); else SWE_LOWT(2, 3); }
    else { if (cap == 2) SWE_LOWT(1, 5); else if (cap) SWE_LOWT(1, 4); else SWE_LOWT(1, 3); }
#undef SWE_LOWT
    return;
  }
#define SWE_LOW(BB, MB)                                                                                  \
  k_low_mix<BB, LAMIN, MB><<<row_grid(k_low_mix<BB, LAMIN, MB>, a.G.n_rows, block, mode), block, 0, s>>>( \
      a.G, a.C, a.St, a.u, a.w.alpha, a.w.dmu, a.w, a.w.res, a.err)
  if (batch >= 2) { if (cap == 2) SWE_LOW(2, 5); else if (cap) SWE_LOW(2, 4); else SWE_LOW(2, 3); }
  else { if (cap == 2) SWE_LOW(1, 5); else if (cap) SWE_LOW(1, 4); else SWE_LOW(1, 3); }
#undef SWE_LOW
}

bool kind_has_tiles(int kind) { return kind >= 0 && kind <= 4; }

void launch_kernel_mix(int kind, const StageArgsMix& a, const KernelTune& t, cudaStream_t s) {
  const int64_t n = a.G.n_rows;
  switch (kind) {
    case 1: if (t.tiled[1] && a.tiles) {
              SWE_DISPATCH_TILE(t.batch[1], k_node_tile, t.block[1], *a.tiles, n, a.G, a.C, a.St, a.u, a.w.alpha, *a.tiles);
            } else {
              SWE_DISPATCH_B(t.batch[1], k_node_mix, n, t.block[1], t.grid[1], a.G, a.C, a.St, a.u, a.w.alpha)
            }
            break;
    case 2: if (a.rk_stage == 1 && a.w.dlam)   // stage 1 follows k_dt_mix on the same state
              launch_low<true>(a, t.batch[2], t.cap_low, t.grid[2], t.block[2], t.tiled[2], s);
            else
              launch_low<false>(a, t.batch[2], t.cap_low, t.grid[2], t.block[2], t.tiled[2], s);
            break;
    case 3: if (t.tiled[3] && a.tiles) {
              SWE_DISPATCH_TILE(t.batch[3], k_fct_tile, t.block[3], *a.tiles, n, a.G, a.C, a.St, a.u, a.w.dmu, a.w, a.w.res, a.err,
                                *a.tiles);
            } else {
              SWE_DISPATCH_B(t.batch[3], k_fct_mix, n, t.block[3], t.grid[3], a.G, a.C, a.St, a.u, a.w.dmu, a.w,
                             a.w.res, a.err)
            }
            break;
    case 4: if (t.tiled[4] && a.tiles) {
              SWE_DISPATCH_TILE(t.batch[4], k_update_tile, t.block[4], *a.tiles, n, a.G, a.C, a.St, a.u, a.w.dmu, a.w, a.w.res,
                                a.u0, a.out, a.rk_stage, a.err, *a.tiles);
            } else {
              SWE_DISPATCH_B(t.batch[4], k_update_mix, n, t.block[4], t.grid[4], a.G, a.C, a.St, a.u, a.w.dmu, a.w,
                             a.w.res, a.u0, a.out, a.rk_stage, a.err)
            }
            break;
    default: break;
  }
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

void launch_refresh_z(const Graph& G, StateMix u, cudaStream_t s) {
  k_refresh_z<<<nblk(G.n_rows, 256), 256, 0, s>>>(G, u);
}

void launch_mass_mix(const Graph& G, const float2* h, double* acc, cudaStream_t s) {
  k_mass_mix<<<nblk(G.n_rows, 256), 256, 0, s>>>(G, h, acc);
}

}  // namespace swe
