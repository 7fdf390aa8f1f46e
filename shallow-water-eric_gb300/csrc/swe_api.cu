// C-ABI layer (include/swe_gpu.h): context, device buffers, permuting
// transfers, the per-call operators mirroring MODULE update / MODULE fct, and
// the device-resident SSP-RK3 loop captured in a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/swe_gpu.h"
#include "swe_kernels.hpp"
#include "swe_setup.hpp"

#define SWE_API extern "C" __attribute__((visibility("default")))

using namespace swe;

namespace {

struct DevBuf {
  std::vector<void*> ptrs;
  template <typename T> T* alloc(size_t n, cudaError_t& st) {
    void* p = nullptr;
    if (st != cudaSuccess) return nullptr;
    st = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
    if (st == cudaSuccess) { ptrs.push_back(p); cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T)); }
    return (T*)p;
  }
  void release() { for (void* p : ptrs) cudaFree(p); ptrs.clear(); }
};

}  // namespace

struct swe_ctx {
  int dev = 0;
  cudaStream_t stream = nullptr;
  // state transfers: chunks copied on their own streams (several copy engines)
  // and permuted on `stream` as each lands
  static constexpr int kMaxCopyChunks = 8;
  cudaStream_t copy_stream[kMaxCopyChunks] = {};
  cudaEvent_t copy_ev[kMaxCopyChunks] = {}, copy_go = nullptr;
  int copy_chunks = 0;
  int n_inst = 0, S = 3, precision = 0;
  std::vector<HostMesh> meshes;
  std::vector<swe_params> params;
  Layout L;
  std::vector<int64_t> node_off;         // concatenated host node offsets, n_inst+1
  DevBuf buf;
  Graph G{};
  InstConst* d_C = nullptr;
  InstState* d_St = nullptr;
  unsigned* d_err = nullptr;
  int* d_row_of_node = nullptr;          // concatenated host node -> device row
  double* d_stage = nullptr;             // staging (S, total nodes), reference layout
  uint8_t* d_dir_mask = nullptr;
  double* d_dir_val = nullptr;
  std::vector<uint8_t> h_dir_mask;
  std::vector<double> h_dir_val;
  uint8_t* d_dir_anal = nullptr;         // analytic Dirichlet components per row (on first use)
  double* d_rr_row = nullptr;            // node coordinates per row (with d_dir_anal)
  std::vector<uint8_t> h_dir_anal;
  // FP64 path
  StateF64 A{}, B{}, Cs{};
  WorkF64 w{};
  double* d_lij = nullptr;
  // mixed path
  StateMix mA{}, mB{}, mC{};
  WorkMix wm{};
  TileCtl tiles{};                       // row tiles of the shared-memory variants
  bool tiles_ok = false;
  double* d_mass_acc = nullptr;
  double* d_mass_part = nullptr;         // per-slice partial sums of swe_mass
  int64_t* d_inst_slice = nullptr;       // n_inst + 1 slice offsets
  // diagnostics: per-instance element lists and Gauss weights, on first use
  std::vector<int*> d_jj_inst;
  std::vector<double*> d_rj_inst;
  double* d_norm_acc = nullptr;
  double* d_fanal = nullptr;
  size_t fanal_cap = 0;
  double* d_norm_part = nullptr;     // per-warp partial sums of k_norms
  size_t norm_part_cap = 0;
  // graph of `graph_steps` time steps
  cudaGraphExec_t gexec = nullptr;
  int graph_steps = 0;
  cudaGraphExec_t gexec1 = nullptr;      // one time step (the remainder of a call)
  // movie frames (swe_frame_async): device fields and page-locked host copies
  // in two slots, written to files by a worker thread
  struct FrameJob {
    int slot, inst;
    std::string paths[2];
  };
  double* d_frame = nullptr;             // 2 slots x (hpz, h) x frame_np
  double* h_frame = nullptr;             // same, page-locked
  int64_t frame_np = 0;
  cudaEvent_t frame_ev[2] = {};
  bool frame_busy[2] = {false, false};
  std::vector<std::vector<int>> jj1;     // 1-based element lists per instance (writer input)
  std::deque<FrameJob> frame_queue;
  std::thread frame_worker;
  std::mutex frame_mu;
  std::condition_variable frame_cv;
  bool frame_stop = false;
  int frame_err = 0;
  std::string frame_errmsg;
  // gauges (main.f90:102-117): per gauge its instance, the device rows of its
  // element's three nodes and the P1 weights there; a device ring of
  // (time, h, h + bath) rows appended by k_gauges at the end of every step
  int n_gauges = 0;
  int* d_gauge_inst = nullptr;
  int* d_gauge_rows = nullptr;           // 3 per gauge
  double* d_gauge_w = nullptr;           // 3 per gauge
  double* d_gauge_rec = nullptr;         // kGaugeRing x n_gauges x 3
  unsigned long long* d_gauge_count = nullptr;
  unsigned long long gauge_read = 0;     // rows handed to the caller so far
  static constexpr int kGaugeRing = 4096;
  int block = 128;
  KernelTune tune;
  bool tuned = false;
  long long last_launches = 0;
  double last_ms = 0.0;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  bool euler_done = false;
  int euler_inst = -1;
  std::string err;
  std::string tuning = "thread-per-row SELL-32, block 128";
};

// NVTX range over an API call (host timeline in nsys / ncu; no cost without a tool)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

static int fail(swe_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

static int cuda_check(swe_ctx* c, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return SWE_OK;
  return fail(c, SWE_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(expr)                                                   \
  do {                                                             \
    int _rc = cuda_check(c, (expr), #expr);                        \
    if (_rc) return _rc;                                           \
  } while (0)

// mixed contexts: SWE_PREC_MIXED and its FP64 precision split share the
// FP32 data layout and kernels
static bool is_mixed(const swe_ctx* c) { return c->precision != SWE_PREC_FP64; }
static bool is_split(const swe_ctx* c) { return c->precision == SWE_PREC_MIXED_F64; }

static InstConst make_const(const swe_params& p) {
  InstConst k{};
  k.g = p.gravity; k.htiny = p.htiny; k.cfl = p.cfl; k.mannings = p.mannings; k.lambda_sgn = p.lambda_sgn;
  // Malpasset (type 9): the time loop sets htiny = 1e-3 before every step
  // (main.f90:67-68), so every euler call of that case sees it
  if (p.type_test == 9) k.htiny = 1.e-3;
  k.max_water_h = p.max_water_h;
  k.rescale_floor = 1.e-10 * p.gravity * (p.max_water_h * p.max_water_h);   // update.f90:866
  k.type_test = p.type_test; k.S = p.syst_size; k.visc = p.viscosity_type; k.viscous_type = p.viscous_type;
  k.alpha_limit = p.if_alpha_limit; k.roundoff_fix = p.if_roundoff_fix;
  k.gf = (float)k.g;
  k.htinyf = (float)k.htiny;
  k.htiny_lo = (float)(k.htiny - (double)k.htinyf);
  k.fricf = (float)(k.g * k.mannings * k.mannings);
  k.lambda_sgnf = (float)k.lambda_sgn;
  k.rescale_floorf = (float)k.rescale_floor;
  return k;
}

// some instance runs 'viscous' with viscous_type 'type1' (the mixed path's k_low_type1)
static bool has_type1(const swe_ctx* c) {
  for (const auto& p : c->params)
    if (p.viscous_type == 1 && p.viscosity_type == SWE_VISC_VISCOUS) return true;
  return false;
}

static bool has_entropy(const swe_ctx* c) {
  for (const swe_params& p : c->params)
    if (p.viscosity_type == SWE_VISC_ENTROPY) return true;
  return false;
}

static int check_params(swe_ctx* c, const swe_params& p) {
  if (p.syst_size != 3 && p.syst_size != 5) return fail(c, SWE_ERR_ARG, "syst_size must be 3 or 5");
  if ((p.syst_size == 5) != (p.type_test == 13)) return fail(c, SWE_ERR_ARG, "syst_size 5 goes with type_test 13");
  if (!p.if_lumped) return fail(c, SWE_ERR_ARG, "only the lumped-mass step is supported (if_lumped)");
  if (p.viscosity_type < SWE_VISC_GALERKIN || p.viscosity_type > SWE_VISC_FCT)
    return fail(c, SWE_ERR_ARG, "viscosity_type must be galerkin, viscous, entropy_visc or fct");
  if (p.viscous_type != 1 && p.viscous_type != 2) return fail(c, SWE_ERR_ARG, "viscous_type must be 1 or 2");
  // the reference STOPs on these combinations (update.f90:244-245, 264-266)
  if (p.viscous_type == 1 && p.viscosity_type == SWE_VISC_ENTROPY)
    return fail(c, SWE_ERR_ARG, "Bug: entropy viscosity programmed only with type 2");
  if (p.viscous_type == 1 && p.viscosity_type == SWE_VISC_FCT)
    return fail(c, SWE_ERR_ARG, "BUG: FCT programmed with type2 only");
  if (p.precision != SWE_PREC_FP64 && p.precision != SWE_PREC_MIXED && p.precision != SWE_PREC_MIXED_F64)
    return fail(c, SWE_ERR_ARG, "bad precision");
  if (p.precision != SWE_PREC_FP64 && p.viscous_type == 1 && p.viscosity_type == SWE_VISC_VISCOUS &&
      p.syst_size != 3)
    return fail(c, SWE_ERR_ARG, "mixed precision builds 'viscous' with 'type1' for 3-component systems");
  if (!(p.htiny >= 0.0) || !(p.gravity > 0.0)) return fail(c, SWE_ERR_ARG, "gravity must be > 0, htiny >= 0");
  return SWE_OK;
}

static int alloc_state_f64(swe_ctx* c, StateF64& s, cudaError_t& st) {
  const size_t n = c->L.n_rows;
  s.h = c->buf.alloc<double>(n, st); s.q1 = c->buf.alloc<double>(n, st); s.q2 = c->buf.alloc<double>(n, st);
  if (c->S == 5) { s.q3 = c->buf.alloc<double>(n, st); s.q4 = c->buf.alloc<double>(n, st); }
  return st == cudaSuccess ? SWE_OK : SWE_ERR_CUDA;
}

static int alloc_state_mix(swe_ctx* c, StateMix& s, cudaError_t& st) {
  const size_t n = c->L.n_rows;
  s.h = c->buf.alloc<float2>(n, st);
  s.nq = c->buf.alloc<float4>(n, st);
  if (c->S == 5) { s.q3 = c->buf.alloc<float>(n, st); s.q4 = c->buf.alloc<float>(n, st); }
  return st == cudaSuccess ? SWE_OK : SWE_ERR_CUDA;
}

template <typename T>
static T* upload_vec(swe_ctx* c, const std::vector<T>& v, cudaError_t& st) {
  T* d = c->buf.alloc<T>(v.size(), st);
  if (st == cudaSuccess && !v.empty()) st = cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return d;
}

// Bathymetry as a double-float pair hi + lo (hi = z rounded to FP32): the
// mixed kernels form the free surface eta = h + z from it.
static float2 bath_df(double z) {
  const float hi = (float)z;
  return make_float2(hi, (float)(z - (double)hi));
}

static int build_device(swe_ctx* c, const std::vector<std::vector<double>>& baths) {
  c->L = build_layout(c->meshes, baths);
  const Layout& L = c->L;
  cudaError_t st = cudaSuccess;
  Graph& G = c->G;
  G.n_rows = L.n_rows;
  G.slice_ptr = upload_vec(c, L.slice_ptr, st);
  G.slice_inst = upload_vec(c, L.slice_inst, st);
  G.col = upload_vec(c, L.col, st);
  G.len = upload_vec(c, L.len, st);
  G.dpos = upload_vec(c, L.dpos, st);
  G.lumped = upload_vec(c, L.lumped, st);
  std::vector<double> inv(L.n_rows);
  for (int64_t r = 0; r < L.n_rows; r++) inv[r] = 1.0 / L.lumped[r];
  G.inv_lumped = upload_vec(c, inv, st);
  if (is_mixed(c)) {
    std::vector<float> lf(L.n_rows), ilf(L.n_rows);
    for (int64_t r = 0; r < L.n_rows; r++) { lf[r] = (float)L.lumped[r]; ilf[r] = (float)inv[r]; }
    G.lumpedf = upload_vec(c, lf, st);
    G.inv_lumpedf = upload_vec(c, ilf, st);
  }
  G.bath = upload_vec(c, L.bath, st);
  if (c->precision == SWE_PREC_FP64) {
    G.cx = upload_vec(c, L.cx, st);
    G.cy = upload_vec(c, L.cy, st);
    {   // compute_dij's norm = SQRT(c.c) and normal c/norm per entry (update.f90:309-312),
        // the same IEEE operations as a kernel would do per use
      std::vector<double> nrm(L.n_entries), nx(L.n_entries), ny(L.n_entries);
      for (int64_t e = 0; e < L.n_entries; e++) {
        const double cx = L.cx[e], cy = L.cy[e];
        const double cc = cx * cx + cy * cy;
        nrm[e] = std::sqrt(cc);
        nx[e] = cx / nrm[e];                       // padding entries (never read): 0/0
        ny[e] = cy / nrm[e];
      }
      G.cnorm = upload_vec(c, nrm, st);
      G.cnx = upload_vec(c, nx, st);
      G.cny = upload_vec(c, ny, st);
    }
    G.cxii = upload_vec(c, L.cxii, st);
    G.cyii = upload_vec(c, L.cyii, st);
  } else {
    std::vector<float2> f(L.n_entries);
    for (int64_t e = 0; e < L.n_entries; e++) f[e] = make_float2((float)L.cx[e], (float)L.cy[e]);
    G.cf = upload_vec(c, f, st);
    std::vector<float> fr(L.n_rows);
    for (int64_t r = 0; r < L.n_rows; r++) fr[r] = (float)L.cxii[r];
    G.cxiif = upload_vec(c, fr, st);
    for (int64_t r = 0; r < L.n_rows; r++) fr[r] = (float)L.cyii[r];
    G.cyiif = upload_vec(c, fr, st);
    std::vector<float2> bdf(L.n_rows);
    for (int64_t r = 0; r < L.n_rows; r++) bdf[r] = bath_df(L.bath[r]);
    G.bathdf = upload_vec(c, bdf, st);
  }
  c->h_dir_mask.assign(L.n_rows, 0);
  c->h_dir_val.assign((size_t)c->S * L.n_rows, 0.0);
  c->d_dir_mask = c->buf.alloc<uint8_t>(L.n_rows, st);
  c->d_dir_val = c->buf.alloc<double>((size_t)c->S * L.n_rows, st);
  G.dir_mask = c->d_dir_mask;
  G.dir_val = c->d_dir_val;
  // per-instance constants and state
  std::vector<InstConst> hc(c->n_inst);
  std::vector<InstState> hs(c->n_inst);
  for (int b = 0; b < c->n_inst; b++) {
    hc[b] = make_const(c->params[b]);
    hs[b] = InstState{};
    inst_set_dt(hs[b], c->params[b].dt);
    hs[b].t_final = 1e300;
  }
  c->d_C = upload_vec(c, hc, st);
  c->d_St = upload_vec(c, hs, st);
  c->d_err = c->buf.alloc<unsigned>(1, st);
  // host node -> device row map, staging buffer
  c->node_off.assign(c->n_inst + 1, 0);
  for (int b = 0; b < c->n_inst; b++) c->node_off[b + 1] = c->node_off[b] + c->meshes[b].np;
  std::vector<int> row_of_node(c->node_off[c->n_inst]);
  for (int b = 0; b < c->n_inst; b++)
    for (int i = 0; i < c->meshes[b].np; i++) row_of_node[c->node_off[b] + i] = L.new_of_old[b][i];
  c->d_row_of_node = upload_vec(c, row_of_node, st);
  c->d_stage = c->buf.alloc<double>((size_t)c->S * c->node_off[c->n_inst], st);
  c->d_mass_acc = c->buf.alloc<double>(2 * (size_t)c->n_inst, st);
  c->d_mass_part = c->buf.alloc<double>(2 * (size_t)L.n_slices, st);
  {
    std::vector<int64_t> inst_slice(c->n_inst + 1);
    for (int b = 0; b <= c->n_inst; b++) inst_slice[b] = L.row_off[b] / 32;
    c->d_inst_slice = upload_vec(c, inst_slice, st);
  }
  const size_t n = L.n_rows, ne = L.n_entries;
  if (c->precision == SWE_PREC_FP64) {
    alloc_state_f64(c, c->A, st); alloc_state_f64(c, c->B, st); alloc_state_f64(c, c->Cs, st);
    WorkF64& w = c->w;
    w.ovh = c->buf.alloc<double>(n, st); w.v1 = c->buf.alloc<double>(n, st); w.v2 = c->buf.alloc<double>(n, st);
    w.ent = c->buf.alloc<double>(n, st); w.alpha = c->buf.alloc<double>(n, st);
    w.sqgh = c->buf.alloc<double>(n, st);
    w.dL = c->buf.alloc<double>(ne, st); w.muL = c->buf.alloc<double>(ne, st); w.fct = c->buf.alloc<double>(ne, st);
    w.dLii = c->buf.alloc<double>(n, st); w.muLii = c->buf.alloc<double>(n, st);
    w.res = c->buf.alloc<double>(n, st); w.rminus = c->buf.alloc<double>(n, st);
    alloc_state_f64(c, w.uL, st);
    c->d_lij = c->buf.alloc<double>(ne, st);
  } else {
    alloc_state_mix(c, c->mA, st); alloc_state_mix(c, c->mB, st); alloc_state_mix(c, c->mC, st);
    WorkMix& w = c->wm;
    w.alpha = c->buf.alloc<float>(n, st); w.res = c->buf.alloc<float>(n, st);
    w.rminus = c->buf.alloc<float>(n, st);
    w.dmu = c->buf.alloc<float2>(ne, st);
    w.dlam = c->buf.alloc<float>(ne, st);
    w.hL = c->buf.alloc<float2>(n, st);
    if (is_split(c)) {     // FP64 low-order depth in hL's 8 bytes per row, FP64 R^-
      w.hL64 = reinterpret_cast<double*>(w.hL);
      w.rminus64 = c->buf.alloc<double>(n, st);
    }
    w.qL = c->buf.alloc<float2>(n, st);
    if (c->S == 5) { w.q3L = c->buf.alloc<float>(n, st); w.q4L = c->buf.alloc<float>(n, st); }
    // row tiles of the shared-memory kernel variants (SWE_TILE rows, default
    // 256; 0 disables), while the tile and its halo fit in 48 KB
    const char* ft = getenv("SWE_TILE");
    const int tile = ft ? atoi(ft) : 256;
    RowTiles F;
    TileCtl probe{};
    if (c->S == 3 && tile > 0 && build_row_tiles(L, tile, F) &&
        (probe.tile_rows = F.tile, probe.halo_cap = F.halo_cap, tile_smem_bytes(probe, true) <= 48 * 1024)) {
      c->tiles.loc = upload_vec(c, F.loc, st);
      c->tiles.halo_ptr = upload_vec(c, F.halo_ptr, st);
      c->tiles.halo_rows = upload_vec(c, F.halo_rows, st);
      c->tiles.tile_rows = F.tile;
      c->tiles.halo_cap = F.halo_cap;
      c->tiles_ok = true;
    }
  }
  if (st != cudaSuccess) return fail(c, SWE_ERR_CUDA, std::string("device allocation: ") + cudaGetErrorString(st));
  return SWE_OK;
}

// ---- permuting transfers (reference layout <-> SoA device rows) ----
__global__ void k_scatter_in(const double* __restrict__ stage, const int* __restrict__ row_of_node, int64_t n_nodes,
                             int S, StateF64 a) {
  int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  const int64_t r = row_of_node[n];
  double* comp[5] = {a.h, a.q1, a.q2, a.q3, a.q4};
  for (int k = 0; k < S; k++) comp[k][r] = stage[n * S + k];
}
__global__ void k_gather_out(double* __restrict__ stage, const int* __restrict__ row_of_node, int64_t n_nodes, int S,
                             StateF64 a) {
  int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  const int64_t r = row_of_node[n];
  const double* comp[5] = {a.h, a.q1, a.q2, a.q3, a.q4};
  for (int k = 0; k < S; k++) stage[n * S + k] = comp[k][r];
}
__global__ void k_scatter_in_mix(const double* __restrict__ stage, const int* __restrict__ row_of_node,
                                 int64_t n_nodes, int S, StateMix a, const int* __restrict__ slice_inst,
                                 const InstConst* __restrict__ C, const float2* __restrict__ bathdf) {
  int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  const int64_t r = row_of_node[n];
  const double h = stage[n * S];
  const float2 hdf = df_from_double(h);
  a.h[r] = hdf;
  // free surface eta = h + z rounded once, as the stage kernels form it
  a.nq[r] = make_float4(shadow_depth(h, C[slice_inst[r >> 5]].htiny), (float)stage[n * S + 1],
                        (float)stage[n * S + 2], df_add(hdf, bathdf[r]).x);
  if (S == 5) { a.q3[r] = (float)stage[n * S + 3]; a.q4[r] = (float)stage[n * S + 4]; }
}
// mixed state (sm) or the mixed low-order state (w) back to the reference layout
__global__ void k_gather_out_mix(double* __restrict__ stage, const int* __restrict__ row_of_node, int64_t n_nodes,
                                 int S, StateMix a, WorkMix w, int low) {
  int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  const int64_t r = row_of_node[n];
  if (!low) {
    const float4 v = a.nq[r];
    stage[n * S] = df_to_double(a.h[r]);
    stage[n * S + 1] = v.y;
    stage[n * S + 2] = v.z;
    if (S == 5) { stage[n * S + 3] = a.q3[r]; stage[n * S + 4] = a.q4[r]; }
  } else {
    const float2 v = w.qL[r];
    stage[n * S] = w.hL64 ? w.hL64[r] : df_to_double(w.hL[r]);
    stage[n * S + 1] = v.x;
    stage[n * S + 2] = v.y;
    if (S == 5) { stage[n * S + 3] = w.q3L[r]; stage[n * S + 4] = w.q4L[r]; }
  }
}

// Node ranges of the transfer chunks: k of `chunks` equal parts of [b, e).
static inline int64_t chunk_at(int64_t b, int64_t e, int k, int chunks) { return b + (e - b) * k / chunks; }

// Copy streams and events on first use (SWE_COPY_CHUNKS, default 4, 1..8).
static int copy_setup(swe_ctx* c) {
  if (c->copy_chunks) return SWE_OK;
  const char* env = getenv("SWE_COPY_CHUNKS");
  int k = env ? atoi(env) : 4;
  k = std::max(1, std::min(k, (int)swe_ctx::kMaxCopyChunks));
  for (int i = 0; i < k; i++) {
    CK(cudaStreamCreateWithFlags(&c->copy_stream[i], cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->copy_ev[i], cudaEventDisableTiming));
  }
  CK(cudaEventCreateWithFlags(&c->copy_go, cudaEventDisableTiming));
  c->copy_chunks = k;
  return SWE_OK;
}

// Waits for every copy stream and the context's stream: after an error, so
// that no transfer still reads or writes a caller's buffer once the call has
// returned.
static void drain(swe_ctx* c) {
  for (int k = 0; k < c->copy_chunks; k++) cudaStreamSynchronize(c->copy_stream[k]);
  cudaStreamSynchronize(c->stream);
}

static int to_device(swe_ctx* c, const double* un, bool device_src, int64_t node_begin, int64_t node_end) {
  const int64_t nn = node_end - node_begin;
  if (nn <= 0) return SWE_OK;
  int rc = copy_setup(c);
  if (rc) return rc;
  const int K = nn >= 1024 ? c->copy_chunks : 1;
  // chunk k: copy on copy_stream[k] (after the work already on `stream`),
  // then its permutation into the rows on `stream` once it has landed
  CK(cudaEventRecord(c->copy_go, c->stream));
  for (int k = 0; k < K; k++) {
    const int64_t b = chunk_at(node_begin, node_end, k, K), e = chunk_at(node_begin, node_end, k + 1, K);
    CK(cudaStreamWaitEvent(c->copy_stream[k], c->copy_go, 0));
    CK(cudaMemcpyAsync(c->d_stage + (size_t)c->S * b, un + (size_t)c->S * (b - node_begin),
                       (size_t)c->S * (e - b) * sizeof(double),
                       device_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->copy_stream[k]));
    CK(cudaEventRecord(c->copy_ev[k], c->copy_stream[k]));
  }
  for (int k = 0; k < K; k++) {
    const int64_t b = chunk_at(node_begin, node_end, k, K), e = chunk_at(node_begin, node_end, k + 1, K);
    CK(cudaStreamWaitEvent(c->stream, c->copy_ev[k], 0));
    const unsigned nb = (unsigned)((e - b + 255) / 256);
    if (nb == 0) continue;
    if (c->precision == SWE_PREC_FP64)
      k_scatter_in<<<nb, 256, 0, c->stream>>>(c->d_stage + (size_t)c->S * b, c->d_row_of_node + b, e - b, c->S, c->A);
    else
      k_scatter_in_mix<<<nb, 256, 0, c->stream>>>(c->d_stage + (size_t)c->S * b, c->d_row_of_node + b, e - b, c->S,
                                                   c->mA, c->G.slice_inst, c->d_C, c->G.bathdf);
    CK(cudaGetLastError());
  }
  return SWE_OK;
}

static int from_device_state(swe_ctx* c, double* un, bool device_dst, int64_t node_begin, int64_t node_end,
                             const StateF64* sf, const StateMix* sm, bool low_mix = false) {
  const int64_t nn = node_end - node_begin;
  if (nn <= 0) return SWE_OK;
  int rc = copy_setup(c);
  if (rc) return rc;
  const int K = nn >= 1024 ? c->copy_chunks : 1;
  // chunk k: gathered into reference order on `stream`, then copied out on
  // copy_stream[k] while the next chunk is gathered; `stream` waits for every
  // copy, so the caller's synchronisation on it covers the transfer
  for (int k = 0; k < K; k++) {
    const int64_t b = chunk_at(node_begin, node_end, k, K), e = chunk_at(node_begin, node_end, k + 1, K);
    const unsigned nb = (unsigned)((e - b + 255) / 256);
    double* stg = c->d_stage + (size_t)c->S * b;
    if (nb) {
      if (sf) k_gather_out<<<nb, 256, 0, c->stream>>>(stg, c->d_row_of_node + b, e - b, c->S, *sf);
      else k_gather_out_mix<<<nb, 256, 0, c->stream>>>(stg, c->d_row_of_node + b, e - b, c->S, sm ? *sm : c->mA,
                                                        c->wm, low_mix ? 1 : 0);
      CK(cudaGetLastError());
    }
    CK(cudaEventRecord(c->copy_ev[k], c->stream));
    CK(cudaStreamWaitEvent(c->copy_stream[k], c->copy_ev[k], 0));
    CK(cudaMemcpyAsync(un + (size_t)c->S * (b - node_begin), stg, (size_t)c->S * (e - b) * sizeof(double),
                       device_dst ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->copy_stream[k]));
  }
  for (int k = 0; k < K; k++) {
    CK(cudaEventRecord(c->copy_ev[k], c->copy_stream[k]));
    CK(cudaStreamWaitEvent(c->stream, c->copy_ev[k], 0));
  }
  return SWE_OK;
}

// Gauges after a step (main.f90:102-117): SUM(h(jj(:,m)) * ff) and
// SUM((h + bath)(jj(:,m)) * ff) in the reference's order, with the time
// reached.  One block; the row index is the step count before this step.
// Gauges of an instance that did not step (done) record NaN.
__global__ void k_gauges(int n, const int* __restrict__ ginst, const int* __restrict__ grows,
                         const double* __restrict__ gw, const InstState* __restrict__ St, int fp64, StateF64 a,
                         StateMix m, const double* __restrict__ bath, double* __restrict__ rec,
                         unsigned long long* __restrict__ count, int ring) {
  const unsigned long long k = *count;
  for (int g = threadIdx.x; g < n; g += blockDim.x) {
    double* row = rec + ((size_t)(k % (unsigned long long)ring) * n + g) * 3;
    const InstState& st = St[ginst[g]];
    if (st.done) {
      row[0] = row[1] = row[2] = __longlong_as_double(0x7ff8000000000000ll);
      continue;
    }
    double sh = 0.0, se = 0.0;
    for (int v = 0; v < 3; v++) {
      const int r = grows[3 * g + v];
      const double h = fp64 ? a.h[r] : df_to_double(m.h[r]);
      const double w = gw[3 * g + v];
      sh = v ? __dadd_rn(sh, __dmul_rn(h, w)) : __dmul_rn(h, w);
      se = v ? __dadd_rn(se, __dmul_rn(__dadd_rn(h, bath[r]), w)) : __dmul_rn(__dadd_rn(h, bath[r]), w);
    }
    row[0] = st.time;
    row[1] = sh;
    row[2] = se;
  }
  __syncthreads();
  if (threadIdx.x == 0) *count = k + 1;
}

// Movie frame fields of the time loop (main.f90:125-143) in reference node
// order: hpz = h + z, or -1e-7 hmax0 + z where h <= 1e-4 hmax0; h, or 0
// there.  Explicit roundings: the reference forms each product and sum once.
__global__ void k_frame_fields(const int* __restrict__ row_of_node, int64_t n_nodes, int fp64, StateF64 a,
                               StateMix m, const double* __restrict__ bath, double hmax0, double* __restrict__ hpz,
                               double* __restrict__ hout) {
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  const int64_t r = row_of_node[n];
  const double h = fp64 ? a.h[r] : df_to_double(m.h[r]);
  const double z = bath[r];
  if (h <= __dmul_rn(1.e-4, hmax0)) {
    hpz[n] = __dadd_rn(__dmul_rn(-1.e-7, hmax0), z);
    hout[n] = 0.0;
  } else {
    hpz[n] = __dadd_rn(h, z);
    hout[n] = h;
  }
}

static int frames_wait(swe_ctx* c);
static void free_gauges(swe_ctx* c);

static int read_errors(swe_ctx* c) {
  unsigned e = 0;
  CK(cudaMemcpyAsync(&e, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (e) CK(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
  if (e & ERRB_NAN) return fail(c, SWE_ERR_NAN, "non-finite state produced");
  if (e & ERRB_DELTA) return fail(c, SWE_ERR_DELTA, "BUG in compute_lambda_vacc: Delta < 0");
  if (e & ERRB_NEG_H) return fail(c, SWE_ERR_NEG_H, "Min h<0, STOP");
  return SWE_OK;
}

static int set_inst_state_dt(swe_ctx* c, int inst, double dt, int done_others) {
  std::vector<InstState> hs(c->n_inst);
  CK(cudaMemcpyAsync(hs.data(), c->d_St, sizeof(InstState) * c->n_inst, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int b = 0; b < c->n_inst; b++) {
    if (b == inst) { inst_set_dt(hs[b], dt); hs[b].done = 0; }
    else if (done_others) hs[b].done = 1;
  }
  CK(cudaMemcpyAsync(c->d_St, hs.data(), sizeof(InstState) * c->n_inst, cudaMemcpyHostToDevice, c->stream));
  return SWE_OK;
}

static int restore_done(swe_ctx* c, const std::vector<InstState>& saved) {
  CK(cudaMemcpyAsync(c->d_St, saved.data(), sizeof(InstState) * c->n_inst, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

static int save_state(swe_ctx* c, std::vector<InstState>& saved) {
  saved.resize(c->n_inst);
  CK(cudaMemcpyAsync(saved.data(), c->d_St, sizeof(InstState) * c->n_inst, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

// One time step.  With kev/acc (profiling), every kernel is bracketed by an
// event pair and its duration added to acc[kind] after a synchronisation.
static void enqueue_step(swe_ctx* c, const KernelEvents* kev = nullptr, double* acc = nullptr) {
  const cudaStream_t s = c->stream;
  auto harvest = [&](int first, int last) {
    if (!kev) return;
    cudaEventSynchronize(kev->ev[2 * last + 1]);
    for (int k = first; k <= last; k++) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, kev->ev[2 * k], kev->ev[2 * k + 1]);
      acc[k] += ms;
    }
  };
  // FP64: k_node's per-node arrays of the step's state serve k_dt (1/h,
  // sqrt(g |h|)) and stage 1 (which then skips k_node); k_dt keeps every d_ij
  // (in the f_ij array, free until stage 1's k_fct) for stage 1's k_low
  if (c->precision == SWE_PREC_FP64) {
    StageArgs a0{c->G, c->d_C, c->d_St, c->A, c->A, c->B, c->w, 1, nullptr, c->d_err, c->block};
    if (kev) cudaEventRecord(kev->ev[2], s);
    launch_node_f64(a0, s);
    if (kev) cudaEventRecord(kev->ev[3], s);
  }
  if (kev) cudaEventRecord(kev->ev[0], s);
  if (c->precision == SWE_PREC_FP64)
    launch_dt_f64(c->G, c->d_C, c->d_St, c->A, c->w.fct, nullptr, c->d_err, c->block, s, &c->w);
  else launch_dt_mix(c->G, c->d_C, c->d_St, c->mA, c->wm.dlam, c->wm.alpha, c->d_err, c->tune,
                   c->tiles_ok ? &c->tiles : nullptr, s);
  if (kev) cudaEventRecord(kev->ev[1], s);
  harvest(0, 0);                                   // waits for k_dt, the later of the two
  if (c->precision == SWE_PREC_FP64) harvest(1, 1);
  launch_step_begin(c->d_C, c->d_St, c->n_inst, s);
  for (int stage = 1; stage <= 3; stage++) {
    if (c->precision == SWE_PREC_FP64) {
      StageArgs a{c->G, c->d_C, c->d_St, c->A, c->A, c->B, c->w, stage, nullptr, c->d_err, c->block};
      a.entropy = has_entropy(c);
      if (stage == 1) { a.dij_in = c->w.fct; a.skip_node = 1; }
      if (stage == 2) { a.u = c->B; a.out = c->Cs; }
      if (stage == 3) { a.u = c->Cs; a.out = c->A; }
      launch_stage_f64(a, s, kev);
    } else {
      StageArgsMix a{c->G, c->d_C, c->d_St, c->mA, c->mA, c->mB, c->wm, stage, c->d_err, c->block};
      a.tiles = c->tiles_ok ? &c->tiles : nullptr;
      a.f64 = is_split(c);
      a.type1 = has_type1(c);
      if (stage == 2) { a.u = c->mB; a.out = c->mC; }
      if (stage == 3) { a.u = c->mC; a.out = c->mA; }
      launch_stage_mix(a, s, kev, c->tune);
    }
    harvest(1, 4);
  }
  launch_step_end(c->d_St, c->n_inst, s);
  if (c->n_gauges)
    k_gauges<<<1, 256, 0, s>>>(c->n_gauges, c->d_gauge_inst, c->d_gauge_rows, c->d_gauge_w, c->d_St,
                               c->precision == SWE_PREC_FP64 ? 1 : 0, c->A, c->mA, c->G.bath, c->d_gauge_rec,
                               c->d_gauge_count, swe_ctx::kGaugeRing);
}

static int capture_steps(swe_ctx* c, int steps, cudaGraphExec_t* exec) {
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < steps; k++) enqueue_step(c);
  CK(cudaStreamEndCapture(c->stream, &g));
  cudaError_t e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  CK(e);
  return SWE_OK;
}

static int build_graph(swe_ctx* c, int steps) {
  if (c->gexec && c->graph_steps == steps) return SWE_OK;
  if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
  int rc = capture_steps(c, steps, &c->gexec);
  if (rc) return rc;
  c->graph_steps = steps;
  return SWE_OK;
}

// Captured steps depend on the launch configuration; drop them when it
// changes (parameter, bathymetry and Dirichlet updates rewrite device arrays
// in place and keep them valid).
static void drop_graphs(swe_ctx* c) {
  if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; c->graph_steps = 0; }
  if (c->gexec1) { cudaGraphExecDestroy(c->gexec1); c->gexec1 = nullptr; }
}

// ============================== C ABI ======================================

static int create_common(swe_ctx** out, int n_inst, const int* np, const int* me, const int* jj, const double* rr,
                         const double* bath, const swe_params* params) {
  NvtxRange nvtx("swe_create");
  if (!out) return SWE_ERR_ARG;
  *out = nullptr;
  if (n_inst <= 0 || !np || !me || !jj || !rr || !bath || !params) return SWE_ERR_ARG;
  swe_ctx* c = new swe_ctx;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    *out = c;
    return fail(c, SWE_ERR_CUDA, "no CUDA device: this library has no CPU path");
  }
  cudaGetDevice(&c->dev);
  c->n_inst = n_inst;
  c->S = params[0].syst_size;
  c->precision = params[0].precision;
  c->params.assign(params, params + n_inst);
  for (int b = 0; b < n_inst; b++) {
    int rc = check_params(c, params[b]);
    if (!rc && (params[b].syst_size != c->S || params[b].precision != c->precision))
      rc = fail(c, SWE_ERR_ARG, "all instances must share syst_size and precision");
    if (rc) { *out = c; return rc; }
  }
  c->meshes.resize(n_inst);
  std::vector<std::vector<double>> baths(n_inst);
  int64_t joff = 0, roff = 0;
  for (int b = 0; b < n_inst; b++) {
    HostMesh& m = c->meshes[b];
    if (np[b] <= 0 || me[b] <= 0) { *out = c; return fail(c, SWE_ERR_ARG, "empty mesh"); }
    m.np = np[b]; m.me = me[b];
    m.jj.resize((size_t)3 * me[b]);
    for (size_t q = 0; q < m.jj.size(); q++) m.jj[q] = jj[joff + q] - 1;
    m.rr.assign(rr + 2 * roff, rr + 2 * (roff + np[b]));
    baths[b].assign(bath + roff, bath + roff + np[b]);
    joff += (int64_t)3 * me[b];
    roff += np[b];
    std::string e = construct_matrices_device(m);   // CSR pattern + mass/c_ij assembly on the GPU
    if (!e.empty()) {
      *out = c;
      return fail(c, e.rfind("device setup", 0) == 0 ? SWE_ERR_CUDA : SWE_ERR_MESH, e);
    }
  }
  *out = c;
  if (cuda_check(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate")) return SWE_ERR_CUDA;
  int rc = build_device(c, baths);
  if (rc) return rc;
  return cuda_check(c, cudaDeviceSynchronize(), "setup");
}

SWE_API int swe_create(swe_ctx** ctx, int np, int me, const int* jj, const double* rr, const double* bath,
                       const swe_params* params) {
  return create_common(ctx, 1, &np, &me, jj, rr, bath, params);
}

SWE_API int swe_create_batch(swe_ctx** ctx, int n_inst, const int* np, const int* me, const int* jj, const double* rr,
                             const double* bath, const swe_params* params) {
  return create_common(ctx, n_inst, np, me, jj, rr, bath, params);
}

SWE_API void swe_destroy(swe_ctx* c) {
  if (!c) return;
  free_gauges(c);
  if (c->d_frame) {                                   // finish the frames in flight, stop the writer
    frames_wait(c);
    {
      std::lock_guard<std::mutex> lk(c->frame_mu);
      c->frame_stop = true;
      c->frame_cv.notify_all();
    }
    if (c->frame_worker.joinable()) c->frame_worker.join();
    for (int k = 0; k < 2; k++) if (c->frame_ev[k]) cudaEventDestroy(c->frame_ev[k]);
    cudaFreeHost(c->h_frame);
    cudaFree(c->d_frame);
  }
  drop_graphs(c);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  for (int k = 0; k < c->copy_chunks; k++) {
    cudaStreamSynchronize(c->copy_stream[k]);
    cudaStreamDestroy(c->copy_stream[k]);
    cudaEventDestroy(c->copy_ev[k]);
  }
  if (c->copy_go) cudaEventDestroy(c->copy_go);
  c->buf.release();
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

SWE_API const char* swe_last_error(const swe_ctx* c) { return c ? c->err.c_str() : "null context"; }

SWE_API int swe_set_params(swe_ctx* c, int inst, const swe_params* p) {
  if (!c || !p || inst < 0 || inst >= c->n_inst) return fail(c, SWE_ERR_ARG, "bad instance or params");
  int rc = check_params(c, *p);
  if (rc) return rc;
  if (p->syst_size != c->S || p->precision != c->precision)
    return fail(c, SWE_ERR_ARG, "syst_size and precision are fixed at creation");
  c->params[inst] = *p;
  InstConst k = make_const(*p);
  CK(cudaMemcpyAsync(c->d_C + inst, &k, sizeof(InstConst), cudaMemcpyHostToDevice, c->stream));
  std::vector<InstState> hs;
  if ((rc = save_state(c, hs))) return rc;
  inst_set_dt(hs[inst], p->dt);
  return restore_done(c, hs);
}

SWE_API int swe_set_bath(swe_ctx* c, int inst, const double* bath) {
  if (!c || !bath || inst < 0 || inst >= c->n_inst) return fail(c, SWE_ERR_ARG, "bad arguments");
  Layout& L = c->L;
  for (int i = 0; i < c->meshes[inst].np; i++) L.bath[L.new_of_old[inst][i]] = bath[i];
  const int64_t r0 = L.row_off[inst], nr = L.row_off[inst + 1] - r0;
  if (c->precision == SWE_PREC_FP64) {
    CK(cudaMemcpyAsync((double*)c->G.bath + r0, L.bath.data() + r0, nr * sizeof(double), cudaMemcpyHostToDevice,
                       c->stream));
  } else {
    std::vector<float2> bf(nr);
    for (int64_t r = 0; r < nr; r++) bf[r] = bath_df(L.bath[r0 + r]);
    CK(cudaMemcpyAsync((double*)c->G.bath + r0, L.bath.data() + r0, nr * sizeof(double), cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaMemcpyAsync((float2*)c->G.bathdf + r0, bf.data(), nr * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
    launch_refresh_eta(c->G, c->mA, c->stream);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

SWE_API int swe_set_dirichlet_anal(swe_ctx* c, int inst, int comp, int n, const int* js) {
  if (!c || inst < 0 || inst >= c->n_inst || comp < 0 || comp >= c->S || n < 0 || (n > 0 && !js))
    return fail(c, SWE_ERR_ARG, "bad Dirichlet arguments");
  const int tt = c->params[inst].type_test;
  if (tt != 5 && tt != 13) return fail(c, SWE_ERR_ARG, "analytic Dirichlet data are built for type_test 5 and 13");
  if (comp > 2)   // sol_anal leaves type 13's components 4 and 5 undefined for t > 0 (condlim.f90:803-823)
    return fail(c, SWE_ERR_ARG, "analytic Dirichlet data are built for components h, qx, qy");
  const Layout& L = c->L;
  for (int q = 0; q < n; q++)
    if (js[q] < 1 || js[q] > c->meshes[inst].np) return fail(c, SWE_ERR_ARG, "Dirichlet node out of range");
  if (!c->d_dir_anal) {   // on first use: the per-row flags and node coordinates
    cudaError_t st = cudaSuccess;
    c->h_dir_anal.assign(L.n_rows, 0);
    std::vector<double> rr(2 * (size_t)L.n_rows, 0.0);
    for (int b = 0; b < c->n_inst; b++)
      for (int i = 0; i < c->meshes[b].np; i++) {
        const int64_t r = L.new_of_old[b][i];
        rr[2 * r] = c->meshes[b].rr[2 * (size_t)i];
        rr[2 * r + 1] = c->meshes[b].rr[2 * (size_t)i + 1];
      }
    c->d_dir_anal = c->buf.alloc<uint8_t>(L.n_rows, st);
    c->d_rr_row = upload_vec(c, rr, st);
    if (st != cudaSuccess) return fail(c, SWE_ERR_CUDA, std::string("device allocation: ") + cudaGetErrorString(st));
    c->G.dir_anal = c->d_dir_anal;
    c->G.rr_row = c->d_rr_row;
    drop_graphs(c);       // captured launches carry the graph's pointers
  }
  for (int64_t r = L.row_off[inst]; r < L.row_off[inst + 1]; r++) {
    c->h_dir_mask[r] &= (uint8_t)~(1u << comp);
    c->h_dir_anal[r] &= (uint8_t)~(1u << comp);
  }
  for (int q = 0; q < n; q++) {
    const int64_t r = L.new_of_old[inst][js[q] - 1];
    c->h_dir_mask[r] |= (uint8_t)(1u << comp);
    c->h_dir_anal[r] |= (uint8_t)(1u << comp);
  }
  CK(cudaMemcpyAsync(c->d_dir_mask, c->h_dir_mask.data(), L.n_rows, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_dir_anal, c->h_dir_anal.data(), L.n_rows, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

SWE_API int swe_set_dirichlet(swe_ctx* c, int inst, int comp, int n, const int* js, const double* vals) {
  if (!c || inst < 0 || inst >= c->n_inst || comp < 0 || comp >= c->S || n < 0 || (n > 0 && !js))
    return fail(c, SWE_ERR_ARG, "bad Dirichlet arguments");
  const Layout& L = c->L;
  // clear the component on this instance, then set
  for (int q = 0; q < n; q++)
    if (js[q] < 1 || js[q] > c->meshes[inst].np) return fail(c, SWE_ERR_ARG, "Dirichlet node out of range");
  for (int64_t r = L.row_off[inst]; r < L.row_off[inst + 1]; r++) {
    c->h_dir_mask[r] &= (uint8_t)~(1u << comp);
    if (!c->h_dir_anal.empty()) c->h_dir_anal[r] &= (uint8_t)~(1u << comp);
  }
  for (int q = 0; q < n; q++) {
    const int64_t r = L.new_of_old[inst][js[q] - 1];
    c->h_dir_mask[r] |= (uint8_t)(1u << comp);
    c->h_dir_val[(size_t)comp * L.n_rows + r] = vals ? vals[q] : 0.0;
  }
  if (c->d_dir_anal)
    CK(cudaMemcpyAsync(c->d_dir_anal, c->h_dir_anal.data(), L.n_rows, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_dir_mask, c->h_dir_mask.data(), L.n_rows, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_dir_val, c->h_dir_val.data(), c->h_dir_val.size() * sizeof(double), cudaMemcpyHostToDevice,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

SWE_API int swe_sizes(const swe_ctx* c, int inst, int* np, int* nnz) {
  if (!c || inst < 0 || inst >= c->n_inst) return SWE_ERR_ARG;
  if (np) *np = c->meshes[inst].np;
  if (nnz) *nnz = (int)c->meshes[inst].ja.size();
  return SWE_OK;
}

SWE_API int swe_get_matrices(swe_ctx* c, int inst, int* ia, int* ja, double* mass, double* lumped, int* diag,
                             double* cx, double* cy) {
  if (!c || inst < 0 || inst >= c->n_inst) return fail(c, SWE_ERR_ARG, "bad instance");
  const HostMesh& m = c->meshes[inst];
  for (int i = 0; i <= m.np; i++) if (ia) ia[i] = m.ia[i] + 1;
  for (size_t p = 0; p < m.ja.size(); p++) {
    if (ja) ja[p] = m.ja[p] + 1;
    if (mass) mass[p] = m.mass[p];
    if (cx) cx[p] = m.cx[p];
    if (cy) cy[p] = m.cy[p];
  }
  for (int i = 0; i < m.np; i++) {
    if (lumped) lumped[i] = m.lumped[i];
    if (diag) diag[i] = m.diag[i] + 1;
  }
  return SWE_OK;
}

// copy a per-entry device array of one instance back into CSR order; the
// diagonal positions come from a per-row device array (or are 0 if null)
template <typename T> static double comp_of(const T& v, int) { return (double)v; }
static double comp_of(const float2& v, int k) { return (double)(k ? v.y : v.x); }

template <typename T, typename U = T>
static int entries_to_csr(swe_ctx* c, int inst, const T* d_arr, double* out, const U* d_diag_rows = nullptr,
                          int comp = 0) {
  const Layout& L = c->L;
  const int64_t s0 = L.row_off[inst] / 32, s1 = L.row_off[inst + 1] / 32;
  const int64_t e0 = L.slice_ptr[s0], e1 = L.slice_ptr[s1];
  std::vector<T> h(e1 - e0);
  CK(cudaMemcpyAsync(h.data(), d_arr + e0, (e1 - e0) * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
  const int64_t r0 = L.row_off[inst], r1 = L.row_off[inst + 1];
  std::vector<U> hd(r1 - r0, U(0));
  if (d_diag_rows)
    CK(cudaMemcpyAsync(hd.data(), d_diag_rows + r0, (r1 - r0) * sizeof(U), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int64_t e = e0; e < e1; e++)
    if (L.ref_pos[e] >= 0) out[L.ref_pos[e]] = comp_of(h[e - e0], comp);
  for (int64_t r = r0; r < r1; r++)
    if (L.ref_pos_diag[r] >= 0) out[L.ref_pos_diag[r]] = (double)hd[r - r0];
  return SWE_OK;
}

template <typename T>
static int rows_to_nodes(swe_ctx* c, int inst, const T* d_arr, double* out) {
  const Layout& L = c->L;
  const int64_t r0 = L.row_off[inst], r1 = L.row_off[inst + 1];
  std::vector<T> h(r1 - r0);
  CK(cudaMemcpyAsync(h.data(), d_arr + r0, (r1 - r0) * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < c->meshes[inst].np; i++) out[i] = (double)h[L.new_of_old[inst][i] - r0];
  return SWE_OK;
}

SWE_API int swe_compute_dij(swe_ctx* c, int inst, const double* un, double* dij, double* dt_out) {
  if (!c || inst < 0 || inst >= c->n_inst || !un) return fail(c, SWE_ERR_ARG, "bad arguments");
  if (c->precision != SWE_PREC_FP64) return fail(c, SWE_ERR_ARG, "swe_compute_dij is an FP64 operator");
  int rc = to_device(c, un, false, c->node_off[inst], c->node_off[inst + 1]);
  if (rc) { drain(c); return rc; }
  std::vector<InstState> saved;
  if ((rc = save_state(c, saved))) return rc;
  if ((rc = set_inst_state_dt(c, inst, c->params[inst].dt > 0 ? c->params[inst].dt : 1.0, 1))) return rc;
  launch_dt_f64(c->G, c->d_C, c->d_St, c->A, c->w.dL, c->w.dLii, c->d_err, c->block, c->stream);
  CK(cudaGetLastError());
  if ((rc = read_errors(c))) { restore_done(c, saved); return rc; }
  std::vector<double> d(c->meshes[inst].ja.size());
  if ((rc = entries_to_csr(c, inst, c->w.dL, d.data(), c->w.dLii))) return rc;
  if ((rc = restore_done(c, saved))) return rc;
  if (dij) std::copy(d.begin(), d.end(), dij);
  if (dt_out) {
    const HostMesh& m = c->meshes[inst];
    double mx = std::fabs(d[m.diag[0]]) / m.lumped[0];
    for (int i = 1; i < m.np; i++) mx = std::max(mx, std::fabs(d[m.diag[i]]) / m.lumped[i]);
    *dt_out = c->params[inst].cfl * 1 / mx;
  }
  return SWE_OK;
}

SWE_API int swe_euler(swe_ctx* c, int inst, const double* un, double* unext) {
  NvtxRange nvtx("swe_euler");
  if (!c || inst < 0 || inst >= c->n_inst || !un || !unext) return fail(c, SWE_ERR_ARG, "bad arguments");
  if (!(c->params[inst].dt > 0)) return fail(c, SWE_ERR_ARG, "params.dt must be > 0 for swe_euler");
  int rc = to_device(c, un, false, c->node_off[inst], c->node_off[inst + 1]);
  if (rc) { drain(c); return rc; }
  std::vector<InstState> saved;
  if ((rc = save_state(c, saved))) return rc;
  if ((rc = set_inst_state_dt(c, inst, c->params[inst].dt, 1))) return rc;
  if (c->precision == SWE_PREC_FP64) {
    StageArgs a{c->G, c->d_C, c->d_St, c->A, c->A, c->B, c->w, 0, c->d_lij, c->d_err, c->block};
    a.entropy = has_entropy(c);
    launch_stage_f64(a, c->stream);
  } else {
    StageArgsMix a{c->G, c->d_C, c->d_St, c->mA, c->mA, c->mB, c->wm, 0, c->d_err, c->block};
    a.tiles = c->tiles_ok ? &c->tiles : nullptr;
    a.f64 = is_split(c);
    a.type1 = has_type1(c);
    launch_stage_mix(a, c->stream, nullptr, c->tune);
  }
  CK(cudaGetLastError());
  int erc = read_errors(c);
  if ((rc = restore_done(c, saved))) return rc;
  c->euler_done = true;
  c->euler_inst = inst;
  if ((rc = from_device_state(c, unext, false, c->node_off[inst], c->node_off[inst + 1],
                              c->precision == SWE_PREC_FP64 ? &c->B : nullptr,
                              c->precision == SWE_PREC_FP64 ? nullptr : &c->mB))) {
    drain(c);
    return rc;
  }
  CK(cudaStreamSynchronize(c->stream));
  return erc;
}

SWE_API int swe_euler_intermediates(swe_ctx* c, int inst, double* dij_low, double* muij_low, double* alpha,
                                    double* u_low, double* res, double* fctmat, double* rminus, double* lij) {
  if (!c || inst < 0 || inst >= c->n_inst) return fail(c, SWE_ERR_ARG, "bad instance");
  if (!c->euler_done || c->euler_inst != inst) return fail(c, SWE_ERR_ARG, "call swe_euler on this instance first");
  int rc;
  if (c->precision == SWE_PREC_FP64) {
    if (dij_low && (rc = entries_to_csr(c, inst, c->w.dL, dij_low, c->w.dLii))) return rc;
    if (muij_low && (rc = entries_to_csr(c, inst, c->w.muL, muij_low, c->w.muLii))) return rc;
    if (fctmat && (rc = entries_to_csr(c, inst, c->w.fct, fctmat))) return rc;          // f_ii = 0
    if (lij && (rc = entries_to_csr(c, inst, c->d_lij, lij, c->w.rminus))) return rc;   // l_ii = R_i
    if (alpha && (rc = rows_to_nodes(c, inst, c->w.alpha, alpha))) return rc;
    if (res && (rc = rows_to_nodes(c, inst, c->w.res, res))) return rc;
    if (rminus && (rc = rows_to_nodes(c, inst, c->w.rminus, rminus))) return rc;
    if (u_low && (rc = from_device_state(c, u_low, false, c->node_off[inst], c->node_off[inst + 1], &c->w.uL, nullptr))) {
      drain(c);
      return rc;
    }
  } else {
    if (dij_low && (rc = entries_to_csr(c, inst, c->wm.dmu, dij_low, (const float*)nullptr, 0))) return rc;
    if (muij_low && (rc = entries_to_csr(c, inst, c->wm.dmu, muij_low, (const float*)nullptr, 1))) return rc;
    if (alpha && (rc = rows_to_nodes(c, inst, c->wm.alpha, alpha))) return rc;
    if (res && (rc = rows_to_nodes(c, inst, c->wm.res, res))) return rc;
    if (rminus && is_split(c) && (rc = rows_to_nodes(c, inst, c->wm.rminus64, rminus))) return rc;
    if (rminus && !is_split(c) && (rc = rows_to_nodes(c, inst, c->wm.rminus, rminus))) return rc;
    if (u_low && (rc = from_device_state(c, u_low, false, c->node_off[inst], c->node_off[inst + 1], nullptr, nullptr,
                                         true))) {
      drain(c);
      return rc;
    }
  }
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

SWE_API int swe_fct_positivity(swe_ctx* c, int inst, const double* unext, const double* mat, double* lij) {
  if (!c || inst < 0 || inst >= c->n_inst || !unext || !mat || !lij) return fail(c, SWE_ERR_ARG, "bad arguments");
  if (c->precision != SWE_PREC_FP64) return fail(c, SWE_ERR_ARG, "swe_fct_positivity is an FP64 operator");
  const Layout& L = c->L;
  const HostMesh& m = c->meshes[inst];
  std::vector<double> hrow(L.n_rows, 0.0), hdiag(L.n_rows, 0.0), hent(L.n_entries, 0.0);
  for (int i = 0; i < m.np; i++) {
    const int64_t r = L.new_of_old[inst][i];
    hrow[r] = unext[i];
    hdiag[r] = mat[m.diag[i]];
  }
  const int64_t s0 = L.row_off[inst] / 32, s1 = L.row_off[inst + 1] / 32;
  for (int64_t e = L.slice_ptr[s0]; e < L.slice_ptr[s1]; e++)
    if (L.ref_pos[e] >= 0) hent[e] = mat[L.ref_pos[e]];
  CK(cudaMemcpyAsync(c->w.uL.h, hrow.data(), L.n_rows * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->w.dLii, hdiag.data(), L.n_rows * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->w.fct, hent.data(), L.n_entries * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_fct_positivity_f64(c->G, c->d_C, c->w.uL.h, c->w.fct, c->w.dLii, c->w.rminus, c->d_lij, c->stream);
  CK(cudaGetLastError());
  c->euler_done = false;
  return entries_to_csr(c, inst, c->d_lij, lij, c->w.rminus);   // l_ii = R_i
}

SWE_API int swe_fct_generic(swe_ctx* c, int inst, double* unext, const double* maxn, const double* minn,
                            const double* mat, const double* dg) {
  if (!c || inst < 0 || inst >= c->n_inst || !unext || !maxn || !minn || !mat)
    return fail(c, SWE_ERR_ARG, "bad arguments");
  if (c->precision != SWE_PREC_FP64) return fail(c, SWE_ERR_ARG, "swe_fct_generic is an FP64 operator");
  const Layout& L = c->L;
  const HostMesh& m = c->meshes[inst];
  const size_t nr = L.n_rows;
  std::vector<double> hu(nr, 0.0), hmax(nr, 0.0), hmin(nr, 0.0), hdg(nr, 1.0), hdiag(nr, 0.0),
      hent(L.n_entries, 0.0);
  for (int i = 0; i < m.np; i++) {
    const int64_t r = L.new_of_old[inst][i];
    hu[r] = unext[i];
    hmax[r] = maxn[i];
    hmin[r] = minn[i];
    hdg[r] = dg ? dg[i] : m.lumped[i];
    hdiag[r] = mat[m.diag[i]];
  }
  const int64_t s0 = L.row_off[inst] / 32, s1 = L.row_off[inst + 1] / 32;
  for (int64_t e = L.slice_ptr[s0]; e < L.slice_ptr[s1]; e++)
    if (L.ref_pos[e] >= 0) hent[e] = mat[L.ref_pos[e]];
  WorkF64& w = c->w;   // per-stage scratch, reused: u, bounds, dg, R+-, f_ij
  CK(cudaMemcpyAsync(w.uL.h, hu.data(), nr * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(w.v1, hmax.data(), nr * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(w.v2, hmin.data(), nr * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(w.ovh, hdg.data(), nr * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(w.dLii, hdiag.data(), nr * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(w.fct, hent.data(), L.n_entries * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_fct_generic_f64(c->G, w.uL.h, w.v1, w.v2, w.ovh, w.fct, w.dLii, w.ent, w.rminus, c->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(hu.data(), w.uL.h, nr * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < m.np; i++) unext[i] = hu[L.new_of_old[inst][i]];
  c->euler_done = false;
  return SWE_OK;
}

SWE_API int swe_gauss_points(swe_ctx* c, int inst, double* rj, double* rr_gauss) {
  if (!c || inst < 0 || inst >= c->n_inst) return fail(c, SWE_ERR_ARG, "bad instance");
  gauss_points(c->meshes[inst], rj, rr_gauss);
  return SWE_OK;
}

SWE_API int swe_norms(swe_ctx* c, int inst, int field, const double* f_anal, double* l1, double* l2) {
  if (!c || inst < 0 || inst >= c->n_inst) return fail(c, SWE_ERR_ARG, "bad instance");
  if (!((field >= 0 && field < c->S) || field == SWE_FIELD_H32)) return fail(c, SWE_ERR_ARG, "bad field");
  const HostMesh& m = c->meshes[inst];
  cudaError_t st = cudaSuccess;
  if (c->d_jj_inst.empty()) {
    c->d_jj_inst.assign(c->n_inst, nullptr);
    c->d_rj_inst.assign(c->n_inst, nullptr);
    c->d_norm_acc = c->buf.alloc<double>(4, st);
  }
  if (!c->d_jj_inst[inst]) {
    std::vector<double> rj((size_t)3 * m.me);
    gauss_points(m, rj.data(), nullptr);
    c->d_jj_inst[inst] = c->buf.alloc<int>(m.jj.size(), st);
    c->d_rj_inst[inst] = c->buf.alloc<double>(rj.size(), st);
    if (st == cudaSuccess) st = cudaMemcpy(c->d_jj_inst[inst], m.jj.data(), m.jj.size() * sizeof(int),
                                           cudaMemcpyHostToDevice);
    if (st == cudaSuccess) st = cudaMemcpy(c->d_rj_inst[inst], rj.data(), rj.size() * sizeof(double),
                                           cudaMemcpyHostToDevice);
  }
  if (f_anal && c->fanal_cap < (size_t)3 * m.me) {
    c->d_fanal = c->buf.alloc<double>((size_t)3 * m.me, st);
    c->fanal_cap = (size_t)3 * m.me;
  }
  const size_t nparts = 4 * (size_t)norm_partials(m.me);
  if (c->norm_part_cap < nparts) {
    c->d_norm_part = c->buf.alloc<double>(nparts, st);
    c->norm_part_cap = nparts;
  }
  if (st != cudaSuccess) return cuda_check(c, st, "swe_norms allocation");
  if (f_anal)
    CK(cudaMemcpyAsync(c->d_fanal, f_anal, (size_t)3 * m.me * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_norms(field, c->precision == SWE_PREC_FP64 ? 0 : 1, c->A, c->mA, c->d_jj_inst[inst], c->d_rj_inst[inst],
               m.me, c->d_row_of_node + c->node_off[inst], f_anal ? c->d_fanal : nullptr, c->d_norm_part,
               c->d_norm_acc, c->stream);
  CK(cudaGetLastError());
  double acc[4];
  CK(cudaMemcpyAsync(acc, c->d_norm_acc, sizeof acc, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (l1) *l1 = acc[0] + acc[1];
  if (l2) *l2 = std::sqrt(acc[2] + acc[3]);
  return SWE_OK;
}

SWE_API int swe_upload(swe_ctx* c, const double* un) {
  NvtxRange nvtx("swe_upload");
  if (!c || !un) return fail(c, SWE_ERR_ARG, "bad arguments");
  int rc = to_device(c, un, false, 0, c->node_off[c->n_inst]);
  if (rc) { drain(c); return rc; }
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

SWE_API int swe_download(swe_ctx* c, double* un) {
  NvtxRange nvtx("swe_download");
  if (!c || !un) return fail(c, SWE_ERR_ARG, "bad arguments");
  int rc = from_device_state(c, un, false, 0, c->node_off[c->n_inst], c->precision == SWE_PREC_FP64 ? &c->A : nullptr,
                             c->precision == SWE_PREC_FP64 ? nullptr : &c->mA);
  if (rc) { drain(c); return rc; }
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

SWE_API int swe_upload_device(swe_ctx* c, const double* d_un) {
  if (!c || !d_un) return fail(c, SWE_ERR_ARG, "bad arguments");
  int rc = to_device(c, d_un, true, 0, c->node_off[c->n_inst]);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

SWE_API int swe_download_device(swe_ctx* c, double* d_un) {
  if (!c || !d_un) return fail(c, SWE_ERR_ARG, "bad arguments");
  int rc = from_device_state(c, d_un, true, 0, c->node_off[c->n_inst], c->precision == SWE_PREC_FP64 ? &c->A : nullptr,
                             c->precision == SWE_PREC_FP64 ? nullptr : &c->mA);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return SWE_OK;
}

SWE_API int swe_get_time(swe_ctx* c, double* time, double* t_final, double* dt) {
  if (!c) return SWE_ERR_ARG;
  std::vector<InstState> hs;
  int rc = save_state(c, hs);
  if (rc) return rc;
  for (int b = 0; b < c->n_inst; b++) {
    if (time) time[b] = hs[b].time;
    if (t_final) t_final[b] = hs[b].t_final;
    if (dt) dt[b] = hs[b].dt;
  }
  return SWE_OK;
}

SWE_API int swe_set_time(swe_ctx* c, const double* time, const double* t_final) {
  if (!c) return SWE_ERR_ARG;
  std::vector<InstState> hs;
  int rc = save_state(c, hs);
  if (rc) return rc;
  for (int b = 0; b < c->n_inst; b++) {
    if (time) hs[b].time = time[b];
    if (t_final) hs[b].t_final = t_final[b];
    hs[b].done = 0;
    hs[b].steps = 0;
    hs[b].maxd_bits = 0ull;
  }
  return restore_done(c, hs);
}

// Autotuner of the mixed kernels: for every kernel kind, time each (block
// size, entry batch) variant on the current state and keep the fastest.  The
// variants agree to FP32 rounding, and every timed kernel is idempotent on its
// inputs (it only rewrites its own outputs), so the state is unchanged.
// Launch configuration from the autotuner's own description ("dt:block256/
// batch4/resident node:... low:block128/batch2/regs64/tiled ..."), so that a
// profiling run can reproduce the variants a timed run chose.  Kinds not
// named keep their defaults; false on a malformed string.
static bool parse_tuning(const char* spec, bool tiles, KernelTune& t) {
  const char* names[5] = {"dt", "node", "low", "fct", "update"};
  std::string str(spec);
  size_t pos = 0;
  while (pos < str.size()) {
    size_t end = str.find(' ', pos);
    if (end == std::string::npos) end = str.size();
    const std::string tok = str.substr(pos, end - pos);
    pos = end + 1;
    if (tok.empty()) continue;
    const size_t colon = tok.find(':');
    if (colon == std::string::npos) return false;
    int kind = -1;
    for (int k = 0; k < 5; k++)
      if (tok.compare(0, colon, names[k]) == 0) kind = k;
    if (kind < 0) return false;
    int block = 0, batch = 0, cap = 0, grid = 0, tiled = 0;
    size_t p = colon + 1;
    while (p < tok.size()) {
      size_t q = tok.find('/', p);
      if (q == std::string::npos) q = tok.size();
      const std::string f = tok.substr(p, q - p);
      p = q + 1;
      if (f.compare(0, 5, "block") == 0) block = atoi(f.c_str() + 5);
      else if (f.compare(0, 5, "batch") == 0) batch = atoi(f.c_str() + 5);
      else if (f == "regs85") cap = 0;
      else if (f == "regs64") cap = 1;
      else if (f == "regs51") cap = 2;
      else if (f == "resident") grid = 1;
      else if (f == "tiled") tiled = 1;
      else return false;
    }
    if (!(block == 64 || block == 128 || block == 256) || !(batch == 1 || batch == 2 || batch == 4 || batch == 8))
      return false;
    if ((kind == 2 && batch > 2) || (tiled && !tiles)) return false;
    t.block[kind] = block;
    t.batch[kind] = batch;
    t.grid[kind] = grid;
    t.tiled[kind] = tiled;
    if (kind == 2) t.cap_low = cap;
  }
  return true;
}

// A fixed launch configuration (the autotuner's description) instead of timing
static int apply_tuning(swe_ctx* c, const char* spec, const char* what) {
  KernelTune t;
  if (!parse_tuning(spec, c->tiles_ok, t)) return fail(c, SWE_ERR_ARG, std::string("bad ") + what + ": " + spec);
  c->tune = t;
  c->tuned = true;
  c->tuning = std::string("thread-per-row SELL-32; fixed ") + spec;
  drop_graphs(c);
  return SWE_OK;
}

static int autotune(swe_ctx* c) {
  if (!is_mixed(c)) { c->tuned = true; return SWE_OK; }
  if (const char* spec = getenv("SWE_TUNE")) return apply_tuning(c, spec, "SWE_TUNE");
  int rc;
  std::vector<InstState> saved;
  if ((rc = save_state(c, saved))) return rc;
  std::vector<InstState> run = saved;
  for (auto& st : run) { st.done = 0; if (!(st.dt > 0)) inst_set_dt(st, 1e-6); }
  if ((rc = restore_done(c, run))) return rc;
  const cudaStream_t s = c->stream;
  StageArgsMix a{c->G, c->d_C, c->d_St, c->mA, c->mA, c->mB, c->wm, 1, c->d_err, c->block};
  a.tiles = c->tiles_ok ? &c->tiles : nullptr;
  a.f64 = is_split(c);
  a.type1 = has_type1(c);
  KernelTune t = c->tune;
  launch_dt_mix(c->G, c->d_C, c->d_St, c->mA, c->wm.dlam, c->wm.alpha, c->d_err, t, a.tiles, s);   // populate every work array once
  launch_stage_mix(a, s, nullptr, t);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int blocks[3] = {64, 128, 256};
  const int batches[4] = {1, 2, 4, 8};
  // kernels are timed as in stages 2 and 3 (k_low computes lambda_max, k_update
  // reads u0 for the RK combination): two of the three stages of a step
  StageArgsMix a_low = a;
  a_low.rk_stage = 2;
  std::string desc;
  const char* names[5] = {"dt", "node", "low", "fct", "update"};
  // SWE_TILED=0 leaves the shared-memory variants out, SWE_TILED=1 takes them
  const char* tenv = getenv("SWE_TILED");
  for (int kind = 0; kind < 5; kind++) {
    float best = 1e30f;
    int bb = t.block[kind], bt = t.batch[kind], bc = t.cap_low, bg = t.grid[kind], btl = t.tiled[kind];
    // grid modes: a thread per row, resident grid, shared-memory tiles
    const bool tiles = a_low.tiles && kind_has_tiles(kind) && !(tenv && tenv[0] == '0');
    const int gm0 = (tiles && tenv && tenv[0] == '1') ? 2 : 0, n_modes = tiles ? 3 : 2;
    for (int ib = 0; ib < 3; ib++)
      for (int it = 0; it < 4; it++)
        for (int cap = 0; cap < (kind == 2 ? 3 : 1); cap++)
          for (int gm = gm0; gm < n_modes; gm++) {
            if (kind == 2 && batches[it] > 2) continue;
            KernelTune v = t;
            v.block[kind] = blocks[ib];
            v.batch[kind] = batches[it];
            v.grid[kind] = gm == 1;
            v.tiled[kind] = gm == 2;
            if (kind == 2) v.cap_low = cap;
            float tmin = 1e30f;
            for (int rep = 0; rep < 3; rep++) {
              cudaEventRecord(e0, s);
              if (kind == 0) launch_dt_mix(c->G, c->d_C, c->d_St, c->mA, c->wm.dlam, c->wm.alpha, c->d_err, v, a.tiles, s);
              else launch_kernel_mix(kind, a_low, v, s);
              cudaEventRecord(e1, s);
              CK(cudaEventSynchronize(e1));
              float ms = 0.f;
              cudaEventElapsedTime(&ms, e0, e1);
              tmin = std::min(tmin, ms);
            }
            if (tmin < best) {
              best = tmin; bb = blocks[ib]; bt = batches[it]; bg = gm == 1; btl = gm == 2;
              if (kind == 2) bc = cap;
            }
          }
    t.block[kind] = bb;
    t.batch[kind] = bt;
    t.grid[kind] = bg;
    t.tiled[kind] = btl;
    if (kind == 2) t.cap_low = bc;
    char buf[96];
    snprintf(buf, sizeof buf, "%s%s:block%d/batch%d%s%s", kind ? " " : "", names[kind], bb, bt,
             kind == 2 ? (bc == 2 ? "/regs51" : bc ? "/regs64" : "/regs85") : "",
             bg ? "/resident" : (btl ? "/tiled" : ""));
    desc += buf;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(cudaGetLastError());
  CK(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), s));
  if ((rc = restore_done(c, saved))) return rc;
  c->tune = t;
  c->tuned = true;
  c->tuning = "thread-per-row SELL-32; autotuned " + desc;
  drop_graphs(c);
  return SWE_OK;
}

SWE_API int swe_autotune(swe_ctx* c) {
  NvtxRange nvtx("swe_autotune");
  if (!c) return SWE_ERR_ARG;
  return autotune(c);
}

SWE_API int swe_set_tuning(swe_ctx* c, const char* spec) {
  if (!c || !spec) return SWE_ERR_ARG;
  if (!is_mixed(c)) { c->tuned = true; return SWE_OK; }
  return apply_tuning(c, spec, "tuning");
}

// ---- movie frames (main.f90:119-143, sub_plot.f90:1036-1095) ----
static int frame_setup(swe_ctx* c) {
  if (c->d_frame) return SWE_OK;
  int64_t npmax = 0;
  for (const HostMesh& m : c->meshes) npmax = std::max<int64_t>(npmax, m.np);
  CK(cudaMalloc(&c->d_frame, sizeof(double) * 4 * npmax));
  CK(cudaMallocHost(&c->h_frame, sizeof(double) * 4 * npmax));
  for (int k = 0; k < 2; k++) CK(cudaEventCreateWithFlags(&c->frame_ev[k], cudaEventDisableTiming));
  c->frame_np = npmax;
  c->jj1.resize(c->n_inst);
  for (int b = 0; b < c->n_inst; b++) {
    c->jj1[b] = c->meshes[b].jj;
    for (int& v : c->jj1[b]) v += 1;
  }
  const int dev = c->dev;
  c->frame_worker = std::thread([c, dev]() {
    cudaSetDevice(dev);
    for (;;) {
      swe_ctx::FrameJob job;
      {
        std::unique_lock<std::mutex> lk(c->frame_mu);
        c->frame_cv.wait(lk, [c] { return c->frame_stop || !c->frame_queue.empty(); });
        if (c->frame_queue.empty()) return;
        job = c->frame_queue.front();
      }
      const cudaError_t e = cudaEventSynchronize(c->frame_ev[job.slot]);
      int rc = e == cudaSuccess ? SWE_OK : SWE_ERR_CUDA;
      const HostMesh& m = c->meshes[job.inst];
      const double* f = c->h_frame + (size_t)job.slot * 2 * c->frame_np;
      for (int k = 0; k < 2 && rc == SWE_OK; k++) {
        const std::string& path = job.paths[k];
        // title: the file's name in main.f90's CHARACTER(LEN=200) header, blank-padded
        const size_t cut = path.find_last_of('/');
        std::string title = cut == std::string::npos ? path : path.substr(cut + 1);
        if (title.size() < 200) title.resize(200, ' ');
        rc = swe_write_vtk_2d(path.c_str(), title.c_str(), m.np, m.me, c->jj1[job.inst].data(), m.rr.data(),
                              f + (size_t)k * c->frame_np);
      }
      std::lock_guard<std::mutex> lk(c->frame_mu);
      if (rc && !c->frame_err) {
        c->frame_err = rc;
        c->frame_errmsg = rc == SWE_ERR_CUDA ? std::string("frame copy: ") + cudaGetErrorString(e)
                                             : "cannot write " + job.paths[0] + " or " + job.paths[1];
      }
      c->frame_busy[job.slot] = false;
      c->frame_queue.pop_front();
      c->frame_cv.notify_all();
    }
  });
  return SWE_OK;
}

// Fields of slot k computed on the stream and copied to its page-locked
// buffer on a copy stream (event frame_ev[k] marks the copy's end).
static int frame_enqueue(swe_ctx* c, int inst, double hmax0, int k) {
  const int64_t n0 = c->node_off[inst], nn = c->node_off[inst + 1] - n0;
  double* d = c->d_frame + (size_t)k * 2 * c->frame_np;
  double* h = c->h_frame + (size_t)k * 2 * c->frame_np;
  k_frame_fields<<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(
      c->d_row_of_node + n0, nn, c->precision == SWE_PREC_FP64 ? 1 : 0, c->A, c->mA, c->G.bath, hmax0, d,
      d + c->frame_np);
  CK(cudaGetLastError());
  int rc = copy_setup(c);
  if (rc) return rc;
  CK(cudaEventRecord(c->frame_ev[k], c->stream));
  CK(cudaStreamWaitEvent(c->copy_stream[0], c->frame_ev[k], 0));
  CK(cudaMemcpyAsync(h, d, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->copy_stream[0]));
  CK(cudaMemcpyAsync(h + c->frame_np, d + c->frame_np, sizeof(double) * nn, cudaMemcpyDeviceToHost,
                     c->copy_stream[0]));
  CK(cudaEventRecord(c->frame_ev[k], c->copy_stream[0]));
  return SWE_OK;
}

static int frames_wait(swe_ctx* c) {
  if (!c->d_frame) return SWE_OK;
  std::unique_lock<std::mutex> lk(c->frame_mu);
  c->frame_cv.wait(lk, [c] { return c->frame_queue.empty(); });
  if (c->frame_err) {
    const int rc = c->frame_err;
    c->frame_err = 0;
    return fail(c, rc, c->frame_errmsg);
  }
  return SWE_OK;
}

SWE_API int swe_frame_fields(swe_ctx* c, int inst, double hmax0, double* hpz, double* h) {
  if (!c || inst < 0 || inst >= c->n_inst || !hpz || !h) return fail(c, SWE_ERR_ARG, "bad arguments");
  int rc = frame_setup(c);
  if (rc) return rc;
  if ((rc = frames_wait(c))) return rc;              // both slots free
  if ((rc = frame_enqueue(c, inst, hmax0, 0))) return rc;
  CK(cudaEventSynchronize(c->frame_ev[0]));
  const int64_t nn = c->node_off[inst + 1] - c->node_off[inst];
  std::memcpy(hpz, c->h_frame, sizeof(double) * nn);
  std::memcpy(h, c->h_frame + c->frame_np, sizeof(double) * nn);
  return SWE_OK;
}

SWE_API int swe_frame_async(swe_ctx* c, int inst, double hmax0, const char* hpz_path, const char* h_path) {
  NvtxRange nvtx("swe_frame_async");
  if (!c || inst < 0 || inst >= c->n_inst || !hpz_path || !h_path) return fail(c, SWE_ERR_ARG, "bad arguments");
  int rc = frame_setup(c);
  if (rc) return rc;
  int k;
  {
    std::unique_lock<std::mutex> lk(c->frame_mu);    // a free slot (at most two frames in flight)
    c->frame_cv.wait(lk, [c] { return !c->frame_busy[0] || !c->frame_busy[1]; });
    k = c->frame_busy[0] ? 1 : 0;
    c->frame_busy[k] = true;
  }
  if ((rc = frame_enqueue(c, inst, hmax0, k))) {
    std::lock_guard<std::mutex> lk(c->frame_mu);
    c->frame_busy[k] = false;
    return rc;
  }
  std::lock_guard<std::mutex> lk(c->frame_mu);
  c->frame_queue.push_back(swe_ctx::FrameJob{k, inst, {hpz_path, h_path}});
  c->frame_cv.notify_all();
  return SWE_OK;
}

SWE_API int swe_frames_wait(swe_ctx* c) {
  if (!c) return SWE_ERR_ARG;
  return frames_wait(c);
}

// ---- gauges (main.f90:102-117, condlim.f90:273-283) ----
static void free_gauges(swe_ctx* c) {
  cudaFree(c->d_gauge_inst); cudaFree(c->d_gauge_rows); cudaFree(c->d_gauge_w);
  cudaFree(c->d_gauge_rec); cudaFree(c->d_gauge_count);
  c->d_gauge_inst = c->d_gauge_rows = nullptr;
  c->d_gauge_w = c->d_gauge_rec = nullptr;
  c->d_gauge_count = nullptr;
  c->n_gauges = 0;
  c->gauge_read = 0;
}

SWE_API int swe_gauges_set(swe_ctx* c, int n, const int* inst, const double* rr, int* elem_out) {
  if (!c || n < 0 || n > 1024 || (n && (!inst || !rr))) return fail(c, SWE_ERR_ARG, "bad arguments");
  std::vector<int> gi(n), rows(3 * (size_t)n), elems(n);
  std::vector<double> w(3 * (size_t)n);
  for (int g = 0; g < n; g++) {
    if (inst[g] < 0 || inst[g] >= c->n_inst) return fail(c, SWE_ERR_ARG, "bad gauge instance");
    const HostMesh& m = c->meshes[inst[g]];
    const int e = gauge_element(m, rr + 2 * (size_t)g);
    if (e < 0) return fail(c, SWE_ERR_ARG, "gauge " + std::to_string(g) + " lies in no element");
    gauge_weights(m, e, rr + 2 * (size_t)g, &w[3 * (size_t)g]);
    gi[g] = inst[g];
    elems[g] = e + 1;
    for (int v = 0; v < 3; v++)
      rows[3 * (size_t)g + v] = c->L.new_of_old[inst[g]][m.jj[3 * (size_t)e + v]];
  }
  CK(cudaStreamSynchronize(c->stream));
  free_gauges(c);
  drop_graphs(c);                                    // steps now end with k_gauges (or no longer do)
  if (elem_out) std::copy(elems.begin(), elems.end(), elem_out);
  if (n == 0) return SWE_OK;
  // owned by the gauges (freed by free_gauges), not by the context's buffer list
  auto put = [](auto** d, const auto& v, cudaError_t& e) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(d, v.size() * sizeof(v[0]));
    if (e == cudaSuccess) e = cudaMemcpy(*d, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice);
  };
  cudaError_t st = cudaSuccess;
  put(&c->d_gauge_inst, gi, st);
  put(&c->d_gauge_rows, rows, st);
  put(&c->d_gauge_w, w, st);
  if (st == cudaSuccess) st = cudaMalloc(&c->d_gauge_rec, sizeof(double) * 3 * n * (size_t)swe_ctx::kGaugeRing);
  if (st == cudaSuccess) st = cudaMalloc(&c->d_gauge_count, sizeof(unsigned long long));
  if (st == cudaSuccess) st = cudaMemset(c->d_gauge_count, 0, sizeof(unsigned long long));
  if (st != cudaSuccess) { free_gauges(c); return cuda_check(c, st, "gauges"); }
  c->n_gauges = n;
  return SWE_OK;
}

SWE_API int swe_gauges_read(swe_ctx* c, int max_rows, double* out, int* rows, long long* lost) {
  NvtxRange nvtx("swe_gauges_read");
  if (!c || max_rows < 0 || !rows || (max_rows && !out)) return fail(c, SWE_ERR_ARG, "bad arguments");
  *rows = 0;
  if (lost) *lost = 0;
  if (!c->n_gauges) return SWE_OK;
  unsigned long long count = 0;
  CK(cudaMemcpyAsync(&count, c->d_gauge_count, sizeof count, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const unsigned long long ring = swe_ctx::kGaugeRing;
  unsigned long long first = c->gauge_read;
  if (count - first > ring) {                        // overwritten before this read
    if (lost) *lost = (long long)(count - ring - first);
    first = count - ring;
  }
  const unsigned long long take = std::min<unsigned long long>(count - first, (unsigned long long)max_rows);
  const size_t row_bytes = sizeof(double) * 3 * c->n_gauges;
  for (unsigned long long k = 0; k < take;) {         // at most two contiguous pieces of the ring
    const unsigned long long slot = (first + k) % ring, len = std::min(take - k, ring - slot);
    CK(cudaMemcpyAsync(out + (size_t)k * 3 * c->n_gauges, c->d_gauge_rec + (size_t)slot * 3 * c->n_gauges,
                       row_bytes * len, cudaMemcpyDeviceToHost, c->stream));
    k += len;
  }
  CK(cudaStreamSynchronize(c->stream));
  c->gauge_read = first + take;
  *rows = (int)take;
  return SWE_OK;
}

// The steps of swe_rk3_steps enqueued on the context's stream (the autotuner
// runs on the first call, on the state the stream holds by then), between the
// t0 / t1 events.
static int enqueue_rk3_steps(swe_ctx* c, int nsteps) {
  int rc;
  if (!c->tuned) {
    const char* env = getenv("SWE_AUTOTUNE");
    if (env && env[0] == '0') c->tuned = true;
    else if ((rc = autotune(c))) return rc;
  }
  launch_reset_counters(c->d_St, c->n_inst, c->stream);
  const int chunk = nsteps >= 8 ? 8 : 1;
  long long launches = 0;
  if (!c->t0) { CK(cudaEventCreate(&c->t0)); CK(cudaEventCreate(&c->t1)); }
  if (nsteps >= chunk && chunk > 1 && (rc = build_graph(c, chunk))) return rc;
  CK(cudaEventRecord(c->t0, c->stream));
  // the mixed stage 1 takes alpha from k_dt_mix: one k_node launch fewer
  const long long per_step = 3LL * kLaunchesPerStage + kLaunchesPerStepExtra -
                             (is_mixed(c) ? 1 : 0) + (c->n_gauges ? 1 : 0);
  if (nsteps >= chunk && chunk > 1) {
    for (int k = 0; k + chunk <= nsteps; k += chunk) {
      CK(cudaGraphLaunch(c->gexec, c->stream));
      launches += per_step * chunk;
    }
  }
  const int rem = chunk > 1 ? nsteps % chunk : nsteps;
  if (rem && !c->gexec1 && (rc = capture_steps(c, 1, &c->gexec1))) return rc;
  for (int k = 0; k < rem; k++) {
    CK(cudaGraphLaunch(c->gexec1, c->stream));
    launches += per_step;
  }
  CK(cudaEventRecord(c->t1, c->stream));
  CK(cudaGetLastError());
  c->last_launches = launches;
  c->euler_done = false;
  return SWE_OK;
}

// The instances' clocks and the error word after everything enqueued, in one
// synchronisation.
static int finish_rk3_steps(swe_ctx* c, double* time_out, double* dt_out, int* steps_done) {
  std::vector<InstState> out(c->n_inst);
  CK(cudaMemcpyAsync(out.data(), c->d_St, sizeof(InstState) * c->n_inst, cudaMemcpyDeviceToHost, c->stream));
  const int rc = read_errors(c);
  for (int b = 0; b < c->n_inst; b++) {
    if (time_out) time_out[b] = out[b].time;
    if (dt_out) dt_out[b] = out[b].dt;
  }
  if (steps_done) *steps_done = out[0].steps;
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->t0, c->t1));
  c->last_ms = ms;
  return rc;
}

SWE_API int swe_rk3_steps(swe_ctx* c, int nsteps, double* time_out, double* dt_out, int* steps_done) {
  NvtxRange nvtx("swe_rk3_steps");
  if (!c || nsteps < 0) return fail(c, SWE_ERR_ARG, "bad arguments");
  const int rc = enqueue_rk3_steps(c, nsteps);
  if (rc) return rc;
  return finish_rk3_steps(c, time_out, dt_out, steps_done);
}

SWE_API int swe_rk3_steps_host(swe_ctx* c, const double* un, double* unext, int nsteps, double* time_out,
                               double* dt_out, int* steps_done) {
  NvtxRange nvtx("swe_rk3_steps_host");
  if (!c || nsteps < 0) return fail(c, SWE_ERR_ARG, "bad arguments");
  const int64_t nn = c->node_off[c->n_inst];
  int rc;
  if ((un && (rc = to_device(c, un, false, 0, nn))) || (rc = enqueue_rk3_steps(c, nsteps)) ||
      (unext && (rc = from_device_state(c, unext, false, 0, nn, c->precision == SWE_PREC_FP64 ? &c->A : nullptr,
                                        c->precision == SWE_PREC_FP64 ? nullptr : &c->mA)))) {
    drain(c);
    return rc;
  }
  return finish_rk3_steps(c, time_out, dt_out, steps_done);
}

SWE_API double swe_last_device_ms(const swe_ctx* c) { return c ? c->last_ms : 0.0; }

SWE_API int swe_profile_kernels(swe_ctx* c, int nsteps, double* ms_out) {
  if (!c || nsteps <= 0 || !ms_out) return fail(c, SWE_ERR_ARG, "bad arguments");
  KernelEvents kev;
  for (int k = 0; k < 10; k++) CK(cudaEventCreate(&kev.ev[k]));
  double acc[SWE_NKERNELS] = {0, 0, 0, 0, 0};
  for (int n = 0; n < nsteps; n++) enqueue_step(c, &kev, acc);
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 10; k++) cudaEventDestroy(kev.ev[k]);
  ms_out[0] = acc[0] / nsteps;
  for (int k = 1; k < SWE_NKERNELS; k++) ms_out[k] = acc[k] / (3.0 * nsteps);
  return read_errors(c);
}

SWE_API int swe_mass(swe_ctx* c, double* mass_out) {
  if (!c || !mass_out) return fail(c, SWE_ERR_ARG, "bad arguments");
  CK(cudaMemsetAsync(c->d_mass_acc, 0, 2 * sizeof(double) * c->n_inst, c->stream));
  launch_mass(c->G, c->n_inst, c->precision == SWE_PREC_FP64 ? c->A.h : nullptr,
              c->precision == SWE_PREC_FP64 ? nullptr : c->mA.h, c->d_inst_slice, c->d_mass_part, c->d_mass_acc,
              c->stream);
  CK(cudaGetLastError());
  std::vector<double> acc(2 * c->n_inst);
  CK(cudaMemcpyAsync(acc.data(), c->d_mass_acc, acc.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int b = 0; b < c->n_inst; b++) mass_out[b] = acc[2 * b] + acc[2 * b + 1];
  return SWE_OK;
}

SWE_API long long swe_last_launch_count(const swe_ctx* c) { return c ? c->last_launches : 0; }
SWE_API const char* swe_tuning(const swe_ctx* c) { return c ? c->tuning.c_str() : ""; }
