// Declarations shared by the kernel translation units and the C-ABI layer.
#pragma once
#include "swe_device.cuh"

namespace swe {

// FP64 state, SoA per component (h, qx, qy[, h*eta, h*w]) over the padded rows
struct StateF64 {
  double* h;
  double* q1;
  double* q2;
  double* q3;
  double* q4;
};

// Mixed-precision state: h as a double-float pair (hi + lo, about 48
// significant bits: positivity and mass) plus a packed FP32 node record
// {h shadow, qx, qy, eta} that neighbours gather with one 16-byte load (eta =
// h + z rounded once per node); type 13's h*eta and h*w in FP32.
struct StateMix {
  float2* h;
  float4* nq;
  float* q3;
  float* q4;
};

// Work arrays of one stage
struct WorkF64 {
  double *ovh, *v1, *v2, *ent, *alpha;   // per row
  double* sqgh;                          // per row: sqrt(g |h|)
  double *dL, *muL, *fct;                // per off-diagonal entry
  double *dLii, *muLii;                  // per row: the diagonal of dL, muL
  double *res, *rminus;                  // per row
  StateF64 uL;                           // low-order state
};

struct WorkMix {
  float *alpha, *res;                    // per row
  float* rminus;                         // per row: R^-_i
  float2* dmu;                           // per entry: (d_ij, mu_ij), one 8-byte load
  float* dlam;                           // per entry: |c_ij| lambda_max from k_dt_mix (stage 1)
  float2* hL;                            // low-order depth (double-float)
  double* hL64;                          // precision split: the FP64 low-order depth (hL's storage), or null
  double* rminus64;                      // precision split: FP64 R^-_i, or null
  float2* qL;                            // low-order momenta
  float *q3L, *q4L;                      // low-order h*eta, h*w (type 13)
};

struct StageArgs {
  Graph G;
  const InstConst* C;
  InstState* St;
  StateF64 u, u0, out;
  WorkF64 w;
  int rk_stage;
  double* lij_out;
  unsigned* err;
  int block;
  int entropy = 0;   // some instance uses 'entropy_visc': launch k_entropy
  const double* dij_in = nullptr;   // stage 1: d_ij of k_dt on the same state (bit-identical)
  int skip_node = 0;                // stage 1: k_node already ran on this state (before k_dt)
};

// Tiles of rows for the shared-memory variants of the entry loops: a block
// owns `tile_rows` consecutive rows (a compact patch of the mesh in Morton
// order) and first copies the node records of its rows and of its halo (the
// rows outside the tile that its entries reference) into shared memory; the
// entry loops then read neighbours there by tile-local position.
struct TileCtl {
  const int16_t* loc;     // per entry: col - tile start, or tile_rows + halo index
  const int* halo_ptr;    // n_tiles + 1
  const int* halo_rows;   // ascending per tile
  int tile_rows;
  int halo_cap;           // largest halo
};

struct StageArgsMix {
  Graph G;
  const InstConst* C;
  InstState* St;
  StateMix u, u0, out;
  WorkMix w;
  int rk_stage;
  unsigned* err;
  int block;
  const TileCtl* tiles = nullptr;  // row tiles of the shared-memory variants, or null
  bool f64 = false;                 // precision split: h^L, R^- and the depth's limited sum in FP64
  bool type1 = false;               // some instance runs 'viscous' with viscous_type 'type1'
};

// Optional per-kernel event timing: when non-null, ev[2k], ev[2k+1] bracket
// the launch of kernel kind k (0 dt, 1 node, 2 low, 3 fct, 4 update).
struct KernelEvents {
  cudaEvent_t ev[10];
};

void launch_stage_f64(const StageArgs& a, cudaStream_t s, const KernelEvents* kev = nullptr);
void launch_dt_f64(const Graph& G, const InstConst* C, InstState* St, const StateF64& u, double* d_out,
                   double* dii_out, unsigned* err, int block, cudaStream_t s, const WorkF64* node = nullptr);
void launch_node_f64(const StageArgs& a, cudaStream_t s);   // per-node arrays of the state a.u
void launch_step_begin(const InstConst* C, InstState* St, int n_inst, cudaStream_t s);
void launch_step_end(InstState* St, int n_inst, cudaStream_t s);
void launch_reset_counters(InstState* St, int n_inst, cudaStream_t s);
void launch_fct_positivity_f64(const Graph& G, const InstConst* C, const double* unext, const double* mat,
                               const double* matii, double* rtmp, double* lij, cudaStream_t s);
void launch_fct_generic_f64(const Graph& G, double* unext, const double* maxn, const double* minn, const double* dg,
                            const double* mat, const double* matii, double* rplus, double* rminus, cudaStream_t s);

// Launch configuration of the mixed kernels, per kernel kind (0 dt, 1 node,
// 2 low, 3 fct, 4 update): block size, entry batch (1, 2, 4 or 8; 1 or 2
// for low), grid (one thread per row, or a resident grid striding over the
// rows, or one block per tile of rows with shared-memory neighbours), and for
// low a register cap (cap_low 0, 1, 2: at least 3, 4 or 5 resident blocks of
// 256 threads per SM, i.e. at most 85, 64 or 51 registers; the tightest
// spills a little).  Chosen by the autotuner in swe_api.cu.  Every choice
// performs the same IEEE operations in the same entry order (the mixed
// kernels are built without FMA contraction and spell out every fused
// multiply-add), so every choice gives bit-identical results.
struct KernelTune {
  int block[5] = {128, 128, 128, 128, 128};
  int batch[5] = {1, 1, 1, 1, 1};
  int grid[5] = {0, 0, 0, 0, 0};   // 0: a thread per row; k: k resident grids striding over the rows
  int cap_low = 0;
  int tiled[5] = {0, 0, 0, 0, 0};  // 1: the shared-memory tile variant (grid: one block per tile)
};

void launch_stage_mix(const StageArgsMix& a, cudaStream_t s, const KernelEvents* kev, const KernelTune& t);
// dynamic shared memory of one tile block (d: with the FP64 R^- of the precision split)
size_t tile_smem_bytes(const TileCtl& tc, bool d = false);
void launch_kernel_mix(int kind, const StageArgsMix& a, const KernelTune& t, cudaStream_t s);
bool kind_has_tiles(int kind);   // kernel kinds with a shared-memory tile variant
void launch_dt_mix(const Graph& G, const InstConst* C, InstState* St, const StateMix& u, float* dlam, float* alpha,
                   unsigned* err, const KernelTune& t, const TileCtl* tiles, cudaStream_t s);
void launch_refresh_eta(const Graph& G, StateMix u, cudaStream_t s);

// Diagnostics (swe_diag.cu): field index kFieldH32 selects h^(3/2)
constexpr int kFieldH32 = 16;
// per-warp partial sums k_norms writes for me elements (4 doubles each)
int64_t norm_partials(int me);
// Total mass sum m_i h_i per instance in a fixed order (bit-reproducible):
// per-slice double-double partials (part: 2 per slice), then one block per
// instance adds its slices (inst_slice: n_inst + 1 slice offsets) into
// acc[2 b], acc[2 b + 1].  One of h64 (FP64 state) and hdf (mixed) is non-null.
void launch_mass(const Graph& G, int n_inst, const double* h64, const float2* hdf, const int64_t* inst_slice,
                 double* part, double* acc, cudaStream_t s);
void launch_norms(int field, int precision, const StateF64& a, const StateMix& mx, const int* jj, const double* rj,
                  int me, const int* row_of_node, const double* f_anal, double* part, double* acc, cudaStream_t s);

// kernels launched per stage / per step (for launch accounting)
constexpr int kLaunchesPerStage = 4;
constexpr int kLaunchesPerStepExtra = 3;   // k_dt, k_step_begin, k_step_end

}  // namespace swe
