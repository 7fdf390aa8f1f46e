/*
 * swe_gpu.h — C ABI of the GB300 (sm_103a) explicit P1 shallow-water step.
 *
 * This is the drop-in boundary for the public surface of the reference's
 * Fortran modules `update` and `fct` (t-bltg/shallow-water-eric):
 *
 *   MODULE update   SOURCES/update.f90:1-16   construct_matrices, euler,
 *                                             compute_dij; public data dij,
 *                                             lumped, diag
 *   MODULE fct      SOURCES/fct.f90:1-5       FCT_positivity
 *   time loop       SOURCES/main.f90:61-91    COMPUTE_DT (:166-174) + SSP-RK3
 *                                             + bdy (:176-188)
 *
 * Conventions
 *  - Every host pointer is owned by the caller and only borrowed for the
 *    duration of the call.  State arrays use the reference layout
 *    un(syst_size, np): column-major FP64, component fastest, nodes in the
 *    caller's (reference) numbering.  Node/element indices are 1-based.
 *  - Every call returns an int status: SWE_OK or one of SWE_ERR_*.  The
 *    reference STOPs where this layer returns SWE_ERR_NEG_H (check_hmin,
 *    SOURCES/update.f90:810-822) or SWE_ERR_DELTA (compute_lambda_vacc,
 *    SOURCES/condlim.f90:934-937).  swe_last_error() gives the message.
 *  - One context serves one host thread and owns one CUDA stream; calls are
 *    synchronous on return.  There is no CPU fallback: a context cannot be
 *    created without a CUDA device.
 *  - A context holds one mesh, or a batch of independent meshes advanced
 *    together (each with its own parameters, dt and time).
 */
#ifndef SWE_GPU_H
#define SWE_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  SWE_OK = 0,
  SWE_ERR_NEG_H = 1,     /* min h < 0 after a stage (check_hmin)           */
  SWE_ERR_DELTA = 2,     /* Delta < 0 in the lambda_max bound              */
  SWE_ERR_NAN = 3,       /* non-finite value produced                      */
  SWE_ERR_TIMEOUT = 4,   /* a bounded device wait gave up                  */
  SWE_ERR_CUDA = 5,      /* CUDA runtime error                             */
  SWE_ERR_ARG = 6,       /* invalid argument                               */
  SWE_ERR_MESH = 7       /* mesh rejected (row longer than 90 entries, ...) */
};

/* viscosity_type values (SOURCES/read_data.f90:57-58 marker) */
enum { SWE_VISC_GALERKIN = 0, SWE_VISC_VISCOUS = 1, SWE_VISC_ENTROPY = 2, SWE_VISC_FCT = 3 };
/* precision values.  SWE_PREC_MIXED: FP32 fluxes, viscosities, limiter and
 * momenta with a double-float depth (no FP64 instruction per edge or row).
 * SWE_PREC_MIXED_F64: the same FP32 fluxes, with the per-row low-order depth
 * update, the limiter's Q^-, P^-, R^- (and its exact dry test) and the
 * l_ij-weighted depth sum in FP64. */
enum { SWE_PREC_FP64 = 0, SWE_PREC_MIXED = 1, SWE_PREC_MIXED_F64 = 2 };

/* The subset of the reference's `inputs` record (SOURCES/read_data.f90:4-32)
 * and module constants the step reads.  Field order is part of the ABI. */
typedef struct swe_params {
  double gravity;        /* inputs%gravity                                   */
  double dt;             /* inputs%dt (used by the per-call entry points)    */
  double cfl;            /* inputs%CFL                                       */
  double htiny;          /* inputs%htiny = epsilon*max_water_h               */
  double mannings;       /* inputs%mannings (type_test 9, 10)                */
  double lambda_sgn;     /* inputs%lambdaSGN (type_test 13)                  */
  double max_water_h;    /* boundary_conditions max_water_h                  */
  int type_test;         /* selects flux variant and source term             */
  int syst_size;         /* 3, or 5 for type_test 13                         */
  int viscosity_type;    /* SWE_VISC_*                                       */
  int viscous_type;      /* 1 = 'type1', 2 = 'type2'                         */
  int if_alpha_limit;    /* inputs%if_alpha_limit                            */
  int if_lumped;         /* inputs%if_lumped (only lumped is supported)      */
  int if_roundoff_fix;   /* update.f90:15 module constant                    */
  int precision;         /* SWE_PREC_FP64, SWE_PREC_MIXED or _MIXED_F64      */
} swe_params;

typedef struct swe_ctx swe_ctx;

/* construct_matrices (SOURCES/update.f90:18-132) for one mesh: builds the CSR
 * pattern, consistent and lumped mass, diag and c_ij, renumbers the nodes
 * along a Z-order (Morton) curve of their coordinates (SWE_ORDER=rcm: reverse
 * Cuthill-McKee) and uploads the SELL-32 edge graph.
 * jj(3, me) 1-based counter-clockwise triangles, rr(2, np), bath(np). */
int swe_create(swe_ctx** ctx, int np, int me, const int* jj, const double* rr,
               const double* bath, const swe_params* params);

/* Batched variant: n_inst independent meshes, concatenated.  np[b], me[b]
 * give each instance's sizes; jj holds each instance's own 1-based node
 * numbers, instance after instance; rr, bath likewise; params[b] per
 * instance (all instances must share syst_size and precision). */
int swe_create_batch(swe_ctx** ctx, int n_inst, const int* np, const int* me,
                     const int* jj, const double* rr, const double* bath,
                     const swe_params* params);

void swe_destroy(swe_ctx* ctx);
const char* swe_last_error(const swe_ctx* ctx);

/* Replace the parameters of instance `inst` (0-based); dt is the inputs%dt
 * used by swe_euler. */
int swe_set_params(swe_ctx* ctx, int inst, const swe_params* params);

/* Replace the bathymetry of instance `inst` (np values, caller numbering).
 * The reference's driver builds the matrices (construct_matrices,
 * SOURCES/main.f90:21) before init() sets bath (:31), so a Fortran shim
 * creates the context with a zero bathymetry and sets it here. */
int swe_set_bath(swe_ctx* ctx, int inst, const double* bath);

/* Constant Dirichlet data applied after every RK stage by swe_rk3_steps,
 * like bdy (SOURCES/main.f90:176-188) with values that do not depend on t:
 * comp is the 0-based component, js 1-based node numbers of instance
 * `inst`, vals the values (NULL = zeros).  Replaces earlier data for comp. */
int swe_set_dirichlet(swe_ctx* ctx, int inst, int comp, int n, const int* js, const double* vals);

/* Time-dependent Dirichlet data on the device loop, like bdy
 * (SOURCES/main.f90:176-188) with sol_anal (SOURCES/condlim.f90:311-831):
 * after every RK stage swe_rk3_steps writes sol_anal(comp+1, rr(js), t) of
 * the instance's type_test into component comp of nodes js, with t the
 * reference's bdy time of that stage (to + dt, then (to + dt) + dt/2, then
 * (to + dt/2) + dt; main.f90:78, 84, 90).  Built for type_test 5 and 13 and
 * the components h, qx, qy (0-2); others -> SWE_ERR_ARG.  Replaces earlier
 * data for comp, as swe_set_dirichlet does (and is replaced by it). */
int swe_set_dirichlet_anal(swe_ctx* ctx, int inst, int comp, int n, const int* js);

/* Sizes and the assembled matrices in the reference numbering and CSR order
 * (1-based ia/ja, like mass%ia/ja).  Any output pointer may be NULL. */
int swe_sizes(const swe_ctx* ctx, int inst, int* np, int* nnz);
int swe_get_matrices(swe_ctx* ctx, int inst, int* ia, int* ja, double* mass,
                     double* lumped, int* diag, double* cx, double* cy);

/* compute_dij (SOURCES/update.f90:291-326) on instance `inst` for the state
 * un(S, np); dij (nnz, CSR order) and dt_out = CFL/max(|d_ii|/m_i)
 * (COMPUTE_DT, SOURCES/main.f90:166-174) are optional outputs. */
int swe_compute_dij(swe_ctx* ctx, int inst, const double* un, double* dij, double* dt_out);

/* euler (SOURCES/update.f90:134-289): one forward-Euler stage with the
 * instance's viscosity settings and inputs%dt = params.dt. */
int swe_euler(swe_ctx* ctx, int inst, const double* un, double* unext);

/* Intermediates of the last swe_euler call of instance `inst`, in CSR order
 * (nnz) or node order (np); any pointer may be NULL.  dij_low/muij_low are
 * the alpha-limited low-order viscosities (dijL, muijL), res the entropy
 * residual per node, fctmat the antidiffusive matrix, rminus R^-_i, lij the
 * limiter l_ij, u_low the low-order state (S, np). */
int swe_euler_intermediates(swe_ctx* ctx, int inst, double* dij_low, double* muij_low,
                            double* alpha, double* u_low, double* res, double* fctmat,
                            double* rminus, double* lij);

/* FCT_positivity (SOURCES/fct.f90:5-42): unext = (lumped/dt)*h^L (np),
 * mat = f_ij (nnz, CSR order) -> lij (nnz, CSR order). */
int swe_fct_positivity(swe_ctx* ctx, int inst, const double* unext, const double* mat, double* lij);

/* FCT_generic (SOURCES/SAFE/fct.f90:3-43), the two-sided Zalesak limiter with
 * local bounds: unext (np, in/out) is limited in place using maxn, minn (np),
 * the antidiffusive matrix mat (nnz, CSR order, diagonal included) and dg
 * (np; NULL = the lumped mass).  FP64 contexts only. */
int swe_fct_generic(swe_ctx* ctx, int inst, double* unext, const double* maxn, const double* minn,
                    const double* mat, const double* dg);

/* Gauss weights rj (3 per element) and points rr_gauss ((2, 3*me)
 * column-major) of the 3-point rule (SFEMaNS/GAUSS_POINTS_OBJET/
 * gauss_points_2d_p1.f90, r_gauss of SOURCES/main.f90:207), in the caller's
 * element order, to evaluate analytic data for swe_norms.  Either may be
 * NULL. */
int swe_gauss_points(swe_ctx* ctx, int inst, double* rj, double* rr_gauss);

/* Quadrature norms of one field of the device-resident state (after
 * swe_upload / swe_rk3_steps), with no download of the state:
 * l1 = sum |f - f_anal| rj, l2 = sqrt(sum (f - f_anal)^2 rj) over the Gauss
 * points (ns_anal_l1, ns_anal_0, ns_l1: SFEMaNS/FEMSUB_OBJET/
 * fem_tn.f90:1513-1553, 1679-1716).  field: component 0..syst_size-1, or
 * SWE_FIELD_H32 for h^(3/2) (the monitor of SOURCES/main.f90:94-99).
 * f_anal: 3 values per element at the Gauss points, or NULL for zero.
 * l1, l2 may be NULL. */
#define SWE_FIELD_H32 16
int swe_norms(swe_ctx* ctx, int inst, int field, const double* f_anal, double* l1, double* l2);

/* Device-resident fast path.  upload/download move every instance's state;
 * un is the concatenation of the instances' un(S, np_b) blocks. */
int swe_upload(swe_ctx* ctx, const double* un);
int swe_download(swe_ctx* ctx, double* un);
/* Same, with un already in device memory (concatenated reference layout). */
int swe_upload_device(swe_ctx* ctx, const double* d_un);
int swe_download_device(swe_ctx* ctx, double* d_un);

/* Set every instance's time and final time (arrays of n_inst, NULL time =
 * keep). */
int swe_set_time(swe_ctx* ctx, const double* time, const double* t_final);
/* The instances' time, t_final and last dt (n_inst each; any may be null):
 * with swe_download, what a checkpoint needs to resume with swe_upload and
 * swe_set_time. */
int swe_get_time(swe_ctx* ctx, double* time, double* t_final, double* dt);

/* Advance nsteps iterations of the reference time loop (SOURCES/main.f90:
 * 61-91) on the device: per instance, while time < t_final: dt =
 * CFL/max|d_ii|/m_i, three SSP-RK stages, Dirichlet data after each stage,
 * time += dt (dt is not clipped at t_final, as in the reference).  Instances
 * that reached t_final stop.  The step sequence runs as one captured CUDA
 * graph.  time_out / dt_out (n_inst each, nullable) receive the instances'
 * time and last dt; steps_done (nullable) the number of steps instance 0 ran. */
int swe_rk3_steps(swe_ctx* ctx, int nsteps, double* time_out, double* dt_out, int* steps_done);

/* swe_upload(un), swe_rk3_steps(nsteps), swe_download(unext) as one call with
 * one synchronisation: the host-buffer form of the reference's time loop
 * (SOURCES/main.f90:61-91 around euler, SOURCES/update.f90:134-289), where
 * un and unext are host arrays.  The state goes up in chunks on several copy
 * streams, the steps run as the captured graph, and the new state comes back
 * in chunks while the next chunk is permuted.  un == NULL keeps the device
 * state, unext == NULL skips the download; un == unext is allowed.  Results
 * are bit-identical to the three separate calls. */
int swe_rk3_steps_host(swe_ctx* ctx, const double* un, double* unext, int nsteps, double* time_out,
                       double* dt_out, int* steps_done);

/* Total water mass sum_i m_i h_i per instance: double-double sums added in a
 * fixed order, so every call on the same state gives the same bits. */
int swe_mass(swe_ctx* ctx, double* mass_out);

/* Kernel launches issued by the last swe_rk3_steps call (for accounting). */
long long swe_last_launch_count(const swe_ctx* ctx);

/* Device time (ms, CUDA events on the context's stream) of the kernels of the
 * last swe_rk3_steps call. */
double swe_last_device_ms(const swe_ctx* ctx);

/* Runs nsteps time steps kernel by kernel with a CUDA event pair around every
 * launch and returns the average duration (ms) per launch of each kernel
 * kind in ms_out[SWE_NKERNELS] (order: dt, node, low, fct, update). */
enum { SWE_NKERNELS = 5 };
int swe_profile_kernels(swe_ctx* ctx, int nsteps, double* ms_out);

/* Autotuner: times every block-size / entry-batch / grid variant of the
 * mixed kernels (including the shared-memory row-tile variants) on the
 * current state and keeps the fastest per kernel (every variant gives the
 * same bits).  swe_rk3_steps runs it on its first call unless the environment
 * sets SWE_AUTOTUNE=0.  swe_tuning names the chosen configuration; setting
 * SWE_TUNE to that description (the text after "autotuned ") makes a later
 * context launch exactly those variants without timing (a malformed value
 * -> SWE_ERR_ARG). */
int swe_autotune(swe_ctx* ctx);
const char* swe_tuning(const swe_ctx* ctx);
/* Launch exactly the variants of a tuning description (the text after
 * "autotuned " or "fixed " in swe_tuning) without timing, as SWE_TUNE does;
 * a checkpoint stores the description and a resumed run sets it, so the
 * resumed context runs the same launch shapes.  Every variant gives the
 * same bits, so this changes speed only.  No-op on FP64 contexts; a
 * malformed description -> SWE_ERR_ARG. */
int swe_set_tuning(swe_ctx* ctx, const char* spec);

/* FCT_positivity for callers that cannot allocate device memory.
 *
 * No counterpart in the reference: its FCT_positivity (SOURCES/fct.f90:5-42)
 * works on host arrays.  This entry point serves callers that manage device
 * memory themselves (their own pool or arena, or a driver that forbids
 * further cudaMalloc calls): every input and output is a device pointer the
 * caller owns, and the only scratch (R^- per node) lives in a fixed device
 * array compiled into the library.  Nothing is allocated or freed.
 *   np        rows (1..SWE_NOALLOC_MAX_NODES; larger values -> SWE_ERR_ARG)
 *   d_ia      row pointers, np+1 ints, 1-based like mass%ia: ia(1) = 1,
 *             non-decreasing, ia(np+1)-1 entries in d_mat and d_lij
 *   d_ja      column indices, 1-based, each in 1..np (checked on the device:
 *             a column out of range is not read through and the call
 *             returns SWE_ERR_ARG with d_lij unspecified)
 *   d_unext   (lumped/dt)*h^L per row
 *   d_mat     f_ij per CSR entry
 *   htiny     inputs%htiny
 *   d_lij     l_ij per CSR entry (output)
 *   stream    cudaStream_t to launch on (NULL = default stream); the call
 *             synchronises that stream before returning, so it cannot be
 *             recorded into a CUDA graph (stream capture).
 * The scratch array (SWE_NOALLOC_MAX_NODES doubles, 8 MiB) is held by every
 * GPU that loads the library until the process exits and is shared by all
 * calls: calls that overlap on the GPU race, so serialise them.  The first
 * call on a device looks up the array's address for that device (with it
 * current). */
#define SWE_NOALLOC_MAX_NODES (1 << 20)
int swe_fct_positivity_noalloc(int np, const int* d_ia, const int* d_ja, const double* d_unext,
                               const double* d_mat, double htiny, double* d_lij, void* stream);

/* ---- movie frames and VTK output (the frame block of the time loop,
 * SOURCES/main.f90:119-143, and vtk_2d, SFEMaNS/FEMSUB/sub_plot.f90:1036-1095)
 *
 * swe_write_vtk_2d writes one P1 scalar field as the legacy-VTK text that
 * vtk_2d writes, byte for byte (P1 branch): title is the file name vtk_2d
 * puts on its second line, jj (3, me) is 1-based like mesh%jj, rr (2, np)
 * like mesh%rr.  Host only; SWE_ERR_ARG if the file cannot be written.
 *
 * swe_frame_fields computes on the device the two fields of a movie frame
 * from the current state of instance inst, in the reference node order:
 *   hpz = h + bath, or -1e-7 hmax0 + bath where h <= 1e-4 hmax0  (hpz_k.vtk)
 *   h   = h,        or 0                  where h <= 1e-4 hmax0  (h_k.vtk)
 * with hmax0 = MAXVAL of the initial depth (main.f90:32), and copies them to
 * the host arrays (np doubles each).
 *
 * swe_frame_async does the same into one of two page-locked buffers and
 * returns at once; a worker thread writes hpz_path and h_path with
 * swe_write_vtk_2d while the caller keeps stepping (at most two frames in
 * flight: a third call waits for a free buffer).  The title line carries
 * the file's name blank-padded to 200 characters, as main.f90 passes its
 * CHARACTER(LEN=200) header to vtk_2d.  swe_frames_wait returns
 * once every queued frame is on disk, with the first write error if any. */
int swe_write_vtk_2d(const char* path, const char* title, int np, int me, const int* jj, const double* rr,
                     const double* field);
int swe_frame_fields(swe_ctx* ctx, int inst, double hmax0, double* hpz, double* h);
int swe_frame_async(swe_ctx* ctx, int inst, double hmax0, const char* hpz_path, const char* h_path);
int swe_frames_wait(swe_ctx* ctx);

/* ---- gauges (the Malpasset gauge block of the time loop,
 * SOURCES/main.f90:102-117, located as in condlim.f90:273-283)
 *
 * swe_gauges_set places n point gauges (rr (2, n), instance inst[g]): each
 * lies in the first element where the reference's `inside` holds
 * (SFEMaNS/FEMSUB_OBJET/post_interp.f90:492-524) and carries its
 * FE_interpolation weights (:206-255); elem_out (optional) gets the 1-based
 * element numbers.  A gauge in no element -> SWE_ERR_ARG.  From then on every
 * time step ends with one more kernel, which appends a row per gauge to a
 * device ring of 4096 steps: (time, SUM(h(jj(:,m)) ff),
 * SUM((h + bath)(jj(:,m)) ff)); NaN for an instance that did not step.  n = 0
 * removes the gauges.  swe_gauges_read copies the rows recorded since the
 * previous read, oldest first, as out(3, n, rows) (at most max_rows); lost
 * (optional) counts rows overwritten before they were read. */
int swe_gauges_set(swe_ctx* ctx, int n, const int* inst, const double* rr, int* elem_out);
int swe_gauges_read(swe_ctx* ctx, int max_rows, double* out, int* rows, long long* lost);

#ifdef __cplusplus
}
#endif
#endif /* SWE_GPU_H */
