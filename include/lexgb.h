/*
 * lexgb.h - C ABI of lex_gb300, a GB300 (sm_103a) implementation of LEX's fully
 * compressible dynamical-core time step (solver_opt = 2: explicit time splitting,
 * WENO5 advection, Smagorinsky SGS, acoustic sub-steps, pressure gradient, Coriolis,
 * periodic / rigid-lid halos, Wicker-Skamarock RK3).
 *
 * Conventions
 *   - Every call returns int status: LEXGB_OK (0) or an LEXGB_ERR_* code; the message of
 *     the last failure on the calling thread is available from lexgb_last_error().
 *   - Host arrays use the reference's padded C-order [x][y][z] layout (z fastest) with
 *     ngx = ngy = 3 lateral ghost cells and ngz = 1 ghost level:
 *        scalars (theta, pi', qv)  (nx+6) x (ny+6) x (nz+2)
 *        u                         (nx+7) x (ny+6) x (nz+2)
 *        v                         (nx+6) x (ny+7) x (nz+2)
 *        w                         (nx+6) x (ny+6) x (nz+3)
 *     exactly as setup_lex.py:39-49 allocates them.  Ghost values on input are ignored
 *     (they are periodic / edge copies by construction); on output they are filled the way
 *     padding3_array / padding3u_array / padding3v_array + set_w_bc fill them.
 *   - Field order is the reference's phys_state tuple: (theta, u, v, w, pi', qv)
 *     (setup_lex.py:66).
 *   - Device memory is owned by the context.  A context is not thread-safe; all its work
 *     is ordered on one CUDA stream (its own, or the one given to lexgb_set_stream).
 */
#ifndef LEXGB_H
#define LEXGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    LEXGB_OK = 0,
    LEXGB_ERR_ARG = 1,      /* bad dimensions, null pointer, out-of-range option */
    LEXGB_ERR_CUDA = 2,     /* a CUDA runtime call failed */
    LEXGB_ERR_NAN = 3,      /* a non-finite value was found in the state */
    LEXGB_ERR_TIMEOUT = 4,  /* a bounded device-side wait gave up */
    LEXGB_ERR_STATE = 5,    /* call order violated (e.g. stepping before a base state is set) */
    LEXGB_ERR_ALLOC = 6     /* device allocation failed */
};

enum { LEXGB_F32 = 0, LEXGB_F64 = 1 };

typedef struct lexgb_config {
    int nx, ny, nz;          /* interior cells; nx, ny >= 4, nz >= 6 */
    double dx, dy, dz;       /* uniform spacings [m] (namelist_n_constants.py:17-19) */
    double dt;               /* RK3 big-step length [s] (namelist_n_constants.py:7) */
    int n_sound;             /* acoustic sub-steps per big step (namelist_n_constants.py:13) */
    int turb_opt;            /* 0: none, 1: Smagorinsky (namelist_n_constants.py:48) */
    int cor_opt;             /* 0: none, 1: Coriolis, 2: Coriolis + large-scale pressure gradient */
    double f_cor;            /* Coriolis parameter (namelist_n_constants.py:39) */
    double theta_ref;        /* constant subtracted from theta on the device; 0 = use theta0 at the first level */
    int acoustic_pairs;      /* 0 (default): one acoustic sub-step per launch; 1: two per launch (temporal blocking) */
    int l2_persist;          /* 0 (default): keep the acoustic sub-steps' per-stage inputs (R_u, R_v, R_w, theta_rho)
                                in a persisting L2 window; -1: normal caching */
    double cs;               /* Smagorinsky constant; 0 (default): 0.18 (turbulence.py:433) */
    int acoustic_kernel;     /* how the acoustic sub-steps run: LEXGB_ACOUSTIC_AUTO (0, default: the fastest
                                form measured for the grid), _ROWS (one launch per sub-step, float4 rows),
                                _TILE (one launch per sub-step, 32 x 4 x 8 blocks sharing values; nx % 32 == 0,
                                ny % 4 == 0), _PERSISTENT (stages 1 and 2 as one cooperative launch each, pi' kept
                                in shared memory, inputs staged by TMA; nx % 32 == 0, ny % 8 == 0, nz <= 99,
                                a 32 x 8 tile per SM).  A form the grid does not allow falls back to AUTO. */
} lexgb_config;

enum { LEXGB_ACOUSTIC_AUTO = 0, LEXGB_ACOUSTIC_ROWS = 1, LEXGB_ACOUSTIC_TILE = 2, LEXGB_ACOUSTIC_PERSISTENT = 3 };

typedef struct lexgb_ctx lexgb_ctx;

/* Fill *cfg with the reference namelist defaults for solver_opt = 2 (namelist_n_constants.py:6-54). */
int lexgb_default_config(lexgb_config *cfg);

/* Create / destroy a solver context (replaces the jit-compiled closure over the
 * namelist globals that one_sprint_functions.py:9-30 builds). */
int lexgb_create(const lexgb_config *cfg, lexgb_ctx **out);
int lexgb_destroy(lexgb_ctx *ctx);

/* Order all of the context's work on this CUDA stream (cudaStream_t passed as void*). */
int lexgb_set_stream(lexgb_ctx *ctx, void *stream);

/* Base state from the reference's base_state tuple (setup_lex.py:67): horizontally
 * uniform padded FP64 columns of length nz+2 (theta0, qv0, pi0, rho0). */
int lexgb_set_base_columns(lexgb_ctx *ctx, const double *theta0, const double *qv0,
                           const double *pi0, const double *rho0);

/* Hydrostatic base state integrated in FP64 on the GPU from theta0 and qv0 columns
 * (padded, nz+2) with pi = 1 at z = 0 (setup_lex.py:123-132); pi0 and rho0 are written
 * back to the optional host columns. */
int lexgb_integrate_base_state(lexgb_ctx *ctx, const double *theta0, const double *qv0,
                               double *pi0_out, double *rho0_out);

/* Host <-> device transfer of the six prognostic fields in the reference's padded layout
 * (dtype LEXGB_F32 or LEXGB_F64); replaces the host/device boundary at jit dispatch
 * (lex_relay.py:48) and at np.reshape in the writers (write_netcdf.py:56). */
int lexgb_upload_state(lexgb_ctx *ctx, const void *const fields[6], int dtype);
int lexgb_download_state(lexgb_ctx *ctx, void *const fields[6], int dtype);

/* Advance nsteps Wicker-Skamarock RK3 big steps (ws_rk3_big_step, one_sprint_functions.py:10-30;
 * ws_rk3_sprint :109-115 is nsteps = sprint_n).  use_graph != 0 replays a captured CUDA graph
 * of one big step. */
int lexgb_step(lexgb_ctx *ctx, int nsteps, int use_graph);

/* One big step that also keeps each stage's output state and the reference's tendency tuple
 * (d_theta_dt, d_pip_dt, du_dt, dv_dt, dw_dt, d_qv_dt) of rk_sub_step0/1/2
 * (one_step_integration.py:16-447).  Afterwards lexgb_download_stage() returns them. */
int lexgb_step_record(lexgb_ctx *ctx);
/* stage in 0..2; fields (6, padded reference layout) and/or tends (6, interior arrays in
 * reference C order: theta/pi'/qv (nx,ny,nz), u (nx+1,ny,nz), v (nx,ny+1,nz), w (nx,ny,nz+1)).
 * Either pointer array may be NULL.  FP64 host output. */
int lexgb_download_stage(lexgb_ctx *ctx, int stage, double *const fields[6], double *const tends[6]);

/* Single operators evaluated on the current state, for parity checks.  Output is an FP64
 * host array in the reference's C order for that operator's result. */
enum {
    LEXGB_DIAG_MASS_DIV = 0,  /* get_divergence, interior (nx,ny,nz)           advection.py:200 */
    LEXGB_DIAG_ADV_THETA,     /* advection_scalar(theta), (nx,ny,nz)             advection.py:9 */
    LEXGB_DIAG_ADV_QV,        /* advection_scalar(qv), (nx,ny,nz)                advection.py:9 */
    LEXGB_DIAG_ADV_U,         /* advection_u, (nx+1,ny,nz)                       advection.py:37 */
    LEXGB_DIAG_ADV_V,         /* advection_v, (nx,ny+1,nz)                       advection.py:77 */
    LEXGB_DIAG_ADV_W,         /* advection_w, (nx,ny,nz+1)                       advection.py:117 */
    LEXGB_DIAG_BUOY_W,        /* calculate_buoyancy b8w, (nx,ny,nz+1)            pressure_equations.py:162 */
    LEXGB_DIAG_THETA_RHO,     /* density potential temperature, (nx,ny,nz)       one_step_integration.py:269 */
    LEXGB_DIAG_PGF_U,         /* pressure_gradient_force, (nx+1,ny,nz)           pressure_gradient_coriolis.py:7 */
    LEXGB_DIAG_PGF_V,         /* (nx,ny+1,nz) */
    LEXGB_DIAG_PGF_W,         /* (nx,ny,nz+1) */
    LEXGB_DIAG_ADV_PI,        /* advection_pi(pi' of the state, winds of the state), (nx,ny,nz) advection.py:152 */
    LEXGB_DIAG_SGS_U,         /* compute_smag, (nx+1,ny,nz)                      turbulence.py:9 */
    LEXGB_DIAG_SGS_V,
    LEXGB_DIAG_SGS_W,
    LEXGB_DIAG_SGS_THETA,
    LEXGB_DIAG_SGS_QV,
    LEXGB_DIAG_N2,            /* compute_nm, interior (nx,ny,nz)                 turbulence.py:391 */
    LEXGB_DIAG_KM,            /* compute_k km, interior (nx,ny,nz)               turbulence.py:430 */
    LEXGB_DIAG_COUNT
};
int lexgb_diagnose(lexgb_ctx *ctx, int what, double *host_out);

/* FP64 global budgets of the current state (no counterpart in the reference's solver_opt=2
 * path; space_integration, one_step_integration.py:930-938, is its closest analogue):
 * out[0] total air mass  sum rho dV (rho from pi0+pi', theta, qv as get_rho, :941-947)
 * out[1] water vapour mass  sum rho qv dV
 * out[2] kinetic energy  sum 0.5 rho0 (u^2+v^2+w^2) dV (velocities averaged to cell centres)
 * out[3] sum rho0 theta dV
 * out[4] total energy  sum rho (cv T + g z + 0.5 (u^2+v^2+w^2)) dV, T = (pi0+pi') theta, z the cell
 *        centre's height, cv of dry air; written when n_out >= 5.  n_out >= 4. */
int lexgb_budget(lexgb_ctx *ctx, double *out, int n_out);

/* Non-finite check of the state: *n_bad = number of non-finite values (0 = clean). */
int lexgb_check_finite(lexgb_ctx *ctx, long long *n_bad);

/* Wait for the context's stream.  Returns LEXGB_ERR_TIMEOUT (once, then the status is cleared) when a
 * bounded device-side wait of the persistent acoustic kernel gave up since the last check; the state is
 * then invalid and must be uploaded again.  lexgb_download_state, lexgb_check_finite and
 * lexgb_get_state_interior to host memory report the same status. */
int lexgb_synchronize(lexgb_ctx *ctx);

/* Polls a grid-barrier wait of the persistent acoustic kernel makes before it gives up with
 * LEXGB_ERR_TIMEOUT (0: the default, about 2^24 polls of >= 32 ns).  polls < 0 is a test mode: every
 * grid-barrier wait then waits for one arrival more than there are blocks, so it can only give up,
 * after -polls polls (the timeout path, without a fault or a hang).  No reference counterpart: the
 * reference runs each sub-step as separate XLA work (one_step_integration.py:638-675). */
int lexgb_set_barrier_limit(lexgb_ctx *ctx, long long polls);

/* The acoustic form the context runs (LEXGB_ACOUSTIC_ROWS, _TILE or _PERSISTENT) after AUTO and any
 * fallback were resolved.  No reference counterpart. */
int lexgb_acoustic_kernel(lexgb_ctx *ctx, int *kind);

/* Device pointers of the current state in the internal layout (x fastest, interior only,
 * theta stored minus theta_ref, u/v periodic without the duplicated face, w with nz+1 levels). */
int lexgb_state_device_ptrs(lexgb_ctx *ctx, void *ptrs[6]);

/* Kernels of one big step, for timing: the number of kernel nodes in the captured CUDA graph
 * of one big step (captures it if needed). */
int lexgb_step_kernel_count(lexgb_ctx *ctx, int *n_kernels);

/* Time `reps` back-to-back launches of one kernel of the step on the context's stream with CUDA
 * events (state untouched: outputs go to scratch).  *ms_per_launch = average launch duration. */
enum {
    LEXGB_KERNEL_ACOUSTIC = 0,  /* one acoustic sub-step */
    LEXGB_KERNEL_DIV_TRHO,      /* mass divergence + theta_rho (a kernel of its own only where nx % 4 != 0) */
    LEXGB_KERNEL_ADV_SCALARS,   /* theta and qv advection + Euler update; forms the mass divergence and
                                   theta_rho on the way, as a stage runs it */
    LEXGB_KERNEL_ADV_MOMENTUM,  /* u, v, w advection + Coriolis + buoyancy + SGS -> R_u, R_v, R_w */
    LEXGB_KERNEL_SMAG_A,
    LEXGB_KERNEL_SMAG_B,
    LEXGB_KERNEL_ACOUSTIC_PAIR, /* two acoustic sub-steps */
    LEXGB_KERNEL_ACOUSTIC_STAGE,/* the persistent kernel: all n_sound sub-steps of stage 2 in one launch */
    LEXGB_KERNEL_COUNT
};
int lexgb_time_kernel(lexgb_ctx *ctx, int which, int reps, float *ms_per_launch);

/* FP64 budgets without any device allocation (no counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc - code inside a framework that owns all device memory
 * through its own pool, work being recorded into a CUDA graph, or a loop that cannot afford
 * cudaMalloc's implicit synchronisation).  Same four sums as lexgb_budget, for a state the
 * caller holds in device memory in the internal layout (see lexgb_state_device_ptrs: theta
 * minus theta_ref, x fastest, w with nz+1 levels), FP64 padded base columns rho0 and pi0
 * (nz+2, device) and a device output of 4 doubles; enqueued on `stream` (cudaStream_t, NULL =
 * legacy default stream), not synchronised.  Partial sums go to a fixed array of
 * LEXGB_NOALLOC_MAX_BLOCKS x 4 doubles (256 KiB) compiled into the library, one slot per 2048
 * cells: grids above 16,777,216 cells are rejected with LEXGB_ERR_ARG.  The first call on a
 * device looks up that array's device address (make it before any stream capture) and keeps it for
 * the life of the process, so it is not valid after a cudaDeviceReset of that device; all calls
 * share the array, so calls that overlap on the GPU race. */
#define LEXGB_NOALLOC_MAX_BLOCKS 8192
int lexgb_budget_noalloc(int nx, int ny, int nz, double dx, double dy, double dz, double theta_ref,
                         const float *const fields[6], const double *rho0_col, const double *pi0_col,
                         double *out, void *stream);

/* The prognostic state in the device layout: interior only, x fastest; theta, u, v, pi', qv
 * [nz][ny][nx] and w [nz+1][ny][nx], FP32, host (on_device = 0) or device pointers (1, e.g. torch
 * CUDA tensors; ordered on the context's stream), theta in K; on_device = 2: device pointers with theta
 * as the device stores it, theta - theta_ref (no rounding of theta to FP32 kelvin: the exact state).
 * set marks the state as present.
 * The device-pointer form of lexgb_upload_state / lexgb_download_state (no reference counterpart:
 * LEX hands JAX arrays around, one_sprint_functions.py:10-30). */
int lexgb_set_state_interior(lexgb_ctx *ctx, const float *const fields[6], int on_device);
int lexgb_get_state_interior(lexgb_ctx *ctx, float *fields[6], int on_device);

/* Reverse mode (vector-Jacobian product) of the first `nstages` (1..3) WS-RK3 stages of one big
 * step taken from the resident state: given ybar, the adjoint of the state after those stages,
 * writes xbar, the adjoint of the resident state.  The resident state is not modified.  The
 * forward stages are recomputed internally and every intermediate the reverse pass needs (stage
 * states, divergence, theta_rho, slow tendencies and all acoustic sub-step states) is kept in a
 * workspace allocated on first use (about 110 + 4 * (acoustic sub-steps per step) fields).
 * Arrays are interior-only in the device layout, x fastest: theta, u, v, pi', qv [nz][ny][nx],
 * w [nz+1][ny][nx] (u on west faces, v on south faces, w on faces 0..nz), FP32, host pointers
 * (on_device = 0) or device pointers (on_device = 1).
 * Replaces jax.vjp of ws_rk3_big_step (one_sprint_functions.py:10-30) as used by the training
 * loop (lex_dl_train.py:114).  With turb_opt = 1 the Smagorinsky tendencies, taken from the
 * step's input state, are differentiated as well. */
int lexgb_step_vjp(lexgb_ctx *ctx, int nstages, const float *const ybar[6], float *xbar[6], int on_device);

/* One big step that keeps what its reverse mode reads: the resident state advances one step as
 * with lexgb_step(ctx, 1, 0), and the step's input state and all of its intermediates stay in the
 * adjoint workspace.  lexgb_step_vjp_kept then returns the adjoint of that input without
 * recomputing the step (LEXGB_ERR_STATE if there is no kept step: lexgb_step_vjp and a new base
 * state discard it).  Together they are the non-checkpointed forward + reverse of training. */
int lexgb_step_keep(lexgb_ctx *ctx);
/* The Smagorinsky constant Cs (> 0) for the following steps (no counterpart in the reference,
 * where it is the constant of turbulence.py:433).  lexgb_get_cs_grad: the derivative of the
 * reverse-mode seeds' inner product with respect to Cs, accumulated over every lexgb_step_vjp /
 * lexgb_step_vjp_kept call since the last reset (turb_opt 1; FP64 on the device); reset != 0
 * zeroes the accumulator after reading it.  Together with the state adjoints this is the
 * gradient of jax.vjp of the sprint with respect to (state, Cs). */
int lexgb_set_cs(lexgb_ctx *ctx, double cs);
int lexgb_get_cs_grad(lexgb_ctx *ctx, double *grad, int reset);
int lexgb_step_vjp_kept(lexgb_ctx *ctx, const float *const ybar[6], float *xbar[6], int on_device);

/* ---- learned SGS correction: the 3-D CNN of dl_models.py:19-30 (simpleCNN) ----
 * Device pointers, ordered on `stream` (a cudaStream_t; NULL: the default stream).  Activations
 * are channels-innermost [nz][ny][nx][C]; BF16 where `void *`.
 * lexgb_cnn_conv3d: one 3x3x3 zero-padded convolution on the BF16 tensor cores with FP32
 *   accumulation: y = act(conv(x, w) + bias); nx a multiple of 16, cin a multiple of 16 (padding
 *   channels of x zero), cout 8, 16 or 32; w [27][cout][cin] BF16 (offset (dz+1)*9+(dy+1)*3+(dx+1));
 *   optional outputs: pre (FP32 pre-activation), y_bf16, y_f32; gelu: tanh-GELU (flax nn.gelu);
 *   output channels >= creal are written as zero.  With the offsets mirrored and cin/cout swapped
 *   in w it is the gradient with respect to the input.
 * lexgb_cnn_gelu_bwd: g = dy * GELU'(pre) (pre NULL: g = dy), FP32 [npts][c] -> BF16 [npts][cpad].
 * lexgb_cnn_conv3d_dw: dw[27][cout][cin] += sum_p g[p][co] x[p+off][ci], db[cout] += sum_p g[p][co]
 *   (FP32, accumulated: zero them first); g has `gstride` channels per point.  dw is summed on the
 *   tcgen05 tensor cores (BF16 products, FP32 accumulation in tensor memory, any nx, ny, nz) for cin
 *   16 or 32, gstride 16 or 32 and 16-byte aligned x and g, unless lexgb_cnn_set_kernel chose
 *   LEXGB_CNN_MMA, which (like other shapes) takes the FP32 CUDA-core reduction.
 * lexgb_cnn_adam: Adam step `step` (>= 1) of n FP32 parameters with moments m, v; optional BF16 copy.
 * Replace flax's Conv / optax in lex_dl_train.py (the reference trains with optax.lamb). */
int lexgb_cnn_conv3d(int nx, int ny, int nz, int cin, int cout, const void *x, const void *w, const float *bias,
                     float *pre, void *y_bf16, float *y_f32, int gelu, int creal, void *stream);
/* Which kernel the convolutions (lexgb_cnn_conv3d and the correction inside lexgb_step) use,
 * process-wide: LEXGB_CNN_AUTO (default) the tcgen05 kernel (5th-generation tensor cores,
 * accumulators in tensor memory, tiles of 8 x 16 points: nx % 8 == 0, ny % 16 == 0) where the grid
 * fits it and has at least 2^18 points, else the mma.sync kernel; LEXGB_CNN_MMA the mma.sync
 * kernel; LEXGB_CNN_TCGEN05 the
 * tcgen05 kernel only (a grid it does not fit is an error).  Set it before capturing a step graph.
 * lexgb_cnn_take_timeouts: the number of bounded waits of the tcgen05 kernels (convolution and
 * weight gradient) that gave up since the last call (0 in normal operation; such a tile's outputs,
 * or such a block's share of dw, are not written), then reset. */
enum { LEXGB_CNN_AUTO = 0, LEXGB_CNN_MMA = 1, LEXGB_CNN_TCGEN05 = 2 };
int lexgb_cnn_set_kernel(int which);
int lexgb_cnn_take_timeouts(unsigned int *n);
int lexgb_cnn_gelu_bwd(long long npts, int c, int cpad, const float *dy, const float *pre, void *g_bf16,
                       void *stream);
int lexgb_cnn_conv3d_dw(int nx, int ny, int nz, int cin, int cout, int gstride, const void *x, const void *g,
                        float *dw, float *db, void *stream);
int lexgb_cnn_adam(long long n, float *w, const float *gw, float *m, float *v, void *w_bf16, float lr, float beta1,
                   float beta2, float eps, int step, void *stream);

/* Learned SGS correction fused into lexgb_step: after every big step the CNN corrects theta, u,
 * v, w and qv (pi' is not corrected) the way ws_rk3_sprint_dl does (one_sprint_functions.py:118-163):
 *   input  x_f = (value - in_lo[f][l]) / in_range[f][l] on each field's own points (theta in K; l the
 *            level, for w the face level 0..nz), then u, v, w averaged to the cell centre
 *                                                                  (phys_state_tuple2array, dl_models.py:125-155)
 *   output c = CNN(x) (16 -> 32 -> 32 -> 32 -> 8 channels, 5 used)
 *   state += (c staggered) * out_range[f] at the point: theta and qv at the cell; u (v) on the west
 *            (south) face i >= 1 the mean of the two cells beside it, on face 0 the value of face nx-1;
 *            w on the interior faces the mean of the cells below and above    (correct_array2tuple and
 *            stagger_uvw, dl_models.py:158-182; one_sprint_functions.py:139-151)
 * w[l]: BF16 weights [27][cout][cin] of layer l with (cin, cout) = (16,32), (32,32), (32,32),
 * (32,8) (padding rows and columns zero); b[l]: FP32 biases [cout]; in_lo, in_range: FP32 [5][nz+1]
 * (entry nz used by w only); out_range: FP32 [5][nz+1][ny][nx] (level nz used by w's lid face only).
 * All device pointers, copied on the bound stream: a later call replaces the weights and ranges
 * without rebuilding the step graph.  enable = 0 turns the correction off (the other arguments may be
 * NULL).  Needs nx a multiple of 16.  Not applied by lexgb_step_record, lexgb_step_keep or the reverse
 * mode (training differentiates the correction outside the library).  No counterpart function in the
 * reference, which applies the network in Python after each ws_rk3_big_step call. */
int lexgb_set_sgs_net(lexgb_ctx *ctx, const void *const w[4], const float *const b[4], const float *in_lo,
                      const float *in_range, const float *out_range, int enable);

/* Message of the last failure on this thread; returns the untruncated length. */
int lexgb_last_error(char *buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* LEXGB_H */
