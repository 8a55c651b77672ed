/*
 * dyn.h — C ABI of the GB300-native DYNAMITE hot path.
 *
 * One context (dyn_ctx) owns everything the reference keeps in the globals
 * `sim` (SimulationData, include/simulation/simulation_data.hpp:12-55), `rk`
 * (RKData, include/EOMs/rk_data.hpp:9-25) and the model constants
 * (`config`, include/core/config.hpp:18-56; `__constant__ d_p/d_p2/d_lambda`,
 * src/core/device_constants.cu:4-6): the stencil tables, the two-time
 * history, the interpolation results and the RK scratch, all resident on one
 * GPU.  Every function returns a dyn_status; no C++ exception crosses the
 * ABI.  Host buffers are plain pointers owned by the caller; functions whose
 * name ends in `_dev` take device pointers.
 *
 * Thread safety: a context is used from one host thread at a time.
 */
#ifndef DYN_H
#define DYN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DYN_ABI_VERSION 5

typedef enum {
    DYN_OK = 0,
    DYN_ERR_INVALID = -1,     /* bad argument or size */
    DYN_ERR_CUDA = -2,        /* a CUDA call failed; see dyn_last_error() */
    DYN_ERR_NOMEM = -3,       /* device or host allocation failed */
    DYN_ERR_STATE = -4,       /* call not valid in the current state */
    DYN_ERR_UNSUPPORTED = -5, /* option not built into this library */
    DYN_ERR_NONFINITE = -6    /* a step's error estimate came out NaN or infinite: the state
                                 holds non-finite values (overflow of the model terms); the
                                 driver loop stops before its controller acts on it */
} dyn_status;

/* RK methods: values of rk->init (runge_kutta.cu:607-615). */
enum {
    DYN_RK54 = 1,      /* Dormand-Prince 5(4), 7 stages */
    DYN_SSPRK104 = 2,  /* SSPRK(10,4), 10 stages */
    DYN_SERK2_BASE = 2 /* method m >= 3 is SERK2 with q = 2*(m-2) */
};

/* Arithmetic of the O(L^2) gathers and reductions. */
/* DYN_MIXED_DF: the mixed form with its frozen inputs carried as FP32 (hi, lo)
 * pairs (stencil weights, the history mirror, the B1 coefficients) and the
 * gathers summed as exact FP32 products with compensated sums; the rest as
 * DYN_MIXED. */
enum { DYN_FP64 = 0, DYN_MIXED = 1, DYN_MIXED_DF = 2 };

/* Fractional-position search in t1grid. */
enum {
    DYN_SEARCH_BINARY = 0,      /* bsearchPosSorted, search_utils.cpp:13-61 */
    DYN_SEARCH_LOWER_BOUND = 1  /* bsearch_interp_kernel, search_utils.cu:71-112 */
};

/* sparsifyNscale variants (the reference has three). */
enum {
    DYN_SPARSIFY_CPU = 0,       /* CPU-only build, sparsify_utils.cpp:14-97 */
    DYN_SPARSIFY_CUDA_HOST = 1, /* CUDA build, host path, sparsify_utils.cu:38-113 */
    DYN_SPARSIFY_GPU = 2        /* CUDA build, device path, sparsify_utils.cu:154-290 */
};

/* Which materialized interpolation array dyn_get_interp returns. */
enum {
    DYN_QKA1 = 0, DYN_QRA1, DYN_QKA2, DYN_QRA2, DYN_QKB1, DYN_QRB1, DYN_QKB2, DYN_QRB2,
    DYN_SIGMAKA1, DYN_SIGMARA1, DYN_SIGMAKA2, DYN_SIGMARA2,
    DYN_SIGMAKB1, DYN_SIGMARB1, DYN_SIGMAKB2, DYN_SIGMARB2,
    DYN_RINT = 16,    /* [len] */
    DYN_POSB1X = 17,  /* [len] */
    DYN_POSB2X = 18   /* [len*len] */
};

/* Model, grid size and run options (config.hpp:18-56). */
typedef struct {
    int p, p2;              /* f(q) = lambda q^p + (1-lambda) q^p2 */
    double lambda;
    double T0;              /* initial temperature (1e50 = infinite) */
    double Gamma;           /* bath temperature */
    size_t len;             /* L */
    size_t depth;           /* stencil depth m (interp order + 1) */
    double delta_t_min;
    double delta_max;
    int precision;          /* DYN_FP64 | DYN_MIXED | DYN_MIXED_DF */
    int search;             /* DYN_SEARCH_* */
    size_t history_capacity;/* rows to preallocate (0: default) */
    int device;             /* CUDA device ordinal */
    void* stream;           /* cudaStream_t to run on; NULL: the context creates one */
    int use_graph;          /* capture each RK step into a CUDA graph */
    int log_response;       /* 1: QR gathers in log space, the reference's -R option (index_vec.cu:183-395,
                               index_mat.cu:149-227); DYN_FP64 only, fused stage kernels only */
} dyn_config;

/* Grid tables as RG-Evo writes them (grid_cli.cpp:163-215, read back by
 * io_input.cpp:90-110).  Host pointers; copied at dyn_ctx_create. */
typedef struct {
    const double* theta;       /* [len], non-decreasing, theta[len-1] == 1 */
    const double* phi2;        /* [len*len] */
    const double* integ;       /* [len] (int.dat) */
    const int64_t* indsA1y;    /* [len*len] stencil starts */
    const int64_t* indsA2y;
    const int64_t* indsB2y;
    const double* weightsA1y;  /* [len*len*depth] */
    const double* weightsA2y;
    const double* weightsB2y;
} dyn_tables;

/* History in the reference's layout (simulation_data.hpp:32-38); host buffers. */
typedef struct {
    size_t n;                 /* rows */
    double* t1grid;           /* [n] */
    double* delta_t_ratio;    /* [n] */
    double* QK;               /* [n*len] row-major */
    double* QR;
    double* dQK;
    double* dQR;
    double* rvec;             /* [n] */
    double* drvec;            /* [n] */
} dyn_state;

/* Controller variables (config.hpp:18-56: delta, delta_old, loop, delta_t, rk->init). */
typedef struct {
    double delta_t;
    double delta;
    double delta_old;
    int loop;
    int method;
} dyn_controller;

/* What one RK step returns to the driver loop. */
typedef struct {
    double delta;   /* error estimate (runge_kutta.cpp:241-251) */
    double t;       /* t1grid.back() after the step */
    double r;       /* r(t) of the new last row */
    double energy;  /* -(t sum_j w_j f'(C_j) R_j + f'(C_0)/T0) at t (time_steps.cu:641-674) */
    double qk0;     /* C(t, 0) */
    double dr;      /* dr/dt at the step start (drstep2) */
} dyn_step_result;

/* Driver loop options (simulation_runner.cpp:125-304). */
typedef struct {
    int nsteps;               /* controller iterations to run */
    double tmax;              /* stop when t >= tmax (<= 0: no limit) */
    const double* dt_schedule;   /* optional: replay these step sizes (frozen schedule) */
    const int* method_schedule;  /* with dt_schedule: the method of each step */
    int gpu_rollback;         /* 1: the CUDA build's rollback on delta > 2 delta_max (:280-304) */
    /* optional per-step outputs, each [nsteps] */
    double* out_dt;
    int* out_method;
    double* out_delta;
    double* out_t;
    double* out_energy;
    double* out_qk0;
    double* out_r;
    /* periodic sparsify of the driver loop (simulation_runner.cpp:148-237): after
     * every loop that is a multiple of sparsify_every (0: never; the reference
     * uses 100000), up to sparsify_sweeps passes of dyn_sparsify(delta_max,
     * sparsify_variant) while the history shrinks (at most 10; 0: none; -1: the
     * reference's default "auto", 2 when more than half of the device's memory is
     * in use, else 1), then, if delta < delta_max/2 and the last rollback is more
     * than 1000 loops back, delta_t halves and RK54 gives way to SSPRK(10,4) */
    long long sparsify_every;
    int sparsify_sweeps;
    int sparsify_variant;
    /* 1: the QK tail fit of the newest row after every step (the reference's
     * --tail-fit, tail_fit.cpp:46-262, applied at simulation_runner.cpp:135-141);
     * out_energy is then the energy of the fitted row, as the reference records it. */
    int tail_fit;
    /* 1: at the periodic block's step halving a method other than RK54 moves one
     * SERK2 level up (SSPRK(10,4) -> SERK2(2) -> SERK2(4) ...; the GPU loop's
     * init_SERK2(2 (init - 1)), simulation_runner.cpp:222-229, the reference's
     * default --serk2 true), at most to SERK2(16); 0: it stays (RK54 still gives
     * way to SSPRK(10,4)) */
    int use_serk2;
} dyn_run_params;

/* ---------------------------------------------------------------- basics */
int dyn_abi_version(void);
const char* dyn_last_error(void);

/* Replaces import() + copyVectorsToGPU + copyParametersToDevice
 * (io_input.cpp:90-110, gpu_memory_utils.cu:11-146,195-199).  Checks the
 * model (finite lambda and Gamma, T0 > 0, exponents the kernels are built
 * for) and the tables (dyn_check_tables) on the host before any CUDA call:
 * a bad argument returns DYN_ERR_INVALID with the reason in dyn_last_error(). */
dyn_status dyn_ctx_create(const dyn_config* cfg, const dyn_tables* tables, void** ctx);
/* Host-side check of a grid's tables, no GPU needed (what dyn_ctx_create and
 * dyn_batch_create run; io_input.cpp:90-110 reads the same files without a
 * check): theta non-decreasing on [0, 1] with theta[len-1] == 1; every stencil
 * start s of the three families within [0, len - depth], so that every tap
 * s + d (d < depth) lies inside a history row; phi2 within [0, 1] ending at 1;
 * finite weights and int.dat.  Returns DYN_ERR_INVALID with the first failure
 * in dyn_last_error(). */
dyn_status dyn_check_tables(size_t len, size_t depth, const dyn_tables* tables);
dyn_status dyn_ctx_destroy(void* ctx);
dyn_status dyn_sync(void* ctx);

/* t=0 state: initialization.cpp:204-222 (+ the first interpolation, :267-274). */
dyn_status dyn_state_init(void* ctx, double delta_t);
/* Load / read back the history (loadSimulationState / copyVectorsToCPU).
 * dyn_state_upload rejects (DYN_ERR_INVALID, nothing changed) a state whose
 * t1grid is negative or decreasing or whose values are not all finite. */
dyn_status dyn_state_upload(void* ctx, const dyn_state* st);
dyn_status dyn_state_rows(void* ctx, size_t* n);
/* t1grid of the newest row (the current time); 0 before any state */
dyn_status dyn_state_time(void* ctx, double* t);
dyn_status dyn_state_download(void* ctx, dyn_state* st);
dyn_status dyn_controller_get(void* ctx, dyn_controller* c);
dyn_status dyn_controller_set(void* ctx, const dyn_controller* c);

/* ---------------------------------------------------------- the path */
/* interpolateGPU (interpolation_core.cu:63-159): fills the 16 [len*len]
 * arrays, rInt and the positions.  posB1x/posB2x: optional host arrays to
 * use as positions instead of searching (same == 1 in the reference). */
dyn_status dyn_interpolate(void* ctx, const double* posB1x, const double* posB2x);
dyn_status dyn_get_interp(void* ctx, int which, double* host_out);

/* QKRstepGPU (time_steps.cu:327-408) on the materialized arrays. */
dyn_status dyn_qkr_step(void* ctx, double* hK, double* hR);
/* The same right-hand side computed by the fused stage kernel (no arrays). */
dyn_status dyn_rhs(void* ctx, double* hK, double* hR);
/* rstepGPU (time_steps.cu:410-472) of the last row; drstep2GPU (:564-639)
 * on caller rows; energyGPU (:641-674). */
dyn_status dyn_rstep(void* ctx, double* r);
dyn_status dyn_drstep2(void* ctx, const double* qK, const double* qR, const double* dqK,
                       const double* dqR, double t, double* dr);
dyn_status dyn_energy(void* ctx, double* e);
/* The energy of every history row as RG-Evo writes it with a save
 * (computeEnergyHistoryKernel, io_output.cu:61-122), into host e[n_rows]:
 * E_k = -t_k (sum_j w_j f'(QK[k,j]) QR[k,j] + f'(QK[k,0]) / T0). */
dyn_status dyn_energy_history(void* ctx, double* e, size_t n_rows);
/* tailFitBlendCPU / tailFitBlendGPU (tail_fit.cpp:46-262, tail_fit.cu): one QK
 * tail fit of the newest history row, in place.  last_rollback_loop is the loop
 * of the caller's last rollback (-1000: none; a change resets the smoothing).
 * The fit keeps its window and smoothed alpha across calls on the context, as
 * the reference keeps them across a process; dyn_tail_fit_reset forgets them.
 * info (may be NULL; non-NULL synchronizes) receives this call's raw and
 * smoothed alpha, first blended column and whether QK was blended.  On the
 * mixed forms the fit edits the FP64 row and refreshes its FP32 mirror. */
typedef struct {
    double alpha_raw, alpha;
    int j0, applied;
} dyn_tail_info;
dyn_status dyn_tail_fit(void* ctx, int last_rollback_loop, dyn_tail_info* info);
dyn_status dyn_tail_fit_reset(void* ctx);
/* ConvAGPU / ConvRGPU (convolution.cu:64-230): kind 0 = A, 1 = R; f, g,
 * out are device arrays, n = len (1-D) or len*len (2-D). */
dyn_status dyn_conv_dev(void* ctx, int kind, const double* f, const double* g, size_t n, double t,
                        double* out);
/* bsearchPosSortedGPU (search_utils.cu:273-319): out[k] = position of
 * elem[k] * list[nlist-1] in list, device arrays. */
dyn_status dyn_search_dev(void* ctx, const double* list, size_t nlist, const double* elem,
                          size_t nelem, double* out);

/* One RK step: updateGPU / update (runge_kutta.cu:607-615, runge_kutta.cpp:254-261). */
dyn_status dyn_update(void* ctx, int method, double delta_t, dyn_step_result* res);
/* The driver loop (simulation_runner.cpp:125-304) for p->nsteps iterations.
 * Returns DYN_ERR_NONFINITE (after storing that step's outputs) when a step's
 * error estimate is NaN or infinite; the reference's loop would go on with
 * it, its controller comparisons all false. */
dyn_status dyn_run(void* ctx, const dyn_run_params* p, dyn_step_result* last);
/* sparsifyNscale[GPU] (sparsify_utils.*): returns the new row count. */
dyn_status dyn_sparsify(void* ctx, double threshold, int variant, size_t* n_out);
/* rollbackState (simulation_control.cpp:14-123). */
dyn_status dyn_rollback(void* ctx, int nrows);

/* The last history row C(t, theta_j t), R(t, theta_j t) into host buffers
 * (what the driver loop reads after each step, simulation_runner.cpp:306-310). */
dyn_status dyn_last_row(void* ctx, double* qK, double* qR);

/* ------------------------------------------------ device-resident history */
/* The history in the reference's own device layout (SimulationData's
 * d_QKv, d_QRv, d_dQKv, d_dQRv: row-major n x len; d_t1grid,
 * d_delta_t_ratio, d_rvec, d_drvec: n), as device pointers.  For a driver
 * that keeps its thrust vectors (include/simulation/simulation_data.hpp:12-55)
 * and hands them to this library: the drop-in layer of RG-Evo's hot-path
 * symbols exchanges state with RG-Evo through these calls. */
typedef struct {
    size_t n;
    double* t1grid;
    double* delta_t_ratio;
    double* QK;
    double* QR;
    double* dQK;
    double* dQR;
    double* rvec;
    double* drvec;
} dyn_state_dev;
/* Replace the whole history from device arrays (as dyn_state_upload; the
 * times are checked on the host, the values are not read back). */
dyn_status dyn_state_upload_dev(void* ctx, const dyn_state_dev* st);
/* Overwrite rows [row0, row0 + nrows) of the context's history (values,
 * derivatives, r, dr; not the times) from device arrays indexed like the full
 * history (row k at offset k * len): for a caller that edited rows in place,
 * as the reference's tail fit edits the newest row (tail_fit.cu). */
dyn_status dyn_state_rows_load_dev(void* ctx, size_t row0, size_t nrows, const dyn_state_dev* src);
/* Copy rows [row0, row0 + nrows) of the context's history, times included,
 * into device arrays indexed like the full history (appendAllGPU_ptr's
 * effect, time_steps.cu:766-919, when the caller has grown its arrays). */
dyn_status dyn_state_rows_store_dev(void* ctx, size_t row0, size_t nrows, const dyn_state_dev* dst);
/* After dyn_interpolate: materialized array `which` into a device buffer
 * (the sim->d_*int arrays interpolateGPU fills, interpolation_core.cu:63-159). */
dyn_status dyn_get_interp_dev(void* ctx, int which, double* dev_out);
/* The reference-order B1 pair QK_B1, QR_B1 ([len*len] each) of the current
 * state into device buffers: what RG-Evo's saves read back after a step
 * (io_save_compressed.cpp:17-63), without the other fourteen arrays. */
dyn_status dyn_interp_b1_dev(void* ctx, double* qk_b1, double* qr_b1);

/* ----------------------------------------------------------- measurement */
/* Average device time of the two stage kernels for the current state, timed
 * with CUDA events on the context's stream over `reps` launches. */
dyn_status dyn_profile_stage(void* ctx, int reps, float* ms_main, float* ms_epilogue);
/* Measured FP64 FMA throughput of the current device (GFLOP/s, 2 flop/FMA). */
dyn_status dyn_probe_fp64(int device, double* gflops);

/* ------------------------------------------------- allocation-free RHS */
/* No counterpart in the reference.  The right-hand side of dyn_rhs for
 * callers that cannot allocate device memory (a driver working inside a
 * device pool it does not own, or one that has handed all free memory to its
 * history): every input and the output are the caller's device buffers, in
 * this library's layout; the kernels' scratch is a fixed file-scope device
 * array of DYN_NOALLOC_SCRATCH_BYTES per GPU, held from library load to
 * process exit.  The first call on each device resolves that array's address
 * (make it before any stream capture) and keeps it for the process: do not
 * call across a cudaDeviceReset of that device.  Calls that overlap on the
 * GPU race on the array: serialize them.
 * Limits: 4 <= len <= DYN_NOALLOC_MAX_LEN, 2 <= rows <= DYN_NOALLOC_MAX_ROWS,
 * 2 <= depth <= len, search DYN_SEARCH_BINARY or DYN_SEARCH_LOWER_BOUND;
 * anything else is rejected with DYN_ERR_INVALID.
 * The tables live in device memory and are NOT checked here: every stencil
 * start must lie in [0, len - depth] (a larger one reads past a history row),
 * theta and phi2 must be as dyn_check_tables requires.  Run dyn_check_tables
 * on the host copies once before uploading them.
 * Enqueued on `stream` (cudaStream_t, NULL = default stream); the caller
 * synchronizes. */
#define DYN_NOALLOC_MAX_LEN 1024
#define DYN_NOALLOC_MAX_ROWS 16384
#define DYN_NOALLOC_SCRATCH_BYTES 458752   /* 448 KiB */
typedef struct {
    int p, p2;
    double lambda, T0, Gamma;
    size_t len, depth, rows;
    int search;                         /* DYN_SEARCH_* */
    const double* theta;                /* [len] */
    const double* phi2;                 /* [len*len] */
    const double* integ;                /* [len] */
    const int32_t* indsA1y;             /* [len*len] stencil starts */
    const int32_t* indsA2y;
    const int32_t* indsB2y;
    const double* weightsA1y;           /* [len*len*depth] */
    const double* weightsA2y;
    const double* weightsB2y;
    const double* KR;                   /* [rows*len][2]: (QK, QR) pairs, row-major */
    const double* dKR;                  /* [rows*len][2]: (dQK, dQR) pairs */
    const double* t1grid;               /* [rows] */
    const double* delta_t_ratio;        /* [rows] */
    const double* rvec;                 /* [rows] */
    const double* drvec;                /* [rows] */
    double* out;                        /* [len][2]: (hK, hR) pairs */
} dyn_noalloc_rhs;
dyn_status dyn_rhs_noalloc(const dyn_noalloc_rhs* args, void* stream);

/* ---------------------------------------------------- batched quenches */
/* No counterpart in the reference, which runs one quench per process
 * (simulation_runner.cpp:125-304).  A batch holds many quenches, each with
 * its own model, grid (grids of one length are shared), history, step
 * controller and stopping rule, and advances every running quench by one RK
 * stage per "tick": one persistent gather kernel over the target rows of all
 * quenches and one epilogue kernel over their history rows, with the step
 * planner and the controller of dyn_run (its gpu_rollback option included)
 * running on the device, ticks replayed from a CUDA graph.  Arithmetic: the
 * mixed form (DYN_MIXED) of a single context, stage for stage. */
typedef struct {
    size_t len, depth;
    dyn_tables tables;       /* host pointers, copied at creation */
} dyn_batch_grid;

typedef struct {
    int grid;                /* index into the grids array */
    int p, p2;
    double lambda, T0, Gamma;
    double delta_t_min, delta_max;
    double delta_t;          /* first step size (<= 0: delta_t_min) */
    double t_stop;           /* stop once t1grid.back() >= t_stop (<= 0: no limit) */
    long long max_steps;     /* stop after this many steps (<= 0: no limit) */
    size_t capacity;         /* history rows held on the device (0: 4096) */
} dyn_batch_quench;

typedef struct {
    int device;
    void* stream;            /* cudaStream_t; NULL: the batch creates one */
    int search;              /* DYN_SEARCH_* */
    int gpu_rollback;        /* 1: roll back 10 rows on delta > 2 delta_max, as dyn_run */
    int ticks_per_launch;    /* ticks per graph replay (0: 32) */
    int threads;             /* gather CTA threads: 128 or 256 (0: 128) */
    int targets;             /* targets per thread: 1 or 2 (0: 1) */
    int ctas_per_sm;         /* persistent gather CTAs per SM (0: occupancy limit) */
    /* periodic sparsify of every quench, as dyn_run_params (threshold: the
     * quench's delta_max); a quench pauses at the end of such a loop with
     * status DYN_QUENCH_SPARSIFY until the host has compacted its history
     * (dyn_batch_run, dyn_batch_sync) */
    long long sparsify_every;
    int sparsify_sweeps;
    int sparsify_variant;
    int precision;           /* DYN_MIXED_DF (or 0) | DYN_MIXED: the (hi, lo) form is the one whose
                                free step-size controller and sparsify decisions match the FP64
                                form's at delta_max 1e-10; the plain form's controller reads its
                                FP32 stage noise as error and keeps the step far smaller */
    int use_serk2;           /* the periodic block's SERK2 climb, as dyn_run_params */
} dyn_batch_config;

/* Quench status */
enum {
    DYN_QUENCH_RUNNING = 0,
    DYN_QUENCH_DONE = 1,      /* reached t_stop */
    DYN_QUENCH_MAXSTEPS = 2,  /* took max_steps steps */
    DYN_QUENCH_FULL = 3,      /* history capacity reached */
    DYN_QUENCH_SPARSIFY = 4,  /* waiting for its periodic sparsify (transient) */
    DYN_QUENCH_FAILED = 5     /* its error estimate came out NaN or infinite (as DYN_ERR_NONFINITE
                                 of dyn_run); stopped until dyn_batch_upload gives it a new state */
};

typedef struct {
    int status;
    int method;              /* method of the next step */
    int loop;
    int pad;
    long long steps;         /* steps taken since creation / the last upload */
    size_t n;                /* history rows */
    double t;                /* t1grid.back() */
    double delta_t;          /* step size of the next step */
    double delta, delta_old;
    double energy, r, qk0;   /* of the last step (as dyn_step_result) */
} dyn_batch_info;

/* Quenches start from the t=0 state of dyn_state_init. */
dyn_status dyn_batch_create(const dyn_batch_config* cfg, const dyn_batch_grid* grids, int ngrids,
                            const dyn_batch_quench* quenches, int nquench, void** batch);
dyn_status dyn_batch_destroy(void* batch);
/* Replace quench q's history and controller (as dyn_state_upload +
 * dyn_controller_set); its status returns to running, steps to 0. */
dyn_status dyn_batch_upload(void* batch, int q, const dyn_state* st, const dyn_controller* ctl);
dyn_status dyn_batch_download(void* batch, int q, dyn_state* st);
/* Quench q's status and controller as of the last run/sync/upload. */
dyn_status dyn_batch_get_info(void* batch, int q, dyn_batch_info* info);
/* New stopping rule for quench q; a stopped quench that the new rule allows
 * to continue runs again. */
dyn_status dyn_batch_set_limits(void* batch, int q, double t_stop, long long max_steps);
/* Advance until no quench runs or max_ticks ticks have run; *ticks_out =
 * ticks run.  Synchronous. */
dyn_status dyn_batch_run(void* batch, long long max_ticks, long long* ticks_out);
/* Enqueue `ticks` ticks on the batch's stream and return (stopped quenches
 * skip them); dyn_batch_sync waits and refreshes what dyn_batch_get_info
 * reports. */
dyn_status dyn_batch_enqueue(void* batch, long long ticks);
dyn_status dyn_batch_sync(void* batch);
/* Quench q's newest history row C(t, theta_j t), R(t, theta_j t) (as of the
 * last run/sync) into host buffers of its grid length. */
dyn_status dyn_batch_last_row(void* batch, int q, double* qK, double* qR);
/* Autotuner: times the gather kernel over the current states for every
 * tile shape (threads x targets x CTAs per SM), keeps the fastest and
 * returns it.  Changes the order of the partial sums (the results move at
 * the FP32-compensated level), not the algorithm. */
dyn_status dyn_batch_tune(void* batch, int reps, int* threads, int* targets, int* ctas_per_sm, float* ms_best);
/* Average device time of the gather kernel over `reps` launches for the
 * current stage of every running quench (the kernel is idempotent). */
dyn_status dyn_batch_profile(void* batch, int reps, float* ms_gather);

/* ------------------------------------------------------ discrete adjoint */
/* No counterpart in the reference.  Gradients of a final-time objective
 * with respect to the bath temperature Gamma and the mixing coupling lambda,
 * by a hand-written discrete adjoint of the FP64 RK-stepped pipeline
 * (interpolation, convolutions, RHS, r(t), RK stages) on a fixed step
 * schedule.  The history is append-only, so the state before each step is a
 * prefix of the final history: the reverse sweep recomputes one step's
 * stages at a time from it and keeps no other checkpoint.  RK54 and
 * SSPRK(10,4) steps only; FP64 contexts only. */
typedef struct {
    double w_energy;          /* weight of E(t_f) */
    double w_r;               /* weight of r(t_f) */
    const double* c_K;        /* [len] weights on C(t_f, theta_j t_f) of the final row, or NULL
                                 (C(t_f, t_f/2): interpolation weights at theta = 1/2) */
    const double* c_R;        /* [len] weights on R(t_f, theta_j t_f), or NULL */
    const double* c_dK;       /* [len] weights on the final row's dQK, or NULL */
    const double* c_dR;       /* [len] weights on the final row's dQR, or NULL */
    double w_dr;              /* weight of the final row's drvec */
} dyn_adjoint_objective;

typedef struct {
    double ms_forward;        /* wall time of the recorded forward steps */
    double ms_backward;       /* wall time of the reverse sweep (recompute included) */
    size_t device_bytes;      /* device memory the reverse sweep holds (cotangents, snapshot, scratch) */
    int steps;
    long long recompute_mismatch;  /* elements where a recomputed row differed from the forward's (0) */
} dyn_adjoint_stats;

/* dyn_run (no rollback) that records the step schedule it took (dt, method
 * per step) for the reverse sweep; with p->dt_schedule it replays that
 * schedule.  Gradients include the t=0 state's dependence on Gamma and
 * lambda when the run starts from dyn_state_init's single row. */
dyn_status dyn_adjoint_forward(void* ctx, const dyn_run_params* p, dyn_step_result* last);
/* Reverse sweep of the recorded forward: grad[0] = dJ/dGamma, grad[1] =
 * dJ/dlambda for J = w_energy E(t_f) + sum_j c_K[j] C(t_f, theta_j t_f) +
 * w_r r(t_f) (+ the other final-row terms of the objective).  Leaves the history as the forward left it, so several
 * objectives can be differentiated in turn. */
dyn_status dyn_adjoint_backward(void* ctx, const dyn_adjoint_objective* obj, double* grad, dyn_adjoint_stats* stats);
/* After dyn_adjoint_backward: dJ/d(history the recorded forward started
 * from), rows [0, n_start) in dyn_state layout (t1grid, delta_t_ratio
 * untouched).  The t=0 row's dependence on Gamma and lambda is already in
 * grad; these are the sensitivities to an uploaded initial history. */
dyn_status dyn_adjoint_history_grad(void* ctx, dyn_state* grad);

/* ------------------------------------------------------------ tables */
/* `RG-Evo grid -L len -M Tmax -s spline_order -m poly -o interp_order
 * -a alpha -D delta` (grid_cli.cpp:35-258) without the files: fills the
 * tables the solver reads (caller-allocated; phi1 may be NULL; depth =
 * interp_order + 1).  Host only, no GPU needed. */
dyn_status dyn_grid_generate(size_t len, double Tmax, int spline_order, int interp_order, double alpha,
                             double delta, double* theta, double* phi1, double* phi2, double* integ,
                             int64_t* indsA1y, double* weightsA1y, int64_t* indsA2y, double* weightsA2y,
                             int64_t* indsB2y, double* weightsB2y);
/* `RG-Evo grid ... -m rational -o interp_order -f fh_window`: local Floater-Hormann
 * stencils of order interp_order on windows of dyn_grid_rational_depth(len,
 * interp_order, fh_window) = min(len, max(interp_order + 1, fh_window)) points
 * (compute_barycentric_rational_weights, interpolation_weights.cpp:159-280), the
 * polynomial stencil of the window where FH is ill-conditioned.  The weight arrays
 * hold that depth per target; the depth is at most 256. */
int dyn_grid_rational_depth(size_t len, int interp_order, int fh_window);
/* The position grids RG-Evo's Grid_data holds beside the tables (posA1y.dat,
 * posA2y.dat, posB2y.dat; generate_pos_grids, pos_grid.cpp:111-205): the
 * 1-based fractional theta index of phi1, phi2 and theta_i / phi2, each len*len.
 * The solver does not read them; the reference checks that they exist. */
dyn_status dyn_grid_positions(size_t len, double Tmax, double alpha, double delta, double* posA1y, double* posA2y,
                              double* posB2y);
dyn_status dyn_grid_generate_rational(size_t len, double Tmax, int spline_order, int interp_order, int fh_window,
                                      double alpha, double delta, double* theta, double* phi1, double* phi2,
                                      double* integ, int64_t* indsA1y, double* weightsA1y, int64_t* indsA2y,
                                      double* weightsA2y, int64_t* indsB2y, double* weightsB2y);

#ifdef __cplusplus
}
#endif
#endif /* DYN_H */
