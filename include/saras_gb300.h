/*
 * saras_gb300.h -- C ABI of the GB300-native SARAS time-step hot path.
 *
 * One opaque context (saras_ctx) owns every device buffer of one SARAS solver
 * instance (velocity, pressure, temperature, the multigrid level hierarchy and
 * all temporaries) plus one CUDA stream.  Arrays cross the boundary as plain
 * host pointers in the reference layout: C order (k fastest), ghost width 1,
 * logical index range -1 .. n along each axis, so a field with core extent
 * (nx, ny, nz) occupies (nx+2)*(ny+2)*(nz+2) doubles.
 *
 * Every entry point returns an int status (SARAS_OK on success).  Calls are
 * stream-ordered; calls that return a scalar to the host synchronise.
 *
 * Each declaration names the reference interface (file:line, paths inside the
 * roshansamuel/saras repository) whose behaviour it reproduces.
 */
#ifndef SARAS_GB300_H
#define SARAS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum saras_status {
    SARAS_OK = 0,
    SARAS_NOT_CONVERGED = 1,     /* CN Jacobi hit maxIterations (hydro_d3.cc:415-421) */
    SARAS_DIVERGENCE_LIMIT = 2,  /* max divergence > 1e5 (tseries.cc:141-145)        */
    SARAS_BAD_CONFIG = 3,        /* parameter check failed (parser.cc:250-352)        */
    SARAS_CUDA_ERROR = 4,
    SARAS_BAD_ARG = 5,
    SARAS_NO_DEVICE = 6,
    SARAS_NOT_FINITE = 7,        /* NaN/Inf detected in a solver residual            */
    SARAS_TOO_LARGE = 8          /* request exceeds a fixed capacity                 */
};

/* ---------------------------------------------------------------- fields */
enum saras_field {
    SARAS_FIELD_VX = 0,      /* vfield V.Vx  (x face-centred)              vfield.cc:64  */
    SARAS_FIELD_VY = 1,      /* vfield V.Vy                                vfield.cc:65  */
    SARAS_FIELD_VZ = 2,      /* vfield V.Vz                                vfield.cc:66  */
    SARAS_FIELD_P = 3,       /* sfield P (vertex grid)                     hydro.cc:62   */
    SARAS_FIELD_T = 4,       /* sfield T (vertex grid, scalar solver only) scalar.cc:63  */
    SARAS_FIELD_PP = 5,      /* plainsf Pp, pressure correction            hydro.cc:67   */
    SARAS_FIELD_MGRHS = 6,   /* plainsf mgRHS, Poisson right-hand side     hydro.cc:68   */
    SARAS_FIELD_NSE_X = 7,   /* plainvf nseRHS.Vx                          hydro.cc:69   */
    SARAS_FIELD_NSE_Y = 8,
    SARAS_FIELD_NSE_Z = 9,
    SARAS_FIELD_TRHS = 10,   /* plainsf tmpRHS (scalar solver only)        scalar.cc:64  */
    SARAS_FIELD_GRAD_X = 11, /* plainvf pressureGradient.Vx                hydro.cc:71   */
    SARAS_FIELD_GRAD_Y = 12,
    SARAS_FIELD_GRAD_Z = 13,
    SARAS_NUM_FIELDS = 14
};

/* Multigrid modes (GB300 extension; SARAS_MG_REFERENCE is the drop-in). */
enum saras_mg_mode {
    SARAS_MG_REFERENCE = 0,  /* FP64 V-cycles, stop on |delta residual| < tol  poisson.cc:132-148 */
    SARAS_MG_PLAIN_TARGET = 1, /* FP64 V-cycles until max|b-Ap|/max|b| <= target              */
    SARAS_MG_MIXED = 2       /* FP32 V-cycles inside FP64 iterative refinement to the target   */
};

/* Initial guess sources for the pressure-correction solve. */
enum saras_guess {
    SARAS_GUESS_PREVIOUS = 0, /* previous Pp (reference behaviour, poisson.cc:115) */
    SARAS_GUESS_LEARNED = 1,  /* U-Net guess with fallback to the previous Pp      */
    SARAS_GUESS_EXTRAPOLATE = 2, /* 2 Pp(n-1) - Pp(n-2) with the same fallback (ablation) */
    SARAS_GUESS_QUADRATIC = 3,   /* 3 Pp(n-1) - 3 Pp(n-2) + Pp(n-3), same fallback (ablation) */
    SARAS_GUESS_PARITY = 4,      /* Pp(n-1) + Pp(n-2) - Pp(n-3): exact for a linear trend plus a
                                    period-2 oscillation, same fallback (ablation) */
    SARAS_GUESS_NETWORK = 5      /* the U-Net guess in every solve once its histories are
                                    complete, never the per-solve choice of SARAS_GUESS_LEARNED
                                    (ablation: what the network alone buys) */
};

/*
 * Solver parameters: the fields of the reference parser (parser.h:63-123) that
 * the hot path reads, plus the GB300 extensions at the end.  Fill with
 * saras_default_params() and/or saras_parse_yaml().
 */
typedef struct saras_params {
    /* "Program" */
    int probType, icType, rbcType, forceType;
    int xPer, yPer, zPer;            /* from "Domain Type" (parser.cc:406-414) */
    double Re, Ra, Pr, Ro, Ta;
    double Lx, Ly, Lz;
    int nonHgBC;
    double patchRadius;
    /* "Mesh" */
    int xGrid, yGrid, zGrid;         /* 0 uniform, 1/2 tanh (from "Mesh Type") */
    double betaX, betaY, betaZ;
    int xInd, yInd, zInd;
    /* "Parallel" */
    int nThreads, npX, npY;
    /* "Solver" */
    int dScheme, iScheme;
    double cnTolerance;
    int restartFlag, useCFL;
    double courantNumber, tStp, tMax;
    int ioCnt, solnFormat;
    double fwInt, rsInt;
    int readProbes;
    double prInt;
    /* "Multigrid" */
    int vcDepth, vcCount;
    double mgTolerance;
    int gsSmooth, preSmooth, postSmooth, resType, printResidual;
    /* GB300 extensions ("GB300" section of parameters.yaml) */
    int testPoisson;          /* Dirichlet r^2/6 multigrid check (TEST_POISSON build flag) */
    int mgMode;               /* enum saras_mg_mode */
    double mgTarget;          /* residual target of the PLAIN_TARGET / MIXED modes */
    int mgMaxCycles;          /* cap on V-cycles (target modes)                 */
    int mixedCycles;          /* FP32 V-cycles of the first refinement step of a
                                 solve; later steps (and every step with 0) run
                                 the fewest, at most this many, that the measured
                                 contraction per V-cycle predicts to meet mgTarget */
    int guessMode;            /* enum saras_guess                               */
    double jacobiWeight;      /* damping of the Jacobi smoother (1.0 = reference) */
    int seed;
    int fastKernels;          /* 1: fused multiply-add / reciprocal forms of the CN,
                                 RHS, divergence and projection kernels (not
                                 bit-identical to the reference); 2: as 1, with the
                                 CN Jacobi update in split-FP64 form (FP64 values
                                 carried in float pairs, about 1e-14 relative) and
                                 the right-hand side formed straight as that
                                 solve's first iterate, so saras_time_advance
                                 leaves nseRHS unwritten;
                                 0: reference arithmetic (the drop-in)          */
    int smoother;             /* target modes: 0 damped Jacobi (jacobiWeight);
                                 1 Chebyshev: each smoothing phase of n sweeps
                                 is the degree-n Chebyshev polynomial of D^-1 A
                                 on [1/3, 2], applied as n Jacobi sweeps with
                                 the weights 1 / (its roots) (n <= 16)          */
    int coarseSmooth;         /* target modes: sweeps per smoothing phase on the
                                 levels below the finest (0: preSmooth /
                                 postSmooth, as on the finest level)           */
    int coarseCycles;         /* target modes: cycles on the second level per
                                 visit of the finest (0 or 1: V-cycle; 2: a
                                 W-cycle at the second level; at most 4)       */
} saras_params;

typedef struct saras_step_stats {
    int cn_iters[4];          /* Jacobi iterations for Vx, Vy, Vz, T */
    int vcycles;              /* V-cycles in this step (FP64 or FP32) */
    int refine_steps;         /* FP64 refinement steps (mixed mode)  */
    int coarse_iters;         /* coarsest-level Gauss-Seidel iterations */
    double mg_residual;       /* last value of computeError (poisson_d3.cc:391-459) */
    double fine_residual;     /* FP64 max|b-Ap|/max|b| after the solve (target modes) */
    double guess_residual;    /* FP64 residual of the chosen initial guess */
    int guess_source;         /* guess used: 0 previous Pp, else the saras_guess mode that won */
    int status;
} saras_step_stats;

typedef struct saras_ctx saras_ctx;

/* ------------------------------------------------------ setup / teardown */
int saras_default_params(saras_params *p);
/* Reads input/parameters.yaml (parser.cc:69-239) and validates (parser.cc:250-352). */
int saras_parse_yaml(const char *path, saras_params *p, char *err, int errlen);
/* Builds grid, fields, multigrid hierarchy on the current CUDA device
 * (grid.cc:59-136, hydro.cc:60-75, poisson_d3.cc:64-87).  Fields start at 0. */
int saras_create(const saras_params *p, saras_ctx **out);
int saras_destroy(saras_ctx *ctx);
const char *saras_last_error(const saras_ctx *ctx);
/* Padded extents (n+2 per axis) of a field. */
int saras_field_dims(const saras_ctx *ctx, int field, int dims[3]);
/* Coordinates along axis (0 x, 1 y, 2 z) of the staggered (staggered = 1,
 * xStaggr: n+1 core points) or collocated (0, xColloc: n core points) grid,
 * ghosts included: out[0] is index -1 (grid.cc:370-403, 442-519).  count
 * receives the number written (core points + 2); out may be NULL to query it. */
int saras_grid_coords(const saras_ctx *ctx, int axis, int staggered, double *out, int capacity, int *count);
int saras_upload(saras_ctx *ctx, int field, const double *host);
int saras_download(saras_ctx *ctx, int field, double *host);
/* Several fields at once (n <= SARAS_NUM_FIELDS): the copies run concurrently
 * on their own streams, ordered after the context's work (download) or before
 * it (upload), and the call returns when all of them are done, like n calls of
 * saras_upload / saras_download.  Host buffers in page-locked memory let the
 * copy engines work in parallel. */
int saras_upload_fields(saras_ctx *ctx, int n, const int *fields, const double *const *hosts);
int saras_download_fields(saras_ctx *ctx, int n, const int *fields, double *const *hosts);
int saras_synchronize(saras_ctx *ctx);
/* Number of device kernels this context has launched so far. */
long long saras_launch_count(const saras_ctx *ctx);
/* 1 when the finest level's FP32 sweeps and residuals of the target modes run
 * through the TMA plane-streaming kernels (environment SARAS_PLANE_TMA=1 at
 * saras_create and a level that fits), 0 when the column kernels run. */
int saras_plane_tma_active(const saras_ctx *ctx);

/* ------------------------------------------------------ boundary fills */
/* hydro::imposeUBCs/VBCs/WBCs (hydro.cc:386-461), scalar::imposeTBCs (scalar.cc:240-255):
 * syncData (mpidata.cc:278-306, np=1 semantics) followed by the wall objects of
 * hydro::initVBC / scalar::initTBC (hydro.cc:287-371, scalar.cc:185-227). */
int saras_apply_bc(saras_ctx *ctx, int field);
/* field::syncData alone (mpidata.cc:278-306). */
int saras_sync_field(saras_ctx *ctx, int field);

/* ------------------------------------------------------ field operators */
/* vfield::computeDiff(nseRHS) (vfield.cc:104-146): nseRHS(core) += Laplacian(V). */
int saras_vfield_compute_diff(saras_ctx *ctx);
/* vfield::computeNLin(V, nseRHS) (vfield.cc:163-253): nseRHS(core) -= (V.grad)V. */
int saras_vfield_compute_nlin(saras_ctx *ctx);
/* sfield::gradient(pressureGradient, V) of P or Pp (sfield.cc:155-171, plainsf.h:92-98). */
int saras_sfield_gradient(saras_ctx *ctx, int scalar_field);
/* vfield::divergence(mgRHS, P) (vfield.cc:299-320). */
int saras_vfield_divergence(saras_ctx *ctx);
/* sfield::computeDiff / computeNLin of T into tmpRHS (sfield.cc:86-142). */
int saras_tfield_compute_diff(saras_ctx *ctx);
int saras_tfield_compute_nlin(saras_ctx *ctx);
/* Whole-array field arithmetic used by timeAdvance (field.cc:631-715, plainvf.cc:91-224):
 * dst = a*dst + b*src over the padded array (src < 0: no src term). */
int saras_axpby(saras_ctx *ctx, int dst, double a, int src, double b);

/* ------------------------------------------------------ implicit solves */
/* hydro_d3::solveVx/Vy/Vz (hydro_d3.cc:370-533), scalar_d3::solveVx..solveT
 * (scalar_d3.cc:373-591).  component: 0,1,2 = Vx,Vy,Vz, 3 = T. */
int saras_cn_solve(saras_ctx *ctx, int component, int *iters, double *max_error);
/* Allocation-free variant of saras_cn_solve for callers that cannot allocate
 * device memory when they need the solve (fixed memory budgets, pool
 * allocators closed after start-up).  No counterpart in the reference.  v
 * (in/out) and rhs are the caller's device arrays in the padded layout of the
 * component; the second Jacobi iterate and the residual slot live in a fixed
 * 32 MiB device array reserved by the library on every GPU that loads it, so
 * padded fields above 4 Mi points (e.g. beyond 161^3) return SARAS_TOO_LARGE.
 * fastKernels 0 and 1 run the same iteration as saras_cn_solve; fastKernels 2
 * runs the fastKernels 1 iteration (saras_cn_solve's split-FP64 form needs
 * more scratch than the fixed array holds): the same system and stopping
 * rule with different rounding, so results agree to about the tolerance and
 * counts may differ by one.  The first call on a device resolves that array's
 * address: make it before any stream capture.  Calls that overlap on the GPU
 * share the array and race.  stream may be NULL (legacy default stream). */
int saras_cn_solve_noalloc(const saras_params *p, int component, double *v, const double *rhs, void *stream,
                           int *iters, double *max_error);
/* poisson::mgSolve(Pp, mgRHS) (poisson.cc:100-205). */
int saras_mg_solve(saras_ctx *ctx, int *vcycles, double *residual);
int saras_mg_set_mode(saras_ctx *ctx, int mode, double target, int max_cycles);

/* ------------------------------------------------------ time stepping */
/* hydro_d3::timeAdvance (hydro_d3.cc:254-368) or scalar_d3::timeAdvance
 * (scalar_d3.cc:243-370), chosen by probType (main.cc:92-136). */
int saras_time_advance(saras_ctx *ctx, saras_step_stats *stats);
/* tseries::writeTSData (tseries.cc:137-178, 195-246): energy, signed max
 * divergence and (scalar runs) Nusselt number. */
int saras_diagnostics(saras_ctx *ctx, double *energy, double *max_div, double *nusselt);

/* ------------------------------------------------------ time step, probes, restart */
/* vfield::computeTStp (vfield.cc:267-284): dt = courantNumber (dXi / max|Vx| +
 * dEt / max|Vy| + dZt / max|Vz|), the maxima over each padded array
 * (field::fieldMax, field.cc:602-617). */
int saras_compute_tstp(saras_ctx *ctx, double *dt);
/* The time step of the following steps; hydro_d3::solvePDE sets it from
 * computeTStp capped at "Time-Step" when "Use CFL Condition" is true
 * (hydro_d3.cc:196-203). */
int saras_set_dt(saras_ctx *ctx, double dt);
/* parser::parseProbes / testProbes (parser.cc:424-575): the "Probes" sets of a
 * parameters file expanded into (i, j, k) triplets.  *count receives the total;
 * at most `capacity` triplets are written to ijk. */
int saras_parse_probes(const char *path, int *ijk, int capacity, int *count, char *err, int errlen);
/* probes::getData (probes.cc:174-189): out[p * nfields + f] = fields[f] at
 * logical index (i, j, k) of probe p (each index within -1 .. n of its axis). */
int saras_probe(saras_ctx *ctx, int n, const int *ijk, int nfields, const int *fields, double *out);
/* writer::writeRestart (writer.cc:455-540) / reader::readData (reader.cc:213-296):
 * "Time" and the cores of Vx, Vy, Vz, P (and T for the scalar solver), the
 * reference restart file's datasets and core shapes, in a raw little-endian
 * container: "SARASRST", int32 version 1, int32 field count n, float64 time,
 * n x {char name[16], int32 core points along x, y, z}, then the cores as
 * float64 in C order.  Reading fills the cores (ghosts 0) and checks the
 * shapes (reader.cc:338-399); the caller then applies the boundary conditions,
 * as the hydro_d3 / scalar_d3 constructors do. */
int saras_write_restart(saras_ctx *ctx, const char *path, double time);
int saras_read_restart(saras_ctx *ctx, const char *path, double *time);

/* ------------------------------------------------------ multigrid test hooks */
/* multigrid_d3::testProlong / testTransfer / testPeriodic (poisson_d3.cc:689-857)
 * and hydro_d3::testPeriodic (hydro_d3.cc:536-679); each returns the max error. */
int saras_mg_test_prolong(saras_ctx *ctx, double *err);
int saras_mg_test_transfer(saras_ctx *ctx, double *err);
int saras_mg_test_periodic(saras_ctx *ctx, double *err);
int saras_hydro_test_periodic(saras_ctx *ctx, double *err);
/* Level arrays of the hierarchy (poisson.h:70-73): which = 0 pressureData,
 * 1 residualData.  Extents of level l are (2^(ind-l)+1)+2 per axis. */
int saras_mg_level_dims(const saras_ctx *ctx, int level, int dims[3]);
int saras_mg_set_level(saras_ctx *ctx, int level, int which, const double *host);
int saras_mg_get_level(saras_ctx *ctx, int level, int which, double *host);
/* One call of multigrid_d3::smooth(count) at a level (poisson_d3.cc:114-187),
 * computeResidual + coarsen from level to level+1 (poisson_d3.cc:90-111,250-298),
 * prolong from level+1 to level and add the saved level data (poisson_d3.cc:301-388,
 * poisson.cc:271), and computeError at level 0 (poisson_d3.cc:391-459). */
int saras_mg_smooth(saras_ctx *ctx, int level, int count);
int saras_mg_restrict(saras_ctx *ctx, int level);
int saras_mg_prolong_add(saras_ctx *ctx, int level);
int saras_mg_compute_error(saras_ctx *ctx, int norm, double *err);

/* ------------------------------------------------------ learned warm start */
/* Records (divergence, P_prev, P_prev2) -> Pp training pairs from the plain
 * solver, trains the U-Net for `iters` Adam steps, returns the last loss. */
int saras_unet_collect(saras_ctx *ctx);
int saras_unet_train(saras_ctx *ctx, int iters, double lr, double *loss);
int saras_unet_infer(saras_ctx *ctx, int field_out);
int saras_set_guess_mode(saras_ctx *ctx, int mode);
/* The U-Net's parameter count and finest grid (D, H, W: the voxels of one
 * sample of features). */
int saras_unet_shape(saras_ctx *ctx, long long *nparam, int dims[3]);
/* One forward and backward pass of the U-Net with the training kernels and no
 * update: features (D*H*W x 3 FP32, channels last), target (D*H*W) and
 * parameters (nparam FP32 in the layout the training updates; NULL keeps the
 * current ones) in; the network output d (D*H*W), the loss
 * 0.5 mean (d - target)^2 and its gradient with respect to every parameter
 * out (each output may be NULL). */
int saras_unet_grad_check(saras_ctx *ctx, const float *feat, const float *target, const float *params, float *out,
                          double *loss, float *grad);
/* Stand-alone check of the tensor-core 3x3x3 convolution (no context needed).
 * Channels-last BF16 activations (x: D*H*W*cin, dy: D*H*W*cout as raw bf16
 * bits), FP32 weights w[cout][27][cin], bias[cout].  mode 0: forward,
 * out = conv(x) (+bias, ReLU if relu), D*H*W*cout; mode 1: input gradient,
 * out = conv^T(dy), D*H*W*cin; mode 2: weight gradient, out = dW[cout][27][cin]
 * followed by db[cout].  Allocates its own device buffers. */
int saras_conv3d_check(int mode, int D, int H, int W, int cin, int cout, const unsigned short *x,
                       const unsigned short *dy, const float *w, const float *bias, int relu, float *out);

/* ------------------------------------------------------ measurement */
/* Per-kernel CUDA-event timing on the context stream.  kernel ids are listed
 * by saras_profile_name(); only launches at multigrid level 0 are recorded for
 * level kernels.  Bytes are the algorithmic bytes of the recorded launches. */
int saras_profile_enable(saras_ctx *ctx, int kernel_id, int enable);
int saras_profile_read(saras_ctx *ctx, int kernel_id, long long *launches,
                       double *total_ms, double *bytes);
const char *saras_profile_name(int kernel_id);
int saras_profile_count(void);
/* Time the kernels of one replayed target-mode V-cycle in `every` (1: all, the
 * default).  The timing events inside a replayed cycle separate its kernels
 * on the GPU (about 0.14 ms a 257^3 step for the six level-0 sweeps of three
 * cycles); sampled replays keep that cost to 1/every while the timed launches
 * still spread over the whole run.  Launches outside V-cycles are all timed. */
int saras_profile_sample(saras_ctx *ctx, int every);
/* CUDA events on the context stream for whole-step timing: record event
 * `slot` (0..15) now; elapsed milliseconds between two recorded slots. */
int saras_event_record(saras_ctx *ctx, int slot);
int saras_event_elapsed(saras_ctx *ctx, int slot_start, int slot_stop, double *ms);

#ifdef __cplusplus
}
#endif
#endif /* SARAS_GB300_H */
