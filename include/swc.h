/*
 * swc.h -- C ABI of the GB300 dual-particle ("virtual particle") SPH pressure
 * projection.  Drop-in for DualParticleSphLiquid::advance of
 * skytang0205/sand-water-coupling (Cores/Physics/DualParticleSphLiquid.cpp:112-126)
 * and for the projection it performs, VirtualParticle::project
 * (Cores/Structures/VirtualParticle.h:81-87, VirtualParticle.cpp:76-86).
 *
 * Conventions
 *   - One context owns every device buffer of one simulation on one GPU and
 *     one CUDA stream.  Calls on a context are not re-entrant.
 *   - Host arrays are FP64, `dim` components per particle, particle-major: the
 *     layout of the reference's .sav files (Cores/Utilities/IO.h:19-26).  They
 *     are copied in or out and never retained.
 *   - Device state is FP32; CG dot products and norms accumulate in FP64.
 *   - Every call returns an swc_status code.  Nothing exits the process: the
 *     reference's std::exit(-1) on solver failure (Cores/Solvers/IterativeSolver.h:28-31,35-38)
 *     becomes SWC_CG_NOT_CONVERGED / SWC_NAN_DETECTED.
 *   - There is no CPU fallback: without a usable GPU swc_create fails with
 *     SWC_CUDA_ERROR.
 */
#ifndef SWC_H
#define SWC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWC_API_VERSION 1

typedef enum swc_status {
    SWC_OK               = 0,
    SWC_CG_NOT_CONVERGED = 1, /* iteration cap reached above tolerance */
    SWC_NAN_DETECTED     = 2, /* NaN / breakdown in the solve */
    SWC_BAD_ARG          = 3,
    SWC_CUDA_ERROR       = 4,
    SWC_NOT_INITIALIZED  = 5,
    SWC_OUT_OF_MEMORY    = 6
} swc_status;

typedef enum swc_warm_start {
    SWC_WARM_PREFIX  = 0, /* reference: previous pressure vector by position in the active list */
    SWC_WARM_NODE    = 1, /* previous pressure of the same lattice node (0 for new nodes) */
    SWC_WARM_ZERO    = 2,
    SWC_WARM_LEARNED = 3, /* MLP prediction; falls back to NODE when its initial residual is larger */
    SWC_WARM_EXTRAPOLATE = 4 /* the same lattice node's pressure extrapolated in time: 3 p_{n-1} - 3 p_{n-2}
                                + p_{n-3} with three steps of history, 2 p_{n-1} - p_{n-2} with two, NODE
                                with less (the history spans consecutive swc_advance calls) */
} swc_warm_start;

typedef struct swc_ctx swc_ctx;

/* Scene: replaces the reference constructor DualParticleSphLiquid(StaggeredGrid, radius)
 * (Cores/Physics/DualParticleSphLiquid.h:27-29) and the members it fixes. */
typedef struct swc_scene {
    int32_t dim;             /* 2 or 3 */
    int32_t enable_gravity;  /* SmthParticleHydrodLiquid::_enableGravity */
    double  particle_radius; /* r; real and boundary kernel support h = 4 r */
    double  mass;            /* real particle mass m */
    double  boundary_mass;   /* reference sets it to m (DualParticleSphLiquid.cpp:86) */
    double  grid_origin[3];  /* node-grid origin (StaggeredGrid::nodeGrid) */
    double  grid_spacing;    /* node spacing; virtual kernel support H = 4 * spacing */
    int32_t grid_size[3];    /* node counts per axis (z ignored in 2D) */
    int32_t reserved0;
    double  gravity[3];      /* reference: (0, -9.8, 0) */
    double  viscosity;       /* div-free Laplacian coefficient (reference 0.01) */
    double  target_density;  /* <= 0: max rho_i at initialize (reference) */
    double  kappa;           /* < 0: 1 / packed kernel sum (reference) */
} swc_scene;

typedef struct swc_solver_opts {
    double  tolerance;             /* relative residual (reference default 1e-6) */
    int32_t max_iterations;        /* < 0: 2 * N_v (Eigen default) */
    int32_t warm_start;            /* swc_warm_start */
    int32_t check_interval;        /* CG iterations between host convergence checks (0: auto) */
    int32_t keep_virtual_velocity; /* store vbar_I for swc_get_virtual */
    int32_t compute_true_residual; /* evaluate |b - A x| / |b| after each solve */
    int32_t keep_features;         /* keep per-node neighbour counts (learned warm start) */
    int32_t learned_no_fallback;   /* learned start: keep the prediction even when its initial
                                      residual exceeds the base start's (evaluation) */
    int32_t learned_gate;          /* learned start with the residual test: after this many
                                      consecutive rejections of the prediction, skip the network
                                      (base start) for 4 * learned_gate advance steps, then test
                                      it again: one rejection of that test starts the next window,
                                      twice as long (up to 64 * learned_gate steps) until a
                                      prediction is kept; 0: evaluate the network every step */
} swc_solver_opts;

typedef struct swc_stats {
    int64_t n_particles;
    int64_t n_boundary;
    int64_t n_virtual;          /* active virtual particles N_v */
    int32_t active_bricks;
    int32_t cg_iterations;      /* SpMVs inside the CG loop (Eigen's count is one less on convergence) */
    double  rel_residual;       /* recursive |r| / |b| at exit */
    double  true_rel_residual;  /* |b - A x| / |b| (when requested, else -1) */
    double  rhs_norm;           /* |b| = |D| */
    double  initial_rel_residual;
    int32_t warm_start_used;    /* swc_warm_start actually used */
    int32_t status;
    double  device_ms;          /* device time of the call (CUDA events) */
} swc_stats;

/* Defaults: tolerance 1e-6, max_iterations -1, warm start PREFIX. */
void swc_default_solver_opts(swc_solver_opts * opts);
const char * swc_status_str(int status);
const char * swc_last_error(const swc_ctx * ctx);

/* Create / destroy.  Allocates the node-lattice buffers for scene->grid_size. */
int  swc_create(const swc_scene * scene, const swc_solver_opts * opts, swc_ctx ** out);
void swc_destroy(swc_ctx * ctx);
/* Use the caller's cudaStream_t (NULL: the context's own stream). */
int  swc_set_stream(swc_ctx * ctx, void * cuda_stream);
int  swc_set_solver_opts(swc_ctx * ctx, const swc_solver_opts * opts);

/* Particle state (SmthParticleHydrodLiquid::_particles / _velocities; addShape and
 * loadFrame, Cores/Physics/SmthParticleHydrodLiquid.cpp:34-55,124-131). */
int swc_set_particles(swc_ctx * ctx, const double * pos, const double * vel, int64_t n);
int swc_get_particles(swc_ctx * ctx, double * pos, double * vel, int64_t n);
/* Boundary particles with inward normals and velocities
 * (BoundaryParticles::addSurface, Cores/Structures/SmoothedParticles.cpp:111-155). */
int swc_set_boundary(swc_ctx * ctx, const double * pos, const double * normals, const double * vel, int64_t nb);
/* Rigidly rotating part of the boundary: flags[nb] (1 = moving), rotation about the
 * y axis through `center` at angular velocity omega; applied at every advance. */
int swc_set_boundary_motion(swc_ctx * ctx, const uint8_t * moving, const double center[3], double omega);

/* DualParticleSphLiquid::initialize (Cores/Physics/DualParticleSphLiquid.cpp:78-110):
 * rho_i, V_i = m / rho_i, rho0, boundary rho_b / V_b, alpha0 (FP64), kappa. */
int swc_initialize(swc_ctx * ctx);
/* DualParticleSphLiquid::advance(dt) (DualParticleSphLiquid.cpp:112-126):
 * move, rho_i, gravity, viscosity, virtual generation, projection. */
int swc_advance(swc_ctx * ctx, double dt, swc_stats * stats);
/* Projection of the current state: rho_i, virtual generation, then
 * VirtualParticle::project (VirtualParticle.cpp:76-86). */
int swc_project(swc_ctx * ctx, swc_stats * stats);
/* SmthParticleHydrodLiquid::getTimeStep (Cores/Physics/SmthParticleHydrodLiquid.h:39-41):
 * step_rate * 2 r / max |v| (ParticlesAttribute::normMax,
 * Cores/Structures/ParticlesAttribute.h:61-67), the maximum reduced on the device;
 * +inf when every particle is at rest. */
int swc_get_time_step(swc_ctx * ctx, double step_rate, double * dt);

/* Inspection and replay. */
int swc_get_real_info(swc_ctx * ctx, double * rho, double * vol, int64_t n);
int swc_set_volumes(swc_ctx * ctx, const double * vol, int64_t n);
int swc_get_boundary_info(swc_ctx * ctx, double * rho, double * vol, int64_t nb);
int swc_set_boundary_info(swc_ctx * ctx, const double * rho, const double * vol, int64_t nb);
/* Boundary particles as they stand (moving solids turn every advance): positions,
 * inward normals and velocities in the order of swc_set_boundary; any pointer may
 * be NULL (the reference's BoundaryParticles members, SmoothedParticles.h:118-134). */
int swc_get_boundary(swc_ctx * ctx, double * pos, double * normals, double * vel, int64_t nb);
int swc_get_scalars(swc_ctx * ctx, double * rho0, double * alpha0, double * kappa);
int swc_set_scalars(swc_ctx * ctx, double rho0, double alpha0, double kappa);
int64_t swc_num_virtual(swc_ctx * ctx);
/* Active virtual particles in reference order (x-fastest over the node grid):
 * node ids, rho_I, V_I, vbar_I (n x dim; needs keep_virtual_velocity), D_I,
 * alpha_hat_I, p_I.  Any pointer may be NULL.  capacity >= swc_num_virtual. */
int swc_get_virtual(swc_ctx * ctx, int64_t * node_id, double * rho, double * vol, double * vbar, double * div,
                    double * alpha_hat, double * pressure, int64_t capacity);
/* Pressure vector (reference order) used as the next PREFIX warm start. */
int swc_set_pressure(swc_ctx * ctx, const double * p, int64_t n);
/* y = A x with the operator of the last projection (reference order, length N_v). */
int swc_apply_operator(swc_ctx * ctx, const double * x, double * y, int64_t n);

/* Neighbour ids of query points (FP64, nq x dim) found by the product's cell
 * search, for parity checks of the neighbour sets (ParticlesNearbySearcher.cpp:20-35
 * semantics: strict |x_j - q|^2 < R^2).  which: 0 real particles within h
 * (original ids), 1 boundary particles within h (original ids), 2 active virtual
 * nodes within H (node ids).  Call with ids = NULL for the counts, then with
 * CSR offsets (exclusive scan of counts) to receive the ids. */
int swc_debug_neighbors(swc_ctx * ctx, int which, int64_t nq, const double * q, int64_t * counts,
                        const int64_t * offsets, int64_t * ids);

/* Device time of the kernels of the last advance/project by phase (ms):
 * [0] binning, [1] densities, [2] forces, [3] virtual generation (gather +
 * compaction + alpha_hat), [4] warm start, [5] CG, [6] pressure gradient,
 * [7] export.  Requires swc_set_profiling(ctx, 1). */
int swc_set_profiling(swc_ctx * ctx, int on);
int swc_get_phase_times(swc_ctx * ctx, double * ms, int n);
/* Times `reps` back-to-back launches of one kernel on the live state with CUDA
 * events (0: CG SpMV, 1: CG update, 2: virtual gather, 3: pressure gradient,
 * 4: density, 5: forces, 6: CG direction update, 7: learned warm-start forward
 * pass, after a projection that used it); writes the mean ms per launch. */
int swc_time_kernel(swc_ctx * ctx, int which, int reps, double * mean_ms);

/* ---- Learned CG warm start (no counterpart in the reference) -------------
 * A per-virtual-particle MLP 8 -> 64 -> 64 -> 1 (SiLU), BF16 tensor-core
 * forward with FP32 accumulation, predicts a correction of the time-
 * extrapolated pressure of each node.  With p1, p2, p3 the pressures of the
 * same lattice node one, two and three advance steps back (0 where the node
 * was inactive or the history is shorter), the base start is the
 * SWC_WARM_EXTRAPOLATE start
 *   p_base_I = p1 + (p1 - p2) + (p1 - 2 p2 + p3)   (quadratic; the differences
 *              that need more history than the node has are 0).
 * In units w = alpha_hat_I / sD (sD the RMS of D over active nodes):
 *   d1 = (p1 - p2) w (0 without two steps),  d2 = (p1 - 2 p2 + p3) w (0 without three),
 *   q = p1 w,  s = sqrt(d1^2 + d2^2) + SWC_MLP_SCALE_EPS (the node's history scale).
 * Features of active node I (raw, before the normalisation carried with the
 * network):
 *   f0 = D_I / sD     f1 = alpha_hat_I / alpha0    f2 = nreal_I / 32 (real particles within h)
 *   f3 = d1 / s       f4 = d2 / s                  f5 = ln s
 *   f6 = q / (|q| + s)                             f7 = rho_I / rho0
 * Target / prediction, in units of the history scale (so every step weighs the
 * same however small its change):
 *   t = (p_I - p_base_I) w / s,  warm start p0_I = p_base_I + t s / w.
 * Parameters (SWC_MLP_PARAMS floats): W1[64][8], b1[64], W2[64][64], b2[64], w3[64], b3.
 * Normalisation (SWC_MLP_NORM floats): feature mean[8], feature std[8], target mean, target std. */
#define SWC_MLP_IN 8
#define SWC_MLP_PARAMS (64 * SWC_MLP_IN + 64 + 64 * 64 + 64 + 64 + 1)
#define SWC_MLP_NORM (2 * SWC_MLP_IN + 2)
#define SWC_MLP_SCALE_EPS 1e-4f
/* Network used by SWC_WARM_LEARNED.  Each learned solve computes the initial
 * residual of both the prediction and the base start and starts CG from the
 * smaller unless learned_no_fallback is set (stats.warm_start_used tells
 * which: LEARNED, else EXTRAPOLATE or NODE for the base). */
int swc_set_mlp(swc_ctx * ctx, const float * params, const float * norm);
/* Training data of the last projection (needs keep_features): features
 * (n x SWC_MLP_IN, reference order) and targets (n) as defined above.  Returns
 * the count in *n (<= capacity). */
int swc_get_features(swc_ctx * ctx, float * features, float * targets, int64_t capacity, int64_t * n);

/* Device-side training of the network: every batch runs one fused tensor-core
 * pass (forward, backward and weight gradients as BF16 tcgen05 products with
 * FP32 accumulation; the per-CTA shares of the gradient added in a fixed order)
 * and an Adam step with FP32 master weights.  The dataset lives in device memory. */
typedef struct swc_trainer swc_trainer;
int  swc_trainer_create(int64_t capacity, int32_t batch, swc_trainer ** out);
void swc_trainer_destroy(swc_trainer * tr);
int  swc_trainer_add(swc_trainer * tr, const float * features, const float * targets, int64_t n);
int  swc_trainer_set_params(swc_trainer * tr, const float * params, const float * norm);
int  swc_trainer_get_params(swc_trainer * tr, float * params, float * norm);
/* `epochs` passes over the dataset, each in a pseudo-random row order computed on the
 * device (a Feistel permutation keyed by `seed` and the epoch); epoch_loss[e] = mean
 * squared error of the normalised output after epoch e, over the whole dataset. */
int  swc_trainer_fit(swc_trainer * tr, int32_t epochs, float lr, uint64_t seed, float * epoch_loss);
/* Stateless helpers on host arrays (run on the GPU): predictions, and the loss
 * gradient for one batch (the mean squared error of the normalised output in *loss). */
int swc_mlp_forward(const float * params, const float * norm, const float * features, int64_t n, float * out);
int swc_mlp_gradient(const float * params, const float * norm, const float * features, const float * targets,
                     int64_t n, float * grad, float * loss);
/* Same loss gradient as swc_mlp_gradient, for callers that cannot allocate
 * device memory when they need it (frameworks that plan all device memory up
 * front, callers under a fixed memory budget).  No counterpart in the reference.
 * It allocates nothing: all pointers are device pointers supplied by the caller
 * (params[SWC_MLP_PARAMS], norm[SWC_MLP_NORM], features[n][SWC_MLP_IN], targets[n],
 * grad[SWC_MLP_PARAMS] and loss[1] out), work is queued on `stream` (NULL: the
 * default stream) and its scratch lives in fixed device arrays for at most
 * SWC_MLP_NOALLOC_MAX_ROWS rows (about 0.7 MB per device, held until the process
 * exits).  n above the limit returns SWC_BAD_ARG.  The first call on a device
 * resolves the arrays' device addresses and sets the kernel's shared-memory
 * attribute, so make it before any stream capture; the resolved addresses do
 * not survive a cudaDeviceReset of that device.  All calls share the arrays:
 * calls that overlap on the GPU race.  A failure of the tensor-core pass shows
 * as loss = NaN. */
#define SWC_MLP_NOALLOC_MAX_ROWS 2048
int swc_mlp_gradient_noalloc(const float * params, const float * norm, const float * features,
                             const float * targets, int64_t n, float * grad, float * loss, void * stream);

/* Test hook for the failure paths (no counterpart in the reference): the device
 * allocation `after` allocations from now (0: the next one) made by any context of
 * this library, liquid or sand, fails with SWC_OUT_OF_MEMORY instead of calling
 * cudaMalloc; a negative value disarms it.  Process-wide, meant for tests. */
int swc_debug_fail_alloc(int64_t after);

/* Pinned host memory helpers for callers that stream state every step. */
void * swc_host_alloc(size_t bytes);
void   swc_host_free(void * p);

#ifdef __cplusplus
}
#endif

#endif /* SWC_H */
