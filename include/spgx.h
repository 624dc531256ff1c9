/*
 * spgx.h — C ABI of the GB300 (sm_103a) Vertex Block Descent and XPBD solvers.
 *
 * This is the drop-in boundary for SPG's solver plugin point. A host C++ adapter that
 * derives from spg::solver::BaseSolver (spg/include/spg/sim/solver/baseSolver.h:14-41)
 * packs each ParticleGroup and its energies into an spgx_scene_desc and forwards step()
 * to spgx_vbd_step() / spgx_xpbd_step(). Plain pointers and sizes only; no C++ or CUDA
 * types cross this boundary and no exception escapes it.
 *
 * Reference interfaces replaced (paths inside the spg project):
 *   spgx_vbd_*   spg::solver::VBD   spg/include/spg/sim/solver/vbd.h:14-41,
 *                                   spg/source/sim/solver/vbd.cpp:12-268
 *   spgx_xpbd_*  spg::solver::XPBD  spg/include/spg/sim/solver/xpbd.h:13-27,
 *                                   spg/source/sim/solver/xpbd.cpp:16-160
 *   spgx_implicit_*  spg::solver::ImplicitEulerNewtonDx  implicitEulerNewtonDx.cpp:11-65,
 *                                   implicitEulerBase.cpp:102-240
 *   spgx_energy_desc   the five Energy<ParticleGroup> implementations on the hot path and
 *                      their precomputed per-stencil data (energy.h:21-369)
 *
 * Threading: a handle owns one CUDA stream; calls on one handle must be serialised by the
 * caller (the reference solvers are not re-entrant either). Distinct handles are
 * independent. Every call returns after its GPU work has finished unless stated otherwise.
 */
#ifndef SPGX_H
#define SPGX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPGX_API_VERSION 1

typedef enum spgx_status {
    SPGX_OK = 0,
    SPGX_ERR_INVALID_ARG = 1,        /* mirrors the reference's setup-time std::runtime_error */
    SPGX_ERR_UNSUPPORTED_ENERGY = 2, /* energy type outside the five below */
    SPGX_ERR_CUDA = 3,               /* CUDA runtime error (message in spgx_last_error_string) */
    SPGX_ERR_NONFINITE = 4,          /* a vertex update produced NaN/Inf; the update was not stored */
    SPGX_ERR_TIMEOUT = 5,            /* a bounded device-side wait gave up (dataflow kernel) */
    SPGX_ERR_NO_DEVICE = 6           /* no CUDA device, or not an sm_103 device */
} spgx_status;

/* Energy types (the reference classes whose precomputed data the params carry). */
typedef enum spgx_energy_type {
    SPGX_ENERGY_SPRING = 1,             /* spg::SpringEnergy             springEnergy.h:9 */
    SPGX_ENERGY_SPRING_ANCHOR = 2,      /* spg::SpringAnchorEnergy       springAnchorEnergy.h:7 */
    SPGX_ENERGY_DISCRETE_BENDING = 3,   /* spg::DiscreteBendingEnergy    discreteBendingEnergy.h:9 */
    SPGX_ENERGY_MEMBRANE_STVK = 4,      /* spg::MembraneStvkEnergy       membraneStvkEnergy.h:9 */
    SPGX_ENERGY_STABLE_NEO_HOOKEAN = 5, /* spg::StableNeoHookeanEnergy   stableNeoHookeanEnergy.h:10 */
    /* The types below take their per-vertex blocks from forward-mode derivatives on the device
     * (every VBD kernel); XPBD accepts 6-13 (the static load has no constraint form, and the
     * reference throws for it too). */
    SPGX_ENERGY_STVK = 6,                         /* spg::StvkEnergy (tet)              stvkEnergy.h */
    SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN = 7,   /* spg::StableSquaredNeoHookeanEnergy */
    SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN = 8,       /* spg::MembraneBaraffWitkinEnergy */
    SPGX_ENERGY_MEMBRANE_CHOI = 9,                /* spg::MembraneChoiEnergy */
    SPGX_ENERGY_BARAFF_WITKIN_BENDING = 10,       /* spg::BaraffWitkinBendingEnergy */
    SPGX_ENERGY_QUADRATIC_BENDING = 11,           /* spg::QuadraticBendingEnergy */
    SPGX_ENERGY_SPRING_CONTINUUM = 12,            /* spg::SpringContinuumEnergy */
    SPGX_ENERGY_SPRING_SQUARED_CONTINUUM = 13,    /* spg::SpringSquaredContinuumEnergy */
    SPGX_ENERGY_STATIC_LOAD = 14                  /* spg::StaticLoadEnergy */
} spgx_energy_type;

/*
 * One energy: n_stencils stencils of spgx_stencil_size(type) vertex indices each (the
 * reference's flatStencils(), energy.h:102-110) and spgx_param_count(type) doubles per
 * stencil, in this order:
 *   SPRING            [restLength, effectiveStiffness, effectiveCompliance]
 *   SPRING_ANCHOR     [anchor.x, anchor.y, anchor.z, modelStiffness, effectiveCompliance]
 *   DISCRETE_BENDING  [restTheta, effectiveStiffness, effectiveCompliance]
 *   MEMBRANE_STVK     [inverseReferenceMat (2x2 row-major), effectiveStiffness (3x3 row-major),
 *                      effectiveCompliance (3x3 row-major)]
 *   STABLE_NEO_HOOKEAN [inverseReferenceMat (3x3 row-major), effectiveStiffness(0,0),
 *                      effectiveStiffness(1,1), hydrostaticCorrectionTerm,
 *                      effectiveCompliance(0,0), effectiveCompliance(1,1)]
 *   STVK, STABLE_SQUARED_NEO_HOOKEAN
 *                     [inverseReferenceMat (3x3 row-major), effectiveStiffness(0,0) (lambda V),
 *                      effectiveStiffness(1,1) (mu V), effectiveCompliance(0,0), (1,1)]
 *   MEMBRANE_BARAFF_WITKIN [inverseReferenceMat (2x2 row-major), effectiveStiffness diagonal (3),
 *                      effectiveCompliance diagonal (3)]
 *   MEMBRANE_CHOI     [inverseReferenceMat (2x2 row-major), effectiveStiffness diagonal (4),
 *                      effectiveCompliance diagonal (4)]
 *   BARAFF_WITKIN_BENDING [restTheta, effectiveStiffness, effectiveCompliance]
 *   QUADRATIC_BENDING [laplacian weights c0..c3 (laplacians()[i](0, 0), (0, 3), (0, 6), (0, 9)),
 *                      effectiveStiffness(0,0), effectiveCompliance(0,0)]
 *   SPRING_CONTINUUM, SPRING_SQUARED_CONTINUUM [restLength, effectiveStiffness, effectiveCompliance]
 *   STATIC_LOAD       [modelStiffness, loadDirection.x, .y, .z]
 * i.e. the values the reference holds after addStencil() and preparePrecomputations(). The
 * stiffness matrices of types 6-13 are diagonal, so only their diagonals are passed.
 */
typedef struct spgx_energy_desc {
    int32_t type;
    int32_t n_stencils;
    const int32_t *stencils;
    const double *params;
} spgx_energy_desc;

/* One ParticleGroup (particleGroup.h:14-60): positions, velocities (NULL = zero), masses. */
typedef struct spgx_object_desc {
    int32_t n_vertices;
    const double *x;    /* 3 * n_vertices */
    const double *v;    /* 3 * n_vertices or NULL */
    const double *mass; /* n_vertices */
    int32_t n_energies;
    const spgx_energy_desc *energies; /* in obj.energies() order */
} spgx_object_desc;

/* A solver's object list (BaseSolver::m_objects particle groups). Objects are independent
 * and are solved together, colour by colour, in one launch per colour. */
typedef struct spgx_scene_desc {
    int32_t n_objects;
    const spgx_object_desc *objects;
} spgx_scene_desc;

int32_t spgx_stencil_size(int32_t type);
int32_t spgx_param_count(int32_t type);
int32_t spgx_api_version(void);

/* Last error message of the calling thread ("" if none). */
const char *spgx_last_error_string(void);

/* ------------------------------------------------------------------------------------ */
/* Host-only setup (no device needed)                                                     */

/* Greedy vertex colouring of one object, bit-exact with coloring::colorVertices
 * (graphColoring.cpp:72-84 -> Graph::greedyColoring :21-49). colors: n_vertices. */
spgx_status spgx_color_vertices(const spgx_object_desc *obj, int32_t *colors);
/* Greedy stencil colouring of one energy, bit-exact with coloring::colorStencils
 * (graphColoring.cpp:51-70). colors: n_stencils. */
spgx_status spgx_color_stencils(const spgx_energy_desc *energy, int32_t *colors);
/* Per-vertex incidence lists of one object in reference order (VBD::computeStencilInfoPerVertex,
 * vbd.cpp:231-268): counts[v * n_energies + e] and (stencilIdx, vertexIdxInStencil) pairs. */
spgx_status spgx_incidences(const spgx_object_desc *obj, int32_t *counts, int32_t *entries, int64_t *total);

/* ------------------------------------------------------------------------------------ */
/* Device-side setup for topology changes                                               */

/* Values per stencil that addStencil() takes, for spgx_precompute_params:
 *   SPRING, SPRING_CONTINUUM, SPRING_SQUARED_CONTINUUM  [restLength, stiffness]
 *                       (restLength <= 0 takes |x0[s0] - x0[s1]|)
 *   SPRING_ANCHOR       [anchor.x, anchor.y, anchor.z, stiffness]
 *   DISCRETE_BENDING, BARAFF_WITKIN_BENDING, QUADRATIC_BENDING  [restTheta, stiffness]
 *                       (restTheta is validated as addStencil does, then replaced by the rest angle)
 *   MEMBRANE_STVK, STABLE_NEO_HOOKEAN, STVK, STABLE_SQUARED_NEO_HOOKEAN  [young, poisson]
 *   MEMBRANE_BARAFF_WITKIN, MEMBRANE_CHOI  [kWeft, kWarp, kBias]
 *   STATIC_LOAD         [stiffness, direction.x, .y, .z]
 * Returns 0 for an unknown type. */
int32_t spgx_material_count(int32_t type);
/* The energies' addStencil + preparePrecomputations on the GPU: fills params (n_stencils x
 * spgx_param_count(type), the layout above) from the rest positions x0 (3 * n_vertices) and
 * per-stencil material values (material_stride doubles apart; 0 = one row for all stencils).
 * Every value equals the host classes' to the last bit, except the rest angles of the
 * bending energies (atan2, within a few ulp). A stencil the reference would reject (rest
 * length, angle, area or volume) fails the call with the reference's message. */
spgx_status spgx_precompute_params(int32_t type, int32_t n_stencils, const int32_t *stencils, int32_t n_vertices,
                                   const double *x0, const double *material, int32_t material_stride,
                                   double *params, int32_t device);
/* The same on the host, through the host energy classes' addStencil + preparePrecomputations
 * (the reference's setup path); the baseline spgx_precompute_params replaces. */
spgx_status spgx_precompute_params_host(int32_t type, int32_t n_stencils, const int32_t *stencils,
                                        int32_t n_vertices, const double *x0, const double *material,
                                        int32_t material_stride, double *params);
/* spgx_incidences computed on the GPU (counting pass, scan, scatter, per-bucket ordering):
 * the same counts and entries, bit for bit. With counts and entries NULL only *total is set. */
spgx_status spgx_incidences_device(const spgx_object_desc *obj, int32_t device, int32_t *counts, int32_t *entries,
                                   int64_t *total);

/* ------------------------------------------------------------------------------------ */
/* Vertex Block Descent                                                                  */

typedef struct spgx_vbd spgx_vbd;

typedef struct spgx_vbd_params {
    double dt;                 /* BaseSolver::setDt (baseSolver.h:26) */
    int32_t substeps;          /* BaseSolver::setNumSubsteps (baseSolver.h:28) */
    int32_t iterations;        /* VBD::m_iterations (vbd.h:33; fixed at 1 in the reference) */
    double gravity[3];         /* BaseSolver::setGravity (baseSolver.h:32) */
    double tolerance;          /* > 0: iterate until ||r|| <= tolerance * ||r(y)||, see below */
    int32_t max_iterations;    /* cap per substep when tolerance > 0 */
    int32_t check_interval;    /* iterations between residual checks when tolerance > 0; once two
                                * checks give a decay rate, the last interval is cut to the
                                * iterations that rate needs (5 % margin, at least 10) */
    double fallback_condition; /* 3x3 blocks whose condition estimate exceeds this are solved in FP64 */
    int32_t lanes_per_vertex;  /* 0 = autotune; else 1, 2, 4, 8, 16 or 32 */
    int32_t block_size;        /* 0 = autotune; else a multiple of 32 up to 256 (lanes kernel) */
    int32_t use_graph;         /* 1 = replay the iteration loop as a CUDA graph */
    int32_t device;            /* CUDA device ordinal */
    int32_t kernel;            /* 0 = autotune, 1 = lanes-per-vertex kernel, 2 = shared-memory tile kernel
                                * (one launch per colour), 3 = dataflow tile kernel (one persistent
                                * cooperative launch runs all sweeps; a tile starts as soon as its
                                * neighbour tiles finished the sweeps it reads; no CUDA graph needed) */
    int32_t tile_vertices;     /* vertices per tile of the tile kernels (1..128; 0 = autotune over 32
                                * and 64); the chosen size is block_size / lanes_per_vertex */
} spgx_vbd_params;

/* Defaults: dt 0.01, 1 substep, 1 iteration, gravity (0,-9.8,0) (baseSolver.h:36-38),
 * tolerance 0, max_iterations 1000, check_interval 10, fallback_condition 1e6, autotune,
 * use_graph 1, device 0, kernel and tile size autotuned. */
void spgx_vbd_params_default(spgx_vbd_params *p);

typedef struct spgx_step_stats {
    int32_t iterations;        /* VBD iterations run in the step, summed over substeps */
    int32_t fallback_solves;   /* 3x3 solves redone in FP64 */
    int32_t skipped_solves;    /* vertices skipped by the det(H) > 1e-10 guard (vbd.cpp:139) */
    int32_t converged;         /* tolerance mode: every substep reached the tolerance */
    double residual_initial;   /* ||r(y)|| of the last substep (tolerance mode, else 0) */
    double residual_final;     /* ||r(x)|| at the end of the last substep (tolerance mode) */
    double device_ms;          /* CUDA-event time of the step on the handle's stream */
    int32_t warm_accepted;         /* substeps started from the learned guess */
    int32_t extrapolated_accepted; /* substeps started from the extrapolated guess */
    double residual_warm;          /* ||r|| of the last substep's learned guess (mode 1) or extrapolated
                                    * guess (mode 2); tolerance mode */
    double residual_extrapolated;  /* ||r|| of the last substep's extrapolated guess; tolerance mode */
} spgx_step_stats;

/*
 * Creates a solver for the scene. The scene is copied (positions become FP32 on the device,
 * element data FP32); the caller keeps ownership of every array. Setup mirrors the
 * reference's first step(): greedy vertex colouring per object (vbd.cpp:203-229, bit-exact
 * with graphColoring.cpp:21-84) and the per-vertex incidence lists (vbd.cpp:231-268).
 */
spgx_status spgx_vbd_create(const spgx_scene_desc *scene, const spgx_vbd_params *params, spgx_vbd **out);
spgx_status spgx_vbd_destroy(spgx_vbd *h);
spgx_status spgx_vbd_set_params(spgx_vbd *h, const spgx_vbd_params *params);

/*
 * One VBD::step() (vbd.cpp:12-195) for every object: per substep, inertial prediction,
 * `iterations` colour sweeps of per-vertex 3x3 Newton updates (or, with tolerance > 0, sweeps
 * until the incremental-potential residual r = M/h^2 (x - y) + grad E(x), reduced in FP64,
 * satisfies ||r|| <= tolerance * ||r(y)||), then the velocity update. stats may be NULL.
 */
spgx_status spgx_vbd_step(spgx_vbd *h, spgx_step_stats *stats);

/* Host <-> device state of one object (3 * n_vertices doubles each; NULL skips). */
spgx_status spgx_vbd_get_state(spgx_vbd *h, int32_t object, double *x, double *v);
spgx_status spgx_vbd_set_state(spgx_vbd *h, int32_t object, const double *x, const double *v);

/* BaseSolver::reset (baseSolver.cpp:23-32): positions back to those given at create,
 * velocities to zero. */
spgx_status spgx_vbd_reset(spgx_vbd *h);

/* FP64-reduced residual norm over all objects at the current state against the inertial
 * target of the most recent substep (zero target before the first step). */
spgx_status spgx_vbd_residual(spgx_vbd *h, double *norm);

/* Introspection for parity checks. object -1 gives the number of colour phases of the
 * whole scene (the maximum over objects). */
spgx_status spgx_vbd_num_colors(spgx_vbd *h, int32_t object, int32_t *n);
spgx_status spgx_vbd_get_colors(spgx_vbd *h, int32_t object, int32_t *colors);
/* Incidence lists in reference order: counts[v * n_energies + e] and, in the same order,
 * (stencilIdx, vertexIdxInStencil) pairs. Pass entries == NULL to query *total first. */
spgx_status spgx_vbd_get_adjacency(spgx_vbd *h, int32_t object, int32_t *counts, int32_t *entries, int64_t *total);
/* Launch configuration the solver uses (after autotuning): the kernel (1, 2 or 3), lanes per
 * vertex and threads per CTA. */
spgx_status spgx_vbd_get_launch(spgx_vbd *h, int32_t *kernel, int32_t *lanes_per_vertex, int32_t *block_size);
/* Dynamic anchors for interactive picking (apps/solverCompare.cpp:717-726 adds a one-stencil
 * SpringAnchorEnergy to the picked ParticleGroup, :1524 moves it with updateAnchor, :1499
 * removes it; each change flags a VBD topology update). Replaces the set of picks: pick q
 * pulls vertex vertex[q] of object object[q] towards target[3q..3q+2] with stiffness[q], as a
 * one-stencil SpringAnchorEnergy appended after the object's energies would. Takes effect at
 * the next step, with no rebuild of colours, incidences or tiles (an anchor adds no graph
 * edge, so the reference's recolouring gives the same colours). n = 0 removes every pick. */
/* Failure-detection test hook (dataflow kernel only): marks one tile's sweep counter as never
 * reached, so that the next step's waits on that tile run out their bounded polls (about a
 * second). Every CTA then leaves the kernel, the step returns SPGX_ERR_TIMEOUT, the
 * counters are reset, and the handle keeps working; nothing faults or hangs. */
spgx_status spgx_vbd_test_stall_tile(spgx_vbd *h, int32_t tile);
#define SPGX_MAX_PICKS 16
spgx_status spgx_vbd_set_picks(spgx_vbd *h, int32_t n, const int32_t *object, const int32_t *vertex,
                               const double *target, const double *stiffness);
/* Runs `iterations` colour sweeps with a CUDA event pair around every colour launch on the
 * handle's stream and writes the mean duration (ms) of each colour's launch to color_ms
 * (spgx_vbd_num_colors(h, -1, ...) entries). Advances the positions like the iterations of
 * a step (no inertial or velocity phase). With kernel 3 there are no per-colour launches:
 * color_ms[0] receives the mean time of a whole sweep and the other entries 0. */
spgx_status spgx_vbd_profile_sweeps(spgx_vbd *h, int32_t iterations, double *color_ms);

/* ------------------------------------------------------------------------------------ */
/* Learned warm start. No counterpart in the reference, whose only initial guess is the
 * inertial one (vbd.h:22, InitialGuessType::InertialWithAcceleration; vbd.cpp:78-83).
 *
 * A per-vertex MLP (24 -> 128 -> 128 -> 128 -> 3, GELU; BF16 weights on the tensor cores with
 * FP32 accumulation) maps local features of the displacement history to a correction c of
 * the extrapolated guess x_e = x_n + 2 (x_n - x_{n-1}) - (x_{n-1} - x_{n-2}) (the last
 * step's acceleration carried over): x_w = x_e + l c, in units of l = h^2 * 9.81 m/s^2.
 * Predicting only the remainder keeps the network's BF16 precision from limiting the guess.
 * Features per
 * vertex (24 floats, displacements over l): y - x_n, x_n - x_{n-1}, x_{n-1} - x_{n-2}, the
 * one-ring Laplacians (neighbour mean minus own) of the last two, g / 9.81, the anchored
 * flag, the anchored fraction of the one-ring, the one-ring size / 8, |x_n - x_{n-1}|,
 * |Laplacian of x_n - x_{n-1}| and 1.
 *
 * With the learned warm start every substep evaluates y, x_e and x_w and starts from the one
 * with the lowest ||r|| (FP64-reduced on the device), so the network can only help; a guess
 * is kept only when it lowers the residual below ||r(y)||. The tolerance test stays relative
 * to ||r(y)||, so a guess cannot loosen it. */

typedef struct spgx_mlp spgx_mlp;

/* Parameter count and layout of the flat FP32 weight vector: W1[24][128] b1[128]
 * W2[128][128] b2[128] W3[128][128] b3[128] W4[128][3] b4[3] (row-major, input-major). */
int32_t spgx_mlp_num_params(void);
/* New network with Xavier-uniform weights drawn from `seed` and zero biases. */
spgx_status spgx_mlp_create(uint64_t seed, int32_t device, spgx_mlp **out);
spgx_status spgx_mlp_destroy(spgx_mlp *h);
spgx_status spgx_mlp_get_weights(spgx_mlp *h, float *w);
/* Replaces the weights (FP32 master copy; inference uses their BF16 rounding) and clears the
 * optimizer state. */
spgx_status spgx_mlp_set_weights(spgx_mlp *h, const float *w);
/* y[n][3] = MLP(x[n][24]) on the tensor cores (host arrays). */
spgx_status spgx_mlp_forward(spgx_mlp *h, int32_t n, const float *x, float *y);
/* Mean squared error over the n x 3 outputs against y, and its gradient with respect to the
 * flat weights (FP32 forward/backward with the BF16-rounded weights; the rounding is passed
 * straight through). grad has spgx_mlp_num_params() entries. */
spgx_status spgx_mlp_loss_grad(spgx_mlp *h, int32_t n, const float *x, const float *y, float *loss, float *grad);
/* `steps` Adam steps (beta 0.9 / 0.999, eps 1e-8, learning rate lr) on minibatches of `batch`
 * rows drawn uniformly with replacement (seeded) from the n rows; all on the device.
 * final_loss (may be NULL) is the last minibatch's loss. */
spgx_status spgx_mlp_train(spgx_mlp *h, int32_t n, const float *x, const float *y, int32_t steps, int32_t batch,
                           float lr, uint64_t seed, float *final_loss);

/* Chooses the initial guess of every substep: mode 0 the inertial guess y (the reference's);
 * mode 1 the learned guess (mlp required); mode 2 the previous step's acceleration carried
 * over, x_e = x_n + 2 (x_n - x_{n-1}) - (x_{n-1} - x_{n-2}) (no network; a baseline for
 * the learned guess). Mode 2 keeps x_e only when its residual is below y's. Mode 1 forms
 * x_w = x_e + l * smoothed network correction, runs 40 sweeps from each of x_w and x_e, and
 * continues from the one with the lower residual (the sweeps of the other one are spent and
 * counted in spgx_step_stats.iterations; residual_warm / residual_extrapolated are the
 * residuals after those sweeps).
 * The first call also starts keeping the displacement history (from then on, and after
 * every set_state/reset, seeded with a constant-velocity past). The network must outlive
 * its use by the solver and live on the solver's device; do not train it while the solver
 * steps. */
spgx_status spgx_vbd_set_warm_start(spgx_vbd *h, const spgx_mlp *mlp, int32_t mode);
/* Smoothing passes applied to the network's correction field before the learned guess is
 * formed: each pass replaces a vertex's correction by the mean of itself and its one-ring
 * mean. 0 to 64; the default is 20. The network's error is mostly per-vertex noise, which the
 * stiff springs turn into large forces; the smoothed field keeps its smooth, accurate part. */
spgx_status spgx_vbd_set_warm_start_smoothing(spgx_vbd *h, int32_t passes);
/* One step (one substep only; history started by spgx_vbd_set_warm_start) that also returns,
 * for every vertex of the scene in the solver's internal order, the features at the start of
 * the step (features[n_vertices][24]) and (x - y) / l at its end (targets[n_vertices][3]);
 * the network's training target is that minus (features[3:6] - features[6:9] -
 * features[15:18]), the extrapolated guess's offset from y. */
spgx_status spgx_vbd_step_record(spgx_vbd *h, float *features, float *targets, spgx_step_stats *stats);
/* The solver's internal vertex order (colour-major): ext_of_internal[i] is the index, in the
 * scene's concatenated object-by-object vertex order, of internal vertex i. */
spgx_status spgx_vbd_get_vertex_order(spgx_vbd *h, int32_t *ext_of_internal);

/* ------------------------------------------------------------------------------------ */
/* Element-level evaluation on the GPU with the solver's device code (FP32), for the
 * per-element derivative parity checks. For n incidences of one energy type:
 * X = n * stencil_size * 3 positions, params = n * param_count, slots = n vertex slots.
 * grad = n * 3 (energy gradient segment of the slot), hess = n * 9 (row-major 3x3 block). */
spgx_status spgx_eval_vertex_blocks(int32_t type, int32_t n, const double *X, const double *params,
                                    const int32_t *slots, double *grad, double *hess);
/* Allocation-free variant of spgx_eval_vertex_blocks, for callers that cannot allocate device
 * memory: hosts whose device memory is owned by another allocator (a framework's memory pool
 * that leaves nothing to cudaMalloc), or code paths that must not add allocation latency
 * or fragmentation after start-up. It calls no cudaMalloc, cudaFree or other allocating
 * routine: inputs and outputs are the caller's host arrays, and the device staging is one
 * fixed array inside the library (about 750 KB on each GPU it was called on, until the
 * process exits). Capacity: n <= 4096 incidences per call; larger n returns
 * SPGX_ERR_INVALID_ARG (so do types with more than 4 stencil vertices or 22 parameters; all
 * fourteen fit). The first call on a device loads the library's device code there, which
 * places the array: make it at start-up, before another allocator takes the device's memory.
 * Every call looks up the array's device address (no allocation). The function is never
 * capture-safe: it copies synchronously and launches on the legacy default stream, so it must
 * not be called while any stream of the process is being captured. All calls share the
 * array: calls that overlap on the same GPU race. Results equal spgx_eval_vertex_blocks'. No
 * counterpart in the reference. */
spgx_status spgx_eval_vertex_blocks_noalloc(int32_t type, int32_t n, const double *X, const double *params,
                                            const int32_t *slots, double *grad, double *hess);
/* Constraint values (n * nc) and gradients (n * nc * 3 * stencil_size, constraint-major)
 * as used by the XPBD projection. */
spgx_status spgx_eval_constraints(int32_t type, int32_t n, const double *X, const double *params, double *C,
                                  double *gradC);
int32_t spgx_num_constraints(int32_t type);

/* ------------------------------------------------------------------------------------ */
/* The global solvers of the reference (spg/source/sim/solver/), on ImplicitEulerBase's system
 * force, stiffness matrix and conjugate-gradient solve (implicitEulerBase.cpp:102-240):
 * f = M g - grad E(x), K = -hess E(x) (full element Hessians, no definiteness projection),
 * linear systems by CG with the diagonal preconditioner (relative tolerance cg_threshold,
 * cg_max_iterations, zero start). State, assembly and the CG's vectors and dot products are
 * FP64; the CG's matrix-vector products run in double-float (FP32 pairs, 48-bit significands)
 * unless a matrix value or direction entry exceeds 2^60 in magnitude (or a nonzero diagonal
 * is below 2^-60), in which case that solve's products run in FP64. Per substep of h:
 *   NEWTON_DX       implicitEulerNewtonDx.cpp:31-55     x += v h; (M/h^2 - K) dx = f; x += dx; v = (x - x0)/h
 *   NEWTON_DV       implicitEulerNewtonDv.cpp:31-60     x += v h; (M - h^2 K) dv = h f; v = v0 + dv; x = x0 + v h
 *   NEWTON_ROBUST   implicitEulerNewtonRobust.cpp:33-126 Newton on (M - h^2 K) dv = h f - M (v_i - v0) with a
 *                   halving line search (5 steps), 5 iterations, threshold 1e-5; a failed substep restores
 *                   x0, v0 and scales the persistent step by 0.75; more than 5 successes in a row grow it back
 *   BARAFF_WITKIN   implicitEulerBaraffWitkin.cpp:31-52 (M - h^2 K) dv = h (f + h K v0); v = v0 + dv; x += v h
 *   BDF2            bdf2.cpp:31-74                      (M - 4/9 h^2 K) dv = 1/3 M (v0 - v_-1)
 *                   + 2/3 h (f + 1/3 K (x0 - x_-1 + 2 h v0)); v = v0 + dv; x = 4/3 x0 - 1/3 x_-1 + 2/3 v h
 *   STATIC_NEWTON   staticNewton.cpp:30-45              K dx = -f; x += dx
 *   QUASI_STATIC_NEWTON quasiStaticNewton.cpp:32-49     (M - h^2 K) dx = h^2 f; x += dx
 *   QUASI_STATIC_NEWTON_ROBUST quasiStaticNewtonRobust.cpp:33-136 Newton on (M/h^2 - K) dx = f - M v/h,
 *                   v = (x - x0)/h, line search and step control as NEWTON_ROBUST, threshold 1e-2
 *   SYMPLECTIC_EULER simplecticEuler.cpp:11-62          v += h g + h W (-grad E); x += v h
 * Every energy type is accepted. spgx_step_stats: iterations = CG iterations summed over
 * substeps; converged = every solve reached cg_threshold (robust methods: every substep
 * succeeded); residual_final = the last solve's relative residual |r| / |b| (robust methods:
 * the last Newton residual norm, residual_initial the first); fallback_solves = Newton
 * iterations and skipped_solves = failed substeps (robust methods); warm_accepted = solves
 * whose products ran in FP64. */
typedef enum spgx_implicit_method {
    SPGX_IMPLICIT_NEWTON_DX = 0,          /* spg::solver::ImplicitEulerNewtonDx */
    SPGX_IMPLICIT_NEWTON_DV = 1,          /* spg::solver::ImplicitEulerNewtonDv */
    SPGX_IMPLICIT_NEWTON_ROBUST = 2,      /* spg::solver::ImplicitEulerNewtonRobust */
    SPGX_IMPLICIT_BARAFF_WITKIN = 3,      /* spg::solver::ImplicitEulerBaraffWitkin */
    SPGX_IMPLICIT_BDF2 = 4,               /* spg::solver::BDF2 */
    SPGX_STATIC_NEWTON = 5,               /* spg::solver::StaticNewton */
    SPGX_QUASI_STATIC_NEWTON = 6,         /* spg::solver::QuasiStaticNewton */
    SPGX_QUASI_STATIC_NEWTON_ROBUST = 7,  /* spg::solver::QuasiStaticNewtonRobust */
    SPGX_SYMPLECTIC_EULER = 8             /* spg::solver::SimplecticEuler */
} spgx_implicit_method;

typedef struct spgx_implicit spgx_implicit;

typedef struct spgx_implicit_params {
    double dt;                 /* BaseSolver::setDt */
    int32_t substeps;          /* BaseSolver::setNumSubsteps */
    double gravity[3];         /* BaseSolver::setGravity */
    double cg_threshold;       /* ImplicitEulerBase::m_cgThreshold (1e-5) */
    int32_t cg_max_iterations; /* ImplicitEulerBase::m_cgMaxIterations (300) */
    int32_t device;
    int32_t method;            /* an spgx_implicit_method value; default NEWTON_DX */
    int32_t cg_precision;      /* 0 (default): the CG runs in double-float (FP32 hi/lo pairs, 48
                                * significant bits) on a symmetric matrix, as one launch per solve,
                                * and in FP64 when the system leaves that range (above 2^60);
                                * 1: always FP64 (one launch per kernel). */
} spgx_implicit_params;

void spgx_implicit_params_default(spgx_implicit_params *p);
spgx_status spgx_implicit_create(const spgx_scene_desc *scene, const spgx_implicit_params *params,
                                 spgx_implicit **out);
spgx_status spgx_implicit_destroy(spgx_implicit *h);
spgx_status spgx_implicit_step(spgx_implicit *h, spgx_step_stats *stats);
spgx_status spgx_implicit_get_state(spgx_implicit *h, int32_t object, double *x, double *v);
spgx_status spgx_implicit_set_state(spgx_implicit *h, int32_t object, const double *x, const double *v);
spgx_status spgx_implicit_reset(spgx_implicit *h);
/* New dt, substeps, gravity and CG settings for the following steps (BaseSolver::setDt etc.
 * between steps). The robust methods' step size and BDF2's history carry over, as in the
 * reference. method and device must equal the created ones (else SPGX_ERR_INVALID_ARG). */
spgx_status spgx_implicit_set_params(spgx_implicit *h, const spgx_implicit_params *params);
/* The robust methods' current substep (m_currentDt; -1 before the first step). */
spgx_status spgx_implicit_get_step_size(spgx_implicit *h, double *dt);
/* Failure-detection test hook: the next double-float CG solve starts its grid barrier counter
 * where no barrier completes, so that its bounded waits run out (about a second). The step
 * returns SPGX_ERR_TIMEOUT with the positions of that step incomplete; restore a saved state
 * with spgx_implicit_set_state and step on. Nothing faults or hangs. */
spgx_status spgx_implicit_test_stall(spgx_implicit *h);

/* ------------------------------------------------------------------------------------ */
/* XPBD (one projection sweep per substep, xpbd.h:13-15)                                  */

typedef struct spgx_xpbd spgx_xpbd;

typedef struct spgx_xpbd_params {
    double dt;
    int32_t substeps;
    double gravity[3];
    int32_t block_size; /* one launch per phase: threads per block, 0 = default (32) */
    int32_t use_graph;  /* one launch per phase: replay the step as a CUDA graph */
    int32_t device;
    int32_t kernel;     /* 0 = default (1); 1 = one launch per (energy, stencil colour) phase;
                         * 2 = dataflow: every substep of a step in one persistent cooperative
                         * launch, where a chunk of a phase starts once the chunks of earlier
                         * phases that touch its vertices have finished (same result, bit for
                         * bit; slower on the 513x513 cloth, whose chain of about 28 phases per
                         * substep it runs task by task); 3 = synchronised: every substep of a
                         * step in one persistent cooperative launch with a grid barrier after
                         * each phase (same result, bit for bit). A wait of kernel 2 or 3 that
                         * runs out returns SPGX_ERR_TIMEOUT. */
} spgx_xpbd_params;

void spgx_xpbd_params_default(spgx_xpbd_params *p);
spgx_status spgx_xpbd_create(const spgx_scene_desc *scene, const spgx_xpbd_params *params, spgx_xpbd **out);
spgx_status spgx_xpbd_destroy(spgx_xpbd *h);
spgx_status spgx_xpbd_set_params(spgx_xpbd *h, const spgx_xpbd_params *params);
spgx_status spgx_xpbd_step(spgx_xpbd *h, spgx_step_stats *stats);
spgx_status spgx_xpbd_get_state(spgx_xpbd *h, int32_t object, double *x, double *v);
spgx_status spgx_xpbd_set_state(spgx_xpbd *h, int32_t object, const double *x, const double *v);
spgx_status spgx_xpbd_reset(spgx_xpbd *h);
/* Failure-detection test hook (kernels 2 and 3): with kernel 2 it marks one chunk's substep
 * counter as never reached, with kernel 3 it starts the next launch's grid barrier counter
 * where no barrier completes, so that the next step's waits run out their bounded polls
 * (about a second). The step returns SPGX_ERR_TIMEOUT, the counters are reset and the handle
 * keeps working; nothing faults or hangs. */
spgx_status spgx_xpbd_test_stall(spgx_xpbd *h);
/* Stencil colours of one energy (colorStencils, graphColoring.cpp:51-70). */
spgx_status spgx_xpbd_get_stencil_colors(spgx_xpbd *h, int32_t object, int32_t energy, int32_t *colors);

#ifdef __cplusplus
}
#endif

#endif /* SPGX_H */
