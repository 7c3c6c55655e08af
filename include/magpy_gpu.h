/* magpy_gpu.h -- C-ABI of the GB300 sLLG ensemble integrator.
 *
 * Drop-in boundary for magpy's stochastic Landau-Lifshitz-Gilbert path:
 *   magpy.core.simulate (magpy/core.pyx:128-203)
 *     -> simulation::full_dynamics (lib/simulation.cpp:476-624, physical units)
 *     -> simulation::full_dynamics (lib/simulation.cpp:132-429, reduced units, Rng&)
 *     -> integrator::heun / integrator::implicit_midpoint (lib/integrators.cpp:372, 576)
 * and the ensemble fan-out of EnsembleModel.simulate (magpy/model.py:159-208),
 * which the reference runs as one joblib process per member and which this
 * library runs as one batched GPU launch.
 *
 * Conventions (all entry points):
 *   - plain pointers and sizes, int64_t for every count; no exceptions cross
 *     the boundary; every entry point returns MAGPY_SUCCESS (0) or a negative
 *     error code, and magpy_last_error_string() describes the last failure of
 *     the calling thread;
 *   - host pointers unless a descriptor flag says the buffers are device
 *     pointers; results are written into caller-owned buffers;
 *   - three-vectors are stored x,y,z consecutively ([n][3], row-major);
 *   - field shapes use the reference's enum values (include/field.hpp:94-96):
 *     SINE = 0, SQUARE = 1, CONSTANT = 2.
 */
#ifndef MAGPY_GPU_H
#define MAGPY_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ---- */
#define MAGPY_SUCCESS 0
#define MAGPY_ERR_INVALID_ARGUMENT (-1)
#define MAGPY_ERR_CUDA (-2)
#define MAGPY_ERR_NOISE_TOO_SHORT (-3)
#define MAGPY_ERR_UNSUPPORTED (-4)
#define MAGPY_ERR_OUT_OF_MEMORY (-5)
#define MAGPY_ERR_IO (-6)

/* ---- per-member status bits (magpy_ensemble_out.status) ----
 * The reference builds but never throws the implicit solver's error
 * (lib/simulation.cpp:368-369); this library reports it per member. */
#define MAGPY_STATUS_OK 0
#define MAGPY_STATUS_NEWTON_MAXITER 1  /* optimisation::MAX_ITERATIONS_ERR   */
#define MAGPY_STATUS_SINGULAR 2        /* optimisation::LAPACK_ERR (dgesv)    */
#define MAGPY_STATUS_NONFINITE 4       /* a state component became NaN / Inf */
#define MAGPY_STATUS_NOISE_EXHAUSTED 8 /* RngArray out_of_range, lib/rng.cpp:93 */
#define MAGPY_STATUS_WATCHDOG 16       /* a bounded wait on the tensor cores ran out */
#define MAGPY_STATUS_STEP_LIMIT 32     /* the two-state integrator hit its step bound  */

/* ---- field shapes: include/field.hpp:94-96 ---- */
#define MAGPY_FIELD_SINE 0
#define MAGPY_FIELD_SQUARE 1
#define MAGPY_FIELD_CONSTANT 2
/* finite Fourier series of a square wave (field::square_fourier,
 * lib/field.cpp:67-79); two-state model only, as in magpy/core.pyx:245-248 */
#define MAGPY_FIELD_SQUARE_FOURIER 3

/* ---- precision of the state update ---- */
#define MAGPY_PRECISION_FP64 0  /* FP64 throughout, same operation order as the reference */
#define MAGPY_PRECISION_MIXED 1 /* Heun: FP32 evaluation, compensated FP32 state;
                                   implicit midpoint: FP64 state, residual and
                                   convergence test; the dipolar pair sum (partial
                                   sums over 32 sources added in FP64), the
                                   quasi-Jacobian and the 3x3 solve in FP32 */
#define MAGPY_PRECISION_MIXED_TC 2 /* as MIXED, with the dipolar field on the tensor cores
                                      (members sharing one geometry, 2 <= n_particles <= 672;
                                      above 64 particles one thread-block cluster of
                                      ceil(n/42) CTAs per 64 or 32 members) */

/* Ensemble of clusters (EnsembleModel.simulate, magpy/model.py:159-208).
 * Every member has n_particles particles.  Per-particle inputs are either
 * shared by all members (per_member_geometry = 0: arrays of n_particles rows)
 * or given per member (per_member_geometry = 1: member-major arrays of
 * n_members * n_particles rows).  Per-member scalars are either a scalar
 * (pointer NULL) or an array of n_members values.  All inputs are SI units as
 * in Model(...) (magpy/model.py:47-58). */
typedef struct magpy_ensemble_desc {
    int64_t n_members;                      /* E */
    int64_t n_particles;                    /* N */
    int32_t per_member_geometry;
    const double *radius;                   /* [N] or [E][N] (m)            */
    const double *anisotropy;               /* [N] or [E][N] (J/m^3)        */
    const double *anisotropy_axis;          /* [N][3] or [E][N][3]          */
    const double *magnetisation_direction;  /* [N][3] or [E][N][3]          */
    const double *location;                 /* [N][3] or [E][N][3] (m)      */
    double magnetisation;                   /* Ms (A/m)                     */
    double damping;                         /* alpha                        */
    double temperature;                     /* T (K)                        */
    double field_amplitude;                 /* H0 (A/m)                     */
    double field_frequency;                 /* f (Hz)                       */
    int32_t field_shape;                    /* MAGPY_FIELD_*                */
    const double *magnetisation_per_member; /* optional [E]                 */
    const double *damping_per_member;       /* optional [E]                 */
    const double *temperature_per_member;   /* optional [E]                 */
    const double *field_amplitude_per_member; /* optional [E]               */
    const double *field_frequency_per_member; /* optional [E]               */
    int32_t renorm;                         /* magpy/model.py:70 renorm     */
    int32_t interactions;                   /* dipolar coupling on/off      */
    int32_t use_implicit;                   /* 1: implicit midpoint, 0: Heun */
    double eps;                             /* Newton tolerance (implicit_tol) */
    int64_t max_iter;                       /* Newton limit; <= 0 -> 1000 (simulation.cpp:204) */
    double time_step;                       /* dt (s)                       */
    double end_time;                        /* (s)                          */
    int64_t max_samples;                    /* S >= 1 regularly spaced samples */
    const int64_t *seeds;                   /* [E] noise seeds              */
    const double *noise;                    /* optional injected increments,
                                               [E][noise_per_member]; step k of a
                                               member uses entries [(k-1)*3N, k*3N),
                                               particle-major x,y,z (the order of
                                               lib/simulation.cpp:358-359)        */
    int64_t noise_per_member;
    int32_t precision;                      /* MAGPY_PRECISION_*            */
    int32_t buffers_on_device;              /* 1: every pointer in this desc and in
                                               the out struct is a device pointer */
} magpy_ensemble_desc;

typedef struct magpy_ensemble_out {
    double *mx, *my, *mz; /* [S][E*N] sample-major magnetisation (A/m); particle
                             g = e*N + i.  NULL skips the trajectory copy-out.  */
    double *time;         /* [E][S] sample times (s); may be NULL                */
    double *field;        /* [E][S] applied field at the samples (A/m); may be NULL */
    int32_t *status;      /* [E] MAGPY_STATUS_* bits; may be NULL                */
    int64_t *steps;       /* [E] integration steps taken; may be NULL            */
} magpy_ensemble_out;

/* Replaces: the per-member loop of EnsembleModel.simulate (magpy/model.py:202-207)
 * over Model.simulate -> core.simulate -> simulation::full_dynamics
 * (lib/simulation.cpp:476).  One launch for the whole ensemble.  stream may be
 * NULL (legacy default stream). */
int magpy_ensemble_dynamics(const magpy_ensemble_desc *desc, magpy_ensemble_out *out,
                            void *stream);

/* Reusable launch plan: the physical-to-reduced conversion, pair tables,
 * sample schedule and device buffers of one ensemble, built once and run
 * any number of times (no reference counterpart: the reference rebuilds all
 * of it inside every simulation::full_dynamics call, lib/simulation.cpp:476).
 * magpy_plan_create copies everything it needs; the descriptor may be
 * released afterwards.  Trajectories stay on the device, [S][E*N]
 * sample-major, reduced units times the per-member Ms. */
typedef struct magpy_plan magpy_plan;
int magpy_plan_create(const magpy_ensemble_desc *desc, magpy_plan **plan, void *stream);
/* Runs the plan on stream (asynchronous; the caller synchronises). */
int magpy_plan_run(magpy_plan *plan, void *stream);
/* Device pointers of the plan's outputs (any argument may be NULL). */
int magpy_plan_device_outputs(magpy_plan *plan, double **mx, double **my, double **mz,
                              int32_t **status, int64_t **steps);
/* Copies the plan's outputs into out (host or device per the plan's
 * buffers_on_device flag) and synchronises the stream. */
int magpy_plan_copy_out(magpy_plan *plan, magpy_ensemble_out *out, void *stream);
/* Number of members, particles per member, samples, and the largest step
 * count of any member. */
int magpy_plan_shape(const magpy_plan *plan, int64_t *n_members, int64_t *n_particles,
                     int64_t *n_samples, int64_t *max_steps);
/* Launch shape of the warp-packed kernels (clusters of <= 32 particles):
 * warps per CTA and members per warp (0 = as many as fit).  For larger
 * clusters in MAGPY_PRECISION_MIXED whose members share one cluster,
 * members_per_warp = 2 or 4 puts that many members in one CTA.  In
 * MAGPY_PRECISION_MIXED_TC with more than 64 particles (and in its implicit
 * mode), members_per_warp = 32, 40, 48 (Heun only) or 64
 * puts that many members in each thread-block cluster; 0 takes the count
 * with the fewest waves of resident clusters, then the fewest members (a
 * wave's time grows with its clusters' members). */
int magpy_plan_set_launch(magpy_plan *plan, int32_t block_warps, int32_t members_per_warp);
/* No counterpart in the reference.  Bound of the tensor-core kernel's waits
 * for its MMA completions (MAGPY_PRECISION_MIXED_TC), in polls of the
 * mbarrier (each poll may itself block for a short hardware-defined time);
 * default 2^24.  A wait that runs out sets MAGPY_STATUS_WATCHDOG for the
 * CTA's members, stops them (their remaining samples NaN), waits for the
 * MMAs still in flight with the long default bound and frees the tensor
 * memory, so the context stays usable.  A short limit exists to test that
 * path; 0 makes the first wait give up. */
int magpy_plan_set_wait_limit(magpy_plan *plan, int64_t polls);
int magpy_plan_destroy(magpy_plan *plan);

/* Batched ensembles of uneven cluster sizes (no reference counterpart: the
 * reference runs every member as its own joblib process, magpy/model.py:204-207).
 * groups[g] describes one uniform-size ensemble (any precision); the batch
 * builds one plan per group and captures all of them as the parallel
 * branches of one CUDA graph, so magpy_batch_run is a single graph launch.
 * With autotune = 1 the launch configuration of each group is chosen by
 * timing the candidates on a short window of that group's own ensemble:
 * for MAGPY_PRECISION_MIXED / _MIXED_TC groups the kernel (FP32 CUDA-core or
 * tensor-core dipolar field), and for clusters of <= 32 particles the number
 * of warps per CTA (1, 2, 4 or 8) and of members packed per warp (all that
 * fit, a quarter of that, or one).  Choices are cached per process.  For a
 * group on the cluster tensor-core kernel (65 or more particles) the members
 * per thread-block cluster (64, 48 or 32) set how many SMs the group holds
 * beside the others, so that count is chosen by timing the whole graph.
 * A group that chose the CUDA-core kernel alone but fits the single-CTA
 * tensor-core kernel (2..64 particles) is moved to it when that makes the
 * whole graph faster (alone, a kernel spread over every SM wins; beside the
 * other groups, the SM time it takes counts).
 * The branches run at stream priorities ranked by each group's time alone
 * (longest highest; the graph honours its nodes' priorities), so the group
 * on the critical path takes its SMs before the shorter ones fill the rest. */
typedef struct magpy_batch magpy_batch;
int magpy_batch_create(const magpy_ensemble_desc *groups, int64_t n_groups, int32_t autotune,
                       magpy_batch **batch, void *stream);
int magpy_batch_run(magpy_batch *batch, void *stream);
/* The plan of one group (owned by the batch): outputs, statistics. */
int magpy_batch_group_plan(magpy_batch *batch, int64_t group, magpy_plan **plan);
/* The configuration chosen for a group and its tuned time per step (ms; 0
 * when not tuned). */
int magpy_batch_group_choice(const magpy_batch *batch, int64_t group, int32_t *precision,
                             int32_t *block_warps, int32_t *members_per_warp,
                             double *ms_per_step);
int magpy_batch_destroy(magpy_batch *batch);

/* Pathwise adjoint of the stochastic Heun step over fixed noise (no
 * reference counterpart: the reference computes no gradients).  For an
 * ensemble whose members share one geometry and all parameters (Heun, no
 * renormalisation, in-kernel increments, at most 512 particles per member),
 * magpy_adjoint_forward integrates in
 * mixed precision keeping a float-float checkpoint every checkpoint_every
 * steps, and writes the samples into the plan (magpy_adjoint_plan; its
 * ensemble statistics apply).  For an objective J of the ensemble
 * magnetisation samples M_s = (1/E) sum_e sum_q m_z (A/m), given dJ/dM_s,
 * magpy_adjoint_backward recomputes each segment from its checkpoint and
 * sweeps it backward, returning grad_theta = dJ/d(K, alpha, H0) (J/m^3,
 * damping, A/m; K is the mean anisotropy with all K_i scaled together) and
 * the sensitivities to the reduced quantities (dt, sqrt(dt), alpha, happ,
 * dipolar prefactor).  Any direct dependence of J on the field (as in the
 * energy dissipated) is the caller's to add. */
typedef struct magpy_adjoint magpy_adjoint;
int magpy_adjoint_create(const magpy_ensemble_desc *desc, int64_t checkpoint_every,
                         magpy_adjoint **adjoint, void *stream);
int magpy_adjoint_forward(magpy_adjoint *adjoint, void *stream);
int magpy_adjoint_plan(magpy_adjoint *adjoint, magpy_plan **plan);
int magpy_adjoint_backward(magpy_adjoint *adjoint, const double *dJ_dM, double *grad_theta,
                           double *grad_reduced, void *stream);
int magpy_adjoint_destroy(magpy_adjoint *adjoint);

/* Replaces: EnsembleResults.ensemble_magnetisation (magpy/results.py:134-151;
 * cluster sums of magpy/results.py:61-75): the mean over members of the summed
 * particle moments, per sample, FP64 on the device from the plan's last run.
 * direction 0, 1, 2 = x, y, z.  out: [S] host doubles (A/m). */
int magpy_plan_ensemble_magnetisation(magpy_plan *plan, int32_t direction, double *out,
                                      void *stream);

/* Replaces: EnsembleResults.energy_dissipated (magpy/results.py:167-191):
 * -mu0 * integral of H dM (trapezoid rule over the samples whose time lies
 * in [start_time, end_time]; pass NaN for an open bound), FP64, using member
 * 0's sample times and field as the reference does (magpy/results.py:118-119).
 * *out: host double (J/m^3). */
int magpy_plan_energy_dissipated(magpy_plan *plan, double start_time, double end_time,
                                 double *out, void *stream);

/* No counterpart in the reference.  Runs an ensemble like
 * magpy_ensemble_dynamics (mixed-precision Heun kernel only) without
 * allocating any device memory: no cudaMalloc, cudaFree or other allocating
 * routine is called.  It exists for callers that cannot have a library
 * allocate on the device behind their back -- a host framework that manages
 * all GPU memory through its own pool and budget, or a latency-critical loop
 * in which cudaFree (and sometimes cudaMalloc) would wait for the whole
 * device to go idle.
 *   - desc->buffers_on_device must be 1: inputs, optional injected noise and
 *     every output in out are the caller's device buffers;
 *   - the library's own tables (member parameters, per-particle arrays, pair
 *     tables, sample schedule, field table) live in one static device array of
 *     MAGPY_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library
 *     keeps until the process exits; ensembles needing more are rejected with
 *     MAGPY_ERR_INVALID_ARGUMENT and a message giving the bytes needed;
 *   - every call looks up the array's device address (cudaGetSymbolAddress)
 *     with the caller's device and context current; the call reads its
 *     inputs and runs on `stream` and returns after synchronising it, so it
 *     is not meant to be issued while `stream` is being captured;
 *   - out->mx, out->my and out->mz are all set or all NULL;
 *   - all calls share the one array and rewrite every part of it they read,
 *     so calls that overlap on the GPU (other streams, other host threads on
 *     the same device) race with each other: serialise them;
 *   - returns after the results are in the caller's buffers (it synchronises
 *     stream). */
#define MAGPY_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int magpy_ensemble_dynamics_noalloc(const magpy_ensemble_desc *desc, magpy_ensemble_out *out,
                                    void *stream);

/* Replaces: simulation::full_dynamics, physical units (lib/simulation.cpp:476-624;
 * signature include/simulation.hpp:74-94), as bound by magpy/core.pyx:72-93.
 * Outputs in the reference's layout: mx/my/mz [n][max_samples], field/time
 * [max_samples], SI units.  noise: optional injected increments (NULL draws
 * from the counter-based generator keyed by seed).  Returns MAGPY_SUCCESS or
 * an error code; *status receives the MAGPY_STATUS_* bits (may be NULL). */
int magpy_full_dynamics(int64_t n_particles, const double *radius, const double *anisotropy,
                        const double *anisotropy_axis, const double *magnetisation_direction,
                        const double *location, double magnetisation, double damping,
                        double temperature, int32_t renorm, int32_t interactions,
                        int32_t use_implicit, double eps, double time_step, double end_time,
                        int64_t max_samples, int64_t seed, int32_t field_shape,
                        double field_amplitude, double field_frequency, const double *noise,
                        int64_t noise_len, int32_t precision, double *mx, double *my,
                        double *mz, double *field, double *time, int32_t *status);

/* Replaces: simulation::full_dynamics, reduced units with a caller-supplied
 * Rng& (lib/simulation.cpp:132-429; include/simulation.hpp:51-72), driven by
 * an RngArray of injected increments (lib/rng.cpp:67-94).  Inputs are the
 * reduced quantities that overload takes; unit_distances [n][n][3] and
 * reduced_distance_magnitudes [n][n].  Outputs are reduced (no SI
 * conversion), layout as magpy_full_dynamics.  max_iter <= 0 means 1000. */
int magpy_full_dynamics_reduced(
    int64_t n_particles, const double *thermal_field_strengths,
    const double *reduced_anisotropy_constants, const double *reduced_particle_volumes,
    const double *anisotropy_unit_axes, const double *initial_magnetisations,
    const double *interparticle_unit_distances,
    const double *interparticle_reduced_distance_magnitudes, int32_t field_shape,
    double reduced_field_amplitude, double reduced_field_frequency, double average_anisotropy,
    double average_volume, double damping_constant, double saturation_magnetisation,
    double time_step, double end_time, const double *noise, int64_t noise_len, int32_t renorm,
    int32_t interactions, int32_t use_implicit, double eps, int64_t max_iter,
    int64_t max_samples, int32_t precision, double *mx, double *my, double *mz, double *field,
    double *time, int32_t *status, int64_t *steps);

/* Component evaluation on the device (the functions pinned by
 * test/tests.cpp:23-132 and :842): for each of n states, writes
 *   drift [n][3]      llg::drift           (lib/llg.cpp:14-29)
 *   diffusion [n][9]  llg::diffusion       (lib/llg.cpp:92-106)
 *   drift_jac [n][9]  llg::drift_jacobian  (lib/llg.cpp:68-81), with field Jacobian hj [n][9]
 *   diff_jac [n][27]  llg::diffusion_jacobian (lib/llg.cpp:118-158)
 *   anis [n][3]       field::uniaxial_anisotropy (lib/field.cpp:97-105)
 * from m [n][3], h [n][3], axis [n][3], alpha [n], sr [n].  Host buffers.
 * Any output pointer may be NULL. */
int magpy_llg_components(int64_t n, const double *m, const double *h, const double *hj,
                         const double *axis, const double *alpha, const double *sr,
                         double *drift, double *diffusion, double *drift_jac,
                         double *diff_jac, double *anis);

/* Replaces: field::multi_add_dipolar (lib/field.cpp:187-203) for n_members
 * clusters that share one geometry, evaluated as one matrix product on the
 * tensor cores (FP16 hi/lo split, FP32 accumulation, ~22 significant bits).
 * Same inputs as the reference function (saturation magnetisation ms, average
 * anisotropy k_av, reduced volumes [n], unit distances [n][n][3], reduced
 * cubed distances [n][n]); mag [n_members][n][3]; the dipolar field is ADDED
 * to field [n_members][n][3], as the reference adds it.  Host buffers;
 * 2 <= n <= 672 (n > 64: D split over a thread-block cluster of ceil(n/42)
 * CTAs, the same kernel path as the integrator's). */
int magpy_dipolar_field_tc(int64_t n, int64_t n_members, double ms, double k_av,
                           const double *v_reduced, const double *unit_distances,
                           const double *distance_cubes, const double *mag, double *field);

/* The Wiener increments the in-kernel generator produces for one member:
 * out [n_steps][3*n_particles], steps 1..n_steps, particle-major x,y,z.
 * Host buffer.  Lets a caller replay the generator's numbers through any
 * CPU implementation (no reference counterpart: the reference draws
 * std::normal_distribution from std::mt19937_64, include/rng.hpp:36-37). */
int magpy_wiener_increments(int64_t seed, int64_t n_particles, int64_t n_steps, double *out);

/* Number of integration steps full_dynamics takes for a (reduced) time step,
 * end time and sample count (lib/simulation.cpp:342-355), and the minimum
 * injected-noise length per member (steps * 3 * n_particles). */
int magpy_step_count(double time_step, double end_time, int64_t max_samples, int64_t *steps);

/* Two-state master equation of single uniaxial particles (DOModel,
 * magpy/model.py:211-295 -> magpy/core.pyx:205-278 simulate_dom ->
 * simulation::dom_ensemble_dynamics, lib/simulation.cpp:659-767): the
 * probabilities of the up and down states under Neel-Brown rates
 * (lib/dom.cpp:33-59), integrated by adaptive Cash-Karp RK45
 * (lib/integrators.cpp:152-251) with the reference's step control
 * (tolerance = time_step, first step 0.01 time_step, steps at most
 * end_time / 1000) and first-order-hold sampling.  A batch of independent
 * particles runs in one launch, one thread per particle, in FP64.
 * Per-particle inputs are arrays of n_particles values (SI units, as
 * simulate_dom takes them; volume = 4/3 pi r^3 as DOModel computes it). */
typedef struct magpy_dom_desc {
    int64_t n_particles;                 /* E                                   */
    const double *volume;                /* [E] m^3                             */
    const double *anisotropy;            /* [E] J/m^3                           */
    const double *temperature;           /* [E] K                               */
    const double *magnetisation;         /* [E] A/m                             */
    const double *damping;               /* [E]                                 */
    const double *initial_probabilities; /* [E][2] (down, up as DOModel names them) */
    const double *field_amplitude;       /* [E] A/m, along the anisotropy axis   */
    const double *field_frequency;       /* [E] Hz                              */
    int32_t field_shape;                 /* MAGPY_FIELD_*                       */
    int64_t field_n_components;          /* MAGPY_FIELD_SQUARE_FOURIER terms    */
    double time_step;                    /* s: integrator tolerance and first step */
    double end_time;                     /* s                                   */
    int64_t max_samples;                 /* >= 1, or -1: int(end/dt) + 1 samples */
    int64_t max_steps;                   /* per particle; 0: 100,000,000        */
} magpy_dom_desc;
/* Outputs (host, caller-owned) [E][n_samples]: mz = p0 - p1 (reduced), field
 * (A/m), time (s); status [E] (0, MAGPY_STATUS_NONFINITE or
 * MAGPY_STATUS_STEP_LIMIT: the particle stopped and its remaining samples
 * are NaN; the reference loops forever there), steps [E] (any may be NULL). */
int magpy_dom_dynamics(const magpy_dom_desc *desc, double *mz, double *field, double *time,
                       int32_t *status, int64_t *steps, void *stream);

/* Seeded cluster geometries for batched ensembles (the reference draws them
 * on the host with numpy's global generator: magpy/initial_conditions.py:4-37
 * uniform_random_axes, magpy/geometry/coordinates.py chain_coordinates).
 * Per member, from a counter-based generator keyed by seeds[e]: radii
 * log-normal (median_radius * exp(sigma_log_radius * z)); easy axes uniform
 * on the sphere; initial moments along the axes (moments = 0) or uniform
 * (moments = 1); locations either a random packing in a sphere sized for the
 * packing fraction of exclusion spheres of radius spacing * mean(r) / 2, each
 * pair at least spacing * (r_i + r_j) / 2 apart (layout = 0), or a chain
 * along z with pitch spacing * mean(r) (layout = 1).  Outputs are member-major
 * ([E][N] radius, [E][N][3] axes, moments, locations), the per-member geometry
 * layout of magpy_ensemble_desc; status [E] is 1 where the packing found no
 * place for a particle within max_rounds rounds of 256 candidates (its
 * remaining locations are NaN).  Deterministic for given seeds. */
#define MAGPY_LAYOUT_SPHERE 0
#define MAGPY_LAYOUT_CHAIN 1
typedef struct magpy_geometry_desc {
    int64_t n_members;        /* E                                           */
    int64_t n_particles;      /* N, 1..1024                                  */
    int32_t layout;           /* MAGPY_LAYOUT_*                              */
    int32_t moments;          /* 0: along the easy axes, 1: uniform          */
    double median_radius;     /* m                                           */
    double sigma_log_radius;  /* >= 0                                        */
    double spacing;           /* minimum centre distance / mean pair radius  */
    double packing_fraction;  /* (0, 0.6]                                    */
    int64_t max_rounds;       /* per particle; 0: 4096                       */
    const int64_t *seeds;     /* [E]                                         */
    int32_t buffers_on_device;  /* 1: seeds and outputs are device pointers  */
} magpy_geometry_desc;
int magpy_generate_clusters(const magpy_geometry_desc *desc, double *radius,
                            double *anisotropy_axis, double *magnetisation_direction,
                            double *location, int32_t *status, void *stream);

/* Binary results: the format of simulation::save_results
 * (lib/simulation.cpp:38-63, include/io.hpp:13-27): for a prefix 'foo' the
 * files foo.mx, foo.my, foo.mz, foo.field and foo.time, each n_samples raw
 * native-endian doubles.  Where the reference throws std::runtime_error on a
 * failed write this returns MAGPY_ERR_IO. */
int magpy_save_results(const char *prefix, const double *mx, const double *my, const double *mz,
                       const double *field, const double *time, int64_t n_samples);
/* The same files for every particle i of members [member_begin, member_end)
 * of a plan, written straight from the plan's device trajectories (one
 * device-to-host copy per sample block), named '<prefix>_<e>_<i>.mx' etc. */
int magpy_plan_save_results(magpy_plan *plan, const char *prefix, int64_t member_begin,
                            int64_t member_end, void *stream);

/* Description of the last error on the calling thread (never NULL). */
const char *magpy_last_error_string(void);

/* Library version string. */
const char *magpy_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MAGPY_GPU_H */
