/*
 * nbg.h - C ABI of the GB300 force-and-integration engine for the
 * NBodySimulator.jl API (libnbg.so, CUDA sm_103a).
 *
 * The engine is a drop-in for the ODE right-hand side that NBodySimulator.jl
 * builds in src/nbody_to_ode.jl, plus a fused velocity-Verlet / Euler-Maruyama
 * loop that keeps the state resident on one GPU.
 *
 * Conventions shared by every entry point
 *  - Arrays of vectors use the reference's layout: a column-major 3 x n Float64
 *    matrix, i.e. x,y,z of atom i at [3i], [3i+1], [3i+2]
 *    (src/nbody_to_ode.jl:1-20, the u0/v0 built by
 *    gather_bodies_initial_coordinates).
 *  - With the Nose-Hoover thermostat the state has one extra column (3 x (n+1)),
 *    the thermostat variable zeta is u[3n] and its rate is v[3n]
 *    (src/nbody_to_ode.jl:6-8, :419 "gamma_ind = 3n + 1").
 *  - Water systems order atoms O,H1,H2 per molecule (src/nbody_to_ode.jl:46).
 *  - Pointers named host_* or documented as host buffers are ordinary host
 *    memory owned by the caller and never retained after the call returns.
 *  - Every function returns an int status: NBG_OK (0) or a negative nbg_status;
 *    nbg_last_error(ctx) returns a message for the last failure on ctx.
 *  - A context is not re-entrant: call it from one host thread at a time.
 *    Distinct contexts may be used concurrently; each owns its CUDA stream.
 *  - The library has no CPU fallback. A system it does not implement returns
 *    NBG_ERR_UNSUPPORTED so that the caller can keep the problem on its own
 *    CPU path.
 */
#ifndef NBG_H
#define NBG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBG_ABI_VERSION 1

#if defined(__GNUC__)
#define NBG_API __attribute__((visibility("default")))
#else
#define NBG_API
#endif

typedef enum nbg_status {
    NBG_OK = 0,
    NBG_ERR_ARG = -1,          /* invalid argument or descriptor field */
    NBG_ERR_CUDA = -2,         /* a CUDA runtime call failed */
    NBG_ERR_CAPACITY = -3,     /* cell / neighbour capacity could not be grown */
    NBG_ERR_NONFINITE = -4,    /* NaN or Inf in accelerations or state */
    NBG_ERR_TIMEOUT = -5,      /* a bounded device-side wait gave up */
    NBG_ERR_UNSUPPORTED = -6,  /* system/option not implemented on the GPU */
    NBG_ERR_RANGE = -7,        /* minimum-image loop exceeded its iteration cap */
    NBG_ERR_NOMEM = -8,        /* device allocation failed */
    NBG_ERR_INDEX = -9         /* a neighbour or cell index out of range (checked by debug builds only) */
} nbg_status;

/* Boundary conditions (src/boundary_conditions.jl). */
typedef enum nbg_bc {
    NBG_BC_INFINITE = 0, /* InfiniteBox: plain difference, boundary_conditions.jl:167-172 */
    NBG_BC_CUBIC = 1,    /* CubicPeriodicBoundaryConditions(L): minimum image by
                            repeated +-L, boundary_conditions.jl:138-165 */
    NBG_BC_PERIODIC = 2  /* PeriodicBoundaryConditions([lo,hi] x 3): the reference
                            maps each difference into [lo,hi), :111-136 */
} nbg_bc;

/* System families (src/nbody_system.jl). */
typedef enum nbg_system_kind {
    NBG_SYSTEM_POTENTIAL = 0, /* PotentialNBodySystem / GravitationalSystem /
                                 ChargedParticles, nbody_system.jl:32-150 */
    NBG_SYSTEM_WATER = 1      /* WaterSPCFw, nbody_system.jl:182-191 */
} nbg_system_kind;

/* Potentials of a PotentialNBodySystem (bitmask). */
typedef enum nbg_potential {
    NBG_POT_LJ = 1,   /* LennardJonesParameters, basic_potentials.jl:240-272 */
    NBG_POT_EL = 2,   /* ElectrostaticParameters, basic_potentials.jl:274-304 */
    NBG_POT_GRAV = 4, /* GravitationalParameters, basic_potentials.jl:306-331 */
    NBG_POT_MAG = 8   /* MagnetostaticParameters, basic_potentials.jl:333-365 */
} nbg_potential;

/* Thermostats (src/thermostats.jl). */
typedef enum nbg_thermostat {
    NBG_THERMO_NULL = 0,
    NBG_THERMO_ANDERSEN = 1,   /* nbody_simulation_result.jl:504-540 */
    NBG_THERMO_BERENDSEN = 2,  /* thermostats.jl:76-83 */
    NBG_THERMO_NOSEHOOVER = 3, /* thermostats.jl:121-128 */
    NBG_THERMO_LANGEVIN = 4    /* nbody_to_ode.jl:567-680 (SDE, Euler-Maruyama) */
} nbg_thermostat;

/*
 * Everything the reference's marshalling functions (obtain_data_for_*,
 * nbody_to_ode.jl:263-433, get_masses nbody_simulation_result.jl:121-139)
 * extract from an NBodySimulation, as plain values.
 */
typedef struct nbg_system_desc {
    int32_t abi_version;  /* must be NBG_ABI_VERSION */
    int32_t kind;         /* nbg_system_kind */
    int64_t n;            /* atoms (columns), excluding the Nose-Hoover column */
    const double* mass;   /* [n] masses (get_masses order) */
    const double* charge; /* [n] charges; required with NBG_POT_EL or WATER */
    const double* dipole; /* [3n] magnetic moments; required with NBG_POT_MAG */
    uint32_t potentials;  /* nbg_potential bitmask (ignored for WATER) */
    /* LennardJonesParameters(eps, sigma, R); R may be +Inf. For WATER only the
       O atoms take part (obtain_data_for_lennard_jones_interaction, :302-314). */
    double lj_epsilon, lj_sigma, lj_cutoff;
    /* ElectrostaticParameters(k, R); R may be +Inf. eps_rf selects reaction
       field: 1.0 reproduces the reference's truncated Coulomb exactly. */
    double el_k, el_cutoff, el_eps_rf;
    double grav_G;        /* GravitationalParameters(G) */
    double mag_mu_4pi;    /* MagnetostaticParameters(mu/4pi) */
    /* SPCFwParameters(rOH, aHOH, kb, ka) for WATER */
    double water_rOH, water_aHOH, water_kb, water_ka;
    int32_t bc;           /* nbg_bc */
    double box[6];        /* CUBIC: box[0] = L. PERIODIC: lo_x,hi_x,lo_y,hi_y,lo_z,hi_z */
    int32_t thermostat;   /* nbg_thermostat */
    double thermo_T;      /* target temperature */
    double thermo_param;  /* tau (Berendsen, Nose-Hoover), nu (Andersen), gamma (Langevin) */
    double kb;            /* Boltzmann constant of the simulation (nbody_simulation.jl:7) */
    uint64_t seed;        /* Philox key for Andersen / Langevin noise */
    /* Verlet list: list radius = cutoff + skin; rebuilt every rebuild_every
       steps or as soon as an atom moved more than skin/2 since the last build. */
    double skin;
    int32_t rebuild_every;
    int32_t flags;        /* NBG_FLAG_* */
} nbg_system_desc;

/* Force the all-pairs path even where a cell/Verlet list applies. */
#define NBG_FLAG_ALL_PAIRS 1
/* Gravity: plain FP32 position differences (no hi/lo compensation). */
#define NBG_FLAG_GRAV_PLAIN 2
/* Langevin thermostat integrated by BAOAB (velocity-Verlet splitting with an
   exact Ornstein-Uhlenbeck step, Leimkuhler & Matthews 2013) instead of the
   reference's Euler-Maruyama; stable at the step sizes of velocity Verlet. */
#define NBG_FLAG_LANGEVIN_BAOAB 4

typedef struct nbg_ctx nbg_ctx;

/* Energies with the reference's definitions (nbody_simulation_result.jl:
   209-212 kinetic, 293-319 LJ with r^2 clamped to R^2, 321-351 electrostatic,
   353-372 bonds, 374-397 angles). gravity is the project's own
   -G sum_{i<j} m_i m_j / r_ij (the reference defines none). */
typedef struct nbg_energies {
    double kinetic, lennard_jones, electrostatic, bonds, angles, gravity;
    double potential, total;
    double temperature; /* md_temperature with the system's n and Nc (thermostats.jl:87-91) */
} nbg_energies;

typedef struct nbg_run_stats {
    int64_t steps;            /* steps taken */
    int64_t list_builds;      /* Verlet-list rebuilds */
    int64_t kernel_launches;  /* CUDA kernels launched by the call */
    double device_ms;         /* device time of the call (CUDA events) */
} nbg_run_stats;

/* Library identity. */
NBG_API const char* nbg_version(void);
NBG_API int nbg_abi_version(void);

/* Build a context for one system on CUDA device `device`. The descriptor and
   the arrays it points to are copied; the caller may free them afterwards.
   Replaces the closure construction of SciMLBase.SecondOrderODEProblem(sim)
   (src/nbody_to_ode.jl:460-536). */
NBG_API int nbg_create(const nbg_system_desc* desc, int device, nbg_ctx** out);

/* A batch of independent replicas (uneven sizes, own box, temperature and
   seed) advanced together in one launch sequence. All replicas must share
   kind, potentials, thermostat kind and cutoffs. */
NBG_API int nbg_create_batch(const nbg_system_desc* descs, int32_t n_replicas, int device,
                     nbg_ctx** out);

NBG_API void nbg_destroy(nbg_ctx* ctx);
NBG_API const char* nbg_last_error(const nbg_ctx* ctx);

/* Run the context's work on a caller-provided cudaStream_t (NULL restores the
   context's own stream). */
NBG_API int nbg_set_stream(nbg_ctx* ctx, void* cuda_stream);

/* Number of CUDA kernels this context has launched so far. */
NBG_API int64_t nbg_kernel_launches(const nbg_ctx* ctx);

/*
 * The right-hand side soode_system!(dv, v, u, p, t) of
 * SciMLBase.SecondOrderODEProblem(sim) (src/nbody_to_ode.jl:474-488 and
 * :502-532 for water), on host buffers. dv, v, u hold 3 x n doubles
 * (3 x (n+1) with Nose-Hoover). As in the reference, the Nose-Hoover term
 * writes the thermostat rate into v[3n] (thermostats.jl:126): v is the only
 * input that is modified. Replaces one call of the closure SciML's solvers
 * make per stage. Page-locked u and dv (cudaHostAlloc / cudaHostRegister
 * memory, mapped) are read and written by the device in place on the
 * small-system path; other buffers go through the context's pinned staging.
 */
NBG_API int nbg_accel(nbg_ctx* ctx, double* dv, double* v, const double* u, double t);

/* Copy a state (3 x n doubles each, 3 x (n+1) with Nose-Hoover) to and from
   the device-resident state. For batches the replicas' columns are
   concatenated in replica order. A state set here restarts every schedule
   that depends on past steps (list builds, the gravity sort), so runs from
   the same state give the same bits. */
NBG_API int nbg_set_state(nbg_ctx* ctx, const double* u, const double* v);
NBG_API int nbg_get_state(nbg_ctx* ctx, double* u, double* v);

/* The context's step counter: steps taken on the resident state since the
   context was created or the counter was last set. It keys the Philox noise
   of the Andersen and Langevin thermostats (counter (atom, step)), and it
   keeps running across nbg_advance / nbg_run calls, so that every run draws
   fresh noise, as each run_simulation call of the reference does
   (nbody_simulation_result.jl:504-540, nbody_to_ode.jl:567-598). A
   checkpoint is nbg_get_state + nbg_get_step; nbg_set_state + nbg_set_step
   resume it. Resuming at a multiple of rebuild_every (where the uninterrupted
   run rebuilds its lists too) continues the run bit for bit. */
NBG_API int nbg_get_step(nbg_ctx* ctx, int64_t* step);
NBG_API int nbg_set_step(nbg_ctx* ctx, int64_t step);

/* Accelerations of the resident state into the resident acceleration buffer
   (no host traffic); the unit the force roofline is measured on. */
NBG_API int nbg_compute_forces(nbg_ctx* ctx);
NBG_API int nbg_get_accel(nbg_ctx* ctx, double* dv);

/*
 * Advance the resident state nsteps with velocity Verlet at step dt
 * (run_simulation(sim, VelocityVerlet(), dt=dt), nbody_simulation_result.jl:
 * 468-487), applying the thermostat. With NBG_THERMO_LANGEVIN it advances the
 * first-order SDE with Euler-Maruyama instead (calculate_simulation_sde,
 * :489-492). No host traffic; asynchronous on the context's stream: the call
 * returns once its steps are queued, without waiting for them. Steps run in
 * chunks of 512 whose status word is read before the next chunk; the last
 * chunk's status is read by the next call on the context (or nbg_sync), which
 * returns that chunk's error, or, after a list overflow, undoes the chunk,
 * grows the lists and runs it again before doing its own work.
 */
NBG_API int nbg_advance(nbg_ctx* ctx, double dt, int64_t nsteps);

/* Wait for the context's queued work and return the status of its last
   nbg_advance (see there). */
NBG_API int nbg_sync(nbg_ctx* ctx);

/*
 * Host-buffer driver: upload u, v; take nsteps steps; every save_every steps
 * (and at the end) copy the state into traj_u / traj_v (each of
 * (nsteps/save_every + 1) x 3 x n doubles, frame 0 = the initial state; either
 * may be NULL); download the final state into u, v. save_every <= 0 saves only
 * the first and last frames. The steps write the frames into a device buffer
 * (up to 1 GiB of them at a time), copied out once per such segment: saving
 * every step costs about one small kernel per step, and no host round trip.
 */
NBG_API int nbg_run(nbg_ctx* ctx, double* u, double* v, double dt, int64_t nsteps,
            int64_t save_every, double* traj_u, double* traj_v, nbg_run_stats* stats);

/* Energies and temperature of (u, v) (host buffers). */
NBG_API int nbg_energy(nbg_ctx* ctx, const double* u, const double* v, nbg_energies* out);

/*
 * The pair set the force kernels used for (u): every ordered pair (i, j),
 * j != i, with r^2 < R^2 in the reference's Float64 arithmetic
 * (basic_potentials.jl:253-258 for NBG_POT_LJ, :288-292 for NBG_POT_EL).
 * Pairs are written as (i, j) int32 couples sorted by i then j; *count gets
 * the total even when it exceeds cap.
 */
NBG_API int nbg_pair_list(nbg_ctx* ctx, const double* u, int32_t which, int32_t* pairs,
                  int64_t cap, int64_t* count);

/*
 * Profiling support (no reference counterpart). With profiling on, CUDA
 * events bracket every launch of the context's dominant force kernel
 * (gravity all-pairs, Verlet-list pair forces or the all-pairs kernel; for a
 * context on the cluster step loop, the whole multi-step cluster launch);
 * nbg_force_kernel_time returns their summed duration and count since the
 * last reset and resets them.
 */
NBG_API int nbg_set_profiling(nbg_ctx* ctx, int on);
NBG_API int nbg_force_kernel_time(nbg_ctx* ctx, double* total_ms, int64_t* launches);

/*
 * Small systems (no reference counterpart): one potential system under cubic
 * boundaries without thermostat, up to 2048 atoms, runs velocity Verlet as one
 * persistent launch per chunk of steps over a thread-block cluster (the
 * positions shared in distributed shared memory, one cluster barrier per
 * step) instead of a CUDA graph of kernels. Returns 1 and the cluster's CTAs
 * and lanes per atom when the context uses it, 0 otherwise (either pointer
 * may be NULL). The environment variable NBG_NO_CLUSTER, read at creation,
 * keeps such a system on the graph step loop.
 */
NBG_API int nbg_cluster_shape(nbg_ctx* ctx, int32_t* ctas, int32_t* lanes);

/* The launch floor of that cluster shape (measurement): an empty kernel with
 * the same CTAs, threads, shared memory and cluster, which passes one
 * cluster barrier, timed with CUDA events on the context's stream: 200
 * launches back to back (*us_per_launch) and 200 one at a time with the host
 * waiting for each (*us_single). NBG_ERR_UNSUPPORTED off the cluster path. */
NBG_API int nbg_cluster_launch_floor(nbg_ctx* ctx, double* us_single, double* us_per_launch);

/*
 * All-pairs gravity accelerations that allocate no device memory. It has no
 * counterpart in the reference: it is for callers that cannot let a library
 * allocate (a host integrator calling the right-hand side at a high rate,
 * where cudaMalloc/cudaFree would synchronise the device, or a process whose
 * device memory is owned by another allocator). x (3 x n, the reference's
 * column-major layout), mass (n) and a (3 x n) are device buffers of the
 * current device; a_i = -G sum_{j != i} m_j (x_i - x_j) / |x_i - x_j|^3.
 * The scratch is a fixed device array of the library, held by every GPU that
 * loads it until the process exits, and sized for n <= 16384 bodies; larger n
 * returns NBG_ERR_CAPACITY. The first call on a device looks up that array's
 * device address, so make the first call before any stream capture. All calls
 * share the array: calls that overlap on the GPU (other streams or threads)
 * race and must be serialised by the caller. Synchronous on `stream` (a
 * cudaStream_t, NULL for the default stream). Errors are described by
 * nbg_last_error(NULL). The looked-up address is kept for the life of the
 * process: the entry point assumes each device's primary context (the CUDA
 * runtime's) throughout, so do not call it after cudaDeviceReset or from a
 * non-primary driver context on the same device.
 */
NBG_API int nbg_gravity_accel_noalloc(const double* x, const double* mass, int64_t n, double G, double* a,
                                      void* stream);

/* The Verlet-list force kernel's current form (no reference counterpart):
   *lanes = lanes per atom (1: a thread per atom), *fixed_point = 1 when the
   fixed-point kernel with its lists staged into shared memory by the tensor
   memory accelerator runs, 0 for the split-position kernels. Either pointer
   may be NULL. NBG_ERR_UNSUPPORTED off the list path. */
NBG_API int nbg_force_form(nbg_ctx* ctx, int32_t* lanes, int32_t* fixed_point);

/* Replica ensembles (no reference counterpart: the reference runs one
   simulation per call). A batch of potential systems under cubic boundaries
   with the Langevin thermostat integrated by BAOAB, or without thermostat,
   and replicas of at most 9216 atoms, advances as one persistent launch per
   chunk of steps: a CTA per replica (largest first) runs the replica's whole
   step loop (integration, in-launch Verlet-list rebuilds from a
   shared-memory cell sort, pair forces gathering neighbours from shared
   memory), synchronising only its own threads. nbg_ensemble_form returns 1
   and the form (lanes per atom, threads per replica, cells: 1 = of at least
   the list radius over 3^3 cells, 2 = of half of it over 5^3) when the batch
   runs it, 0 otherwise (any pointer may be NULL). NBG_NO_ENSEMBLE_LOOP at
   creation keeps a batch on the step graphs. */
NBG_API int nbg_ensemble_form(nbg_ctx* ctx, int32_t* lanes, int32_t* threads, int32_t* cells);
/* Autotuner of the loop: forms f = 0..11 (lanes 4 or 8 = f / 6; threads 512,
   768, 1024 = (f / 2) % 3; cells 1 or 2 = 1 + f % 2) and f = 12, the batch's
   per-step kernels in CUDA graphs, each run `steps` steps from the resident
   state with a full list build at the first, timed (ms per step into ms[13],
   may be NULL); the state and the step counter are restored after each, and
   the fastest form is kept and written to form[3] (lanes, threads, cells),
   or {0, 0, 0} when the step graphs win (the batch then leaves the loop
   until it is tuned again). */
NBG_API int nbg_ensemble_tune(nbg_ctx* ctx, int32_t steps, int32_t* form, double* ms);

/* Measured FP32 FMA throughput of a device in TFLOP/s (an FMA counts 2):
   the roofline denominator of the FP32-bound gravity kernel. */
NBG_API int nbg_probe_fp32_peak(int device, double* tflops);

/* ------------------------------------------------------------------------
 * Learned short-range model and r-RESPA (engine extension: the reference has
 * no learned model and no multiple-time-step integrator, so none of these
 * replaces a reference interface). One SPC/Fw water system on the
 * Verlet-list path in a cubic box.
 *
 * Model, per species (0 = O, 1 = H), on 64 invariant descriptors of each
 * atom's environment within 0.6 nm (24 radial Gaussians per neighbour
 * species and 16 angular invariants): an MLP 64 -> 128 -> 128 -> 1 (tanh)
 * giving the atom's short-range energy; inference and its backward to the
 * forces run in BF16 on the tensor cores. Parameters of one species are
 * NBG_ML_NPARAM floats in this order: W1 [64][128], b1 [128], W2 [128][128],
 * b2 [128], w3 [128], b3, then the normalisation mean_D [64], sd_D [64],
 * mean_E, sd_E. Training target: E_i = 1/2 sum_j phi(r_ij) S(r_ij) over atoms
 * of other molecules, phi = LJ (O-O) + k q_i q_j erfc(4 r / nm) / r (the
 * real-space part of an Ewald-type split), S = 1 below 0.45 nm with a C2
 * switch to 0 at 0.6 nm.
 * ------------------------------------------------------------------------ */
#define NBG_ML_NPARAM 25091
#define NBG_ML_NTRAIN 24961 /* leading trainable parameters of a species */

typedef struct nbg_respa_stats {
    int64_t outer_mts;       /* outer steps integrated by r-RESPA */
    int64_t outer_fallback;  /* outer steps re-integrated by velocity Verlet (judge over threshold) */
    int64_t judged;          /* outer steps whose judge value entered the mean */
    double judge_mean;       /* mean over r-RESPA outer steps of ||F_ml - F_sr|| / ||F_sr|| */
    double judge_max;
    double judge_last;       /* largest judge value of the last chunk */
} nbg_respa_stats;

NBG_API int nbg_ml_param_count(void);
/* Allocate the model (normalisation mean 0, sd 1; weights 0) and its buffers. */
NBG_API int nbg_ml_enable(nbg_ctx* ctx);
NBG_API int nbg_ml_set_params(nbg_ctx* ctx, int32_t species, const float* theta);
NBG_API int nbg_ml_get_params(nbg_ctx* ctx, int32_t species, float* theta);
/* Random weights (W1 ~ N(0, (w1_scale/8)^2), W2, w3 ~ N(0, 1/128), biases 0)
   for both species; the normalisation is kept. Resets the Adam state. */
NBG_API int nbg_ml_init_params(nbg_ctx* ctx, uint64_t seed, double w1_scale);
/* At positions u (3n): descriptors [n][64], raw or standardised by the model's mean/sd. */
NBG_API int nbg_ml_descriptors(nbg_ctx* ctx, const double* u, int32_t standardised, float* desc);
/* At positions u: learned per-atom energies [n] and forces [3n] (either may be NULL). */
NBG_API int nbg_ml_eval(nbg_ctx* ctx, const double* u, float* energies, double* forces);
/* At positions u: exact short-range per-atom energies [n] and forces [3n] (FP32). */
NBG_API int nbg_ml_labels(nbg_ctx* ctx, const double* u, float* energies, float* forces);
/* Training set on the device with room for `frames` configurations (empties it). */
NBG_API int nbg_ml_reserve(nbg_ctx* ctx, int64_t frames);
/* Append the resident state's raw descriptors and labels; rows[2] = rows per species. */
NBG_API int nbg_ml_collect(nbg_ctx* ctx, int64_t* rows);
NBG_API int nbg_ml_rows(nbg_ctx* ctx, int64_t* rows);
/* Set both species' mean_D, sd_D, mean_E, sd_E from the training set. */
NBG_API int nbg_ml_normalize(nbg_ctx* ctx);
/* Adam on the mean squared error of standardised energies over random batches
   (per species `steps` steps, learning rate lr with a cosine decay over the
   call). loss[2]: mean loss of the last min(steps, 100) batches. */
NBG_API int nbg_ml_train(nbg_ctx* ctx, int64_t steps, int32_t batch, double lr, uint64_t seed, double* loss);
/* Loss and gradient (NBG_ML_NTRAIN floats) of one species' parameters on a
   batch of standardised inputs x [B][64] and standardised targets y [B]. */
NBG_API int nbg_ml_batch_gradient(nbg_ctx* ctx, int32_t species, const float* x, const float* y, int32_t B,
                                  float* grad, double* loss);
/* Advance the resident state by `outer` r-RESPA steps of inner * dt: the fast
   force (bonded + learned) every dt, the slow force (exact non-bonded minus
   learned) every inner * dt (Tuckerman, Berne & Martyna 1992). Every outer
   step the exact short-range force judges the learned one; a chunk of outer
   steps whose largest relative RMS error exceeds `threshold` (> 0) is undone
   and integrated again by velocity Verlet at dt with the exact force.
   Thermostat: none or Berendsen (applied with the slow kicks). With
   NBG_RESPA_EXACT_SPLIT the fast force uses the exact short-range force in
   place of the learned one (the classical split the model stands in for). */
#define NBG_RESPA_EXACT_SPLIT 1
/* With NBG_RESPA_NO_FAST_FORCE the fast force is the bonded terms alone and
   the slow force all of the non-bonded one: the integrator's own cost per
   outer step, an upper bound of the speed of any fast non-bonded model in
   this scheme (the dynamics is not meant to be accurate). */
#define NBG_RESPA_NO_FAST_FORCE 2
NBG_API int nbg_respa_run(nbg_ctx* ctx, double dt, int32_t inner, int64_t outer, double threshold, int32_t flags,
                          nbg_respa_stats* stats);

/* Autotuner of the Verlet-list force kernel: times every lanes-per-atom form
   (index 0: a thread per atom; 1..4: 4, 8, 16, 32 lanes per atom) over `reps`
   launches on the resident positions, writes the times (ms, may be NULL) to
   ms[5] and keeps the fastest form for the context (*lpa: 1, 4, 8, 16 or 32).
   Results do not depend on the choice beyond FP32 summation order. */
NBG_API int nbg_autotune(nbg_ctx* ctx, int32_t reps, int32_t* lpa, double* ms);

/* Change a replica's thermostat target temperature (the reference builds a
   new simulation with another thermostat; this keeps the context). */
NBG_API int nbg_set_thermostat_target(nbg_ctx* ctx, int32_t replica, double T);
/* Device time (ms, averaged over `reps` runs on the resident positions) of
   the learned-force kernels: [0] short list, [1] descriptors, [2] MLP
   forward and backward (BF16 tensor cores), [3] force scatter. */
NBG_API int nbg_ml_kernel_times(nbg_ctx* ctx, int32_t reps, double* ms);

/* Pair histogram of the radial distribution function (replaces the loops of
   rdf, nbody_simulation_result.jl:664-709; the normalisation to g(r) stays
   with the caller). frames: nframes x ncols x 3 positions (the reference's
   3 x N columns per saved time), idx: the nidx participant columns (host
   memory; the reference's LJ participants), cubic boundaries of side L.
   For every frame and every unordered pair of participants with minimum-image
   distance r, r^2 < (L/2)^2 and bin = ceil(r / (L / maxbin)) in 2..maxbin,
   hist[bin - 1] += 2: the reference's counts exactly (FP32 screening, FP64
   arithmetic of the reference for every pair near a bin edge). frames and
   hist may be host or device memory of `device` (device frames are read on
   the legacy default stream); 1 <= maxbin <= 16384.
   NBG_ERR_NONFINITE for a non-finite coordinate, NBG_ERR_RANGE for one more
   than 16384 boxes out. Context-free; calls are serialised. */
NBG_API int nbg_rdf_histogram(const double* frames, int64_t nframes, int64_t ncols, const int32_t* idx,
                              int64_t nidx, double L, int32_t maxbin, int device, double* hist);
/* Device time (ms, CUDA events on the launching stream) of the last
   nbg_rdf_histogram call's kernels: [0] position split, [1] pair histogram.
   For host frames, which go up in chunks with each chunk's kernels running
   behind its copy, [0] is 0 and [1] spans the whole pipeline. */
NBG_API int nbg_rdf_kernel_times(double* ms);

#ifdef __cplusplus
}
#endif

#endif /* NBG_H */
