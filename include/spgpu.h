/*
 * spgpu.h — C ABI of the GB300 SpatialPy simulation engine (libspgpu.so).
 *
 * The reference engine has no in-process ABI: spatialpy.Solver generates a C++
 * model file, builds `ssa_sdpd.exe` with SCons and runs one process per
 * trajectory (spatialpy/solvers/solver.py:443-507 compile, :510-607 run), which
 * writes `outputN.vtk` files (src/output.cpp:104-229).  This header replaces
 * that process + file boundary with plain C calls over caller-owned arrays:
 *
 *   sp_create    replaces Solver.compile() + the generated model file
 *                (solver.py:100-158 __create_propensity_file, :208-288
 *                __get_input_constants, :375-419 __get_system_config) and the
 *                engine set-up in propensity_file_template.cpp:101-142
 *                (init_all_particles, initialize_rdme).
 *   sp_run       replaces the per-trajectory subprocess loop of Solver.run
 *                (solver.py:547-605) and the engine main loop run_simulation
 *                (src/simulate_threads.cpp:171-312), including the NSM event
 *                loop (src/simulate_rdme.cpp:211-472) and the SDPD particle
 *                step (src/simulate.cpp:56-173, src/model.cpp:39-329).
 *   sp_status    replaces the engine's exit codes / printf diagnostics on
 *                negative counts and NaN state (simulate_rdme.cpp:288-294,
 *                395-400; particle.cpp:88-126): errors are reported per
 *                trajectory instead of exit(1).
 *   sp_last_error  replaces the stdout text Solver.run streams back
 *                (solver.py:32-43) when it raises SimulationError.
 *   sp_destroy   replaces Solver.__del__ removing build_dir (solver.py:90-98).
 *
 * All arrays are caller-owned.  Every entry point returns SP_OK (0) or a
 * negative SP_E* code; sp_last_error() then describes the failure.  No
 * callbacks are made into the caller.  A handle is used by one host thread at a
 * time; separate handles are independent.
 */
#ifndef SPGPU_H
#define SPGPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SP_ABI_VERSION 4

/* ---- return codes ------------------------------------------------------ */
#define SP_OK              0
#define SP_E_INVALID     (-1)   /* bad argument (sizes, NULL, out-of-range index) */
#define SP_E_CUDA        (-2)   /* a CUDA runtime call failed */
#define SP_E_NOMEM       (-3)   /* device allocation failed */
#define SP_E_UNSUPPORTED (-4)   /* model feature outside this engine (e.g. custom propensity) */
#define SP_E_TRAJECTORY  (-5)   /* at least one trajectory ended with an error status */
#define SP_E_TIMEOUT     (-6)   /* the caller's wall-clock limit ran out */

/* ---- per-trajectory status words (sp_traj_status.code) ----------------- */
#define SP_TRAJ_OK               0
#define SP_TRAJ_NEG_COUNT        1  /* a count went negative (simulate_rdme.cpp:288-294, 395-400) */
#define SP_TRAJ_NAN_STATE        2  /* NaN/inf in particle state (particle.cpp:88-126) */
#define SP_TRAJ_SELECT_OVERFLOW  3  /* no channel could be selected (simulate_rdme.cpp:277-279, 381-389) */
#define SP_TRAJ_BUDGET_EXHAUSTED 4  /* event budget / deadline of one launch ran out; resumable */

/* ---- mass-action reaction kinds ----------------------------------------
 * Propensity forms generated by Reaction._create_mass_action
 * (spatialpy/core/reaction.py:260-313) and evaluated in the generated C++
 * with left-to-right operator order:                                       */
#define SP_RXN_ZERO   0   /* k * vol                       (0th order)     */
#define SP_RXN_FIRST  1   /* k * x[a]                      (1st order)     */
#define SP_RXN_SECOND 2   /* k * x[a] * x[b] / vol         (a != b)        */
#define SP_RXN_DIMER  3   /* k * x[a] * (x[a] - 1) / vol   (2a -> ...)     */
#define SP_RXN_CUSTOM 4   /* a custom propensity_function, evaluated from a
                             stack program (see sp_scenario.rxn_code)        */

/* ---- custom propensity programs -------------------------------------------
 * A reaction's propensity_function (the expression the reference compiles
 * into its generated C++, solver.py:344-373) as postfix code of int32 words,
 * evaluated in double and rounded to float.  Operands follow their opcode.
 * The engine checks every program (operands in range, stack depth at most
 * SP_PROG_MAX_STACK, END reached) before use.                               */
#define SP_OP_END    0
#define SP_OP_CONST  1   /* k: push rxn_consts[k] */
#define SP_OP_X      2   /* s: push the count of species s */
#define SP_OP_VOL    3   /* push vol = m / rho */
#define SP_OP_T      4   /* push the time */
#define SP_OP_TYPE   5   /* push the particle type (sd) */
#define SP_OP_DATA   6   /* i: push data function i at this particle */
#define SP_OP_ADD   10
#define SP_OP_SUB   11
#define SP_OP_MUL   12
#define SP_OP_DIV   13
#define SP_OP_POW   14
#define SP_OP_NEG   15
#define SP_OP_POWI  16   /* n (|n| <= 64): integer power by repeated products */
#define SP_OP_EXP   20   /* .. SP_OP_CEIL: exp log sqrt sin cos tan fabs log10 floor ceil */
#define SP_OP_CEIL  29
#define SP_OP_LT    30   /* .. SP_OP_NE: < <= > >= == != as 1.0 / 0.0 */
#define SP_OP_NE    35
#define SP_OP_AND   36
#define SP_OP_OR    37
#define SP_OP_NOT   38
#define SP_PROG_MAX_STACK 16

/* ---- NSM selection rule -------------------------------------------------- */
#define SP_SELECT_EXACT     0  /* uniform rescaled for the channel choice; the
                                  event past a step boundary is not executed */
#define SP_SELECT_REFERENCE 1  /* reproduces simulate_rdme.cpp: rand1 reused
                                  unscaled (:253-261, :317-321) and one event
                                  past each step boundary executed (:233-238) */

/* ---- SDPD arithmetic ------------------------------------------------------ */
#define SP_PREC_F32 0
#define SP_PREC_F64 1

/*
 * One model instance: the arrays Model.compile_prep() + Solver.compile()
 * bake into the generated C++ (solver.py:208-288, 312-331, 375-419).
 * Layout follows ParticleSystem/Particle (include/particle_system.hpp:44-107,
 * include/particle.hpp:43-100), as structure-of-arrays.
 */
typedef struct sp_scenario {
    int32_t dimension;            /* 1, 2 or 3 (ParticleSystem::dimension) */
    int32_t num_particles;        /* N: particles == voxels */
    const double*  x;             /* [N*3] positions */
    const double*  v;             /* [N*3] initial velocities; NULL = zero */
    const int32_t* type;          /* [N] type id in 1..num_types */
    const double*  mass;          /* [N] */
    const double*  rho;           /* [N] */
    const double*  nu;            /* [N] */
    const uint8_t* fixed;         /* [N] solidTag (1 = fixed/wall particle) */
    int32_t num_types;            /* T: type ids 1..T (type 0 = unassigned, rejected) */

    int32_t num_species;          /* S */
    int32_t num_reactions;        /* R */
    const double*  rxn_rate;      /* [R] mass-action rate constant k */
    const int32_t* rxn_kind;      /* [R] SP_RXN_* */
    const int32_t* rxn_reactants; /* [R*2] species a, b (-1 when unused) */
    const uint8_t* rxn_allowed;   /* [R*(T+1)] 1 if reaction fires in type t (restrict_to); NULL = all */
    const int64_t* jcN;           /* [R+1] stoichiometry CSC column pointers (model.py:252-268) */
    const int64_t* irN;           /* [jcN[R]] species index of each change */
    const int32_t* prN;           /* [jcN[R]] change in copy number */
    const double*  diffusion;     /* [S*T] D(s,t) = diffusion[s*T + t-1] (solver.py:269-286) */

    double h;                     /* SPH support radius (Domain.find_h, domain.py:751-769) */
    double rho0, c0, P0;          /* reference density, sound speed, background pressure */
    double gravity[3];
    double dt;                    /* TimeSpan.timestep_size */
    int32_t num_steps;            /* nt (TimeSpan.num_timesteps) */
    int32_t static_domain;        /* Model.staticDomain */
    int32_t num_outputs;          /* len(TimeSpan.output_steps) */
    const int32_t* output_steps;  /* [num_outputs] ascending step indices */

    /* custom propensities (reactions of kind SP_RXN_CUSTOM); NULL if none */
    const int32_t* rxn_code;      /* programs of all reactions, concatenated */
    const int64_t* rxn_code_off;  /* [R+1]: reaction r's program is code[off[r] .. off[r+1]) */
    const double*  rxn_consts;    /* [num_consts] constants the programs push */
    int32_t num_consts;
    int32_t num_data_fn;          /* DataFunction values at the initial positions */
    const double*  data_fn;       /* [num_data_fn * N], function-major (solver.py:239-249) */

    /* deterministic chemistry (Model.enable_pde): concentrations C[N*S] that
       start at u0 and follow the reactions' ode_propensity_function and SPH
       diffusion (model.cpp:151-189, simulate.cpp:81-85, 167-169) */
    int32_t enable_pde;
    const int32_t* ode_code;      /* programs as rxn_code, one per reaction; SP_OP_X reads C */
    const int64_t* ode_code_off;  /* [R+1] */
    const double*  ode_consts;
    int32_t num_ode_consts;
    /* boundary conditions (BoundaryCondition.expression, boundarycondition.py:121-167),
       applied in order after the predictor and after the corrector */
    int32_t num_bcs;
    const double*  bc_box;        /* [num_bcs*6] xmin xmax ymin ymax zmin zmax (+-inf: none) */
    const int32_t* bc_type;       /* [num_bcs] particle type the condition needs, 0 = any */
    const int32_t* bc_target;     /* [num_bcs] SP_BC_V, SP_BC_NU, SP_BC_RHO or SP_BC_C + s */
    const double*  bc_value;      /* [num_bcs*3] value (v uses all three) */
} sp_scenario;

#define SP_BC_V   0
#define SP_BC_NU  1
#define SP_BC_RHO 2
#define SP_BC_C   3   /* + species index: a deterministic concentration */

typedef struct sp_options {
    int32_t device;               /* CUDA device ordinal */
    int32_t sdpd_precision;       /* SP_PREC_F32 (default) or SP_PREC_F64 */
    int32_t nsm_variant;          /* 0 = chosen per run: register-resident network when
                                     S <= 8 and R <= 16, speculative 32-event batches
                                     for domains of >= 2,048 voxels (static domains:
                                     larger and smaller domains of one run go to the
                                     two kernels, launched concurrently);
                                     1 = generic sequential warp kernel;
                                     2 = speculative batches wherever supported;
                                     3 = sequential register kernel;
                                     4 / 5 = speculative batches with 2 / 4 warps
                                     per trajectory */
    int32_t sdpd_self_pair;       /* how a moved particle meets its own start-of-step
                                     point in the force pass (particle.cpp:240-294 on a
                                     kd-tree of start-of-step points):
                                     0 = FP64 from the rounded positions, as the
                                     reference (no pair when the step rounds away);
                                     FP32 at the distance |dt vt| of the step itself;
                                     1 = at |dt vt| in both precisions */
    int64_t event_budget;         /* max events per trajectory per launch (0 = default) */
} sp_options;

/*
 * One ensemble run (Solver.run(number_of_trajectories, seed), solver.py:510).
 * Trajectory j runs instance `instance[j]` (NULL = instance 0) with Philox key
 * `seeds[j]` (the reference uses seed+j, solver.py:558-559).
 */
typedef struct sp_run_args {
    int32_t num_trajectories;
    int32_t selection;            /* SP_SELECT_* */
    const int32_t*  instance;     /* [ntraj] or NULL */
    const uint64_t* seeds;        /* [ntraj] */
    const uint32_t* const* u0;    /* [num_instances] -> [N_i*S_i] initial counts, voxel-major */
    int32_t buffers_on_device;    /* 1: every pointer in sp_outputs/u0 is device memory */
    int32_t want_counts;          /* write per-output counts */
    int32_t want_moments;         /* write per-instance moment sums over trajectories */
    int32_t want_particles;       /* write per-output particle state (non-static) */
    int32_t want_chem;            /* write per-output deterministic concentrations */
    double  timeout_s;            /* 0 = none; else SP_E_TIMEOUT once exceeded */
} sp_run_args;

typedef struct sp_outputs {
    /* [sum_j num_outputs_j * N_j * S_j] int32, trajectory-major then output, voxel, species */
    int32_t* counts;
    /* [sum_i num_outputs_i * N_i * S_i * 2] int64: (sum x, sum x^2) over the
       trajectories of instance i */
    int64_t* moments;
    /* [sum_i num_outputs_i * N_i * 3] positions / velocities, [.. * N_i] rho */
    double* particle_x;
    double* particle_v;
    double* particle_rho;
    /* [ntraj*2] (reaction events, diffusion events) — the engine counters
       total_reactions / total_diffusion (simulate_rdme.cpp:310, 445) */
    int64_t* event_counts;
    /* [sum_i num_outputs_i * N_i * S_i] deterministic concentrations C of the
       instances with enable_pde (written when want_chem), instance-major */
    double* chem;
} sp_outputs;

typedef struct sp_traj_status {
    int32_t code;                 /* SP_TRAJ_* */
    int32_t voxel;                /* voxel of the failing event, -1 if none */
    double  time;                 /* simulation time reached */
    int64_t events;               /* events executed */
    int64_t batches;              /* speculative batches run (0 for sequential kernels) */
    int64_t candidates;           /* candidate events examined by those batches */
} sp_traj_status;

typedef struct sp_handle sp_handle;

int         sp_abi_version(void);
int         sp_create(const sp_scenario* scenarios, int32_t num_scenarios,
                      const sp_options* opts, sp_handle** out);
int         sp_run(sp_handle* h, const sp_run_args* args, sp_outputs* out);
/*
 * sp_run in three parts, for callers that advance an ensemble output by
 * output (progress reporting, timing): sp_run_start uploads u0, builds the
 * event queues and writes the outputs at step 0; sp_run_continue advances
 * through the next `num_outputs` outputs that need events; sp_run_finish
 * copies results to host buffers and fills out->event_counts.  sp_run =
 * start + continue(all) + finish.  Same replacement as sp_run
 * (solver.py:547-605, simulate_threads.cpp:232-281).
 */
int         sp_run_start(sp_handle* h, const sp_run_args* args, sp_outputs* out);
int         sp_run_continue(sp_handle* h, int32_t num_outputs);
int         sp_run_finish(sp_handle* h);
int         sp_status(sp_handle* h, int32_t trajectory, sp_traj_status* st);
const char* sp_last_error(sp_handle* h);
void        sp_destroy(sp_handle* h);

/*
 * Inspection entry points (test and tooling use).  They copy device state of
 * instance `inst` into caller buffers.
 *
 * sp_get_neighbors mirrors Particle::neighbors after find_neighbors
 * (particle.cpp:150-210, 240-294): for particle i, count[i] entries at
 * idx/dist/dWdr/Dij[i*kmax ...] in ascending distance order (ties by index).
 * Returns SP_E_INVALID if any particle has more than kmax neighbours.
 */
int sp_get_neighbors(sp_handle* h, int32_t inst, int32_t kmax, int32_t* count,
                     int32_t* idx, double* dist, double* dWdr, double* Dij);
/* Ddiag[i*S+s] (nsm_core__initialize_diff_propensities, simulate_rdme.cpp:131-152) */
int sp_get_ddiag(sp_handle* h, int32_t inst, double* ddiag);
/* Current particle state of instance inst: x[N*3], v[N*3], rho[N]. */
int sp_get_particles(sp_handle* h, int32_t inst, double* x, double* v, double* rho);
/* Advance the SDPD flow of instance inst by nsteps without species
   (take_step substeps 0-2, simulate.cpp:33-48), from its current state. */
int sp_sdpd_advance(sp_handle* h, int32_t inst, int32_t nsteps);
/* Device time in milliseconds of the last sp_run / sp_run_continue /
   sp_sdpd_advance (CUDA events on the handle's stream) and kernel launches
   issued by it. */
int sp_last_timing(sp_handle* h, double* ms, int64_t* launches);

/* Same, split by kernel: kernel_ms = the NSM event-loop (or SDPD step)
   kernels alone, timed by CUDA events around each launch. */
typedef struct sp_profile {
    double total_ms;
    double kernel_ms;
    int64_t launches;
    int64_t kernel;     /* event-loop kernel of the last run: SP_KERNEL_* */
} sp_profile;
#define SP_KERNEL_NONE 0
#define SP_KERNEL_GENERIC 1      /* nsm_advance_generic: any network, one warp per trajectory */
#define SP_KERNEL_SEQUENTIAL 2   /* nsm_advance_small: register-resident network */
#define SP_KERNEL_BATCH 3        /* nsm_advance_batch: speculative 32-event batches */
#define SP_KERNEL_MIXED 4        /* batch kernel for domains of >= 2,048 voxels and
                                    nsm_advance_small for the rest, concurrently */
#define SP_KERNEL_BATCH_W2 5     /* nsm_advance_batchw: 2 warps per trajectory, 64-event batches */
#define SP_KERNEL_BATCH_W4 6     /* nsm_advance_batchw: 4 warps per trajectory, 128-event batches */
int sp_last_profile(sp_handle* h, sp_profile* p);

/*
 * sp_neighbors_noalloc — the neighbour lists of sp_get_neighbors (same
 * predicate, order and values), computed without allocating device memory.
 * It has no counterpart in the reference.  It is for callers that cannot
 * call cudaMalloc while they run: hosts that hand out all device memory from
 * their own fixed arena (once the arena holds the device a side allocation
 * fails, or escapes the host's accounting), and loops that cannot take the
 * device-wide synchronisation that cudaMalloc and cudaFree imply while other
 * streams are busy.
 *
 * Every array is a device pointer the caller owns: x[n*3], mass[n], rho[n];
 * outputs count[n] and idx/dist/dWdr/Dij[n*kmax] (dist, dWdr, Dij may be
 * NULL).  lo[3]/hi[3] are host arrays bounding the points (points outside
 * fall into edge cells and are still found).  Work is queued on `stream`
 * (NULL = default stream); the call synchronises `stream` to read back its
 * overflow flag and returns after its work completes.
 *
 * Limits: n <= 262,144 particles, at most 524,288 cells of edge h inside
 * [lo, hi], kmax <= 256; larger sizes, a non-finite or inverted box and a
 * non-finite h return SP_E_INVALID with a message in err (errlen bytes, may
 * be NULL) before any device work.  SP_E_UNSUPPORTED: some particle has
 * more than kmax neighbours.
 *
 * The cell-list scratch is one file-scope device array of 8.4 MB that every
 * GPU loading the library holds until the process exits.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress) with the
 * device current; make that first call before any stream capture.  All calls
 * share the array, which keeps the last call's contents (each call clears
 * what must start at zero): calls that overlap on the GPU (different streams
 * or host threads) race, so serialise them.
 */
int sp_neighbors_noalloc(const double* x, int32_t n, int32_t dim, double h,
                         const double* mass, const double* rho, const double* lo,
                         const double* hi, int32_t kmax, int32_t* count, int32_t* idx,
                         double* dist, double* dWdr, double* Dij, void* stream,
                         char* err, int32_t errlen);

/* ---- learned surrogate: the FiLM-conditioned Fourier neural operator ----
 *
 * No counterpart in the reference.  A network that maps a lattice's input
 * fields and a conditioning vector (log rate constants, time) to per-voxel
 * output fields, run and trained by this library's own kernels
 * (csrc/fno.cu): forward, backward and Adam, with bf16 weights and fp32
 * arithmetic and accumulation.
 *
 *   h0      = lift(x)                               pointwise, in_ch -> width
 *   g       = W2 GELU(W1 cond + b1) + b2            [layers][2][width]
 *   u_k     = S_k(h_k) + L_k h_k + l_k              k = 0 .. layers-1
 *   h_{k+1} = GELU(u_k * (1 + g[k][0]) + g[k][1])
 *   out     = P2 GELU(P1 h_L + p1) + p2             width -> hidden -> out_ch
 *
 * S_k is the spectral convolution: the real 2-D DFT of each channel,
 * truncated to the modes kx in [0, modes) U [n-modes, n), ky in [0, modes),
 * mixed across channels by one complex width x width matrix per mode, and
 * transformed back (the inverse real DFT of the truncated spectrum).  Fields
 * are [batch][channel][n*n] fp32 (row-major x, y).
 *
 * Parameters are one flat fp32 array, in this order (row-major, [out][in]
 * for the matrices):
 *   lift_w [width][in_ch], lift_b [width]
 *   per layer: spec_w [2*modes*modes][width_in][width_out][2] (mode index
 *              kxi*modes + ky, kxi < modes: kx = kxi, else kx = n-2*modes+kxi;
 *              [2] = real, imaginary), lin_w [width][width], lin_b [width]
 *   film1_w [hidden][cond], film1_b [hidden],
 *   film2_w [2*layers*width][hidden], film2_b [2*layers*width]
 *   proj1_w [hidden][width], proj1_b [hidden], proj2_w [out_ch][hidden],
 *   proj2_b [out_ch]
 * The forward pass reads a bf16 copy (round to nearest even) of every
 * parameter; gradients are taken with respect to those values and applied
 * to the fp32 array by Adam, which refreshes the copy.
 *
 * Device pointers: x, cond, target, out.  x may be one input shared by the
 * whole batch (x_shared = 1) or one per sample.  All calls are asynchronous
 * on `stream` (NULL = the default stream) except the sp_fno_get_* and
 * sp_fno_set_params copies and sp_fno_loss, which synchronise.
 */
typedef struct sp_fno_shape {
    int32_t n;          /* lattice edge, 4 <= n <= 64 */
    int32_t width;      /* channels, <= 64 */
    int32_t modes;      /* 1 <= modes, 2*modes <= n */
    int32_t layers;     /* 1 .. 8 */
    int32_t in_ch;      /* 1 .. 16 */
    int32_t out_ch;     /* 1 .. 16 */
    int32_t cond;       /* 1 .. 16 */
    int32_t hidden;     /* 1 .. 64: projection and conditioning MLP */
    int32_t max_batch;  /* 1 .. 1024 samples per call */
} sp_fno_shape;

typedef struct sp_fno sp_fno;

int         sp_fno_create(const sp_fno_shape* shape, sp_fno** out);
int64_t     sp_fno_num_params(const sp_fno* f);
/* fp32 parameters from the host; resets the Adam moments and step count */
int         sp_fno_set_params(sp_fno* f, const float* params, int64_t count);
int         sp_fno_get_params(sp_fno* f, float* params, int64_t count);
/* gradients of the last sp_fno_backward (or training step) */
int         sp_fno_get_grads(sp_fno* f, float* grads, int64_t count);
/* out [batch][out_ch][n*n] */
int         sp_fno_forward(sp_fno* f, const float* x, int32_t x_shared, const float* cond,
                           int32_t batch, float* out, void* stream);
/* after sp_fno_forward on the same batch: the mean squared error against
   target [batch][out_ch][n*n] and the gradient of every parameter */
int         sp_fno_backward(sp_fno* f, const float* target, int32_t batch, void* stream);
/* one Adam step (PyTorch's Adam: beta1, beta2, eps, no weight decay) */
int         sp_fno_adam(sp_fno* f, float lr, float beta1, float beta2, float eps, void* stream);
/* gather rows idx[batch] (host array, each in 0 .. rows-1) of cond
   [rows][cond], target [rows][out_ch][n*n] and, unless x_shared, x
   [rows][in_ch][n*n]; then forward, backward and Adam, replayed as one CUDA
   graph per (arrays, batch size) */
int         sp_fno_train_step(sp_fno* f, const float* x, int32_t x_shared, const float* cond,
                              const float* target, int32_t rows, const int32_t* idx,
                              int32_t batch, float lr, float beta1, float beta2, float eps,
                              void* stream);
/* loss of the last backward pass (synchronises) */
int         sp_fno_loss(sp_fno* f, float* loss);
const char* sp_fno_last_error(sp_fno* f);
void        sp_fno_destroy(sp_fno* f);

#ifdef __cplusplus
}
#endif
#endif /* SPGPU_H */
