/*
 * simmd.h -- C ABI of libsimmd, the GB300 (sm_103a) molecular-dynamics hot
 * path of SimulationCode.jl behind a plain C interface (Julia reaches it by
 * ccall; Python by ctypes).  No CUDA, C++ or torch types cross this boundary:
 * only plain pointers to host memory, sizes and an opaque context.
 *
 * Reference interfaces replaced (paths relative to the SimulationCode.jl
 * project):
 *   initialize_neighbor_struct(skin, L, rc, N, D, dims; maxneighbours=200)
 *        src/DataStructs.jl:349-378            -> simmd_create
 *   update_neighbor_lists!(arrays, parameters, output, neighborlist)
 *        src/NeighborLists.jl:24-53            -> simmd_rebuild
 *   calculate_new_forces!(arrays, parameters, neighborlist)
 *        src/MD.jl:262-316                     -> simmd_forces
 *   do_time_step(arrays, parameters, output, neighborlist, system)
 *        src/MD.jl:429-471, 499-554            -> simmd_step (nsteps = 1)
 *   the step loop of perform_molecular_dynamics!
 *        src/MD.jl:704-715                     -> simmd_step (nsteps = N_steps)
 *   calculate_full_energy / find_kinetic_energy
 *        src/AuxiliaryFunctions.jl:22-34, 57-65 -> simmd_energy
 *   compute_potential_energy!
 *        src/AuxiliaryFunctions.jl:186-196     -> simmd_potential_energy_array
 *   NeighborListStruct.neighbor_list_half / _full (layout only)
 *        src/DataStructs.jl:243-257            -> simmd_export_pairs
 *   OutputStruct.N_neighbor_list_rebuilds, steps_done
 *        src/DataStructs.jl:291-315            -> simmd_stats
 *
 * Array layout: every per-particle vector array is the reference's
 * ArrayStruct field reinterpreted as Float64, i.e. AoS dims x N, particle i's
 * components at [i*dims + k] (Julia: reinterpret(reshape, Float64, r_array)).
 * Lists are Julia's Array{Int64,2}(maxK, N): column-major, 1-based ids.
 *
 * Every call returns an int status (SIMMD_OK = 0); the Julia shim raises
 * error() on nonzero, as the reference raises on neighbour overflow
 * (BoundsError) or a bad dimension ("To be implemented").  Calls are
 * blocking at the ABI level unless stated; one context per host thread.
 */
#ifndef SIMMD_H
#define SIMMD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum simmd_status {
    SIMMD_OK = 0,
    SIMMD_ERR_BAD_ARG = 1,            /* invalid parameter (dims not 2/3, N<1, ...) */
    SIMMD_ERR_CUDA = 2,               /* CUDA runtime error (message: simmd_last_error) */
    SIMMD_ERR_OOM = 3,                /* device allocation failed */
    SIMMD_ERR_NEIGHBOR_OVERFLOW = 4,  /* a particle has more than max_neighbors entries */
    SIMMD_ERR_NONFINITE = 5,          /* NaN/Inf position or displacement */
    SIMMD_ERR_NOISE_RANGE = 6,        /* host noise array shorter than the steps taken */
    SIMMD_ERR_BUDGET = 7,             /* replica does not fit the memory budget / capacity */
    SIMMD_ERR_NOT_FOUND = 8,          /* unknown replica id */
    SIMMD_ERR_NO_DEVICE = 9,          /* no CUDA device */
    SIMMD_ERR_NOT_CONVERGED = 10      /* minimiser reached max_iterations */
};

enum { SIMMD_POT_LJ = 0, SIMMD_POT_BERTHIER = 1 };
enum { SIMMD_NEWTONIAN = 0, SIMMD_LANGEVIN = 1, SIMMD_BROWNIAN = 2 };
enum { SIMMD_FP64 = 0, SIMMD_FP32_SPLIT = 1 };

/* ParameterStruct + System + potential scalars + neighbour-list skin
 * (src/DataStructs.jl:10-87, 138-153, 244). */
typedef struct simmd_params {
    int32_t dims;                /* 2 or 3 (system.dims) */
    int32_t potential;           /* SIMMD_POT_* (interaction_potential) */
    int32_t dynamics;            /* SIMMD_NEWTONIAN / _LANGEVIN / _BROWNIAN (typeof(system)) */
    int32_t precision;           /* SIMMD_FP64 (reference arithmetic) or SIMMD_FP32_SPLIT */
    int64_t N;                   /* parameters.N */
    double box_size;             /* parameters.box_size (cubic box) */
    double force_cutoff2;        /* parameters.force_cutoff2 = rc^2 */
    double skin;                 /* neighborlist.skin_distance */
    double verlet_force_cutoff;  /* force_cutoff argument of initialize_neighbor_struct (rc) */
    double lj_eps, lj_sigma, lj_Uc;          /* LJ(eps, sigma, rc) fields */
    double b_c0, b_c2, b_c4, b_zeta;         /* Berthier fields */
    double kBT, gamma, dt, m;                /* system fields (gamma unused for Newtonian) */
    int32_t rescale_temperature; /* Newtonian.rescale_temperature */
    int32_t max_neighbors;       /* maxneighbours (rows of the list); 0 -> 200 */
    uint64_t seed;               /* Philox key of the production noise stream */
} simmd_params;

typedef struct simmd_stats {
    int64_t steps_done;          /* time steps taken through simmd_step */
    int64_t rebuilds;            /* neighbour-list rebuilds (N_neighbor_list_rebuilds) */
    int64_t noise_draws;         /* Philox counter: random-force evaluations so far */
    int32_t max_neighbors;       /* list rows allocated */
    int32_t max_count;           /* largest list length seen since creation */
    int32_t overflow;            /* sticky neighbour-overflow flag */
    int32_t nonfinite;           /* sticky NaN/Inf flag */
    double epot, virial, ekin;   /* last values from simmd_energy */
    int64_t list_entries;        /* force-list entries (both directions) at the last rebuild */
} simmd_stats;

typedef struct simmd_ctx simmd_ctx;

const char* simmd_version(void);
const char* simmd_status_string(int status);
const char* simmd_last_error(void);
int simmd_device_count(int32_t* n);

/* ---- single system (drop-in; replica 0 of the context) ------------------ */

/* initialize_neighbor_struct: allocate device state for one system of N
 * particles on the current CUDA device.  The list of maxneighbours rows is
 * allocated as in the reference. */
int simmd_create(const simmd_params* p, simmd_ctx** out);
int simmd_destroy(simmd_ctx* ctx);

/* Copy ArrayStruct fields to the device (r, D required; v, F, disp may be
 * NULL = zeros).  The stale F is used by the first kick, as in the reference.
 * Schedules a list rebuild before the next force evaluation. */
int simmd_upload(simmd_ctx* ctx, const double* r, const double* v, const double* F,
                 const double* D, const double* disp);
/* Overwrite positions / velocities / forces / displacements in place (any
 * pointer may be NULL), keeping the neighbour lists and the skin bookkeeping:
 * the ArrayStruct fields a Julia caller edited between calls. */
int simmd_set_state(simmd_ctx* ctx, const double* r, const double* v, const double* F,
                    const double* disp);
/* Copy the device state back (any pointer may be NULL). */
int simmd_download(simmd_ctx* ctx, double* r, double* v, double* F, double* disp);

/* update_neighbor_lists!: rebuild every replica's lists now (resets the
 * displacements, counts a rebuild). */
int simmd_rebuild(simmd_ctx* ctx);

/* calculate_new_forces!: pair forces + random force (Langevin: -gamma v +
 * sqrt(2 kBT gamma/dt) xi; Brownian: sqrt(2 kBT gamma/dt) xi).  noise: host
 * array dims x N of N(0,1) deviates for this call (NULL: Philox stream).
 * F_out (may be NULL) receives the forces. */
int simmd_forces(simmd_ctx* ctx, const double* noise, double* F_out);

/* do_time_step x nsteps for every replica of the context.  noise: NULL for
 * the Philox stream, or (single-replica contexts) a host array
 * [nsteps][N][dims] of N(0,1) deviates, the reference's random_displacement
 * for each step. */
int simmd_step(simmd_ctx* ctx, int64_t nsteps, const double* noise);

/* Set-up relaxation (not a reference routine): nsteps of steepest descent
 * r += step_size * F with each particle's move capped at max_disp, FP64, no noise, for
 * every replica; removes the overlaps of random initial positions before
 * dynamics (the role of find_random_initial_configuration!'s MC sweeps,
 * src/InitialConfiguration.jl:43-114).  Velocities are kept; F holds the
 * last relaxation forces. */
int simmd_relax(simmd_ctx* ctx, int64_t nsteps, double step_size, double max_disp);

/* calculate_full_energy (epot), virial W = sum_pairs r_ij . F_ij, and
 * find_kinetic_energy (ekin) of replica 0; any pointer may be NULL. */
int simmd_energy(simmd_ctx* ctx, double* epot, double* virial, double* ekin);

/* compute_potential_energy!: per-particle energy (half of the pair sum). */
int simmd_potential_energy_array(simmd_ctx* ctx, double* e);

/* Lists as of the last rebuild, reference layout (maxK, N) column-major,
 * 1-based.  which = 0: the force ("half") list, each pair once, owner = the
 * lower particle id; which = 1: the full Verlet-sphere list (requires
 * simmd_set_full_list(ctx, 1) before the rebuild). */
int simmd_export_pairs(simmd_ctx* ctx, int32_t which, int64_t maxK, int64_t* counts, int64_t* list);
int simmd_set_full_list(simmd_ctx* ctx, int32_t enable);

int simmd_stats_get(simmd_ctx* ctx, simmd_stats* out);

/* ---- many replicas in one context (batching / serving) ------------------ */

int simmd_engine_create(int32_t device, simmd_ctx** out);
/* Pre-size slot, cell and replica capacity (no reallocation -- and no graph
 * re-capture -- while replicas come and go inside it). */
int simmd_reserve(simmd_ctx* ctx, int64_t slots, int64_t cells, int32_t replicas, int32_t max_neighbors);
int simmd_add_replica(simmd_ctx* ctx, const simmd_params* p, const double* r, const double* v,
                      const double* F, const double* D, int32_t* rep_out);
int simmd_remove_replica(simmd_ctx* ctx, int32_t rep);
int simmd_upload_r(simmd_ctx* ctx, int32_t rep, const double* r, const double* v, const double* F,
                   const double* D, const double* disp);
int simmd_download_r(simmd_ctx* ctx, int32_t rep, double* r, double* v, double* F, double* disp);
int simmd_set_state_r(simmd_ctx* ctx, int32_t rep, const double* r, const double* v, const double* F,
                      const double* disp);
/* Batched host transfers (no counterpart in the reference, which holds one
 * system): every replica of the context in one call, with one host <->
 * device copy per array and one synchronisation.  Host layout: the active
 * replicas in increasing replica id, each its ArrayStruct block (dims x N
 * AoS) one after the other; D: each replica's N diameters one after the
 * other.  simmd_transfer_layout returns the total number of doubles of a
 * dims x N array (-1: NULL context) and, if offsets is not NULL, fills
 * offsets[rep] for rep < n with the replica's first double (-1 for ids not
 * in use).  simmd_upload_all = simmd_upload_r of every
 * replica (r, D required; v, F, disp may be NULL = zeros); simmd_set_state_all
 * = simmd_set_state_r of every replica (any pointer may be NULL: the lists
 * and the skin bookkeeping are kept, the segment loop of a caller that holds
 * the state on the host between calls); simmd_download_all =
 * simmd_download_r of every replica (any pointer may be NULL).  Host arrays
 * page-locked with simmd_host_register transfer at full link speed. */
int64_t simmd_transfer_layout(simmd_ctx* ctx, int32_t n, int64_t* offsets);
int simmd_upload_all(simmd_ctx* ctx, const double* r, const double* v, const double* F, const double* D,
                     const double* disp);
int simmd_set_state_all(simmd_ctx* ctx, const double* r, const double* v, const double* F, const double* disp);
int simmd_download_all(simmd_ctx* ctx, double* r, double* v, double* F, double* disp);
/* find_inherent_structure (src/InherentStructure.jl:5-56) for every replica
   of the context, in FP64 with the reference's arithmetic: steepest descent
   v = F*dt, scaled so that max_i |v_i| <= max_step_size, drift with wrap
   and displacement, rebuild on the skin trigger, until max_i |F_i| <=
   tolerance (after that iteration's move).  Pair forces only.  iterations
   (optional) receives each replica's iteration count, indexed by replica id.
   Returns SIMMD_ERR_NOT_CONVERGED if a replica reached max_iterations.
   Velocities are left unchanged (the reference reuses v_array as the step
   buffer). */
int simmd_inherent_structure(simmd_ctx* ctx, double tolerance, int64_t max_iterations, double max_step_size,
                             double dt, int64_t* iterations);
/* Swap Monte Carlo: nsweeps calls of do_MC_step! (src/MC.jl:139-156) with
   do_translation_step! (:21-47) and do_swap_step! (:67-110) for every
   replica of the context, each replica's chain serial as in the reference
   (particles in id order, each move decided on the state the previous ones
   left), FP64 find_energy over the full Verlet list
   (src/AuxiliaryFunctions.jl:546-584), Metropolis at the replica's kBT.  A
   translation displaces by U[-max_displacement, max_displacement) per
   component; with probability swap_probability the move is a swap with a
   uniformly drawn partner instead (the reference's draw ceil(rand()/N)
   always gives particle 1; the uniform partner is its evident intent),
   tried only when the diameters differ by at most 0.2.  Draws: Philox
   keyed by the replica's seed, the particle and the sweep.  The lists are
   rebuilt inside a sweep when a particle's displacement passes skin/2, as
   the reference does.  Enables the full list (simmd_set_full_list).
   simmd_mc_stats: counts4 = {translations accepted, tried, swaps accepted,
   tried} and dE = the sum of the accepted moves' energy changes (what the
   reference adds to output.potential_energy), since the replica was added;
   simmd_download_diameters: the replica's diameters in original order. */
int simmd_mc_sweeps(simmd_ctx* ctx, int64_t nsweeps, double max_displacement, double swap_probability);
int simmd_mc_stats(simmd_ctx* ctx, int32_t rep, int64_t* counts4, double* dE);
int simmd_download_diameters(simmd_ctx* ctx, int32_t rep, double* D);
/* asynchronous dump feed for save_data (src/Dump.jl:60-88): the replica's
   r, v, F (any may be NULL) as of this point of the step sequence are copied
   to the host on a side stream while later steps run (host arrays
   page-locked, see simmd_host_register, for the copy to overlap); one dump
   in flight per context; simmd_dump_wait returns once it has landed */
int simmd_dump_async(simmd_ctx* ctx, int32_t rep, double* r, double* v, double* F);
int simmd_dump_wait(simmd_ctx* ctx);
/* energies of every replica (one pass), then per replica */
int simmd_energy_all(simmd_ctx* ctx);
int simmd_stats_r(simmd_ctx* ctx, int32_t rep, simmd_stats* out);
/* device bytes a replica of this shape needs (admission against a budget) */
int64_t simmd_replica_bytes(const simmd_params* p, int32_t max_neighbors);
/* cap on the context's capacity-sized device memory (0 = none): a grow
   that would pass it is not made and the call that needed it returns
   SIMMD_ERR_BUDGET with the context unchanged.  No counterpart in the
   reference (a serving-layer control). */
int simmd_set_budget(simmd_ctx* ctx, int64_t bytes);

/* ---- energy without device allocation ----------------------------------- */

/* No counterpart in the reference.  For callers that must not allocate
 * device memory -- e.g. a Julia program whose GPU memory belongs to
 * CUDA.jl's pool, a host enforcing its own device-memory budget, or a loop
 * that cannot afford an allocation's latency or implicit synchronisation.
 * Computes, on the caller's stream (NULL: the default stream) and without
 * any cudaMalloc/cudaFree, out[0] = the potential energy of
 * calculate_full_energy, out[1] = the virial W = sum_pairs r_ij . F_ij and
 * out[2] = the number of invalid list entries skipped, from DEVICE arrays the
 * caller owns: r (dims x N AoS), D (N), the full neighbour list as in the
 * reference (counts[N], list[maxK*N] column-major, 1-based) and out[3].
 * Scratch is a fixed array inside the library, shared by every call on a
 * GPU: N must be <= SIMMD_NOALLOC_MAX_N (else SIMMD_ERR_BUDGET, checked
 * before any device work; simmd_last_error says why), and calls
 * that run concurrently on the same GPU race.  The first call on a device
 * performs a one-time symbol lookup, which may load the library's device
 * code onto that GPU (lazy module loading) and so reserve its memory; make
 * that first call before any stream capture and before measuring memory.
 * Later calls allocate nothing.  The looked-up address is kept per device
 * and per CUDA context: after a device reset the next call looks it up
 * again (and is again a first call).
 * Asynchronous: synchronise the stream before reading out. */
#define SIMMD_NOALLOC_MAX_N 1048576
int simmd_energy_virial_noalloc(const simmd_params* p, const double* r, const double* D,
                                const int64_t* counts, const int64_t* list, int64_t maxK,
                                double* out, void* stream);

/* ---- tuning, timing, plumbing ------------------------------------------ */

/* threads per particle in the force pass (1, 2, 4, 8), CUDA-graph capture of
 * the step loop (0/1) and steps per captured graph. */
int simmd_set_tuning(simmd_ctx* ctx, int32_t threads_per_particle, int32_t use_graphs, int32_t graph_steps);
/* tile shape of the force pass: particles per work item (one block of
 * particles x threads_per_particle threads): 128 (a whole tile), 64 or 32,
 * or 0 = automatic (whole tiles, split only when a batch has fewer tiles
 * than SMs).  Results are unchanged. */
int simmd_set_work_item(simmd_ctx* ctx, int32_t particles);
/* change the neighbour-list skin (the rebuild cadence) of one replica (or
 * every replica: rep = -1); the lists are rebuilt before the next force
 * evaluation.  Results are unchanged up to the order of the force sums. */
int simmd_set_skin(simmd_ctx* ctx, int32_t rep, double skin);
/* inner (pruned) neighbour lists for the force pass: after every rebuild,
 * and whenever a particle of the replica has moved more than inner_skin / 2
 * since the last prune, the replica's list is filtered to the pairs within
 * rc_ij + inner_skin (outer-list order kept); the force pass reads the
 * filtered list, and a force pass that finds a replica's filter due reads
 * the full list and writes the filtered one while it sums.  The dropped
 * pairs lie beyond the force cutoff until the next filter and add exactly
 * zero, so every force, energy and trajectory is bit-identical to the
 * unfiltered list's; the rebuild schedule (skin trigger) is unchanged.
 * Needs one thread per particle (simmd_set_tuning tpp = 1).
 * inner_skin > 0 for one replica (or every replica: rep = -1) turns the
 * filtering on for the context (replicas without an inner skin keep every
 * listed pair); 0 on every replica turns it off.  Costs 4K + 20 device
 * bytes per slot (K list rows). */
int simmd_set_prune(simmd_ctx* ctx, int32_t rep, double inner_skin);
/* prunes done and inner-list entries at the last prune of one replica */
int simmd_prune_stats(simmd_ctx* ctx, int32_t rep, int64_t* prunes, int64_t* inner_entries);
int simmd_sync(simmd_ctx* ctx);
void* simmd_stream(simmd_ctx* ctx);          /* the context's cudaStream_t */
int simmd_timer_start(simmd_ctx* ctx);       /* CUDA event on the context stream */
int simmd_timer_stop(simmd_ctx* ctx, float* ms);
int64_t simmd_launch_count(simmd_ctx* ctx);  /* kernels run by this context (synchronises) */
/* force-kernel launches and neighbour-rebuild sequences run so far (a
   captured step loop skips a rebuild sequence's body when no replica's
   trigger fired; synchronises) */
int simmd_kernel_counts(simmd_ctx* ctx, int64_t* force_launches, int64_t* rebuild_sequences);
int64_t simmd_device_bytes(simmd_ctx* ctx);  /* device memory held */
/* time the force pass alone: nrep launches, average ms per launch (CUDA
 * events around the launches on the context stream) */
int simmd_time_force(simmd_ctx* ctx, int32_t nrep, float* ms_per_launch);
/* per-kernel CUDA-event timing of simmd_step (direct launches, events around
 * each kernel group on the context stream).  out[6] = {force ms total, force
 * launches, kick/drift ms, rebuild ms, Brownian-update ms, steps}. */
int simmd_set_profile(simmd_ctx* ctx, int32_t enable);
/* page-lock a caller's host array for fast transfers (cudaHostRegister) */
int simmd_host_register(void* ptr, int64_t bytes);
int simmd_host_unregister(void* ptr);
int simmd_profile_get(simmd_ctx* ctx, double* out6);
/* self-check of the split-precision kernels' float <-> double conversions
 * (bit operations on the integer pipes) against the hardware converter on
 * the current device: n hashed float and double bit patterns (all classes,
 * rounding ties, the float range edges); *mismatches = patterns whose
 * result bits differ.
 * No context needed. */
int simmd_check_conversions(int64_t n, uint64_t seed, int64_t* mismatches);

#ifdef __cplusplus
}
#endif
#endif
