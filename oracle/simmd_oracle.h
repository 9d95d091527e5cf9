/*
 * simmd_oracle.h -- CPU oracle for the SimulationCode.jl molecular-dynamics
 * hot path.  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the
 * CPU-baseline leg of bench.py call it to compare against; the product library
 * (libsimmd.so) never links or calls it.
 *
 * It is a plain-C, serial, FP64 restatement of the reference Julia routines
 * (paths are relative to the SimulationCode.jl project):
 *   src/InteractionPotential.jl:1-11, 17-46, 87-107   pair diameter, V, F/r
 *   src/DataStructs.jl:10-19, 45-60, 349-378          LJ/Berthier constants, list sizing
 *   src/NeighborLists.jl:24-104                       list rebuild + add_pair!
 *   src/MD.jl:30-82, 85-316, 391-402, 429-471, 499-554 forces, noise, integrators
 *   src/AuxiliaryFunctions.jl:22-65, 86-110, 186-196, 311-315, 381-584
 *   src/InitialConfiguration.jl:1-11, 43-114; src/MC.jl:21-47, 139-156 (fixtures)
 *   src/InherentStructure.jl:5-56                     steepest-descent minimiser
 *   src/MC.jl:21-156                                  swap Monte Carlo (translation and swap moves)
 *
 * Parity status: UNPINNED.  The reference is pure Julia, ships no tests, no
 * golden vectors and no fixtures, and Julia is not available where this
 * oracle is built, so no output of the reference itself pins these routines.
 * They are pinned instead by analytic known-answer tests (zero LJ force at
 * r = 2^(1/6) sigma, Berthier V = F = 0 at the cutoff, Newton's third law,
 * F = -grad E and W = -dE/dlnL by finite differences, brute-force vs
 * cell-list pair sets).  The cell-list pair enumeration of the third-party
 * package CellListMap (called at src/NeighborLists.jl:31, 46-52; version not
 * pinned by the reference: no Manifest.toml, no [compat]) is restated
 * geometrically: every minimum-image pair with d2 <= verlet_sphere_size^2,
 * with d2 computed by the reference's own calculate_squared_distance
 * (src/AuxiliaryFunctions.jl:311-315).
 *
 * Build with -O2 -ffp-contract=off (no FMA contraction) so every
 * floating-point operation is rounded as written.
 */
#ifndef SIMMD_ORACLE_H
#define SIMMD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_POT_LJ = 0, ORC_POT_BERTHIER = 1 };
enum { ORC_NEWTONIAN = 0, ORC_LANGEVIN = 1, ORC_BROWNIAN = 2 };

/* Scalars of ParameterStruct / System / potential (src/DataStructs.jl:10-87,
 * 138-153) plus the neighbor-list skin (src/DataStructs.jl:244). */
typedef struct orc_params {
    int32_t dims;                /* 2 or 3 */
    int32_t potential;           /* ORC_POT_* */
    int32_t dynamics;            /* ORC_NEWTONIAN / ORC_LANGEVIN / ORC_BROWNIAN */
    int32_t rescale_temperature; /* Newtonian.rescale_temperature */
    int64_t N;
    double box_size;
    double force_cutoff2;        /* ParameterStruct.force_cutoff2 = rc^2 */
    double skin;                 /* NeighborListStruct.skin_distance */
    double lj_eps, lj_sigma, lj_rc, lj_Uc;
    double b_c0, b_c2, b_c4, b_zeta;
    double kBT, gamma, dt, m;
} orc_params;

/* NeighborListStruct (src/DataStructs.jl:243-257): column-major lists,
 * entry (k, i) at list[k + maxK*i]; particle ids are 0-based here. */
typedef struct orc_nlist {
    int64_t maxK;
    int64_t *nn_full, *nn_half;      /* [N] */
    int64_t *list_full, *list_half;  /* [maxK*N] */
    double *disp;                    /* [dims*N] displacement since rebuild */
    double *disp2;                   /* [N] */
    double verlet_sphere_size;
    int64_t rebuilds;                /* OutputStruct.N_neighbor_list_rebuilds */
    int32_t overflow;                /* set instead of Julia's BoundsError */
    int32_t use_cells;               /* 1: cell-list enumeration, 0: all pairs */
} orc_nlist;

/* constants */
void orc_berthier_constants(int64_t n, double rc, double *c0, double *c2, double *c4);
double orc_lj_Uc(double eps, double sigma, double rc);
double orc_verlet_sphere_size(double skin, double force_cutoff, const double *D, int64_t N);

/* pair physics */
double orc_find_mean_D(const orc_params *p, double Di, double Dj);
double orc_pair_potential(const orc_params *p, double r2, double md2);
double orc_pair_force(const orc_params *p, double r2, double md2);
double orc_squared_distance(const orc_params *p, const double *ri, const double *rj);

/* neighbor lists */
int orc_update_neighbor_lists(const orc_params *p, const double *r, const double *D, orc_nlist *nl);

/* forces, energies, virial */
void orc_calculate_new_forces(const orc_params *p, const double *r, const double *v,
                              const double *D, const orc_nlist *nl, const double *noise,
                              double *F);
void orc_pair_forces_only(const orc_params *p, const double *r, const double *D,
                          const orc_nlist *nl, double *F);
double orc_find_energy(const orc_params *p, int64_t i, const double *ri, double Di,
                       const double *r, const double *D, const orc_nlist *nl);
double orc_calculate_full_energy(const orc_params *p, const double *r, const double *D,
                                 const orc_nlist *nl);
void orc_compute_potential_energy(const orc_params *p, const double *r, const double *D,
                                  const orc_nlist *nl, double *e);
double orc_energy_no_neigh(const orc_params *p, const double *r, const double *D);
double orc_kinetic_energy(const orc_params *p, const double *v);
double orc_virial(const orc_params *p, const double *r, const double *D, const orc_nlist *nl);
void orc_rescale_velocities(const orc_params *p, double *v);

/* integrators; noise = dims*N normals for this step (NULL only for Newtonian) */
int orc_do_time_step(const orc_params *p, double *r, double *v, double *F, const double *D,
                     orc_nlist *nl, const double *noise);
/* nsteps steps; noise either host array [nsteps][N][dims] or (if NULL) Philox
 * normals keyed by (seed, step0 + s).  Returns the first nonzero status. */
int orc_run_steps(const orc_params *p, double *r, double *v, double *F, const double *D,
                  orc_nlist *nl, int64_t nsteps, const double *noise, uint64_t seed,
                  uint64_t step0);

/* counter-based normals shared with the device generator */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_philox_normals(uint64_t seed, uint64_t step, int64_t N, int32_t dims, double *out);

/* fixtures */
uint64_t orc_splitmix64(uint64_t *state);
double orc_uniform01(uint64_t *state);
void orc_generate_diameters_berthier(int64_t N, double sigma_ratio, uint64_t seed, double *D);
int orc_random_initial_configuration(const orc_params *p, double *r, double *D, orc_nlist *nl,
                                     int64_t steps, double max_disp, uint64_t seed,
                                     double *final_energy);
/* swap Monte Carlo sweeps (do_MC_step!, src/MC.jl:21-156), Philox-keyed draws */
void orc_mc_uniforms(uint64_t seed, uint64_t sweep, int64_t i, double u[6]);
int orc_mc_sweeps(const orc_params *p, double *r, double *D, orc_nlist *nl, int64_t nsweeps, double max_disp,
                  double swap_prob, uint64_t seed, uint64_t sweep0, int64_t counts[4], double *dE_sum);
int orc_relax_capped(const orc_params *p, double *r, double *F, const double *D, orc_nlist *nl,
                     int64_t steps, double step_size, double max_disp);
int orc_find_inherent_structure(const orc_params *p, double *r, double *v, double *F,
                                const double *D, orc_nlist *nl, double tolerance,
                                int64_t max_iterations, double max_step_size, double dt,
                                int64_t *iterations);

#ifdef __cplusplus
}
#endif
#endif
