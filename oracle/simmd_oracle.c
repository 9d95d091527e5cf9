/*
 * simmd_oracle.c -- serial FP64 restatement of the SimulationCode.jl MD hot
 * path.  TEST INFRASTRUCTURE ONLY; see simmd_oracle.h for the
 * routine-by-routine reference map and the parity status ("unpinned": no
 * Julia and no reference golden vectors exist for this path).
 *
 * Arithmetic is written in the reference's operation order, and the file is
 * compiled with -ffp-contract=off, so each expression rounds as the Julia
 * source reads (LoopVectorization's @turbo may contract to FMA in the
 * reference; that last-ulp freedom is inside the 1e-12 relative tolerance).
 * Julia's round(x) is round-half-even: nearbyint() in the default rounding
 * mode.  Particle ids are 0-based.
 */
#include "simmd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* constants                                                           */
/* ------------------------------------------------------------------ */

/* Berthier(; n=12, rc=1.25, ...) inner constructor, src/DataStructs.jl:53-59 */
void orc_berthier_constants(int64_t n, double rc, double *c0, double *c2, double *c4)
{
    double dn = (double)n;
    *c0 = -(1.0 / 8.0) * (double)(8 + 6 * n + n * n) * pow(rc, -dn);
    *c2 = 1.0 / 4.0 * dn * (double)(4 + n) * pow(rc, -2.0 - dn);
    *c4 = -(1.0 / 8.0) * dn * (double)(2 + n) * pow(rc, -4.0 - dn);
}

/* LJ(eps, sigma, rc): Uc = 4eps((sigma/rc)^12 - (sigma/rc)^6), src/DataStructs.jl:15-18 */
double orc_lj_Uc(double eps, double sigma, double rc)
{
    double x = sigma / rc;
    return 4.0 * eps * (pow(x, 12.0) - pow(x, 6.0));
}

/* verlet_sphere_size = skin + force_cutoff * maximum(D), src/DataStructs.jl:351-352 */
double orc_verlet_sphere_size(double skin, double force_cutoff, const double *D, int64_t N)
{
    double smax = D[0];
    for (int64_t i = 1; i < N; i++)
        if (D[i] > smax) smax = D[i];
    return skin + force_cutoff * smax;
}

/* ------------------------------------------------------------------ */
/* pair physics, src/InteractionPotential.jl                           */
/* ------------------------------------------------------------------ */

/* find_mean_D, src/InteractionPotential.jl:5-11.  Note the LJ method returns
 * sigma^2 (not sigma); the reference's generic paths square it again. */
double orc_find_mean_D(const orc_params *p, double Di, double Dj)
{
    if (p->potential == ORC_POT_LJ) return p->lj_sigma * p->lj_sigma;
    return (Di + Dj) * 0.5 * (1.0 - p->b_zeta * fabs(Di - Dj));
}

/* potential(r2, md2, U), src/InteractionPotential.jl:17-25 (LJ), 87-95 (Berthier) */
double orc_pair_potential(const orc_params *p, double r2, double md2)
{
    if (p->potential == ORC_POT_LJ) {
        double xi2 = md2 / r2;
        double xi4 = xi2 * xi2;
        double xi6 = xi2 * xi4;
        double xi12 = xi6 * xi6;
        return 4.0 * p->lj_eps * (xi12 - xi6) - p->lj_Uc;
    }
    double invxi2 = r2 / md2;
    double invxi4 = invxi2 * invxi2;
    double xi12 = 1.0 / (invxi4 * invxi4 * invxi4);
    return xi12 + p->b_c4 * invxi4 + p->b_c2 * invxi2 + p->b_c0;
}

/* force(r2, md2, U) = F/r, src/InteractionPotential.jl:39-46 (LJ), 98-107 (Berthier) */
double orc_pair_force(const orc_params *p, double r2, double md2)
{
    if (p->potential == ORC_POT_LJ) {
        double inv_r2 = 1.0 / r2;
        double xi2 = md2 * inv_r2;
        double xi6 = xi2 * xi2 * xi2;
        double xi12 = xi6 * xi6;
        return p->lj_eps * (48.0 * xi12 - 24.0 * xi6) * inv_r2;
    }
    double inv_md2 = 1.0 / md2;
    double invxi2 = r2 * inv_md2;
    double invxi4 = invxi2 * invxi2;
    double xi14 = 1.0 / (invxi4 * invxi4 * invxi4 * invxi2);
    return -2.0 * inv_md2 * (p->b_c2 + 2.0 * p->b_c4 * invxi2 - 6.0 * xi14);
}

/* minimum-image difference dx - round(dx/L)*L, src/MD.jl:115-117 */
static inline double min_image(double dx, double L)
{
    return dx - nearbyint(dx / L) * L;
}

/* calculate_squared_distance, src/AuxiliaryFunctions.jl:311-315 */
double orc_squared_distance(const orc_params *p, const double *ri, const double *rj)
{
    double L = p->box_size;
    double dx = min_image(ri[0] - rj[0], L);
    double dy = min_image(ri[1] - rj[1], L);
    if (p->dims == 2) return dx * dx + dy * dy;
    double dz = min_image(ri[2] - rj[2], L);
    return dx * dx + dy * dy + dz * dz;
}

/* ------------------------------------------------------------------ */
/* neighbor lists, src/NeighborLists.jl                                */
/* ------------------------------------------------------------------ */

/* add_pair!, src/NeighborLists.jl:82-104 (Julia raises BoundsError on
 * overflow; here the overflow flag is set and the entry dropped) */
static void add_pair(const orc_params *p, int64_t i, int64_t j, double d2, orc_nlist *nl,
                     const double *D, double r_cutoff)
{
    int64_t K = nl->maxK;
    int64_t n = nl->nn_full[i] + 1;
    nl->nn_full[i] = n;
    if (n <= K) nl->list_full[(n - 1) + K * i] = j; else nl->overflow = 1;

    double mean_d = orc_find_mean_D(p, D[i], D[j]);
    double t = r_cutoff * mean_d + p->skin;
    if (d2 < t * t) {
        n = nl->nn_half[i] + 1;
        nl->nn_half[i] = n;
        if (n <= K) nl->list_half[(n - 1) + K * i] = j; else nl->overflow = 1;
    }

    n = nl->nn_full[j] + 1;
    nl->nn_full[j] = n;
    if (n <= K) nl->list_full[(n - 1) + K * j] = i; else nl->overflow = 1;
}

/* update_neighbor_lists!, src/NeighborLists.jl:24-53.  The CellListMap pair
 * enumeration (:31, :46-52) is restated as: all unordered pairs (i<j) whose
 * minimum-image d2 <= verlet_sphere_size^2; add_pair!(i, j) is called with
 * the lower id first.  With use_cells the pairs are found through a cell grid
 * of floor(L/verlet) cells per axis (src/DataStructs.jl:353); the pair SET is
 * identical to the all-pairs search (tested). */
int orc_update_neighbor_lists(const orc_params *p, const double *r, const double *D, orc_nlist *nl)
{
    const int64_t N = p->N;
    const int d = p->dims;
    nl->rebuilds += 1;
    nl->overflow = 0;
    memset(nl->nn_full, 0, sizeof(int64_t) * N);
    memset(nl->nn_half, 0, sizeof(int64_t) * N);
    memset(nl->disp, 0, sizeof(double) * d * N);
    memset(nl->disp2, 0, sizeof(double) * N);

    const double r_cutoff = sqrt(p->force_cutoff2);
    const double rv = nl->verlet_sphere_size;
    const double rv2 = rv * rv;
    const double L = p->box_size;
    int64_t nc = (int64_t)floor(L / rv);

    if (!nl->use_cells || nc < 3) {
        for (int64_t i = 0; i < N; i++)
            for (int64_t j = i + 1; j < N; j++) {
                double d2 = orc_squared_distance(p, r + d * i, r + d * j);
                if (d2 <= rv2) add_pair(p, i, j, d2, nl, D, r_cutoff);
            }
        return nl->overflow ? 1 : 0;
    }

    /* cell grid */
    double cs = L / (double)nc;
    int64_t ncell = nc * nc * (d == 3 ? nc : 1);
    int64_t *head = (int64_t *)malloc(sizeof(int64_t) * ncell);
    int64_t *next = (int64_t *)malloc(sizeof(int64_t) * N);
    int64_t *cellof = (int64_t *)malloc(sizeof(int64_t) * N);
    for (int64_t c = 0; c < ncell; c++) head[c] = -1;
    for (int64_t i = N - 1; i >= 0; i--) {
        int64_t cc[3] = {0, 0, 0};
        for (int k = 0; k < d; k++) {
            int64_t c = (int64_t)floor(r[d * i + k] / cs);
            if (c < 0) c = 0;
            if (c >= nc) c = nc - 1;
            cc[k] = c;
        }
        int64_t lin = cc[0] + nc * (cc[1] + nc * cc[2]);
        cellof[i] = lin;
        next[i] = head[lin];
        head[lin] = i;
    }
    for (int64_t i = 0; i < N; i++) {
        int64_t lin = cellof[i];
        int64_t cx = lin % nc, cy = (lin / nc) % nc, cz = lin / (nc * nc);
        int zr = (d == 3) ? 1 : 0;
        for (int oz = -zr; oz <= zr; oz++)
            for (int oy = -1; oy <= 1; oy++)
                for (int ox = -1; ox <= 1; ox++) {
                    int64_t x = (cx + ox + nc) % nc, y = (cy + oy + nc) % nc;
                    int64_t z = (d == 3) ? (cz + oz + nc) % nc : 0;
                    for (int64_t j = head[x + nc * (y + nc * z)]; j >= 0; j = next[j]) {
                        if (j <= i) continue;
                        double d2 = orc_squared_distance(p, r + d * i, r + d * j);
                        if (d2 <= rv2) add_pair(p, i, j, d2, nl, D, r_cutoff);
                    }
                }
    }
    free(head);
    free(next);
    free(cellof);
    return nl->overflow ? 1 : 0;
}

/* ------------------------------------------------------------------ */
/* forces, src/MD.jl:85-316                                            */
/* ------------------------------------------------------------------ */

/* compute_forces_berthier_3d / _2d (src/MD.jl:85-137, 194-238) and
 * compute_forces_lj_3d (src/MD.jl:140-191): the per-particle @turbo loops,
 * Newton-3 scatter to j, accumulation into i after the loop. */
static void forces_particle_specialized(const orc_params *p, int64_t i, const double *r,
                                        const double *D, const orc_nlist *nl, double *F)
{
    const int d = p->dims;
    const double L = p->box_size;
    const double rc2 = p->force_cutoff2;
    const int64_t K = nl->maxK;
    const int64_t nn = nl->nn_half[i];
    const double xi = r[d * i], yi = r[d * i + 1], zi = (d == 3) ? r[d * i + 2] : 0.0;
    const double Di = D[i];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int64_t n = 0; n < nn; n++) {
        int64_t j = nl->list_half[n + K * i];
        double dx = min_image(xi - r[d * j], L);
        double dy = min_image(yi - r[d * j + 1], L);
        double dz = 0.0, rij2;
        if (d == 3) {
            dz = min_image(zi - r[d * j + 2], L);
            rij2 = dx * dx + dy * dy + dz * dz;
        } else {
            rij2 = dx * dx + dy * dy;
        }
        double Fr;
        if (p->potential == ORC_POT_BERTHIER) {
            double Dj = D[j];
            double mean_d = (Di + Dj) * 0.5 * (1.0 - p->b_zeta * fabs(Di - Dj));
            double mds = mean_d * mean_d;
            double inv_md2 = 1.0 / mds;
            double invxi2 = rij2 * inv_md2;
            double invxi4 = invxi2 * invxi2;
            double xi14 = 1.0 / (invxi4 * invxi4 * invxi4 * invxi2);
            Fr = (rc2 * mds < rij2) ? 0.0
                 : -2.0 * inv_md2 * (p->b_c2 + 2.0 * p->b_c4 * invxi2 - 6.0 * xi14);
        } else { /* LJ 3D */
            double s2 = p->lj_sigma * p->lj_sigma;
            double xi2 = s2 / rij2;
            double xi6 = xi2 * xi2 * xi2;
            double xi12 = xi6 * xi6;
            Fr = (rc2 < rij2) ? 0.0 : p->lj_eps * (48.0 * xi12 - 24.0 * xi6) / rij2;
        }
        fx += Fr * dx;
        fy += Fr * dy;
        F[d * j] -= Fr * dx;
        F[d * j + 1] -= Fr * dy;
        if (d == 3) {
            fz += Fr * dz;
            F[d * j + 2] -= Fr * dz;
        }
    }
    F[d * i] += fx;
    F[d * i + 1] += fy;
    if (d == 3) F[d * i + 2] += fz;
}

/* generic fallback of calculate_new_forces! (src/MD.jl:291-309), reached by
 * 2D LJ: mean_d = find_mean_D = sigma^2, squared again, strict '>' test */
static void forces_particle_generic(const orc_params *p, int64_t i, const double *r,
                                    const double *D, const orc_nlist *nl, double *F)
{
    const int d = p->dims;
    const double L = p->box_size;
    const double rc2 = p->force_cutoff2;
    const int64_t K = nl->maxK;
    const int64_t nn = nl->nn_half[i];
    double f[3] = {0.0, 0.0, 0.0};
    for (int64_t n = 0; n < nn; n++) {
        int64_t j = nl->list_half[n + K * i];
        double dr[3] = {0.0, 0.0, 0.0};
        double rij2 = 0.0;
        for (int k = 0; k < d; k++) dr[k] = min_image(r[d * i + k] - r[d * j + k], L);
        rij2 = dr[0] * dr[0] + dr[1] * dr[1];
        if (d == 3) rij2 = rij2 + dr[2] * dr[2];
        double mean_d = orc_find_mean_D(p, D[i], D[j]);
        double mds = mean_d * mean_d;
        if (rc2 * mds > rij2) {
            double Fr = orc_pair_force(p, rij2, mds);
            for (int k = 0; k < d; k++) {
                f[k] += Fr * dr[k];
                F[d * j + k] -= Fr * dr[k];
            }
        }
    }
    for (int k = 0; k < d; k++) F[d * i + k] += f[k];
}

/* pair part of calculate_new_forces!, src/MD.jl:262-311 */
void orc_pair_forces_only(const orc_params *p, const double *r, const double *D,
                          const orc_nlist *nl, double *F)
{
    const int64_t N = p->N;
    const int d = p->dims;
    memset(F, 0, sizeof(double) * d * N);
    int specialized = (d == 3) || (p->potential == ORC_POT_BERTHIER);
    for (int64_t i = 0; i < N; i++) {
        if (nl->nn_half[i] == 0) continue;
        if (specialized) forces_particle_specialized(p, i, r, D, nl, F);
        else forces_particle_generic(p, i, r, D, nl, F);
    }
}

/* calculate_new_forces! (src/MD.jl:262-316) including add_new_random_force!
 * (src/MD.jl:30-82): Langevin F += -gamma v + sqrt(2kBT gamma/dt) xi,
 * Brownian F += sqrt(2kBT gamma/dt) xi, Newtonian nothing. */
void orc_calculate_new_forces(const orc_params *p, const double *r, const double *v,
                              const double *D, const orc_nlist *nl, const double *noise,
                              double *F)
{
    orc_pair_forces_only(p, r, D, nl, F);
    const int64_t n = p->N * p->dims;
    if (p->dynamics == ORC_LANGEVIN) {
        double factor = sqrt(2.0 * p->kBT * p->gamma / p->dt);
        for (int64_t k = 0; k < n; k++) F[k] += -p->gamma * v[k] + factor * noise[k];
    } else if (p->dynamics == ORC_BROWNIAN) {
        double factor = sqrt(2.0 * p->kBT * p->gamma / p->dt);
        for (int64_t k = 0; k < n; k++) F[k] += factor * noise[k];
    }
}

/* ------------------------------------------------------------------ */
/* energies, src/AuxiliaryFunctions.jl                                 */
/* ------------------------------------------------------------------ */

/* find_energy (src/AuxiliaryFunctions.jl:546-584) over the FULL list with the
 * specialised inner loops berthier_inner_loop3/2 (:381-444), LJ_inner_loop
 * (:477-507) and the generic fallback (2D LJ). */
double orc_find_energy(const orc_params *p, int64_t i, const double *ri, double Di,
                       const double *r, const double *D, const orc_nlist *nl)
{
    const int d = p->dims;
    const double L = p->box_size;
    const double rc2 = p->force_cutoff2;
    const int64_t K = nl->maxK;
    const int64_t nn = nl->nn_full[i];
    if (nn == 0) return 0.0;
    double energy = 0.0;
    int specialized = (d == 3) || (p->potential == ORC_POT_BERTHIER);
    for (int64_t n = 0; n < nn; n++) {
        int64_t j = nl->list_full[n + K * i];
        double dx = min_image(ri[0] - r[d * j], L);
        double dy = min_image(ri[1] - r[d * j + 1], L);
        double rij2;
        if (d == 3) {
            double dz = min_image(ri[2] - r[d * j + 2], L);
            rij2 = dx * dx + dy * dy + dz * dz;
        } else {
            rij2 = dx * dx + dy * dy;
        }
        if (specialized) {
            if (p->potential == ORC_POT_BERTHIER) {
                double Dj = D[j];
                double mean_d = (Di + Dj) * 0.5 * (1.0 - p->b_zeta * fabs(Di - Dj));
                double mds = mean_d * mean_d;
                double invxi2 = rij2 / mds;
                double invxi4 = invxi2 * invxi2;
                double xi12 = 1.0 / (invxi4 * invxi4 * invxi4);
                energy += (rc2 * mds < rij2) ? 0.0
                          : xi12 + p->b_c4 * invxi4 + p->b_c2 * invxi2 + p->b_c0;
            } else {
                double mds = p->lj_sigma * p->lj_sigma;
                double xi2 = mds / rij2;
                double xi6 = xi2 * xi2 * xi2;
                double xi12 = xi6 * xi6;
                energy += (rc2 * mds < rij2) ? 0.0
                          : 4.0 * p->lj_eps * (xi12 - xi6) - p->lj_Uc;
            }
        } else {
            double mean_d = orc_find_mean_D(p, Di, D[j]);
            double mds = mean_d * mean_d;
            if (rc2 * mds > rij2) energy += orc_pair_potential(p, rij2, mds);
        }
    }
    return energy;
}

/* calculate_full_energy, src/AuxiliaryFunctions.jl:22-34 */
double orc_calculate_full_energy(const orc_params *p, const double *r, const double *D,
                                 const orc_nlist *nl)
{
    double energy = 0.0;
    for (int64_t i = 0; i < p->N; i++)
        energy += orc_find_energy(p, i, r + p->dims * i, D[i], r, D, nl);
    return energy / 2.0;
}

/* compute_potential_energy!, src/AuxiliaryFunctions.jl:186-196 */
void orc_compute_potential_energy(const orc_params *p, const double *r, const double *D,
                                  const orc_nlist *nl, double *e)
{
    for (int64_t i = 0; i < p->N; i++)
        e[i] = orc_find_energy(p, i, r + p->dims * i, D[i], r, D, nl) / 2.0;
}

/* calculate_full_energy_no_neigh, src/AuxiliaryFunctions.jl:86-110 */
double orc_energy_no_neigh(const orc_params *p, const double *r, const double *D)
{
    const int d = p->dims;
    double energy = 0.0;
    for (int64_t i = 0; i < p->N; i++)
        for (int64_t j = 0; j < p->N; j++) {
            if (i == j) continue;
            double rij2 = orc_squared_distance(p, r + d * i, r + d * j);
            double mean_d = orc_find_mean_D(p, D[i], D[j]);
            double mds = mean_d * mean_d;
            energy += (p->force_cutoff2 * mds < rij2) ? 0.0 : orc_pair_potential(p, rij2, mds);
        }
    return energy / 2.0;
}

/* find_kinetic_energy, src/AuxiliaryFunctions.jl:57-65 */
double orc_kinetic_energy(const orc_params *p, const double *v)
{
    const int d = p->dims;
    double ekin = 0.0;
    for (int64_t i = 0; i < p->N; i++) {
        double s = v[d * i] * v[d * i] + v[d * i + 1] * v[d * i + 1];
        if (d == 3) s = s + v[d * i + 2] * v[d * i + 2];
        ekin += s;
    }
    return ekin * (p->m / 2.0);
}

/* Virial W = sum over pairs of r_ij . F_ij = sum (F/r) r_ij^2, over the half
 * list with the same per-pair force expression and cutoff test as the force
 * pass.  The reference computes no virial; this definition is new and is
 * pinned by W = -dE/dlambda under uniform scaling r -> lambda r, L -> lambda L. */
double orc_virial(const orc_params *p, const double *r, const double *D, const orc_nlist *nl)
{
    const int d = p->dims;
    const double L = p->box_size;
    const double rc2 = p->force_cutoff2;
    const int64_t K = nl->maxK;
    int specialized = (d == 3) || (p->potential == ORC_POT_BERTHIER);
    double W = 0.0;
    for (int64_t i = 0; i < p->N; i++) {
        for (int64_t n = 0; n < nl->nn_half[i]; n++) {
            int64_t j = nl->list_half[n + K * i];
            double dx = min_image(r[d * i] - r[d * j], L);
            double dy = min_image(r[d * i + 1] - r[d * j + 1], L);
            double rij2;
            if (d == 3) {
                double dz = min_image(r[d * i + 2] - r[d * j + 2], L);
                rij2 = dx * dx + dy * dy + dz * dz;
            } else {
                rij2 = dx * dx + dy * dy;
            }
            double Fr = 0.0;
            if (specialized) {
                if (p->potential == ORC_POT_BERTHIER) {
                    double mean_d = (D[i] + D[j]) * 0.5 * (1.0 - p->b_zeta * fabs(D[i] - D[j]));
                    double mds = mean_d * mean_d;
                    if (!(rc2 * mds < rij2)) Fr = orc_pair_force(p, rij2, mds);
                } else {
                    double s2 = p->lj_sigma * p->lj_sigma;
                    double xi2 = s2 / rij2;
                    double xi6 = xi2 * xi2 * xi2;
                    double xi12 = xi6 * xi6;
                    if (!(rc2 < rij2)) Fr = p->lj_eps * (48.0 * xi12 - 24.0 * xi6) / rij2;
                }
            } else {
                double mean_d = orc_find_mean_D(p, D[i], D[j]);
                double mds = mean_d * mean_d;
                if (rc2 * mds > rij2) Fr = orc_pair_force(p, rij2, mds);
            }
            W += Fr * rij2;
        }
    }
    return W;
}

/* rescale_velocities!, src/MD.jl:391-402 (and the inline copy at :543-553) */
void orc_rescale_velocities(const orc_params *p, double *v)
{
    double ekin = 0.0;
    const int d = p->dims;
    for (int64_t i = 0; i < p->N; i++) {
        double s = v[d * i] * v[d * i] + v[d * i + 1] * v[d * i + 1];
        if (d == 3) s = s + v[d * i + 2] * v[d * i + 2];
        ekin += s;
    }
    ekin *= p->m / 2.0;
    double kbt_cur = 2.0 * ekin / (double)(d * p->N);
    double factor = sqrt(p->kBT / kbt_cur);
    for (int64_t k = 0; k < d * p->N; k++) v[k] *= factor;
}

/* ------------------------------------------------------------------ */
/* integrators, src/MD.jl                                              */
/* ------------------------------------------------------------------ */

static int skin_exceeded(const orc_params *p, const orc_nlist *nl)
{
    double mx = 0.0;
    for (int64_t i = 0; i < p->N; i++)
        if (nl->disp2[i] > mx) mx = nl->disp2[i];
    double h = p->skin / 2.0;
    return mx > h * h;
}

/* drift with periodic wrap + displacement bookkeeping; src/MD.jl:515-522 */
static void drift_particle(const orc_params *p, int64_t i, const double *dr, double *r, orc_nlist *nl)
{
    const int d = p->dims;
    const double L = p->box_size;
    double s = 0.0;
    for (int k = 0; k < d; k++) nl->disp[d * i + k] += dr[k];
    s = nl->disp[d * i] * nl->disp[d * i] + nl->disp[d * i + 1] * nl->disp[d * i + 1];
    if (d == 3) s = s + nl->disp[d * i + 2] * nl->disp[d * i + 2];
    nl->disp2[i] = s;
    for (int k = 0; k < d; k++) {
        double rnew = r[d * i + k] + dr[k];
        rnew -= floor(rnew / L) * L;
        r[d * i + k] = rnew;
    }
}

/* do_time_step(::Union{Newtonian,Langevin}), src/MD.jl:499-554;
 * do_time_step(::Brownian), src/MD.jl:429-471, as the code intends: the
 * reference method cannot run (it calls a 4-argument calculate_new_forces!
 * that does not exist, and wraps into an undefined xnew); here the forces
 * come from the 3-argument method, the wrapped rnew is stored, and 2D is
 * allowed. */
int orc_do_time_step(const orc_params *p, double *r, double *v, double *F, const double *D,
                     orc_nlist *nl, const double *noise)
{
    const int64_t N = p->N;
    const int d = p->dims;
    const double dt = p->dt;
    int st = 0;
    if (p->dynamics == ORC_BROWNIAN) {
        orc_calculate_new_forces(p, r, v, D, nl, noise, F);
        double Fmean[3] = {0.0, 0.0, 0.0};
        for (int64_t i = 0; i < N; i++)
            for (int k = 0; k < d; k++) Fmean[k] += F[d * i + k];
        for (int k = 0; k < d; k++) Fmean[k] /= (double)N;
        for (int64_t i = 0; i < N; i++)
            for (int k = 0; k < d; k++) F[d * i + k] -= Fmean[k];
        double factor = dt / p->gamma;
        for (int64_t i = 0; i < N; i++) {
            double dr[3];
            for (int k = 0; k < d; k++) dr[k] = factor * F[d * i + k];
            drift_particle(p, i, dr, r, nl);
        }
        if (skin_exceeded(p, nl)) st = orc_update_neighbor_lists(p, r, D, nl);
        return st;
    }
    const double m = p->m;
    for (int64_t k = 0; k < d * N; k++) v[k] = v[k] + dt * F[k] / (2.0 * m);
    for (int64_t i = 0; i < N; i++) {
        double dr[3];
        for (int k = 0; k < d; k++) dr[k] = dt * v[d * i + k];
        drift_particle(p, i, dr, r, nl);
    }
    if (skin_exceeded(p, nl)) st = orc_update_neighbor_lists(p, r, D, nl);
    orc_calculate_new_forces(p, r, v, D, nl, noise, F);
    for (int64_t k = 0; k < d * N; k++) v[k] = v[k] + dt * F[k] / (2.0 * m);
    double vmean[3] = {0.0, 0.0, 0.0};
    for (int64_t i = 0; i < N; i++)
        for (int k = 0; k < d; k++) vmean[k] += v[d * i + k];
    for (int k = 0; k < d; k++) vmean[k] /= (double)N;
    for (int64_t i = 0; i < N; i++)
        for (int k = 0; k < d; k++) v[d * i + k] -= vmean[k];
    if (p->dynamics == ORC_NEWTONIAN && p->rescale_temperature) orc_rescale_velocities(p, v);
    return st;
}

int orc_run_steps(const orc_params *p, double *r, double *v, double *F, const double *D,
                  orc_nlist *nl, int64_t nsteps, const double *noise, uint64_t seed,
                  uint64_t step0)
{
    const int64_t n = p->N * p->dims;
    double *buf = NULL;
    int need = (p->dynamics != ORC_NEWTONIAN);
    if (need && !noise) buf = (double *)malloc(sizeof(double) * n);
    int st = 0;
    for (int64_t s = 0; s < nsteps; s++) {
        const double *xi = NULL;
        if (need) {
            if (noise) xi = noise + s * n;
            else {
                orc_philox_normals(seed, step0 + (uint64_t)s, p->N, p->dims, buf);
                xi = buf;
            }
        }
        int rc = orc_do_time_step(p, r, v, F, D, nl, xi);
        if (rc && !st) st = rc;
    }
    free(buf);
    return st;
}

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) + Box-Muller       */
/* ------------------------------------------------------------------ */

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; round++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* N(0,1) noise keyed by (seed, step, particle, component pair): counter
 * (particle, pair, step_lo, step_hi), key (seed_lo, seed_hi); two 53-bit
 * uniforms u in (0,1], w in [0,1); z0 = sqrt(-2 ln u) cos(2 pi w),
 * z1 = sqrt(-2 ln u) sin(2 pi w).  Component k of particle i uses pair k/2,
 * slot k%2.  Layout out[i*dims + k] (the reference's random_displacement). */
void orc_philox_normals(uint64_t seed, uint64_t step, int64_t N, int32_t dims, double *out)
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int64_t i = 0; i < N; i++) {
        for (int pair = 0; pair * 2 < dims; pair++) {
            uint32_t ctr[4] = {(uint32_t)i, (uint32_t)pair, (uint32_t)step, (uint32_t)(step >> 32)};
            uint32_t o[4];
            orc_philox4x32_10(ctr, key, o);
            uint64_t a = ((uint64_t)o[0] << 21) | (o[1] >> 11);
            uint64_t b = ((uint64_t)o[2] << 21) | (o[3] >> 11);
            double u = ((double)a + 1.0) * 0x1.0p-53;
            double w = (double)b * 0x1.0p-53;
            double rad = sqrt(-2.0 * log(u));
            double ang = 2.0 * M_PI * w;
            out[i * dims + 2 * pair] = rad * cos(ang);
            if (2 * pair + 1 < dims) out[i * dims + 2 * pair + 1] = rad * sin(ang);
        }
    }
}

/* ------------------------------------------------------------------ */
/* fixtures: src/InitialConfiguration.jl, src/MC.jl                    */
/* ------------------------------------------------------------------ */

uint64_t orc_splitmix64(uint64_t *state)
{
    uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double orc_uniform01(uint64_t *state)
{
    return (double)(orc_splitmix64(state) >> 11) * 0x1.0p-53;
}

/* generate_diameters!(::Berthier), src/InitialConfiguration.jl:1-11: regular
 * inverse-CDF quantiles of P(D) ~ D^-3 on [sigma_min, sigma_min*sigma_ratio],
 * then a seeded Fisher-Yates shuffle (Julia's shuffle stream is not
 * reproducible outside Julia). */
void orc_generate_diameters_berthier(int64_t N, double sigma_ratio, uint64_t seed, double *D)
{
    double A = 1.0 / 2.0 + 1.0 / (sigma_ratio - 1.0);
    double smin = (1.0 + sigma_ratio) / (2.0 * sigma_ratio);
    double a = 1.0 / (2.0 * (double)N), b = 1.0 - 1.0 / (2.0 * (double)N);
    for (int64_t k = 0; k < N; k++) {
        double P = (N == 1) ? a : a + (double)k * (b - a) / (double)(N - 1);
        D[k] = sqrt(1.0 / (pow(smin, -2.0) - 2.0 * P / A));
    }
    uint64_t st = seed;
    for (int64_t k = N - 1; k > 0; k--) {
        int64_t j = (int64_t)(orc_splitmix64(&st) % (uint64_t)(k + 1));
        double t = D[k]; D[k] = D[j]; D[j] = t;
    }
}

/* find_random_initial_configuration! (src/InitialConfiguration.jl:43-114)
 * with do_MC_step! / do_translation_step! (src/MC.jl:21-47, 139-156) at
 * swap_probability 0: uniform random positions, then steps+1 sweeps of
 * Metropolis translations at kBT = 10 using find_energy over the full list,
 * rebuilding when a particle's displacement exceeds skin/2. */
int orc_random_initial_configuration(const orc_params *p0, double *r, double *D, orc_nlist *nl,
                                     int64_t steps, double max_disp, uint64_t seed,
                                     double *final_energy)
{
    orc_params p = *p0;
    p.kBT = 10.0;
    const int d = p.dims;
    const double L = p.box_size;
    uint64_t st = seed;
    (void)D;
    for (int64_t i = 0; i < p.N * d; i++) r[i] = orc_uniform01(&st) * L;
    int status = orc_update_neighbor_lists(&p, r, D, nl);
    double energy = orc_calculate_full_energy(&p, r, D, nl);
    double *disp = (double *)malloc(sizeof(double) * d * p.N);
    double h = p.skin / 2.0;
    for (int64_t s = 0; s <= steps; s++) {
        for (int64_t k = 0; k < d * p.N; k++)
            disp[k] = orc_uniform01(&st) * 2.0 * max_disp - max_disp;
        for (int64_t i = 0; i < p.N; i++) {
            (void)orc_uniform01(&st); /* rand() > swap_probability (always a translation) */
            double rold[3], rnew[3];
            for (int k = 0; k < d; k++) rold[k] = r[d * i + k];
            double e_old = orc_find_energy(&p, i, rold, D[i], r, D, nl);
            for (int k = 0; k < d; k++) {
                double x = rold[k] + disp[d * i + k];
                x -= floor(x / L) * L;
                rnew[k] = x;
            }
            double e_new = orc_find_energy(&p, i, rnew, D[i], r, D, nl);
            double dE = e_new - e_old;
            double bf = exp(-dE / p.kBT);
            if (bf > 1.0) bf = 1.0;
            if (bf > orc_uniform01(&st)) {
                double s2 = 0.0;
                for (int k = 0; k < d; k++) {
                    r[d * i + k] = rnew[k];
                    nl->disp[d * i + k] += disp[d * i + k];
                }
                s2 = nl->disp[d * i] * nl->disp[d * i] + nl->disp[d * i + 1] * nl->disp[d * i + 1];
                if (d == 3) s2 = s2 + nl->disp[d * i + 2] * nl->disp[d * i + 2];
                nl->disp2[i] = s2;
                energy += dE;
            }
            if (nl->disp2[i] > h * h) {
                int rc = orc_update_neighbor_lists(&p, r, D, nl);
                if (rc && !status) status = rc;
            }
        }
    }
    free(disp);
    if (final_energy) *final_energy = energy;
    return status;
}

/* ------------------------------------------------------------------ */
/* swap Monte Carlo: do_MC_step! (src/MC.jl:139-156) with               */
/* do_translation_step! (:21-47) and do_swap_step! (:67-110)            */
/* ------------------------------------------------------------------ */

/* the six uniforms in [0,1) of particle i in MC sweep `sweep`: counter
 * (i, 2 + k, sweep_lo, sweep_hi) for k = 0, 1, 2, key (seed_lo, seed_hi);
 * u[0] move choice, u[1] acceptance, u[2..4] the displacement components,
 * u[5] the swap partner */
void orc_mc_uniforms(uint64_t seed, uint64_t sweep, int64_t i, double u[6])
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (uint32_t k = 0; k < 3; k++) {
        uint32_t ctr[4] = {(uint32_t)i, 2u + k, (uint32_t)sweep, (uint32_t)(sweep >> 32)};
        uint32_t o[4];
        orc_philox4x32_10(ctr, key, o);
        u[2 * k] = (double)(((uint64_t)o[0] << 21) | (o[1] >> 11)) * 0x1.0p-53;
        u[2 * k + 1] = (double)(((uint64_t)o[2] << 21) | (o[3] >> 11)) * 0x1.0p-53;
    }
}

/* nsweeps calls of do_MC_step! on the system (r, D, nl with the full list).
 * Random numbers from orc_mc_uniforms(seed, sweep0 + s, i) instead of the
 * global generator; the displacement component is u * 2 * max_disp -
 * max_disp as populate_random_displacement_array! (src/AuxiliaryFunctions.jl:
 * 610-615); the swap partner is floor(u * N) (0-based), the evident intent of
 * the reference's ceil(Int64, rand()/N), which always gives particle 1.
 * counts[4] += {translations accepted, translations tried, swaps accepted,
 * swaps tried}; *dE_sum += the energy changes of accepted moves in order
 * (output.potential_energy += dE). */
int orc_mc_sweeps(const orc_params *p, double *r, double *D, orc_nlist *nl, int64_t nsweeps, double max_disp,
                  double swap_prob, uint64_t seed, uint64_t sweep0, int64_t counts[4], double *dE_sum)
{
    const int d = p->dims;
    const double L = p->box_size;
    const double h = p->skin / 2.0;
    int status = 0;
    for (int64_t s = 0; s < nsweeps; s++) {
        for (int64_t i = 0; i < p->N; i++) {
            double u[6];
            orc_mc_uniforms(seed, sweep0 + (uint64_t)s, i, u);
            if (u[0] > swap_prob) {  /* do_translation_step! */
                double rold[3] = {0, 0, 0}, rnew[3] = {0, 0, 0}, dr[3] = {0, 0, 0};
                for (int k = 0; k < d; k++) {
                    rold[k] = r[d * i + k];
                    dr[k] = u[2 + k] * 2.0 * max_disp - max_disp;
                }
                double e_old = orc_find_energy(p, i, rold, D[i], r, D, nl);
                for (int k = 0; k < d; k++) {
                    double x = rold[k] + dr[k];
                    x -= floor(x / L) * L;
                    rnew[k] = x;
                }
                double e_new = orc_find_energy(p, i, rnew, D[i], r, D, nl);
                double dE = e_new - e_old;
                double bf = exp(-dE / p->kBT);
                if (bf > 1.0) bf = 1.0;
                counts[1]++;
                if (bf > u[1]) {
                    counts[0]++;
                    for (int k = 0; k < d; k++) {
                        r[d * i + k] = rnew[k];
                        nl->disp[d * i + k] += dr[k];
                    }
                    double s2 = nl->disp[d * i] * nl->disp[d * i] + nl->disp[d * i + 1] * nl->disp[d * i + 1];
                    if (d == 3) s2 = s2 + nl->disp[d * i + 2] * nl->disp[d * i + 2];
                    nl->disp2[i] = s2;
                    *dE_sum += dE;
                }
                if (nl->disp2[i] > h * h) {
                    int rc = orc_update_neighbor_lists(p, r, D, nl);
                    if (rc && !status) status = rc;
                }
            } else {  /* do_swap_step! */
                int64_t j = (int64_t)(u[5] * (double)p->N);
                if (j >= p->N) j = p->N - 1;
                if (j == i) continue;
                const double Di = D[i], Dj = D[j];
                if (fabs(Di - Dj) > 0.2) continue;
                double ei_old = orc_find_energy(p, i, r + d * i, Di, r, D, nl);
                double ej_old = orc_find_energy(p, j, r + d * j, Dj, r, D, nl);
                D[i] = Dj;
                D[j] = Di;
                double ei_new = orc_find_energy(p, i, r + d * i, D[i], r, D, nl);
                double ej_new = orc_find_energy(p, j, r + d * j, D[j], r, D, nl);
                double dE = (ei_new + ej_new) - (ei_old + ej_old);
                double bf = exp(-dE / p->kBT);
                if (bf > 1.0) bf = 1.0;
                counts[3]++;
                if (bf > u[1]) {
                    counts[2]++;
                    *dE_sum += dE;
                } else {
                    D[i] = Di;
                    D[j] = Dj;
                }
            }
        }
    }
    return status;
}

/* Set-up only, no counterpart in the reference: capped steepest descent of
 * random starts, r += step_size*F with |dr_i| <= max_disp per particle, wrap,
 * displacement, rebuild on the skin trigger (the benchmark relaxes its
 * random initial positions this way; the reference uses MC at kBT = 10,
 * too slow for millions of particles). */
int orc_relax_capped(const orc_params *p, double *r, double *F, const double *D, orc_nlist *nl,
                     int64_t steps, double step_size, double max_disp)
{
    const int d = p->dims;
    const int64_t N = p->N;
    int st = orc_update_neighbor_lists(p, r, D, nl);
    for (int64_t it = 0; it < steps && !st; it++) {
        orc_pair_forces_only(p, r, D, nl, F);
        for (int64_t i = 0; i < N; i++) {
            double dr[3] = {0.0, 0.0, 0.0};
            double len2 = 0.0;
            for (int k = 0; k < d; k++) {
                dr[k] = step_size * F[d * i + k];
                len2 += dr[k] * dr[k];
            }
            const double len = sqrt(len2);
            if (!(len <= max_disp)) {
                const double sc = (len > 0.0 && isfinite(len)) ? max_disp / len : 0.0;
                for (int k = 0; k < d; k++) dr[k] *= sc;
            }
            drift_particle(p, i, dr, r, nl);
        }
        if (skin_exceeded(p, nl)) st = orc_update_neighbor_lists(p, r, D, nl);
    }
    return st;
}

/* find_inherent_structure, src/InherentStructure.jl:5-56 (steepest descent,
 * step v = F dt capped so that max |v| <= max_step_size).  Pair forces only
 * (the reference calls calculate_new_forces! with a Newtonian system, whose
 * random force is a no-op).  Returns 2 if max_iterations is exceeded. */
int orc_find_inherent_structure(const orc_params *p, double *r, double *v, double *F,
                                const double *D, orc_nlist *nl, double tolerance,
                                int64_t max_iterations, double max_step_size, double dt,
                                int64_t *iterations)
{
    const int d = p->dims;
    const int64_t N = p->N;
    double err = tolerance * 2.0;
    int st = orc_update_neighbor_lists(p, r, D, nl);
    int64_t it = 0;
    while (err > tolerance) {
        it += 1;
        if (it > max_iterations) { st = 2; break; }
        orc_pair_forces_only(p, r, D, nl, F);
        for (int64_t k = 0; k < d * N; k++) v[k] = F[k] * dt;
        double stepsize = 0.0;
        for (int64_t i = 0; i < N; i++) {
            double s = v[d * i] * v[d * i] + v[d * i + 1] * v[d * i + 1];
            if (d == 3) s = s + v[d * i + 2] * v[d * i + 2];
            double q = sqrt(s);
            if (q > stepsize) stepsize = q;
        }
        if (stepsize > max_step_size)
            for (int64_t k = 0; k < d * N; k++) v[k] *= max_step_size / stepsize;
        for (int64_t i = 0; i < N; i++) drift_particle(p, i, v + d * i, r, nl);
        if (skin_exceeded(p, nl)) {
            int rc = orc_update_neighbor_lists(p, r, D, nl);
            if (rc && !st) st = rc;
        }
        double maxforce = 0.0;
        for (int64_t i = 0; i < N; i++) {
            double s = F[d * i] * F[d * i] + F[d * i + 1] * F[d * i + 1];
            if (d == 3) s = s + F[d * i + 2] * F[d * i + 2];
            double q = sqrt(s);
            if (q > maxforce) maxforce = q;
        }
        err = maxforce > stepsize ? maxforce : stepsize;
    }
    if (iterations) *iterations = it;
    return st;
}
