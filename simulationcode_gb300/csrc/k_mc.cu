// k_mc.cu -- swap Monte Carlo on the device: do_MC_step! with its
// translation and swap moves (SimulationCode.jl src/MC.jl:21-156), for every
// replica of a context at once.
//
// The Markov chain stays the reference's: within a replica the particles
// are visited one after another in id order, each move is decided on the
// state the previous moves left.  Replicas are independent, so one warp runs
// one replica's chain; the warp's lanes share each move's energies
// (find_energy, src/AuxiliaryFunctions.jl:546-584, over the full Verlet
// list: berthier_inner_loop3/2 :381-444, LJ_inner_loop :477-507 and the
// generic 2D form) and a butterfly sum combines them in a fixed order.
// Arithmetic is FP64 in the reference's operation order.
//
// Random numbers: the six uniforms of particle i in sweep s come from
// Philox4x32-10 with counter (i, 2 + k, s) and the replica's seed (k = 0, 1,
// 2): move choice, acceptance, the displacement components, the swap
// partner (floor(u N), the evident intent of the reference's
// ceil(Int64, rand()/N), which always gives particle 1).
//
// A translation that takes the particle's displacement past skin/2 needs a
// list rebuild before the next move (src/MC.jl:147-149): the warp records
// where its sweep stands, requests the rebuild and stops; the host runs the
// rebuild sequence and launches the kernel again, and the chain continues.
#include "simmd_internal.cuh"

namespace simmd {

// pair energy of find_energy's inner loops (the FP64 energy of k_force.cu's
// pair code, the same operation order)
template <int DIM, int POT>
__device__ __forceinline__ double mc_pair_energy(const RepDesc& d, double r2, double Di, double Dj)
{
    if (POT == POT_BERTHIER) {
        const double md = dmul(dmul(dadd(Di, Dj), 0.5), dsub(1.0, dmul(d.zeta, fabs(dsub(Di, Dj)))));
        const double mds = dmul(md, md);
        if (dmul(d.rc2, mds) < r2) return 0.0;
        const double jx2 = ddiv(r2, mds);
        const double jx4 = dmul(jx2, jx2);
        const double xi12 = drcp(dmul(dmul(jx4, jx4), jx4));
        return dadd(dadd(dadd(xi12, dmul(d.c4, jx4)), dmul(d.c2, jx2)), d.c0);
    } else if (DIM == 3) {
        if (d.lj_cut2 < r2) return 0.0;
        const double xi2 = ddiv(d.sigma2, r2);
        const double xi6 = dmul(dmul(xi2, xi2), xi2);
        const double xi12 = dmul(xi6, xi6);
        return dsub(dmul(dmul(4.0, d.eps), dsub(xi12, xi6)), d.Uc);
    } else {
        if (!(d.lj_cut2 > r2)) return 0.0;
        const double y2 = ddiv(d.sigma4, r2);
        const double y4 = dmul(y2, y2);
        const double y6 = dmul(y2, y4);
        const double y12 = dmul(y6, y6);
        return dsub(dmul(dmul(4.0, d.eps), dsub(y12, y6)), d.Uc);
    }
}

template <int DIM>
__device__ __forceinline__ double mc_r2(const RepDesc& d, long long halfLb, const double* a, const double4_32a& pj)
{
    const double dx = min_image_f64(dsub(a[0], pj.x), halfLb, d.L);
    const double dy = min_image_f64(dsub(a[1], pj.y), halfLb, d.L);
    double r2 = dadd(dmul(dx, dx), dmul(dy, dy));
    if (DIM == 3) {
        const double dz = min_image_f64(dsub(a[2], pj.z), halfLb, d.L);
        r2 = dadd(r2, dmul(dz, dz));
    }
    return r2;
}

// the energies of the particle in slot s over its full list for two states
// (a: position pa, diameter Da; b: position pb, diameter Db, and neighbour
// slot sx, if >= 0, with diameter Dx instead of its own); every lane gets
// both sums
template <int DIM, int POT>
__device__ __forceinline__ void mc_energy2(const Batch& b, const RepDesc& d, const unsigned* nbr_full,
                                           const int* ncnt_full, long long s, const double* pa, double Da,
                                           const double* pb, double Db, long long sx, double Dx, double& ea,
                                           double& eb)
{
    const int lane = threadIdx.x & 31;
    const long long halfLb = __double_as_longlong(d.halfL);
    const int cnt = ncnt_full[s];
    double sa = 0.0, sb = 0.0;
    for (int k = lane; k < cnt; k += 32) {
        const long long j = (long long)(nbr_full[(size_t)k * (size_t)b.S + (size_t)s] & IDX_MASK);
        const double4_32a pj = b.s.posD[j];
        sa = dadd(sa, mc_pair_energy<DIM, POT>(d, mc_r2<DIM>(d, halfLb, pa, pj), Da, pj.w));
        sb = dadd(sb, mc_pair_energy<DIM, POT>(d, mc_r2<DIM>(d, halfLb, pb, pj), Db, j == sx ? Dx : pj.w));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sa = dadd(sa, __shfl_xor_sync(0xffffffffu, sa, o));
        sb = dadd(sb, __shfl_xor_sync(0xffffffffu, sb, o));
    }
    ea = sa;
    eb = sb;
}

__device__ __forceinline__ void mc_uniforms(unsigned long long seed, long long sweep, int i, double (&u)[6])
{
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint4 o = philox4x32_10(make_uint4((unsigned)i, 2u + (unsigned)k, (unsigned)sweep,
                                                 (unsigned)((unsigned long long)sweep >> 32)),
                                      make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
        u[2 * k] = (double)(((unsigned long long)o.x << 21) | (o.y >> 11)) * 0x1.0p-53;
        u[2 * k + 1] = (double)(((unsigned long long)o.z << 21) | (o.w >> 11)) * 0x1.0p-53;
    }
}

// min(1, exp(-dE/kBT)) > u: the reference's Metropolis test
__device__ __forceinline__ bool mc_accept(double dE, double kBT, double u)
{
    double bf = exp(ddiv(-dE, kBT));
    bf = bf > 1.0 ? 1.0 : bf;
    return bf > u;
}

template <int DIM, int POT>
__device__ void mc_chain(const Batch& b, const RepDesc& d, RepState& st, const unsigned* nbr_full,
                         const int* ncnt_full, double max_disp, double swap_prob)
{
    const int lane = threadIdx.x & 31;
    const Slots& S = b.s;  // the pointers are const, the arrays they point to are written
    const int N = d.n;
    while (st.mc_sweep < st.mc_target) {
        const long long sweep = st.mc_sweep;
        for (int i = st.mc_next; i < N; i++) {
            double u[6];
            mc_uniforms(d.seed, sweep, i, u);
            const long long si = S.inv[d.slot0 + i];
            const double4_32a pi = S.posD[si];
            const double ri[3] = {pi.x, pi.y, pi.z};
            if (u[0] > swap_prob) {  // do_translation_step! (src/MC.jl:21-47)
                double dr[3] = {0.0, 0.0, 0.0}, rn[3] = {pi.x, pi.y, pi.z};
#pragma unroll
                for (int k = 0; k < DIM; k++) {
                    dr[k] = dsub(dmul(dmul(u[2 + k], 2.0), max_disp), max_disp);
                    const double x = dadd(ri[k], dr[k]);
                    rn[k] = dsub(x, dmul(floor(ddiv(x, d.L)), d.L));
                }
                double eo, en;
                mc_energy2<DIM, POT>(b, d, nbr_full, ncnt_full, si, ri, pi.w, rn, pi.w, -1, 0.0, eo, en);
                const double dE = dsub(en, eo);
                const bool acc = mc_accept(dE, d.kBT, u[1]);
                bool rebuild = false;
                if (lane == 0) {
                    st.mc_counts[1] += 1;
                    if (acc) {
                        st.mc_counts[0] += 1;
                        st.mc_dE = dadd(st.mc_dE, dE);
                        S.posD[si] = make_double4_32a(rn[0], rn[1], rn[2], pi.w);
                        if (d.prec == PREC_FP32 || d.prune) S.rec[si] = fix_rec(rn[0], rn[1], rn[2], pi.w, d);
                        if (d.prec == PREC_FP64) {
                            const double ux = dadd(S.ux[si], dr[0]), uy = dadd(S.uy[si], dr[1]);
                            S.ux[si] = ux;
                            S.uy[si] = uy;
                            double u2 = dadd(dmul(ux, ux), dmul(uy, uy));
                            if (DIM == 3) {
                                const double uz = dadd(S.uz[si], dr[2]);
                                S.uz[si] = uz;
                                u2 = dadd(u2, dmul(uz, uz));
                            }
                            rebuild = u2 > d.skin_half2;
                        } else {  // split precision: the fixed-point displacement since the rebuild
                            rebuild = fix_dist2(S.rec[si], S.recb[si]) > d.skin_thr;
                        }
                    }
                    if (rebuild) {  // src/MC.jl:147-149: rebuild before the next move
                        st.mc_next = i + 1;
                        st.force_rebuild = 1;
                    }
                }
                __syncwarp();
                if (__shfl_sync(0xffffffffu, rebuild ? 1 : 0, 0)) return;
            } else {  // do_swap_step! (src/MC.jl:67-110)
                int j = (int)(u[5] * (double)N);
                j = j >= N ? N - 1 : j;
                if (j == i) continue;
                const long long sj = S.inv[d.slot0 + j];
                const double4_32a pj = S.posD[sj];
                const double Di = pi.w, Dj = pj.w;
                if (fabs(dsub(Di, Dj)) > 0.2) continue;
                const double rj[3] = {pj.x, pj.y, pj.z};
                double ei_old, ei_new, ej_old, ej_new;
                mc_energy2<DIM, POT>(b, d, nbr_full, ncnt_full, si, ri, Di, ri, Dj, sj, Di, ei_old, ei_new);
                mc_energy2<DIM, POT>(b, d, nbr_full, ncnt_full, sj, rj, Dj, rj, Di, si, Dj, ej_old, ej_new);
                const double dE = dsub(dadd(ei_new, ej_new), dadd(ei_old, ej_old));
                const bool acc = mc_accept(dE, d.kBT, u[1]);
                if (lane == 0) {
                    st.mc_counts[3] += 1;
                    if (acc) {
                        st.mc_counts[2] += 1;
                        st.mc_dE = dadd(st.mc_dE, dE);
                        S.posD[si] = make_double4_32a(pi.x, pi.y, pi.z, Dj);
                        S.posD[sj] = make_double4_32a(pj.x, pj.y, pj.z, Di);
                        if (d.prec == PREC_FP32 || d.prune) {
                            S.rec[si].d = d2f_rn(Dj);
                            S.rec[sj].d = d2f_rn(Di);
                        }
                    }
                }
                __syncwarp();
            }
        }
        if (lane == 0) {
            st.mc_next = 0;
            st.mc_sweep += 1;
        }
        __syncwarp();
    }
}

// one warp per replica; returns at the end of the requested sweeps or at a
// rebuild request
__global__ void __launch_bounds__(128) k_mc_sweeps(Batch b, const unsigned* nbr_full, const int* ncnt_full,
                                                   double max_disp, double swap_prob)
{
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= b.nreps) return;
    const RepDesc& d = b.desc[r];
    RepState& st = b.state[r];
    if (!d.active || !st.mc_active || st.force_rebuild || st.nonfinite) return;
    if (d.dims == 3) {
        if (d.pot == POT_BERTHIER) mc_chain<3, POT_BERTHIER>(b, d, st, nbr_full, ncnt_full, max_disp, swap_prob);
        else mc_chain<3, POT_LJ>(b, d, st, nbr_full, ncnt_full, max_disp, swap_prob);
    } else {
        if (d.pot == POT_BERTHIER) mc_chain<2, POT_BERTHIER>(b, d, st, nbr_full, ncnt_full, max_disp, swap_prob);
        else mc_chain<2, POT_LJ>(b, d, st, nbr_full, ncnt_full, max_disp, swap_prob);
    }
}

void launch_mc_sweeps_impl(const Batch& b, const LaunchCfg& lc, const unsigned* nbr_full, const int* ncnt_full,
                           double max_disp, double swap_prob)
{
    const int wpb = 4;
    k_mc_sweeps<<<(b.nreps + wpb - 1) / wpb, 32 * wpb, 0, lc.stream>>>(b, nbr_full, ncnt_full, max_disp, swap_prob);
    if (lc.launches) *lc.launches += 1;
}

}  // namespace simmd
