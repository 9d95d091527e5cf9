// k_force.cu -- pair forces, energies and virial for LJ and the polydisperse
// non-additive soft-sphere ("Berthier") potential, 2D and 3D, with the
// Langevin/Brownian random force and the second velocity half-kick fused in.
//
// Reference (SimulationCode.jl):
//   calculate_new_forces!              src/MD.jl:262-316
//   compute_forces_berthier_3d / _2d   src/MD.jl:85-137, 194-238
//   compute_forces_lj_3d               src/MD.jl:140-191
//   generic fallback (2D LJ)           src/MD.jl:291-309
//   add_new_random_force!              src/MD.jl:30-82
//   kick2 + centre-of-mass removal     src/MD.jl:528-542
//   find_energy inner loops            src/AuxiliaryFunctions.jl:381-444, 477-507, 571-581
//
// One persistent kernel per launch: blocks pull 128-slot tiles from an atomic
// work queue; a tile belongs to one replica, so (precision, dims, potential,
// dynamics) are uniform per block.  T threads per particle split the
// particle's list (interleaved ELL) and combine with __shfl_xor.  Every pair
// is visited from both sides (no atomics, deterministic sums).
//
// FP64 path: the reference's per-pair operation order with explicit
// round-to-nearest intrinsics, so each pair force is bit-identical to the
// reference expression; only the order of the per-particle sum differs.
// FP32 split path: pair arithmetic in FP32 on cell-relative FP32 offsets plus
// an exact integer cell shift carried in the list entry; per-particle sums in
// FP32, converted to FP64 for integration.
#include "simmd_internal.cuh"
#include "simmd_reduce.cuh"

namespace simmd {

template <int DIM, int POT, bool EN>
__device__ __forceinline__ void pairs_f64(const Batch& b, const RepDesc& d, long long i, int sub, int T,
                                          const double4_32a pi, int cnt, double& fx, double& fy, double& fz,
                                          double& e, double& w)
{
    const long long halfLb = __double_as_longlong(d.halfL);
    const double L = d.L, rc2 = d.rc2;
    const unsigned* __restrict__ nbr = b.s.nbr;
    const double4_32a* __restrict__ posD = b.s.posD;
    for (int n = sub; n < cnt; n += T) {
        const unsigned ent = __ldg(nbr + nbr_addr(n, i, T, b.S));
        const double4_32a pj = posD[ent & IDX_MASK];
        const double dx = min_image_f64(dsub(pi.x, pj.x), halfLb, L);
        const double dy = min_image_f64(dsub(pi.y, pj.y), halfLb, L);
        double dz = 0.0, r2;
        if (DIM == 3) {
            dz = min_image_f64(dsub(pi.z, pj.z), halfLb, L);
            r2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
        } else {
            r2 = dadd(dmul(dx, dx), dmul(dy, dy));
        }
        double Fr = 0.0, V = 0.0;
        if (POT == POT_BERTHIER) {
            const double md = dmul(dmul(dadd(pi.w, pj.w), 0.5), dsub(1.0, dmul(d.zeta, fabs(dsub(pi.w, pj.w)))));
            const double mds = dmul(md, md);
            const bool out = dmul(rc2, mds) < r2;
            const double inv = drcp(mds);
            const double ix2 = dmul(r2, inv);
            const double ix4 = dmul(ix2, ix2);
            const double xi14 = drcp(dmul(dmul(dmul(ix4, ix4), ix4), ix2));
            Fr = out ? 0.0 : dmul(dmul(-2.0, inv), dsub(dadd(d.c2, dmul(dmul(2.0, d.c4), ix2)), dmul(6.0, xi14)));
            if (EN && !out) {  // berthier_inner_loop3/2: invxi2 = rij2 / mean_d2
                const double jx2 = ddiv(r2, mds);
                const double jx4 = dmul(jx2, jx2);
                const double xi12 = drcp(dmul(dmul(jx4, jx4), jx4));
                V = dadd(dadd(dadd(xi12, dmul(d.c4, jx4)), dmul(d.c2, jx2)), d.c0);
            }
        } else if (DIM == 3) {  // compute_forces_lj_3d / LJ_inner_loop
            const double xi2 = ddiv(d.sigma2, r2);
            const double xi6 = dmul(dmul(xi2, xi2), xi2);
            const double xi12 = dmul(xi6, xi6);
            Fr = (rc2 < r2) ? 0.0 : ddiv(dmul(d.eps, dsub(dmul(48.0, xi12), dmul(24.0, xi6))), r2);
            if (EN && !(d.lj_cut2 < r2)) V = dsub(dmul(dmul(4.0, d.eps), dsub(xi12, xi6)), d.Uc);
        } else {  // generic path: mean_d = find_mean_D = sigma^2, squared; strict '>'
            const double mds = d.sigma4;
            if (d.lj_cut2 > r2) {
                const double inv = drcp(r2);
                const double xi2 = dmul(mds, inv);
                const double xi6 = dmul(dmul(xi2, xi2), xi2);
                const double xi12 = dmul(xi6, xi6);
                Fr = dmul(dmul(d.eps, dsub(dmul(48.0, xi12), dmul(24.0, xi6))), inv);
                if (EN) {
                    const double y2 = ddiv(mds, r2);
                    const double y4 = dmul(y2, y2);
                    const double y6 = dmul(y2, y4);
                    const double y12 = dmul(y6, y6);
                    V = dsub(dmul(dmul(4.0, d.eps), dsub(y12, y6)), d.Uc);
                }
            }
        }
        fx = dadd(fx, dmul(Fr, dx));
        fy = dadd(fy, dmul(Fr, dy));
        if (DIM == 3) fz = dadd(fz, dmul(Fr, dz));
        if (EN) {
            e = dadd(e, V);
            w = dadd(w, dmul(Fr, r2));
        }
    }
}

template <int DIM, int POT, bool EN>
__device__ __forceinline__ void pairs_f32(const Batch& b, const RepDesc& d, long long i, int sub, int T,
                                          const float4 oi, int cnt, float& fx, float& fy, float& fz,
                                          float& e, float& w)
{
    const float csf = d.csf, Lf = d.Lf, hL = d.halfLf;
    const unsigned* __restrict__ nbr = b.s.nbr;
    const float4* __restrict__ off = b.s.off;
    for (int n = sub; n < cnt; n += T) {
        const unsigned ent = __ldg(nbr + nbr_addr(n, i, T, b.S));
        const float4 oj = __ldg(off + (ent & IDX_MASK));
        const unsigned code = ent >> IDX_BITS;
        const float dx = min_image_f32(oi.x - oj.x + (float)((int)(code & 3u) - 1) * csf, hL, Lf);
        const float dy = min_image_f32(oi.y - oj.y + (float)((int)((code >> 2) & 3u) - 1) * csf, hL, Lf);
        float dz = 0.0f, r2;
        if (DIM == 3) {
            dz = min_image_f32(oi.z - oj.z + (float)((int)((code >> 4) & 3u) - 1) * csf, hL, Lf);
            r2 = dx * dx + dy * dy + dz * dz;
        } else {
            r2 = dx * dx + dy * dy;
        }
        float Fr = 0.0f, V = 0.0f;
        if (POT == POT_BERTHIER) {
            const float md = (oi.w + oj.w) * 0.5f * (1.0f - d.zetaf * fabsf(oi.w - oj.w));
            const float mds = md * md;
            const float inv = __fdividef(1.0f, mds);
            const float ix2 = r2 * inv;
            const float ix4 = ix2 * ix2;
            const float xi12 = __fdividef(1.0f, ix4 * ix4 * ix4);
            const float xi14 = xi12 * __fdividef(1.0f, ix2);
            const bool in = r2 <= d.rc2f * mds;
            Fr = in ? -2.0f * inv * (d.c2f + 2.0f * d.c4f * ix2 - 6.0f * xi14) : 0.0f;
            if (EN && in) V = xi12 + d.c4f * ix4 + d.c2f * ix2 + d.c0f;
        } else {
            const float inv = __fdividef(1.0f, r2);
            const float xi2 = (DIM == 3 ? d.sigma2f : d.sigma4f) * inv;
            const float xi6 = xi2 * xi2 * xi2;
            const float xi12 = xi6 * xi6;
            const bool in = (DIM == 3) ? (r2 <= d.cut2f) : (r2 < d.cut2f);
            Fr = in ? d.epsf * (48.0f * xi12 - 24.0f * xi6) * inv : 0.0f;
            if (EN && in) V = 4.0f * d.epsf * (xi12 - xi6) - d.Ucf;
        }
        fx += Fr * dx;
        fy += Fr * dy;
        if (DIM == 3) fz += Fr * dz;
        if (EN) {
            e += V;
            w += Fr * r2;
        }
    }
}

__device__ __forceinline__ void particle_noise(const RepDesc& d, RepState& st, int oid, double xi[3])
{
    const long long step = st.step;
    xi[0] = xi[1] = xi[2] = 0.0;
    if (d.noise_mode == NOISE_HOST) {
        long long k = step - d.noise_step0;
        if (k < 0 || k >= d.noise_nsteps) {
            st.noise_range_error = 1;
            return;
        }
        const double* q = d.host_noise + (k * d.n + oid) * d.dims;
        for (int c = 0; c < d.dims; c++) xi[c] = q[c];
    } else if (d.prec == PREC_FP64) {
        double z1;
        normal_pair_f64(d.seed, step, oid, 0, xi[0], xi[1]);
        if (d.dims == 3) normal_pair_f64(d.seed, step, oid, 1, xi[2], z1);
    } else {
        float a, c, z1;
        normal_pair_f32(d.seed, step, oid, 0, a, c);
        xi[0] = a;
        xi[1] = c;
        if (d.dims == 3) {
            normal_pair_f32(d.seed, step, oid, 1, a, z1);
            xi[2] = a;
        }
    }
}

template <bool EN>
__device__ __forceinline__ void particle_pairs(const Batch& b, const RepDesc& d, long long i, int sub, int T,
                                               double& fx, double& fy, double& fz, double& e, double& w)
{
    const int cnt = b.s.ncnt[i];
    if (d.prec == PREC_FP64) {
        const double4_32a pi = b.s.posD[i];
        if (d.dims == 3) {
            if (d.pot == POT_BERTHIER) pairs_f64<3, POT_BERTHIER, EN>(b, d, i, sub, T, pi, cnt, fx, fy, fz, e, w);
            else pairs_f64<3, POT_LJ, EN>(b, d, i, sub, T, pi, cnt, fx, fy, fz, e, w);
        } else {
            if (d.pot == POT_BERTHIER) pairs_f64<2, POT_BERTHIER, EN>(b, d, i, sub, T, pi, cnt, fx, fy, fz, e, w);
            else pairs_f64<2, POT_LJ, EN>(b, d, i, sub, T, pi, cnt, fx, fy, fz, e, w);
        }
    } else {
        const float4 oi = b.s.off[i];
        float gx = 0.f, gy = 0.f, gz = 0.f, ge = 0.f, gw = 0.f;
        if (d.dims == 3) {
            if (d.pot == POT_BERTHIER) pairs_f32<3, POT_BERTHIER, EN>(b, d, i, sub, T, oi, cnt, gx, gy, gz, ge, gw);
            else pairs_f32<3, POT_LJ, EN>(b, d, i, sub, T, oi, cnt, gx, gy, gz, ge, gw);
        } else {
            if (d.pot == POT_BERTHIER) pairs_f32<2, POT_BERTHIER, EN>(b, d, i, sub, T, oi, cnt, gx, gy, gz, ge, gw);
            else pairs_f32<2, POT_LJ, EN>(b, d, i, sub, T, oi, cnt, gx, gy, gz, ge, gw);
        }
        fx = gx; fy = gy; fz = gz; e = ge; w = gw;
    }
}

template <int MODE>
__global__ void __launch_bounds__(512) k_force(Batch b, double* epp)
{
    constexpr bool EN = (MODE == FMODE_ENERGY || MODE == FMODE_STEP_ENERGY);
    constexpr bool STEP = (MODE == FMODE_STEP || MODE == FMODE_STEP_ENERGY);
    __shared__ int s_tile;
    __shared__ int s_flag;
    __shared__ double s_part[32 * 5];
    const int T = b.tpp;
    const int tid = threadIdx.x;
    const int p = tid / T, sub = tid - p * T;
    for (;;) {
        if (tid == 0) s_tile = atomicAdd(&b.queue[0], 1);
        __syncthreads();
        const int t = s_tile;
        __syncthreads();
        if (t >= b.ntiles) break;
        const int r = b.tile_rep[t];
        if (r < 0) continue;
        const RepDesc& d = b.desc[r];
        RepState& st = b.state[r];
        const long long i = (long long)t * TILE + p;
        const bool real = i < d.slot0 + d.n;
        double fx = 0.0, fy = 0.0, fz = 0.0, e = 0.0, w = 0.0;
        if (real) particle_pairs<EN>(b, d, i, sub, T, fx, fy, fz, e, w);
        for (int o = T >> 1; o > 0; o >>= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, o);
            fy += __shfl_xor_sync(0xffffffffu, fy, o);
            fz += __shfl_xor_sync(0xffffffffu, fz, o);
            if (EN) {
                e += __shfl_xor_sync(0xffffffffu, e, o);
                w += __shfl_xor_sync(0xffffffffu, w, o);
            }
        }
        double pv[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        const bool noise = d.dyn != DYN_NEWTONIAN && MODE != FMODE_ENERGY && d.relax_cap == 0.0;
        if (sub == 0 && real) {
            if (EN) {
                pv[3] = e;
                pv[4] = w;
                if (epp) epp[i] = e / 2.0;
            }
            if (MODE != FMODE_ENERGY) {
                double Fx = fx, Fy = fy, Fz = fz;
                double vx = 0.0, vy = 0.0, vz = 0.0;
                const bool nl = d.dyn != DYN_BROWNIAN;
                if (nl) {
                    vx = b.s.vx[i];
                    vy = b.s.vy[i];
                    if (d.dims == 3) vz = b.s.vz[i];
                }
                if (noise) {
                    double xi[3];
                    particle_noise(d, st, b.s.orig[i], xi);
                    if (d.dyn == DYN_LANGEVIN) {
                        const double mg = -d.gamma;
                        Fx = dadd(Fx, dadd(dmul(mg, vx), dmul(d.noise_factor, xi[0])));
                        Fy = dadd(Fy, dadd(dmul(mg, vy), dmul(d.noise_factor, xi[1])));
                        if (d.dims == 3) Fz = dadd(Fz, dadd(dmul(mg, vz), dmul(d.noise_factor, xi[2])));
                    } else {
                        Fx = dadd(Fx, dmul(d.noise_factor, xi[0]));
                        Fy = dadd(Fy, dmul(d.noise_factor, xi[1]));
                        if (d.dims == 3) Fz = dadd(Fz, dmul(d.noise_factor, xi[2]));
                    }
                }
                b.s.fx[i] = Fx;
                b.s.fy[i] = Fy;
                if (d.dims == 3) b.s.fz[i] = Fz;
                if (STEP) {
                    if (nl) {  // kick2 (src/MD.jl:529-531)
                        vx = dadd(vx, ddiv(dmul(d.dt, Fx), d.two_m));
                        vy = dadd(vy, ddiv(dmul(d.dt, Fy), d.two_m));
                        b.s.vx[i] = vx;
                        b.s.vy[i] = vy;
                        if (d.dims == 3) {
                            vz = dadd(vz, ddiv(dmul(d.dt, Fz), d.two_m));
                            b.s.vz[i] = vz;
                        }
                        pv[0] = vx; pv[1] = vy; pv[2] = vz;
                    } else {
                        pv[0] = Fx; pv[1] = Fy; pv[2] = Fz;
                    }
                }
            }
        }
        double out[5];
        if (tile_reduce<5>(b, t, d, st, pv, out, s_part, &s_flag) && tid == 0) {
            const double nd = (double)d.n;
            if (STEP) {
                if (d.dyn == DYN_BROWNIAN) {
                    st.fmean[0] = ddiv(out[0], nd);
                    st.fmean[1] = ddiv(out[1], nd);
                    st.fmean[2] = ddiv(out[2], nd);
                } else {
                    st.vmean[0] = ddiv(out[0], nd);
                    st.vmean[1] = ddiv(out[1], nd);
                    st.vmean[2] = ddiv(out[2], nd);
                }
            }
            if (EN) {
                st.epot = out[3] / 2.0;
                st.virial = out[4] / 2.0;
            }
            if (noise) st.step += 1;
        }
    }
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&b.queue[1], 1) == (int)gridDim.x - 1) {
            b.queue[0] = 0;
            b.queue[1] = 0;
        }
    }
}

int force_blocks_per_sm(int T, int mode)
{
    int nb = 0;
    const int threads = TILE * T;
    switch (mode) {
        case FMODE_STEP: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force<FMODE_STEP>, threads, 0); break;
        case FMODE_FORCES: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force<FMODE_FORCES>, threads, 0); break;
        case FMODE_ENERGY: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force<FMODE_ENERGY>, threads, 0); break;
        default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force<FMODE_STEP_ENERGY>, threads, 0); break;
    }
    return nb > 0 ? nb : 1;
}

void launch_force_impl(const Batch& b, const LaunchCfg& lc, int mode, int grid, double* epp)
{
    const int threads = TILE * b.tpp;
    switch (mode) {
        case FMODE_STEP: k_force<FMODE_STEP><<<grid, threads, 0, lc.stream>>>(b, epp); break;
        case FMODE_FORCES: k_force<FMODE_FORCES><<<grid, threads, 0, lc.stream>>>(b, epp); break;
        case FMODE_ENERGY: k_force<FMODE_ENERGY><<<grid, threads, 0, lc.stream>>>(b, epp); break;
        default: k_force<FMODE_STEP_ENERGY><<<grid, threads, 0, lc.stream>>>(b, epp); break;
    }
    if (lc.launches) *lc.launches += 1;
}

}  // namespace simmd
