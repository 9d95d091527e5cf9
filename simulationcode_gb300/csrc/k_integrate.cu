// k_integrate.cu -- O(N) streaming kernels of the time step and the host <->
// slot-layout transfers.
//
// Reference (SimulationCode.jl):
//   kick1 / drift / wrap / displacement  src/MD.jl:510-522
//   skin trigger max|disp|^2 > (skin/2)^2 src/MD.jl:523-525 (one atomicMax per warp)
//   centre-of-mass removal               src/MD.jl:532-542 (applied lazily: the vmean
//                                        computed by the force pass is subtracted at the
//                                        start of the next kick1, or by finalize)
//   temperature rescale                  src/MD.jl:543-553, 391-402
//   Brownian update (as intended)        src/MD.jl:444-470
//   find_kinetic_energy                  src/AuxiliaryFunctions.jl:57-65
// All FP64 arithmetic uses explicit round-to-nearest intrinsics in the
// reference's operation order.
#include "simmd_internal.cuh"
#include "simmd_reduce.cuh"

namespace simmd {

// rnew - floor(rnew/L)*L (src/MD.jl:520) with floor(RN(rnew/L)) decided by
// comparisons against 0 and wrap_hi = min{x : RN(x/L) >= 1}: bit-identical to
// the divide for |dr| < L, no FP64 divide on the path
__device__ __forceinline__ double wrap_coord(double x, const RepDesc& d)
{
    // the common case 0 <= x < wrap_hi decided on the bit pattern (integer
    // pipe; non-negative doubles order as integers, x < 0 has the sign bit)
    const long long bits = __double_as_longlong(x);
    if (bits >= 0 && bits < __double_as_longlong(d.wrap_hi)) return x;
    if (x < 0.0 && x >= -d.L) return dsub(x, -d.L);
    if (x >= d.wrap_hi && x < 2.0 * d.wrap_hi) return dsub(x, d.L);  // RN(x/L) in [1, 2)
    return dsub(x, dmul(floor(ddiv(x, d.L)), d.L));
}

// v + dt*F/(2m); one multiply when 2m is a power of two (exact scaling)
__device__ __forceinline__ double half_kick(double v, double F, const RepDesc& d)
{
    if (d.two_m_pow2) return dadd(v, dmul(d.dt_over_two_m, F));
    return dadd(v, ddiv(dmul(d.dt, F), d.two_m));
}

// r += dr with the reference wrap rnew - floor(rnew/L)*L, displacement,
// fixed-point record refresh.  Returns the skin-trigger key: FP64 replicas
// the bits of |disp|^2 (the reference's accumulated displacement, its
// rounding); split-precision replicas the fixed-point |X - X_rebuild|^2,
// exact, with no FP64 displacement arithmetic.  d2in: the fixed-point
// |X - X_prune|^2 when the context keeps inner lists; bad: a non-finite
// position or displacement
__device__ __forceinline__ unsigned long long drift_slot(const Batch& b, const RepDesc& d, long long i, double drx,
                                                         double dry, double drz, unsigned long long& d2in,
                                                         bool& bad)
{
    const Slots& S = b.s;
    unsigned long long key = 0ull;
    if (d.prec == PREC_FP64) {  // the reference's rounding of sum(abs2, disp)
        double ux = dadd(S.ux[i], drx), uy = dadd(S.uy[i], dry), uz = 0.0;
        S.ux[i] = ux;
        S.uy[i] = uy;
        double u2 = dadd(dmul(ux, ux), dmul(uy, uy));
        if (d.dims == 3) {
            uz = dadd(S.uz[i], drz);
            S.uz[i] = uz;
            u2 = dadd(u2, dmul(uz, uz));
        }
        key = (unsigned long long)__double_as_longlong(u2);
        bad = nonfinite_bits(u2);
    }
    double4_32a p = S.posD[i];
    const double x = wrap_coord(dadd(p.x, drx), d);
    const double y = wrap_coord(dadd(p.y, dry), d);
    const double z = (d.dims == 3) ? wrap_coord(dadd(p.z, drz), d) : p.z;
    S.posD[i] = make_double4_32a(x, y, z, p.w);
    if (d.prec == PREC_FP32 || d.prune) {  // the record, rebuilt from the position (no read)
        const FixRec q = fix_rec(x, y, z, p.w, d);
        S.rec[i] = q;
        if (d.prec == PREC_FP32) {
            key = fix_dist2(q, S.recb[i]);
            bad = nonfinite_bits(x) || nonfinite_bits(y) || nonfinite_bits(z);
        }
        if (d.prune) d2in = fix_dist2(q, S.recp[i]);
    }
    return key;
}

// block-level max of the skin-trigger key (FP64: non-negative doubles order
// as integers) and of the fixed-point displacement since the last prune,
// one atomic per tile and only when it raises the replica's max
__device__ __forceinline__ void block_max_to_state(unsigned long long bits, bool bad, unsigned long long d2in,
                                                   const RepDesc& d, RepState& st, unsigned long long* s_max)
{
    if (bad) {
        st.nonfinite = 1;
        bits = 0x7ff0000000000000ull;  // above every threshold of either kind
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long y = __shfl_xor_sync(0xffffffffu, bits, o);
        bits = y > bits ? y : bits;
        if (d.prune) {
            y = __shfl_xor_sync(0xffffffffu, d2in, o);
            d2in = y > d2in ? y : d2in;
        }
    }
    const int w = threadIdx.x >> 5;
    constexpr int NW = TILE / 32;
    if ((threadIdx.x & 31) == 0) {
        s_max[w] = bits;
        s_max[NW + w] = d2in;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = s_max[0], mi = s_max[NW];
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) {
            m = s_max[k] > m ? s_max[k] : m;
            mi = s_max[NW + k] > mi ? s_max[NW + k] : mi;
        }
        if (m > *(volatile unsigned long long*)&st.maxdisp2) atomicMax(&st.maxdisp2, m);
        if (d.prune && mi > *(volatile unsigned long long*)&st.maxdisp_in) atomicMax(&st.maxdisp_in, mi);
    }
    __syncthreads();
}

// the displacement since the last rebuild of slot s, component k: FP64
// replicas the accumulated one, split replicas the fixed-point difference
// X - X_rebuild times u
__device__ __forceinline__ double slot_disp(const Slots& S, const RepDesc& d, long long s, int k)
{
    if (d.prec == PREC_FP64) return k == 0 ? S.ux[s] : (k == 1 ? S.uy[s] : S.uz[s]);
    const FixRec q = S.rec[s], q0 = S.recb[s];
    const unsigned a = k == 0 ? q.x : (k == 1 ? q.y : q.z), a0 = k == 0 ? q0.x : (k == 1 ? q0.y : q0.z);
    return dmul((double)(int)(a - a0), d.fix_ud);
}

// blocks per SM the position updates are compiled for (registers): more
// warps in flight hide the FP64 and memory latency of these streaming passes
#ifndef SIMMD_UPD_MINB
#define SIMMD_UPD_MINB 16
#endif

// kick1 + drift for Newtonian / Langevin replicas (src/MD.jl:510-522)
__global__ void __launch_bounds__(TILE, SIMMD_UPD_MINB) k_kick_drift(Batch b)
{
    __shared__ unsigned long long s_max[2 * (TILE / 32)];
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        int r = b.tile_rep[t];
        if (r < 0) continue;
        const RepDesc& d = b.desc[r];
        if (d.dyn == DYN_BROWNIAN) continue;
        RepState& st = b.state[r];
        long long i = (long long)t * TILE + threadIdx.x;
        unsigned long long u2 = 0ull, d2in = 0ull;
        bool bad = false;
        if (i < d.slot0 + d.n) {
            const Slots& S = b.s;
            const double vs = st.vscale;
            // the rescale multiply only when a rescale is pending (x * 1.0 == x)
            const bool scale = __double_as_longlong(vs) != 0x3ff0000000000000ll;
            double vx = dsub(S.vx[i], st.vmean[0]);
            double vy = dsub(S.vy[i], st.vmean[1]);
            if (scale) {
                vx = dmul(vx, vs);
                vy = dmul(vy, vs);
            }
            vx = half_kick(vx, S.fx[i], d);
            vy = half_kick(vy, S.fy[i], d);
            S.vx[i] = vx;
            S.vy[i] = vy;
            double vz = 0.0;
            if (d.dims == 3) {
                vz = dsub(S.vz[i], st.vmean[2]);
                if (scale) vz = dmul(vz, vs);
                vz = half_kick(vz, S.fz[i], d);
                S.vz[i] = vz;
            }
            u2 = drift_slot(b, d, i, dmul(d.dt, vx), dmul(d.dt, vy), dmul(d.dt, vz), d2in, bad);
        }
        block_max_to_state(u2, bad, d2in, d, st, s_max);
    }
}

// set-up relaxation: |dr| <= cap per particle (out of line: it runs only
// during the relaxation and would otherwise hold registers of the hot path)
__device__ __noinline__ void relax_clamp(double& drx, double& dry, double& drz, double cap)
{
    double m = fmax(fabs(drx), fmax(fabs(dry), fabs(drz)));
    if (m > 0.0) {
        double qx = drx / m, qy = dry / m, qz = drz / m;
        double len = m * sqrt(qx * qx + qy * qy + qz * qz);
        if (!(len <= cap)) {
            double sc = cap / len;
            drx = isfinite(sc) ? drx * sc : 0.0;
            dry = isfinite(sc) ? dry * sc : 0.0;
            drz = isfinite(sc) ? drz * sc : 0.0;
            if (!isfinite(len)) {
                drx = qx * cap;
                dry = qy * cap;
                drz = qz * cap;
            }
        }
    }
}

// Brownian position update (src/MD.jl:444-467 as intended): dr = (dt/gamma)
// (F - <F>), displacement, wrap.  F itself is left as computed (the mean
// subtraction is applied again when F is downloaded), saving a store.
// FP64 replicas: the reference's rounding, (dt/gamma)*(F - <F>); split
// precision: one fused multiply-add (the force is FP32-accurate anyway).
__global__ void __launch_bounds__(TILE, SIMMD_UPD_MINB) k_brownian_update(Batch b)
{
    __shared__ unsigned long long s_max[2 * (TILE / 32)];
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        int r = b.tile_rep[t];
        if (r < 0) continue;
        const RepDesc& d = b.desc[r];
        if (d.dyn != DYN_BROWNIAN) continue;
        RepState& st = b.state[r];
        long long i = (long long)t * TILE + threadIdx.x;
        unsigned long long u2 = 0ull, d2in = 0ull;
        bool bad = false;
        if (i < d.slot0 + d.n) {
            const Slots& S = b.s;
            const double c = d.dt_over_gamma;
            double drx, dry, drz = 0.0;
            if (d.prec == PREC_FP64) {
                drx = dmul(c, dsub(S.fx[i], st.fmean[0]));
                dry = dmul(c, dsub(S.fy[i], st.fmean[1]));
                if (d.dims == 3) drz = dmul(c, dsub(S.fz[i], st.fmean[2]));
            } else {
                drx = fma(c, S.fx[i], st.cfmean[0]);
                dry = fma(c, S.fy[i], st.cfmean[1]);
                if (d.dims == 3) drz = fma(c, S.fz[i], st.cfmean[2]);
            }
            if (d.relax_cap > 0.0) relax_clamp(drx, dry, drz, d.relax_cap);
            u2 = drift_slot(b, d, i, drx, dry, drz, d2in, bad);
        }
        block_max_to_state(u2, bad, d2in, d, st, s_max);
    }
}

// ---------------------------------------------------------------------------
// inherent-structure minimiser (src/InherentStructure.jl:5-56)
// ---------------------------------------------------------------------------
__global__ void k_min_reset(Batch b)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= b.nreps) return;
    RepState& st = b.state[r];
    st.min_fmax = 0ull;
    st.min_step = 0ull;
}

// max_i |F_i| and max_i |F_i dt| (stepsize before scaling), the reference's
// rounding: v = F*dt, |v| = sqrt(v.v)
__global__ void k_min_max(Batch b, double dt)
{
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const int r = b.tile_rep[t];
        if (r < 0) continue;
        const RepDesc& d = b.desc[r];
        RepState& st = b.state[r];
        if (!st.min_active || st.min_done) continue;
        const long long i = (long long)t * TILE + threadIdx.x;
        double qf = 0.0, qs = 0.0;
        if (i < d.slot0 + d.n) {
            const Slots& S = b.s;
            const double fx = S.fx[i], fy = S.fy[i], fz = d.dims == 3 ? S.fz[i] : 0.0;
            double sf = dadd(dmul(fx, fx), dmul(fy, fy));
            const double vx = dmul(fx, dt), vy = dmul(fy, dt), vz = dmul(fz, dt);
            double sv = dadd(dmul(vx, vx), dmul(vy, vy));
            if (d.dims == 3) {
                sf = dadd(sf, dmul(fz, fz));
                sv = dadd(sv, dmul(vz, vz));
            }
            qf = __dsqrt_rn(sf);
            qs = __dsqrt_rn(sv);
        }
        unsigned long long bf = (unsigned long long)__double_as_longlong(qf);
        unsigned long long bs = (unsigned long long)__double_as_longlong(qs);
        if (!(qf == qf) || !(qs == qs)) {
            st.nonfinite = 1;
            bf = bs = 0x7ff0000000000000ull;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long yf = __shfl_xor_sync(0xffffffffu, bf, o);
            const unsigned long long ys = __shfl_xor_sync(0xffffffffu, bs, o);
            bf = yf > bf ? yf : bf;
            bs = ys > bs ? ys : bs;
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMax(&st.min_fmax, bf);
            atomicMax(&st.min_step, bs);
        }
    }
}

// r += v with v = F*dt scaled by max_step/stepsize when stepsize >
// max_step, wrap, displacement, skin max
__global__ void k_min_drift(Batch b, double dt, double max_step)
{
    __shared__ unsigned long long s_max[2 * (TILE / 32)];
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const int r = b.tile_rep[t];
        if (r < 0) continue;
        const RepDesc& d = b.desc[r];
        RepState& st = b.state[r];
        if (!st.min_active || st.min_done) continue;
        const double stepsize = __longlong_as_double((long long)st.min_step);
        const long long i = (long long)t * TILE + threadIdx.x;
        unsigned long long u2 = 0ull, d2in = 0ull;
        bool bad = false;
        if (i < d.slot0 + d.n) {
            const Slots& S = b.s;
            double vx = dmul(S.fx[i], dt), vy = dmul(S.fy[i], dt), vz = d.dims == 3 ? dmul(S.fz[i], dt) : 0.0;
            if (stepsize > max_step) {
                const double sc = ddiv(max_step, stepsize);
                vx = dmul(vx, sc);
                vy = dmul(vy, sc);
                vz = dmul(vz, sc);
            }
            u2 = drift_slot(b, d, i, vx, vy, vz, d2in, bad);
        }
        block_max_to_state(u2, bad, d2in, d, st, s_max);
    }
}

// after the move: the iteration's error max(maxforce, stepsize) ends the
// replica's minimisation when <= tol (one thread per replica, so every
// kernel of an iteration sees the same flag)
__global__ void k_min_decide(Batch b, double tol, long long max_iters)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= b.nreps) return;
    RepState& st = b.state[r];
    if (!b.desc[r].active || !st.min_active || st.min_done) return;
    const double stepsize = __longlong_as_double((long long)st.min_step);
    const double maxforce = __longlong_as_double((long long)st.min_fmax);
    const long long it = st.min_iters + 1;
    st.min_iters = it;
    const double err = maxforce > stepsize ? maxforce : stepsize;
    if (!(err > tol)) st.min_done = 1;
    else if (it >= max_iters) st.min_done = 2;
}

// one iteration after the force pass: maxima, move, decision
void launch_min_iteration_impl(const Batch& b, const LaunchCfg& lc, double dt, double max_step, double tol,
                               long long max_iters)
{
    const int rb = (b.nreps + 127) / 128;
    k_min_reset<<<rb, 128, 0, lc.stream>>>(b);
    k_min_max<<<lc.grid_stream, TILE, 0, lc.stream>>>(b, dt);
    k_min_drift<<<lc.grid_stream, TILE, 0, lc.stream>>>(b, dt, max_step);
    k_min_decide<<<rb, 128, 0, lc.stream>>>(b, tol, max_iters);
    if (lc.launches) *lc.launches += 4;
}

// kinetic energy of (v - vmean) with the pending COM removal applied, and
// (rescale mode) the velocity rescale factor sqrt(kBT / kBT_current)
template <bool RESCALE_ONLY>
__global__ void k_kinetic(Batch b)
{
    __shared__ double s_part[32];
    __shared__ int s_flag;
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        int r = b.tile_rep[t];
        if (r < 0) continue;
        const RepDesc& d = b.desc[r];
        if (d.dyn == DYN_BROWNIAN) continue;
        if (RESCALE_ONLY && !d.rescale) continue;
        RepState& st = b.state[r];
        long long i = (long long)t * TILE + threadIdx.x;
        double v[1] = {0.0};
        if (i < d.slot0 + d.n) {
            const Slots& S = b.s;
            double vx = dsub(S.vx[i], st.vmean[0]), vy = dsub(S.vy[i], st.vmean[1]);
            double s = dadd(dmul(vx, vx), dmul(vy, vy));
            if (d.dims == 3) {
                double vz = dsub(S.vz[i], st.vmean[2]);
                s = dadd(s, dmul(vz, vz));
            }
            v[0] = s;
        }
        double out[1];
        if (tile_reduce<1>(b, t, d, st, v, out, s_part, &s_flag) && threadIdx.x == 0) {
            double ekin = dmul(out[0], d.m_half);
            if (RESCALE_ONLY) {
                double kbt = ddiv(dmul(2.0, ekin), (double)(d.dims * d.n));
                st.vscale = __dsqrt_rn(ddiv(d.kBT, kbt));
            } else {
                st.ekin = ekin;
            }
        }
    }
}

// apply the pending COM removal / rescale (end of a batch of steps)
__global__ void k_finalize(Batch b)
{
    __shared__ double s_part[32];
    __shared__ int s_flag;
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        int r = b.tile_rep[t];
        if (r < 0) continue;
        const RepDesc& d = b.desc[r];
        if (d.dyn == DYN_BROWNIAN) continue;
        RepState& st = b.state[r];
        long long i = (long long)t * TILE + threadIdx.x;
        if (i < d.slot0 + d.n) {
            const Slots& S = b.s;
            const double vs = st.vscale;
            S.vx[i] = dmul(dsub(S.vx[i], st.vmean[0]), vs);
            S.vy[i] = dmul(dsub(S.vy[i], st.vmean[1]), vs);
            if (d.dims == 3) S.vz[i] = dmul(dsub(S.vz[i], st.vmean[2]), vs);
        }
        double v[1] = {0.0}, out[1];
        if (tile_reduce<1>(b, t, d, st, v, out, s_part, &s_flag) && threadIdx.x == 0) {
            st.vmean[0] = st.vmean[1] = st.vmean[2] = 0.0;
            st.vscale = 1.0;
        }
    }
}

void launch_kick_drift_impl(const Batch& b, const LaunchCfg& lc)
{
    k_kick_drift<<<lc.grid_stream, TILE, 0, lc.stream>>>(b);
    if (lc.launches) *lc.launches += 1;
}
void launch_brownian_update_impl(const Batch& b, const LaunchCfg& lc)
{
    k_brownian_update<<<lc.grid_stream, TILE, 0, lc.stream>>>(b);
    if (lc.launches) *lc.launches += 1;
}
void launch_rescale_impl(const Batch& b, const LaunchCfg& lc)
{
    k_kinetic<true><<<lc.grid_stream, TILE, 0, lc.stream>>>(b);
    if (lc.launches) *lc.launches += 1;
}
void launch_kinetic_impl(const Batch& b, const LaunchCfg& lc)
{
    k_kinetic<false><<<lc.grid_stream, TILE, 0, lc.stream>>>(b);
    if (lc.launches) *lc.launches += 1;
}
void launch_finalize_impl(const Batch& b, const LaunchCfg& lc)
{
    k_finalize<<<lc.grid_stream, TILE, 0, lc.stream>>>(b);
    if (lc.launches) *lc.launches += 1;
}

// ---------------------------------------------------------------------------
// host layout (AoS dims x N, original order) <-> slots
// ---------------------------------------------------------------------------
__global__ void k_load_aos(Batch b, int rep, const double* r, const double* v, const double* F,
                           const double* D, const double* disp)
{
    const RepDesc& d = b.desc[rep];
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.npad) return;
    long long s = d.slot0 + k;
    Slots& S = b.s;
    const int dm = d.dims;
    if (k < d.n) {
        double x = r[k * dm], y = r[k * dm + 1], z = dm == 3 ? r[k * dm + 2] : 0.0;
        S.posD[s] = make_double4_32a(x, y, z, D[k]);
        S.vx[s] = v ? v[k * dm] : 0.0;
        S.vy[s] = v ? v[k * dm + 1] : 0.0;
        S.vz[s] = (v && dm == 3) ? v[k * dm + 2] : 0.0;
        S.fx[s] = F ? F[k * dm] : 0.0;
        S.fy[s] = F ? F[k * dm + 1] : 0.0;
        S.fz[s] = (F && dm == 3) ? F[k * dm + 2] : 0.0;
        S.ux[s] = disp ? disp[k * dm] : 0.0;
        S.uy[s] = disp ? disp[k * dm + 1] : 0.0;
        S.uz[s] = (disp && dm == 3) ? disp[k * dm + 2] : 0.0;
        S.orig[s] = (int)k;
        S.inv[s] = (int)s;
    } else {
        S.posD[s] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
        S.vx[s] = S.vy[s] = S.vz[s] = 0.0;
        S.fx[s] = S.fy[s] = S.fz[s] = 0.0;
        S.ux[s] = S.uy[s] = S.uz[s] = 0.0;
        S.orig[s] = -1;
    }
    S.ncnt[s] = 0;
    S.cellc[s] = 0;
    S.rec[s] = FixRec{0u, 0u, 0u, 0.0f};
}

__global__ void k_store_aos(Batch b, int rep, double* r, double* v, double* F, double* disp,
                            const double* epp_src, double* epp)
{
    const RepDesc& d = b.desc[rep];
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    long long s = d.slot0 + k;
    const Slots& S = b.s;
    int o = S.orig[s];
    const int dm = d.dims;
    double4_32a p = S.posD[s];
    if (r) {
        r[o * dm] = p.x;
        r[o * dm + 1] = p.y;
        if (dm == 3) r[o * dm + 2] = p.z;
    }
    if (v) {
        v[o * dm] = S.vx[s];
        v[o * dm + 1] = S.vy[s];
        if (dm == 3) v[o * dm + 2] = S.vz[s];
    }
    if (F) {
        const RepState& st = b.state[rep];
        if (d.dyn == DYN_BROWNIAN && st.fmean_pending) {  // F - <F> of the last Brownian step
            F[o * dm] = dsub(S.fx[s], st.fmean[0]);
            F[o * dm + 1] = dsub(S.fy[s], st.fmean[1]);
            if (dm == 3) F[o * dm + 2] = dsub(S.fz[s], st.fmean[2]);
        } else {
            F[o * dm] = S.fx[s];
            F[o * dm + 1] = S.fy[s];
            if (dm == 3) F[o * dm + 2] = S.fz[s];
        }
    }
    if (disp) {
        disp[o * dm] = slot_disp(S, d, s, 0);
        disp[o * dm + 1] = slot_disp(S, d, s, 1);
        if (dm == 3) disp[o * dm + 2] = slot_disp(S, d, s, 2);
    }
    if (epp && epp_src) epp[o] = epp_src[s];
}

// host arrays (original order) -> current slot order; lists and cells kept
// slot s (original id o) of a replica takes the host's values; r, v, F,
// disp point at the replica's dims x N block (original order) or are NULL.
// The lists and the skin bookkeeping are kept: an edited position keeps its
// displacement since the rebuild (split replicas shift the rebuild-time
// record with it), unless a displacement is given
__device__ __forceinline__ void set_slot_state(const Batch& b, const RepDesc& d, RepState& st, long long s, int o,
                                               const double* r, const double* v, const double* F,
                                               const double* disp)
{
    const Slots& S = b.s;
    const int dm = d.dims;
    if (r) {
        double4_32a p = S.posD[s];
        p.x = r[o * dm];
        p.y = r[o * dm + 1];
        if (dm == 3) p.z = r[o * dm + 2];
        S.posD[s] = p;
        if (d.prec == PREC_FP32 || d.prune) {
            const FixRec q0 = S.rec[s], q = fix_rec(p.x, p.y, p.z, p.w, d);
            S.rec[s] = q;
            if (d.prec == PREC_FP32 && !disp) {  // the displacement since the rebuild is kept
                FixRec qb = S.recb[s];
                qb.x += q.x - q0.x;
                qb.y += q.y - q0.y;
                qb.z += q.z - q0.z;
                S.recb[s] = qb;
            }
        }
    }
    if (v) {
        S.vx[s] = v[o * dm];
        S.vy[s] = v[o * dm + 1];
        if (dm == 3) S.vz[s] = v[o * dm + 2];
    }
    if (F) {
        S.fx[s] = F[o * dm];
        S.fy[s] = F[o * dm + 1];
        if (dm == 3) S.fz[s] = F[o * dm + 2];
        if (s == d.slot0) st.fmean_pending = 0;  // the host's F is final
    }
    if (disp) {
        S.ux[s] = disp[o * dm];
        S.uy[s] = disp[o * dm + 1];
        if (dm == 3) S.uz[s] = disp[o * dm + 2];
        if (d.prec == PREC_FP32) {  // the rebuild-time record: the position minus the displacement
            const double4_32a p = S.posD[s];
            S.recb[s] = fix_rec(dsub(p.x, disp[o * dm]), dsub(p.y, disp[o * dm + 1]),
                                dm == 3 ? dsub(p.z, disp[o * dm + 2]) : 0.0, p.w, d);
        }
    }
}

__global__ void k_set_state(Batch b, int rep, const double* r, const double* v, const double* F,
                            const double* disp)
{
    const RepDesc& d = b.desc[rep];
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    const long long s = d.slot0 + k;
    set_slot_state(b, d, b.state[rep], s, b.s.orig[s], r, v, F, disp);
}

// every active replica at once, batched host layout (replica r's dims x N
// block at xfer_off, replicas in id order); one thread per slot
__global__ void k_set_state_all(Batch b, const double* r, const double* v, const double* F, const double* disp)
{
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const int rep = b.tile_rep[t];
        if (rep < 0) continue;
        const RepDesc& d = b.desc[rep];
        if (!d.active) continue;
        const long long s = (long long)t * TILE + threadIdx.x;
        if (s - d.slot0 >= d.n) continue;
        const long long o = d.xfer_off;
        set_slot_state(b, d, b.state[rep], s, b.s.orig[s], r ? r + o : nullptr, v ? v + o : nullptr,
                       F ? F + o : nullptr, disp ? disp + o : nullptr);
    }
}

// every active replica at once, batched host layout: replica r's dims x N
// block at xfer_off, its N-element block at xfer_soff (replicas in id
// order); one thread per slot of the replicas' tiles
__global__ void k_load_all(Batch b, const double* r, const double* v, const double* F, const double* D,
                           const double* disp)
{
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const int rep = b.tile_rep[t];
        if (rep < 0) continue;
        const RepDesc& d = b.desc[rep];
        if (!d.active) continue;
        const long long s = (long long)t * TILE + threadIdx.x;
        const long long k = s - d.slot0;
        Slots& S = b.s;
        const int dm = d.dims;
        if (k < d.n) {
            const double* rr = r + d.xfer_off + k * dm;
            S.posD[s] = make_double4_32a(rr[0], rr[1], dm == 3 ? rr[2] : 0.0, D[d.xfer_soff + k]);
            const double* vv = v ? v + d.xfer_off + k * dm : nullptr;
            const double* ff = F ? F + d.xfer_off + k * dm : nullptr;
            const double* uu = disp ? disp + d.xfer_off + k * dm : nullptr;
            S.vx[s] = vv ? vv[0] : 0.0;
            S.vy[s] = vv ? vv[1] : 0.0;
            S.vz[s] = (vv && dm == 3) ? vv[2] : 0.0;
            S.fx[s] = ff ? ff[0] : 0.0;
            S.fy[s] = ff ? ff[1] : 0.0;
            S.fz[s] = (ff && dm == 3) ? ff[2] : 0.0;
            S.ux[s] = uu ? uu[0] : 0.0;
            S.uy[s] = uu ? uu[1] : 0.0;
            S.uz[s] = (uu && dm == 3) ? uu[2] : 0.0;
            S.orig[s] = (int)k;
            S.inv[s] = (int)s;
        } else {
            S.posD[s] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
            S.vx[s] = S.vy[s] = S.vz[s] = 0.0;
            S.fx[s] = S.fy[s] = S.fz[s] = 0.0;
            S.ux[s] = S.uy[s] = S.uz[s] = 0.0;
            S.orig[s] = -1;
        }
        S.ncnt[s] = 0;
        S.cellc[s] = 0;
        S.rec[s] = FixRec{0u, 0u, 0u, 0.0f};
    }
}

__global__ void k_store_all(Batch b, double* r, double* v, double* F, double* disp)
{
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const int rep = b.tile_rep[t];
        if (rep < 0) continue;
        const RepDesc& d = b.desc[rep];
        if (!d.active) continue;
        const long long s = (long long)t * TILE + threadIdx.x;
        if (s >= d.slot0 + d.n) continue;
        const Slots& S = b.s;
        const int dm = d.dims;
        const long long o = d.xfer_off + (long long)S.orig[s] * dm;
        if (r) {
            const double4_32a p = S.posD[s];
            r[o] = p.x;
            r[o + 1] = p.y;
            if (dm == 3) r[o + 2] = p.z;
        }
        if (v) {
            v[o] = S.vx[s];
            v[o + 1] = S.vy[s];
            if (dm == 3) v[o + 2] = S.vz[s];
        }
        if (F) {
            const RepState& st = b.state[rep];
            if (d.dyn == DYN_BROWNIAN && st.fmean_pending) {  // F - <F> of the last Brownian step
                F[o] = dsub(S.fx[s], st.fmean[0]);
                F[o + 1] = dsub(S.fy[s], st.fmean[1]);
                if (dm == 3) F[o + 2] = dsub(S.fz[s], st.fmean[2]);
            } else {
                F[o] = S.fx[s];
                F[o + 1] = S.fy[s];
                if (dm == 3) F[o + 2] = S.fz[s];
            }
        }
        if (disp) {
            disp[o] = slot_disp(S, d, s, 0);
            disp[o + 1] = slot_disp(S, d, s, 1);
            if (dm == 3) disp[o + 2] = slot_disp(S, d, s, 2);
        }
    }
}

// max(D) of each replica's block of a batched upload (one block per
// replica; max is order-independent, so the result is exact)
__global__ void k_rep_dmax(Batch b, const double* D, double* out)
{
    const int r = blockIdx.x;
    if (r >= b.nreps) return;
    const RepDesc& d = b.desc[r];
    if (!d.active) return;
    double m = 0.0;
    for (long long k = threadIdx.x; k < d.n; k += blockDim.x) m = fmax(m, D[d.xfer_soff + k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double s_m[32];
    if ((threadIdx.x & 31) == 0) s_m[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = fmax(m, s_m[w]);
        out[r] = m;
    }
}

void launch_rep_dmax_impl(const Batch& b, const LaunchCfg& lc, const double* D, double* out)
{
    k_rep_dmax<<<b.nreps, 256, 0, lc.stream>>>(b, D, out);
    if (lc.launches) *lc.launches += 1;
}

void launch_load_all(const Batch& b, const LaunchCfg& lc, const double* r, const double* v, const double* F,
                     const double* D, const double* disp)
{
    k_load_all<<<lc.grid_stream, TILE, 0, lc.stream>>>(b, r, v, F, D, disp);
    if (lc.launches) *lc.launches += 1;
}

void launch_set_state_all(const Batch& b, const LaunchCfg& lc, const double* r, const double* v, const double* F,
                          const double* disp)
{
    k_set_state_all<<<lc.grid_stream, TILE, 0, lc.stream>>>(b, r, v, F, disp);
    if (lc.launches) *lc.launches += 1;
}

void launch_store_all(const Batch& b, const LaunchCfg& lc, double* r, double* v, double* F, double* disp)
{
    k_store_all<<<lc.grid_stream, TILE, 0, lc.stream>>>(b, r, v, F, disp);
    if (lc.launches) *lc.launches += 1;
}

// the replica's diameters in original order (swap moves exchange them)
__global__ void k_store_diameters(Batch b, int rep, double* D)
{
    const RepDesc& d = b.desc[rep];
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    const long long s = d.slot0 + k;
    D[b.s.orig[s]] = b.s.posD[s].w;
}

void launch_store_diameters_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, double* D)
{
    const int blocks = (hd.n + 127) / 128;
    if (blocks > 0) k_store_diameters<<<blocks, 128, 0, lc.stream>>>(b, rep, D);
    if (lc.launches) *lc.launches += 1;
}

void launch_set_state_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, const double* r,
                           const double* v, const double* F, const double* disp)
{
    int blocks = (hd.n + 127) / 128;
    if (blocks > 0) k_set_state<<<blocks, 128, 0, lc.stream>>>(b, rep, r, v, F, disp);
    if (lc.launches) *lc.launches += 1;
}

void launch_load_aos_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, const double* r,
                          const double* v, const double* F, const double* D, const double* disp)
{
    int blocks = (hd.npad + 127) / 128;
    k_load_aos<<<blocks, 128, 0, lc.stream>>>(b, rep, r, v, F, D, disp);
    if (lc.launches) *lc.launches += 1;
}

void launch_store_aos_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, double* r,
                           double* v, double* F, double* disp, const double* epp_src, double* epp)
{
    int blocks = (hd.n + 127) / 128;
    if (blocks > 0) k_store_aos<<<blocks, 128, 0, lc.stream>>>(b, rep, r, v, F, disp, epp_src, epp);
    if (lc.launches) *lc.launches += 1;
}

}  // namespace simmd
