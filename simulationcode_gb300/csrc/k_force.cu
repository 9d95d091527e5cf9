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
// One persistent kernel per launch and precision: blocks pull work items
// (a 128-slot tile, or a part of one for batches with fewer tiles than SMs)
// from an atomic work queue; a tile belongs to one replica, so (dims,
// potential, dynamics) are uniform per block.  T threads per particle
// (compile-time) split the particle's list (tile-major ELL, entries of one
// particle's T lanes adjacent) and combine with __shfl_xor; the split
// pass stages the first list rows of its particles in shared memory and
// gathers PAIR_UNROLL neighbour records at a time.  Every pair is visited
// from both sides (no atomics, deterministic sums).  Per-replica sums (mean
// force or centre-of-mass velocity, energy, virial) go through the fixed
// reduction tree of simmd_reduce.cuh; a stepping pass over a batch of many
// small replicas only stores its warps' partials and leaves the tree to
// k_replica_means, launched after it.
//
// FP64 path: the reference's per-pair operation order with explicit
// round-to-nearest intrinsics, so each pair force is bit-identical to the
// reference expression; only the order of the per-particle sum differs.
// FP32 split path: pair arithmetic in FP32 on exact integer differences of
// the positions in 32-bit box-periodic fixed point (r^2 exact before one
// rounding; compensated pair diameter); one 16-byte record per neighbour
// gather; per-particle sums, random force (four deviates per Philox call)
// and the mean-force partial sums in FP32, integration in FP64.
#include "simmd_internal.cuh"
#include "simmd_reduce.cuh"

namespace simmd {

// ---------------------------------------------------------------------------
// FP64 pair (reference arithmetic)
// ---------------------------------------------------------------------------
// the inner-list test of a pair (the force pass prunes while it sums):
// |r| <= r_cut (1 + 1e-4) s + inner skin, s the pair diameter (LJ: 1)
__device__ __forceinline__ bool prune_keep(const RepDesc& d, float r2, float s)
{
    const float tt = fmaf(d.prune_rcut_f, s, d.prune_skin_f);
    return r2 <= tt * tt;
}

template <int DIM, int POT, bool EN>
__device__ __forceinline__ void pair_f64(const RepDesc& d, long long halfLb, const double4_32a& pi,
                                         const double4_32a& pj, double& fx, double& fy, double& fz, double& e,
                                         double& w, double& r2o, double& so)
{
    const double L = d.L, rc2 = d.rc2;
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
    r2o = r2;
    so = 1.0;
    if (POT == POT_BERTHIER) {
        const double md = dmul(dmul(dadd(pi.w, pj.w), 0.5), dsub(1.0, dmul(d.zeta, fabs(dsub(pi.w, pj.w)))));
        so = md;
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

// PR: the pass also writes the inner list of the pairs prune_keep accepts
// (in list order; one thread per particle)
template <int DIM, int POT, bool EN, int T, bool PR>
__device__ __forceinline__ void pairs_f64(const Batch& b, const RepDesc& d, long long i, int sub,
                                          const double4_32a pi, const unsigned* __restrict__ nbr, int cnt,
                                          double& fx, double& fy, double& fz, double& e, double& w, int& m)
{
    const long long halfLb = __double_as_longlong(d.halfL);
    const double4_32a* __restrict__ posD = b.s.posD;
    double r2, sd;
    auto keep = [&](unsigned j) {
        if (PR && prune_keep(d, (float)r2, (float)sd)) b.s.nbr_in[nbr_addr(m++, i, 1, b.K)] = j;
    };
    int n = sub;
    for (; n + T < cnt; n += 2 * T) {
        const unsigned j0 = __ldg(nbr + nbr_addr(n, i, T, b.K)) & IDX_MASK;
        const unsigned j1 = __ldg(nbr + nbr_addr(n + T, i, T, b.K)) & IDX_MASK;
        const double4_32a p0 = posD[j0];
        const double4_32a p1 = posD[j1];
        pair_f64<DIM, POT, EN>(d, halfLb, pi, p0, fx, fy, fz, e, w, r2, sd);
        keep(j0);
        pair_f64<DIM, POT, EN>(d, halfLb, pi, p1, fx, fy, fz, e, w, r2, sd);
        keep(j1);
    }
    if (n < cnt) {
        const unsigned j0 = __ldg(nbr + nbr_addr(n, i, T, b.K)) & IDX_MASK;
        pair_f64<DIM, POT, EN>(d, halfLb, pi, posD[j0], fx, fy, fz, e, w, r2, sd);
        keep(j0);
    }
}

// ---------------------------------------------------------------------------
// FP32 split-precision pair
// ---------------------------------------------------------------------------
// Positions are 32-bit box-periodic fixed point, so the minimum-image
// difference of a pair is the exact int32 difference (the wraparound is the
// periodic image) and r^2 is formed exactly in 64-bit integers and rounded
// once.  The soft-sphere pair diameter s^2 = ((D_i + D_j)/2 (1 - zeta
// |D_i - D_j|))^2 and the ratio x = r^2 / s^2 carry their rounding errors
// along (error-free sum and FMA-based product residuals, first order): the
// force's sensitivity to x (about 10 near contact, the r^-14 term) would
// otherwise amplify the ~5 roundings of s^2 into most of the FP32 error.
struct PairS2 {
    float q, eq;  // s^2 = q + eq
    float s;      // s (rounded): the inner-list test
};

__device__ __forceinline__ PairS2 pair_s2_comp(float Di, float Dj, const RepDesc& d)
{
    const float a = fmaxf(Di, Dj), b = fminf(Di, Dj);
    const float S = a + b;
    const float eS = b - (S - a);               // S + eS = Di + Dj exactly (|a| >= |b|)
    const float dd = a - b;                     // |Di - Dj|, exact for D within a factor 2
    const float p = d.zetaf * dd;
    const float ep = fmaf(d.zetaf, dd, -p) + d.zeta_lo * dd;  // zeta |dD| = p + ep
    const float T = 1.0f - p;
    const float eT = ((1.0f - T) - p) - ep;     // T + eT = 1 - zeta |dD|
    float m = S * T;
    float em = fmaf(S, T, -m) + (S * eT + eS * T);
    m *= 0.5f;
    em *= 0.5f;
    PairS2 r;
    r.s = m;
    r.q = m * m;
    r.eq = fmaf(m, m, -r.q) + 2.0f * m * em;
    return r;
}

template <int DIM, int POT, bool EN>
__device__ __forceinline__ void pair_f32(const RepDesc& d, const FixRec& pi, const FixRec& pj, float& fx, float& fy,
                                         float& fz, float& e, float& w, float& r2o, float& so)
{
    const int ix = (int)(pi.x - pj.x), iy = (int)(pi.y - pj.y), iz = DIM == 3 ? (int)(pi.z - pj.z) : 0;
    unsigned long long r2i = (unsigned long long)((long long)ix * ix) + (unsigned long long)((long long)iy * iy);
    if (DIM == 3) r2i += (unsigned long long)((long long)iz * iz);
    const float r2 = __ull2float_rn(r2i) * d.fix_u2;
    r2o = r2;
    so = 1.0f;
    const float dx = (float)ix * d.fix_u, dy = (float)iy * d.fix_u, dz = DIM == 3 ? (float)iz * d.fix_u : 0.0f;
    float Fr = 0.0f, V = 0.0f;
    if (POT == POT_BERTHIER) {
        const PairS2 s2 = pair_s2_comp(pi.d, pj.d, d);
        so = s2.s;
        const float inv = __fdividef(1.0f, s2.q);
        float x = r2 * inv;
        x = fmaf(fmaf(-x, s2.q, r2) - x * s2.eq, inv, x);  // x = r^2 / (q + eq), first order
        const float xsq = x * x;
        const float xi14 = __fdividef(1.0f, xsq * xsq * xsq * x);
        const bool in = r2 <= d.rc2f * s2.q;
        const float B = fmaf(-6.0f, xi14, fmaf(2.0f * d.c4f, x, d.c2f));
        const float F0 = -2.0f * inv * B;
        Fr = in ? fmaf(-F0, s2.eq * inv, F0) : 0.0f;  // -2 B / (q + eq), first order
        if (EN && in) V = xi14 * x + fmaf(d.c4f, xsq, fmaf(d.c2f, x, d.c0f));
    } else {
        const float inv = __fdividef(1.0f, r2);
        const float xi2 = (DIM == 3 ? d.sigma2f : d.sigma4f) * inv;
        const float xi6 = xi2 * xi2 * xi2;
        const float xi12 = xi6 * xi6;
        const bool in = (DIM == 3) ? (r2 <= d.cut2f) : (r2 < d.cut2f);
        Fr = in ? d.epsf * (48.0f * xi12 - 24.0f * xi6) * inv : 0.0f;
        if (EN && in) V = 4.0f * d.epsf * (xi12 - xi6) - d.Ucf;
    }
    fx = fmaf(Fr, dx, fx);
    fy = fmaf(Fr, dy, fy);
    if (DIM == 3) fz = fmaf(Fr, dz, fz);
    if (EN) {
        e += V;
        w = fmaf(Fr, r2, w);
    }
}

// list entry n of the particle: from the tile's rows staged in shared memory
// (rows < nrows), else from global memory
template <int T>
__device__ __forceinline__ unsigned list_entry(const Batch& b, const unsigned* __restrict__ lst,
                                               const unsigned* s_rows, int nrows, long long i, int pl, int ppb, int n)
{
    const int row = n / T;
    if (row < nrows) return s_rows[row * (ppb * T) + pl * T + (n % T)] & IDX_MASK;
    return __ldg(lst + nbr_addr(n, i, T, b.K)) & IDX_MASK;
}

// neighbour records gathered PAIR_UNROLL at a time (all loads issued before
// the arithmetic); the pairs are still summed in list order
#ifndef SIMMD_PAIR_UNROLL
#define SIMMD_PAIR_UNROLL 2
#endif
constexpr int PAIR_UNROLL = SIMMD_PAIR_UNROLL;

// PR: the pass also writes the inner list of the pairs prune_keep accepts
// (in list order; one thread per particle)
template <int DIM, int POT, bool EN, int T, bool PR>
__device__ __forceinline__ void pairs_f32(const Batch& b, const RepDesc& d, long long i, int sub,
                                          const FixRec ri, const unsigned* __restrict__ lst, int cnt, float& fx,
                                          float& fy, float& fz, float& e, float& w, const unsigned* s_rows,
                                          int nrows, int pl, int ppb, int& m)
{
    const FixRec* __restrict__ rec = b.s.rec;
    float r2, sd;
    int n = sub;
    if constexpr (T == 1 && !PR) {
        // the rows staged in shared memory first, by a pointer walk with no
        // per-entry test of where the entry lives; the rest below (pairs in
        // list order either way)
        const int ns = min(cnt, nrows);
        const unsigned* q = s_rows + pl;
        for (; n + PAIR_UNROLL - 1 < ns; n += PAIR_UNROLL, q += PAIR_UNROLL * ppb) {
            unsigned j[PAIR_UNROLL];
            FixRec o[PAIR_UNROLL];
#pragma unroll
            for (int u = 0; u < PAIR_UNROLL; u++) j[u] = q[u * ppb] & IDX_MASK;
#pragma unroll
            for (int u = 0; u < PAIR_UNROLL; u++) o[u] = rec_get(rec + j[u]);
#pragma unroll
            for (int u = 0; u < PAIR_UNROLL; u++) pair_f32<DIM, POT, EN>(d, ri, o[u], fx, fy, fz, e, w, r2, sd);
        }
    }
    for (; n + (PAIR_UNROLL - 1) * T < cnt; n += PAIR_UNROLL * T) {
        unsigned j[PAIR_UNROLL];
        FixRec o[PAIR_UNROLL];
#pragma unroll
        for (int u = 0; u < PAIR_UNROLL; u++) j[u] = list_entry<T>(b, lst, s_rows, nrows, i, pl, ppb, n + u * T);
#pragma unroll
        for (int u = 0; u < PAIR_UNROLL; u++) o[u] = rec_get(rec + j[u]);
#pragma unroll
        for (int u = 0; u < PAIR_UNROLL; u++) {
            pair_f32<DIM, POT, EN>(d, ri, o[u], fx, fy, fz, e, w, r2, sd);
            if (PR && prune_keep(d, r2, sd)) b.s.nbr_in[nbr_addr(m++, i, 1, b.K)] = j[u];
        }
    }
    for (; n < cnt; n += T) {
        const unsigned j0 = list_entry<T>(b, lst, s_rows, nrows, i, pl, ppb, n);
        pair_f32<DIM, POT, EN>(d, ri, rec_get(rec + j0), fx, fy, fz, e, w, r2, sd);
        if (PR && prune_keep(d, r2, sd)) b.s.nbr_in[nbr_addr(m++, i, 1, b.K)] = j0;
    }
}

// v + dt*F/(2m).  When 2m is a power of two the divide is an exact scaling,
// so RN(dt*F)/(2m) == RN((dt/(2m))*F) and one multiply does both
__device__ __forceinline__ double kick(double v, double F, const RepDesc& d)
{
    if (d.two_m_pow2) return dadd(v, dmul(d.dt_over_two_m, F));
    return dadd(v, ddiv(dmul(d.dt, F), d.two_m));
}

// N(0,1) deviates of this particle for the current noise step: the host
// array (parity runs) or the Philox stream keyed by (seed, step, id, pair)
template <int PREC>
__device__ __forceinline__ void particle_noise(const RepDesc& d, RepState& st, int oid, double& x0, double& x1,
                                               double& x2)
{
    const long long step = st.step;
    x0 = x1 = x2 = 0.0;
    if (d.noise_mode == NOISE_HOST) {
        long long k = step - d.noise_step0;
        if (k < 0 || k >= d.noise_nsteps) {
            st.noise_range_error = 1;
            return;
        }
        const double* q = d.host_noise + (k * d.n + oid) * d.dims;
        x0 = q[0];
        x1 = q[1];
        if (d.dims == 3) x2 = q[2];
    } else if (PREC == PREC_FP64) {
        double z1;
        normal_pair_f64(d.seed, step, oid, 0, x0, x1);
        if (d.dims == 3) normal_pair_f64(d.seed, step, oid, 1, x2, z1);
    } else {
        float a, c, z1;
        normal_pair_f32(d.seed, step, oid, 0, a, c);
        x0 = a;
        x1 = c;
        if (d.dims == 3) {
            normal_pair_f32(d.seed, step, oid, 1, a, z1);
            x2 = a;
        }
    }
}

template <int DIM, bool EN, int T, bool PR>
__device__ __forceinline__ void particle_pairs_f64(const Batch& b, const RepDesc& d, long long i, int sub,
                                                   const unsigned* lst, int cnt, double& fx, double& fy, double& fz,
                                                   double& e, double& w, int& m)
{
    const double4_32a pi = b.s.posD[i];
    if (d.pot == POT_BERTHIER) pairs_f64<DIM, POT_BERTHIER, EN, T, PR>(b, d, i, sub, pi, lst, cnt, fx, fy, fz, e, w, m);
    else pairs_f64<DIM, POT_LJ, EN, T, PR>(b, d, i, sub, pi, lst, cnt, fx, fy, fz, e, w, m);
}

template <int DIM, bool EN, int T, bool PR>
__device__ __forceinline__ void particle_pairs_f32(const Batch& b, const RepDesc& d, long long i, int sub,
                                                   const FixRec ri, const unsigned* lst, int cnt, float& fx,
                                                   float& fy, float& fz, float& e, float& w, const unsigned* s_rows,
                                                   int nrows, int pl, int ppb, int& m)
{
    if (d.pot == POT_BERTHIER)
        pairs_f32<DIM, POT_BERTHIER, EN, T, PR>(b, d, i, sub, ri, lst, cnt, fx, fy, fz, e, w, s_rows, nrows, pl, ppb,
                                                m);
    else pairs_f32<DIM, POT_LJ, EN, T, PR>(b, d, i, sub, ri, lst, cnt, fx, fy, fz, e, w, s_rows, nrows, pl, ppb, m);
}

// rows of the tile's list staged in shared memory (16-byte loads, all rows
// issued at once): the pair loop then waits only on the record gathers
#ifndef SIMMD_STAGE_WORDS
#define SIMMD_STAGE_WORDS 2048
#endif
constexpr int STAGE_WORDS = SIMMD_STAGE_WORDS;  // list entries staged per block (8 KB)

// A block covers the ppb particles of one part of a tile; each staged row
// holds their ppb*T entries (one contiguous run of the tile-major row).
template <int T>
__device__ __forceinline__ int stage_rows(const Batch& b, const unsigned* lst, int t, int part, int ppb, int maxcnt,
                                          unsigned* s_rows)
{
    const int row_words = ppb * T, vpr = row_words / 4;
    const int vsh = 31 - __clz(vpr);  // ppb and T are powers of two
    const int nrows = min((maxcnt + T - 1) / T, STAGE_WORDS / row_words);
    const uint4* src = reinterpret_cast<const uint4*>(lst + (size_t)t * ((size_t)TILE * (size_t)b.K) +
                                                      (size_t)part * row_words);
    uint4* dst = reinterpret_cast<uint4*>(s_rows);
    for (int v = threadIdx.x; v < nrows * vpr; v += blockDim.x) {
        const int row = v >> vsh, c4 = v & (vpr - 1);
        dst[v] = __ldg(src + (size_t)row * (TILE * T / 4) + c4);
    }
    return nrows;
}

template <typename R, int T, bool EN>
__device__ __forceinline__ void combine_lanes(R& fx, R& fy, R& fz, R& e, R& w)
{
#pragma unroll
    for (int o = T >> 1; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o);
        fy += __shfl_xor_sync(0xffffffffu, fy, o);
        fz += __shfl_xor_sync(0xffffffffu, fz, o);
        if (EN) {
            e += __shfl_xor_sync(0xffffffffu, e, o);
            w += __shfl_xor_sync(0xffffffffu, w, o);
        }
    }
}

// last tile of a replica: the replica totals -> COM velocity / mean force,
// energy and virial, noise counter
// the replica's inner-list size, one atomic per warp; before the tile
// reduction, whose fence orders it before the replica's last tile reads it
__device__ __forceinline__ void count_inner(RepState& st, int m)
{
    unsigned long long sum = (unsigned long long)m;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0 && sum) {
        atomicAdd(&st.entries_in_acc, sum);
        __threadfence();
    }
}

template <int MODE, int NV>
__device__ __forceinline__ void finish_replica(const RepDesc& d, RepState& st, const double (&out)[NV], bool noise,
                                               bool pruned)
{
    if (pruned) {  // every tile of the replica wrote its inner list in this pass
        st.maxdisp_in = 0ull;
        st.force_prune = 0;
        st.prunes += 1;
        st.list_entries_in = (long long)st.entries_in_acc;
        st.entries_in_acc = 0ull;
    }
    constexpr bool EN = (MODE == FMODE_ENERGY || MODE == FMODE_STEP_ENERGY);
    constexpr bool STEP = (MODE == FMODE_STEP || MODE == FMODE_STEP_ENERGY || MODE == FMODE_STEP_DEFER);
    const double nd = (double)d.n;
    if (STEP) {
        double* m = (d.dyn == DYN_BROWNIAN) ? st.fmean : st.vmean;
        m[0] = ddiv(out[0], nd);
        m[1] = ddiv(out[1], nd);
        m[2] = ddiv(out[2], nd);
        if (d.dyn == DYN_BROWNIAN)
            for (int k = 0; k < 3; k++) st.cfmean[k] = -(d.dt_over_gamma * m[k]);
    }
    if (EN) {
        st.epot = out[NV - 2] / 2.0;
        st.virial = out[NV - 1] / 2.0;
    }
    // Brownian steps leave F - <F> implicit (applied by the position update
    // and by the download); a plain force evaluation leaves F final
    if (MODE != FMODE_ENERGY && d.dyn == DYN_BROWNIAN) st.fmean_pending = STEP ? 1 : 0;
    if (noise) st.step += 1;
}

// a stepping pass (no energy) leaves the tile reduction to k_replica_means:
// lane 0 of each warp stores the warp's sums in the tile's warp slot, with
// no block barrier and no tree climb inside the persistent loop
template <int NV>
__device__ __forceinline__ void step_slot_store(const Batch& b, int t, int part, const double (&pv)[NV])
{
    if ((threadIdx.x & 31) == 0) {
        const int nw = blockDim.x >> 5, wid = threadIdx.x >> 5;
        double* slot = b.warp_part + ((size_t)t * WARP_SLOTS + (size_t)(part * nw + wid)) * NPART;
#pragma unroll
        for (int k = 0; k < NV; k++) slot[k] = pv[k];
    }
}

#ifndef SIMMD_F32_MINB
#define SIMMD_F32_MINB 12
#endif
#ifndef SIMMD_F64_MINB
#define SIMMD_F64_MINB 4
#endif
template <int PREC, int T>
constexpr int force_min_blocks()
{
    return ((PREC == PREC_FP32 ? SIMMD_F32_MINB : SIMMD_F64_MINB) / T) > 0
               ? (PREC == PREC_FP32 ? SIMMD_F32_MINB : SIMMD_F64_MINB) / T
               : 1;
}

template <int MODE, int PREC, int T>
__global__ void __launch_bounds__(TILE * T, force_min_blocks<PREC, T>()) k_force(Batch b, double* epp)
{
    constexpr bool EN = (MODE == FMODE_ENERGY || MODE == FMODE_STEP_ENERGY);
    constexpr bool STEP = (MODE == FMODE_STEP || MODE == FMODE_STEP_ENERGY || MODE == FMODE_STEP_DEFER);
    constexpr int NV = EN ? 5 : 3;
    __shared__ int s_tile;
    __shared__ int s_flag;
    __shared__ int s_maxcnt;
    __shared__ double s_part[32 * NV];
    __shared__ __align__(16) unsigned s_rows[(PREC == PREC_FP32 && STAGE_WORDS >= 4) ? STAGE_WORDS : 4];
    const int tid = threadIdx.x;
    // work item = one part of a tile: parts per tile b.parts (a power of two,
    // > 1 only for small batches, so that every SM gets work), ppb particles
    // per part, blockDim = ppb * T
    const int parts = b.parts, ppb = TILE / parts;
    const int pl = tid / T, sub = tid - pl * T;
    for (;;) {
        if (tid == 0) s_tile = atomicAdd(&b.queue[0], 1);
        __syncthreads();
        const int item = s_tile;
        __syncthreads();
        if (item >= b.ntiles * parts) break;
        const int t = item / parts, part = item - t * parts;
        const int p = part * ppb + pl;
        const int r = b.tile_rep[t];
        if (r < 0) continue;
        const RepDesc& d = b.desc[r];
        if (d.prec != PREC) continue;  // the other precision's launch handles this tile
        RepState& st = b.state[r];
        if (MODE == FMODE_FORCES && st.min_done) continue;  // minimiser: this replica has converged
        const long long i = (long long)t * TILE + p;
        const bool real = i < d.slot0 + d.n;
        const bool noise = d.dyn != DYN_NEWTONIAN && MODE != FMODE_ENERGY && d.relax_cap == 0.0;
        const bool nl = d.dyn != DYN_BROWNIAN;
        // the list of this pass: the inner list when the context keeps one
        // and it is valid; the outer list when a prune is due, the pass then
        // writing the inner list (one thread per particle)
        const bool prn = T == 1 && need_prune(st, d);
        const bool inner = d.prune && !prn;
        const unsigned* lst = inner ? b.s.nbr_in : b.s.nbr;
        int m = 0;
        double pv[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) pv[k] = 0.0;
        double out[NV];
        bool last;
        if constexpr (PREC == PREC_FP32) {
            // ---- split precision: everything per particle in FP32 except the
            // FP64 state updates (force store, velocity kick)
            float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f, w = 0.f;
            const int cnt = real ? (inner ? b.s.ncnt_in[i] : b.s.ncnt[i]) : 0;
            if (tid == 0) s_maxcnt = 0;
            __syncthreads();
            if (sub == 0 && cnt > 0) atomicMax(&s_maxcnt, cnt);
            __syncthreads();
            const int nrows = stage_rows<T>(b, lst, t, part, ppb, s_maxcnt, s_rows);
            __syncthreads();
            if (real) {
                const FixRec ri = rec_get(b.s.rec + i);
                if (prn) {
                    if (d.dims == 3)
                        particle_pairs_f32<3, EN, T, true>(b, d, i, sub, ri, lst, cnt, fx, fy, fz, e, w, s_rows, nrows,
                                                           pl, ppb, m);
                    else
                        particle_pairs_f32<2, EN, T, true>(b, d, i, sub, ri, lst, cnt, fx, fy, fz, e, w, s_rows, nrows,
                                                           pl, ppb, m);
                    b.s.ncnt_in[i] = m;
                    b.s.recp[i] = ri;
                } else if (d.dims == 3) {
                    particle_pairs_f32<3, EN, T, false>(b, d, i, sub, ri, lst, cnt, fx, fy, fz, e, w, s_rows, nrows,
                                                        pl, ppb, m);
                } else {
                    particle_pairs_f32<2, EN, T, false>(b, d, i, sub, ri, lst, cnt, fx, fy, fz, e, w, s_rows, nrows,
                                                        pl, ppb, m);
                }
            }
            if (T > 1) combine_lanes<float, T, EN>(fx, fy, fz, e, w);
            float q0 = 0.f, q1 = 0.f, q2 = 0.f;  // per-particle contribution to the replica sums
            if (sub == 0 && real) {
                if (EN && epp) epp[i] = f2d(e) * 0.5;
                if (MODE != FMODE_ENERGY) {
                    double vx = 0.0, vy = 0.0, vz = 0.0;
                    if (nl) {
                        vx = b.s.vx[i];
                        vy = b.s.vy[i];
                        if (d.dims == 3) vz = b.s.vz[i];
                    }
                    if (noise) {
                        const float nf = d.noisef;
                        float z0, z1, z2 = 0.f, zz;
                        if (d.noise_mode == NOISE_HOST) {
                            double x0, x1, x2;
                            particle_noise<PREC_FP32>(d, st, b.s.orig[i], x0, x1, x2);
                            z0 = (float)x0;
                            z1 = (float)x1;
                            z2 = (float)x2;
                        } else {
                            normal_quad_f32(d.seed, st.step, b.s.orig[i], z0, z1, z2, zz);
                        }
                        fx += nf * z0;
                        fy += nf * z1;
                        fz += nf * z2;
                        if (d.dyn == DYN_LANGEVIN) {
                            const float mg = -d.gammaf;
                            fx += mg * d2f_rn(vx);
                            fy += mg * d2f_rn(vy);
                            fz += mg * d2f_rn(vz);
                        }
                    }
                    const double Fx = f2d(fx), Fy = f2d(fy), Fz = f2d(fz);
                    b.s.fx[i] = Fx;
                    b.s.fy[i] = Fy;
                    if (d.dims == 3) b.s.fz[i] = Fz;
                    if (STEP) {
                        if (nl) {  // kick2 in FP64 (src/MD.jl:529-531)
                            vx = kick(vx, Fx, d);
                            vy = kick(vy, Fy, d);
                            b.s.vx[i] = vx;
                            b.s.vy[i] = vy;
                            if (d.dims == 3) {
                                vz = kick(vz, Fz, d);
                                b.s.vz[i] = vz;
                            }
                            q0 = d2f_rn(vx);
                            q1 = d2f_rn(vy);
                            q2 = d2f_rn(vz);
                        } else {
                            q0 = fx;
                            q1 = fy;
                            q2 = fz;
                        }
                    }
                }
            }
            // per-warp sums in FP32 (the summed quantities carry FP32-level
            // accuracy), energy and virial in FP64; tile and replica sums FP64
            if (STEP) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    q0 += __shfl_xor_sync(0xffffffffu, q0, o);
                    q1 += __shfl_xor_sync(0xffffffffu, q1, o);
                    q2 += __shfl_xor_sync(0xffffffffu, q2, o);
                }
                if ((tid & 31) == 0) {  // only lane 0's value is read (WARP_DONE)
                    pv[0] = f2d(q0);
                    pv[1] = f2d(q1);
                    pv[2] = f2d(q2);
                }
            }
            if (EN) {
                double de = (sub == 0 && real) ? f2d(e) : 0.0, dw = (sub == 0 && real) ? f2d(w) : 0.0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    de += __shfl_xor_sync(0xffffffffu, de, o);
                    dw += __shfl_xor_sync(0xffffffffu, dw, o);
                }
                pv[NV - 2] = de;
                pv[NV - 1] = dw;
            }
            if (prn) count_inner(st, m);
            if (MODE == FMODE_STEP_DEFER) {  // lane 0 holds the warp's sums
                step_slot_store<NV>(b, t, part, pv);
                last = false;
            } else {
                last = tile_reduce<NV, true, 3>(b, item, d, st, pv, out, s_part, &s_flag, parts);
            }
        } else {
            // ---- FP64: the reference's arithmetic
            double fx = 0.0, fy = 0.0, fz = 0.0, e = 0.0, w = 0.0;
            if (real) {
                const int cnt = inner ? b.s.ncnt_in[i] : b.s.ncnt[i];
                if (prn) {
                    if (d.dims == 3) particle_pairs_f64<3, EN, T, true>(b, d, i, sub, lst, cnt, fx, fy, fz, e, w, m);
                    else particle_pairs_f64<2, EN, T, true>(b, d, i, sub, lst, cnt, fx, fy, fz, e, w, m);
                    b.s.ncnt_in[i] = m;
                    b.s.recp[i] = b.s.rec[i];
                } else if (d.dims == 3) {
                    particle_pairs_f64<3, EN, T, false>(b, d, i, sub, lst, cnt, fx, fy, fz, e, w, m);
                } else {
                    particle_pairs_f64<2, EN, T, false>(b, d, i, sub, lst, cnt, fx, fy, fz, e, w, m);
                }
            }
            if (T > 1) combine_lanes<double, T, EN>(fx, fy, fz, e, w);
            if (sub == 0 && real) {
                if (EN) {
                    pv[NV - 2] = e;
                    pv[NV - 1] = w;
                    if (epp) epp[i] = e / 2.0;
                }
                if (MODE != FMODE_ENERGY) {
                    double vx = 0.0, vy = 0.0, vz = 0.0;
                    if (nl) {
                        vx = b.s.vx[i];
                        vy = b.s.vy[i];
                        if (d.dims == 3) vz = b.s.vz[i];
                    }
                    double Fx = fx, Fy = fy, Fz = fz;
                    if (noise) {
                        double x0, x1, x2;
                        particle_noise<PREC_FP64>(d, st, b.s.orig[i], x0, x1, x2);
                        if (d.dyn == DYN_LANGEVIN) {  // F += -gamma v + sqrt(2kBT gamma/dt) xi
                            const double mg = -d.gamma;
                            Fx = dadd(Fx, dadd(dmul(mg, vx), dmul(d.noise_factor, x0)));
                            Fy = dadd(Fy, dadd(dmul(mg, vy), dmul(d.noise_factor, x1)));
                            if (d.dims == 3) Fz = dadd(Fz, dadd(dmul(mg, vz), dmul(d.noise_factor, x2)));
                        } else {
                            Fx = dadd(Fx, dmul(d.noise_factor, x0));
                            Fy = dadd(Fy, dmul(d.noise_factor, x1));
                            if (d.dims == 3) Fz = dadd(Fz, dmul(d.noise_factor, x2));
                        }
                    }
                    b.s.fx[i] = Fx;
                    b.s.fy[i] = Fy;
                    if (d.dims == 3) b.s.fz[i] = Fz;
                    if (STEP) {
                        if (nl) {  // kick2 (src/MD.jl:529-531)
                            vx = kick(vx, Fx, d);
                            vy = kick(vy, Fy, d);
                            b.s.vx[i] = vx;
                            b.s.vy[i] = vy;
                            if (d.dims == 3) {
                                vz = kick(vz, Fz, d);
                                b.s.vz[i] = vz;
                            }
                            pv[0] = vx; pv[1] = vy; pv[2] = vz;
                        } else {
                            pv[0] = Fx; pv[1] = Fy; pv[2] = Fz;
                        }
                    }
                }
            }
            if (prn) count_inner(st, m);
            if (MODE == FMODE_STEP_DEFER) {
                warp_sum<NV>(pv);
                step_slot_store<NV>(b, t, part, pv);
                last = false;
            } else {
                last = tile_reduce<NV, false, 3>(b, item, d, st, pv, out, s_part, &s_flag, parts);
            }
        }
        if (last && tid == 0) finish_replica<MODE, NV>(d, st, out, noise, prn);
    }
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&b.queue[1], 1) == (int)gridDim.x - 1) {
            b.queue[0] = 0;
            b.queue[1] = 0;
        }
    }
}

// after a stepping force pass, one block per replica: the replica's sums
// from the warp slots of its tiles, in the canonical order of the tile
// reduction (each tile its warp slots added in order; then groups of 32
// consecutive tiles -- one warp -- reduced in the tree's fixed shuffle
// order, the mean force / velocity summed plainly as the tile reduction
// sums them, level by level, a level's group results kept in the
// reduction tree's records);
// then what the pass's last tile does in the other modes: the mean force
// (Brownian) or centre-of-mass velocity, the filtered-list bookkeeping and
// the noise counter
constexpr int MEANS_THREADS = 256;

__global__ void __launch_bounds__(MEANS_THREADS) k_replica_means(Batch b)
{
    const int r = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
    const RepDesc& d = b.desc[r];
    RepState& st = b.state[r];
    if (!d.active || d.ntiles < 1) return;  // block-uniform
    const int wpt = (TILE / b.parts) * b.tpp / 32 * b.parts;  // warp slots per tile
    __shared__ double s_fin[6];
    int n = d.ntiles;
    for (int level = 0;; level++) {
        const int ng = (n + 31) >> 5;
        // every warp of the block takes whole groups; the block covers
        // MEANS_THREADS members per round
        for (int base = 0; base < ng * 32; base += MEANS_THREADS) {
            const int idx = base + tid;
            double s[3] = {0.0, 0.0, 0.0}, c[3] = {0.0, 0.0, 0.0};
            if (idx < n) {
                if (level == 0) {  // the tile's sum: its warp slots in order
                    const double* slot = b.warp_part + (size_t)(d.tile0 + idx) * WARP_SLOTS * NPART;
                    for (int w0 = 0; w0 < wpt; w0 += 8) {
                        double v[8][3];
#pragma unroll
                        for (int w = 0; w < 8; w++)
#pragma unroll
                            for (int k = 0; k < 3; k++)
                                v[w][k] = w0 + w < wpt ? __ldcg(slot + (size_t)(w0 + w) * NPART + k) : 0.0;
#pragma unroll
                        for (int w = 0; w < 8; w++)
                            if (w0 + w < wpt)
#pragma unroll
                                for (int k = 0; k < 3; k++) s[k] += v[w][k];
                    }
                } else {
                    const double* src = b.red_val + ((size_t)level * b.ntiles + d.tile0 + idx) * RED_REC;
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        s[k] = __ldcg(src + k);
                        c[k] = __ldcg(src + 3 + k);
                    }
                }
            }
            if (base + (tid & ~31) < ng * 32) {  // a warp of this level's groups
                warp_sum_comp<3, 3>(s, c);
                const int g = (base + tid) >> 5;
                if (lane == 0) {
                    if (ng > 1) {
                        double* dst = b.red_val + ((size_t)(level + 1) * b.ntiles + d.tile0 + g) * RED_REC;
#pragma unroll
                        for (int k = 0; k < 3; k++) {
                            dst[k] = s[k];
                            dst[3 + k] = c[k];
                        }
                    } else {
#pragma unroll
                        for (int k = 0; k < 3; k++) {
                            s_fin[k] = s[k];
                            s_fin[3 + k] = c[k];
                        }
                    }
                }
            }
        }
        __threadfence_block();
        __syncthreads();
        if (ng == 1) break;
        n = ng;
    }
    if (tid != 0) return;
    const bool pruned = b.tpp == 1 && need_prune(st, d);
    if (pruned) {  // every tile of the replica wrote its inner list in this pass
        st.maxdisp_in = 0ull;
        st.force_prune = 0;
        st.prunes += 1;
        st.list_entries_in = (long long)st.entries_in_acc;
        st.entries_in_acc = 0ull;
    }
    const double nd = (double)d.n;
    double* m = (d.dyn == DYN_BROWNIAN) ? st.fmean : st.vmean;
#pragma unroll
    for (int k = 0; k < 3; k++) m[k] = ddiv(s_fin[k] + s_fin[3 + k], nd);
    if (d.dyn == DYN_BROWNIAN) {
        for (int k = 0; k < 3; k++) st.cfmean[k] = -(d.dt_over_gamma * m[k]);
        st.fmean_pending = 1;
    }
    if (d.dyn != DYN_NEWTONIAN && d.relax_cap == 0.0) st.step += 1;
}

// ---------------------------------------------------------------------------
// host side: occupancy and launch, one instantiation per (mode, precision, T)
// ---------------------------------------------------------------------------
template <int MODE, int PREC>
static void* kernel_ptr(int T)
{
    switch (T) {
        case 2: return (void*)k_force<MODE, PREC, 2>;
        case 4: return (void*)k_force<MODE, PREC, 4>;
        case 8: return (void*)k_force<MODE, PREC, 8>;
        default: return (void*)k_force<MODE, PREC, 1>;
    }
}

template <int PREC>
static void* kernel_for(int mode, int T)
{
    switch (mode) {
        case FMODE_STEP: return kernel_ptr<FMODE_STEP, PREC>(T);
        case FMODE_STEP_DEFER: return kernel_ptr<FMODE_STEP_DEFER, PREC>(T);
        case FMODE_FORCES: return kernel_ptr<FMODE_FORCES, PREC>(T);
        case FMODE_ENERGY: return kernel_ptr<FMODE_ENERGY, PREC>(T);
        default: return kernel_ptr<FMODE_STEP_ENERGY, PREC>(T);
    }
}

int force_blocks_per_sm(int T, int mode, int prec, int parts)
{
    int nb = 0;
    void* k = prec == PREC_FP64 ? kernel_for<PREC_FP64>(mode, T) : kernel_for<PREC_FP32>(mode, T);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, (TILE / parts) * T, 0);
    return nb > 0 ? nb : 1;
}

// one launch per precision present in the batch (prec_mask bit 0: FP64, bit 1: FP32 split)
void launch_force_impl(const Batch& b, const LaunchCfg& lc, int mode, int prec_mask, double* epp)
{
    if (mode == FMODE_STEP && b.defer) mode = FMODE_STEP_DEFER;
    for (int prec = 0; prec < 2; prec++) {
        if (!(prec_mask & (1 << prec))) continue;
        void* k = prec == PREC_FP64 ? kernel_for<PREC_FP64>(mode, b.tpp) : kernel_for<PREC_FP32>(mode, b.tpp);
        Batch bb = b;
        double* ep = epp;
        void* args[] = {(void*)&bb, (void*)&ep};
        cudaLaunchKernel(k, dim3(prec == PREC_FP64 ? lc.grid_force64 : lc.grid_force32),
                         dim3((TILE / b.parts) * b.tpp), args, 0, lc.stream);
        if (lc.launches) *lc.launches += 1;
    }
    if (mode == FMODE_STEP_DEFER) {
        k_replica_means<<<b.nreps, MEANS_THREADS, 0, lc.stream>>>(b);
        if (lc.launches) *lc.launches += 1;
    }
}

}  // namespace simmd
