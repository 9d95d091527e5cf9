// simmd_internal.cuh -- device-side data model of libsimmd.
//
// Layout in HBM (one engine = one CUDA stream, many replicas):
//   * a flat SLOT space; replica r owns slots [slot0, slot0 + npad), npad a
//     multiple of TILE; slots hold particles in cell-sorted order after each
//     rebuild, padding slots (orig < 0) never appear in a cell or a list;
//   * per-slot SoA FP64 arrays v, F, displacement; an AoS double4_32a (x,y,z,D)
//     gathered by neighbours; a 32-byte split-precision record (FP32 offsets
//     from a power-of-two grid point, D, the grid point); packed rebuild-time
//     cell coordinates; the original particle id;
//   * a padded ELL neighbour list, tile-major (see nbr_addr; T = threads per
//     particle), each entry the slot of j (low 26 bits);
//   * per-replica descriptors (read-only) and states (flags, counters,
//     reductions), a tile -> replica table and per-warp partial-sum slots.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace simmd {

constexpr int TILE = 128;                       // slots per tile (work unit)
constexpr int IDX_BITS = 26;
constexpr unsigned IDX_MASK = (1u << IDX_BITS) - 1u;
constexpr int MAX_CELLS_AXIS = 1023;
constexpr int NPART = 8;                        // doubles per partial-sum record
constexpr int MAX_PARTS = 16;                   // work items per tile in the force pass
constexpr int MAX_TPP = 8;                      // threads per particle: 1, 2, 4 or 8
constexpr int RED_REC = 16;                     // doubles per reduction-tree record (sum, error) x <= 8 values
constexpr int RED_LEVELS = 4;                   // tree levels: 32^4 tiles >= 2^24 particles
constexpr int WARP_SLOTS = TILE * MAX_TPP / 32; // warp partial-sum slots per tile

enum { POT_LJ = 0, POT_BERTHIER = 1 };
enum { DYN_NEWTONIAN = 0, DYN_LANGEVIN = 1, DYN_BROWNIAN = 2 };
enum { PREC_FP64 = 0, PREC_FP32 = 1 };
enum { NOISE_PHILOX = 0, NOISE_HOST = 1 };

struct RepDesc {
    long long slot0;
    int n, npad;
    int tile0, ntiles;
    int cell0, ncell;          // cells [cell0, cell0+ncell) + pad cell + end marker
    int dims, pot, dyn, prec;
    int nc;                    // cells per axis (1 or >= 3); cubic box
    int rescale;
    int noise_mode;
    int active;
    double L, halfL, cs, inv_cs;
    double rc2, rcut, skin, rv2, skin_half2;
    double sigma2, sigma4, lj_cut2, eps, Uc, c0, c2, c4, zeta;
    double kBT, gamma, dt, m, noise_factor, dt_over_gamma, two_m, m_half;
    double relax_cap;          // > 0: capped steepest descent (set-up relaxation), no noise
    double wrap_hi;            // smallest x with RN(x/L) >= 1: floor(x/L) without a divide
    double inv_two_m;          // 1/(2m), used when 2m is a power of two (exact)
    double dt_over_two_m;      // dt/(2m) when 2m is a power of two (exact): one multiply per kick
    int two_m_pow2;
    int build_wrap;            // 0: stencil candidates never need the minimum image (2 cs + h < L/2)
    // split precision: FP32 offsets from a power-of-two grid h (exact integer shifts)
    double h, inv_h;
    float hf, Lhi_f, Llo_f, rv2f;
    float Lf, halfLf, csf, rc2f, rcutf, skinf, sigma2f, sigma4f, cut2f, epsf, Ucf, c0f, c2f, c4f, zetaf;
    float noisef, gammaf;      // noise_factor, gamma rounded to FP32
    unsigned long long seed;
    long long xfer_off;        // batched host transfers: offset of this replica's dims x N block
    long long xfer_soff;       // ... and of its N-element block (D)
    const double* host_noise;  // [noise_nsteps][n][dims], original order
    long long noise_step0;
    int noise_nsteps;
    int pad_;
};

struct RepState {
    unsigned long long maxdisp2;  // bits of the max |disp|^2 (non-negative double)
    int force_rebuild;
    int overflow;
    int nonfinite;
    int done_count;
    int maxcount;
    int noise_range_error;
    int fmean_pending;            // Brownian: F holds F before the mean-force subtraction
    int in_plan;                  // listed by the current rebuild sequence's plan
    long long step;               // noise draws so far (Philox counter)
    long long rebuilds;
    long long list_entries;       // total list length at the last rebuild
    double vmean[3];              // pending centre-of-mass velocity (Newtonian/Langevin)
    double fmean[3];              // mean force (Brownian)
    double cfmean[3];             // -(dt/gamma) * fmean (split-precision position update)
    double vscale;                // pending velocity rescale factor
    double epot, virial, ekin;
    double fmax;
    // inherent-structure minimiser
    unsigned long long min_fmax;  // bits of max_i |F_i| this iteration
    unsigned long long min_step;  // bits of max_i |F_i dt| this iteration
    long long min_iters;
    int min_done;                 // 1 converged, 2 iteration limit
    int min_active;               // replica takes part in the minimisation
};

// split-precision gather record (one 32-byte sector): FP32 offsets of the
// FP64 position from its grid point, FP32 diameter, packed grid index
struct __align__(32) SplitRec {
    float4 o;   // x, y, z offsets from the grid point, D
    float4 g;   // grid point m*h per axis (exact in FP32), unused
};

struct Slots {
    double4_32a* posD;                // x, y, z, D
    double *vx, *vy, *vz;
    double *fx, *fy, *fz;
    double *ux, *uy, *uz;         // displacement since the last rebuild
    SplitRec* rec;                // split precision: offsets + D + grid index
    int* cellc;                   // packed rebuild-time cell coords (10 bits each)
    int* orig;                    // original id, -1 for padding
    unsigned* nbr;                // ELL neighbour list
    int* ncnt;                    // neighbours per slot
    // rebuild scratch
    int* bin_cell;
    int* bin_rank;
    int* src;
    double4_32a* t_posD;
    double *t_vx, *t_vy, *t_vz, *t_fx, *t_fy, *t_fz;
    int* t_orig;
    int* cell_count;              // per cell (+ pad cell)
    int* cell_start;              // per cell (+ pad cell + end)
};

struct Batch {
    const RepDesc* desc;
    RepState* state;
    const int* tile_rep;          // tile -> replica (-1: unused)
    int ntiles;                   // tiles in the slot space
    int nreps;                    // replica table size
    long long S;                  // slot capacity
    int K;                        // list rows
    int tpp;                      // threads per particle (list interleave)
    int parts;                    // force pass: work items per tile (power of two, <= MAX_PARTS)
    Slots s;
    double* red_val;              // [RED_LEVELS][ntiles][RED_REC] reduction tree values (sum, error)
    int* red_cnt;                 // [RED_LEVELS][ntiles] members of a tree group done (reset by the last)
    double* warp_part;            // [ntiles][WARP_SLOTS][NPART] warp partials of split tiles
    int* tile_cnt;                // [ntiles] parts of a split tile done (reset by the last)
    int* queue;                   // work-queue heads [4]
    // rebuild plan: tiles and cells of the replicas rebuilding this step
    int* plan_tiles;              // [ntiles]
    int2* plan_cells;             // [cell capacity] (replica, cell)
    int* plan_cnt;                // [0] tiles, [1] cells
};

// ---------------------------------------------------------------------------
// exact FP64 helpers: explicit round-to-nearest intrinsics, never contracted
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double drcp(double a) { return __drcp_rn(a); }

// dx - round(dx/L)*L for |dx| < L, decided on the bit pattern (integer pipe):
// identical to the reference whenever |dx| is not within an ulp of L/2, i.e.
// for every pair closer than L/2.
__device__ __forceinline__ double min_image_f64(double dx, long long halfL_bits, double L)
{
    long long b = __double_as_longlong(dx);
    long long a = b & 0x7fffffffffffffffLL;
    double sh = (a > halfL_bits) ? ((b < 0) ? -L : L) : 0.0;
    return dsub(dx, sh);
}

__device__ __forceinline__ float min_image_f32(float dx, float halfL, float L)
{
    dx = (dx > halfL) ? dx - L : dx;
    dx = (dx < -halfL) ? dx + L : dx;
    return dx;
}

// float <-> double conversions on the integer pipes.  GB300 runs FP64
// arithmetic and FP64 conversions on one narrow pipe (about 1/70 of the FP32
// rate), so the split-precision kernels widen and narrow with bit operations:
// f2d is exact, d2f_rn rounds to nearest even; both give the converter's
// result bit for bit.  Zero and normal numbers take the inline path; the
// rest (subnormal, out of range, inf, nan) go to the converter.
__device__ __forceinline__ double f2d(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned a = u & 0x7fffffffu;
    if (a - 0x00800000u < 0x7f000000u)  // exponent field 1..254
        return __hiloint2double((int)((u & 0x80000000u) | ((a >> 3) + (896u << 20))), (int)(u << 29));
    if (a == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)f;
}

__device__ __forceinline__ float d2f_rn(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned ah = hi & 0x7fffffffu;
    const int e = (int)(ah >> 20) - 896;  // the float exponent field
    if (e >= 1 && e <= 254) {
        unsigned f = ((unsigned)e << 23) | ((ah & 0xfffffu) << 3) | (lo >> 29);
        const unsigned r = lo & 0x1fffffffu;  // the 29 dropped bits
        f += (r > 0x10000000u || (r == 0x10000000u && (f & 1u))) ? 1u : 0u;  // carry may reach inf: correct
        return __uint_as_float((hi & 0x80000000u) | f);
    }
    if (ah == 0u && lo == 0u) return __uint_as_float(hi & 0x80000000u);
    return (float)x;
}

// non-finite test on the bit pattern (no FP64 compare)
__device__ __forceinline__ bool nonfinite_bits(double x)
{
    return (__double_as_longlong(x) & 0x7fffffffffffffffll) >= 0x7ff0000000000000ll;
}

// split precision: grid index of the FP32 offset origin (power-of-two grid
// h), the FP64 form floor(x/h + 0.5) clamped to [0, 1023] (h a power of two, so
// x/h is exact), computed on the integer pipes with the same result for every
// x: with y = x/h in [2^j, 2^(j+1)), y + 0.5 is exact unless it crosses into
// the next binade, and there no integer is within the rounding's reach --
// except at j = -2, where y = 0.5 - 2^-54 rounds y + 0.5 up to 1
__device__ __forceinline__ int grid_index(double x, const RepDesc& d)
{
    const long long b = __double_as_longlong(x);
    if (b <= 0) return 0;  // +0, negatives, NaNs with the sign bit
    const int ex = (int)(b >> 52);
    const long long mant = b & 0xfffffffffffffll;
    if (ex == 0x7ff) return mant ? 0 : 1023;  // NaN, +inf
    if (ex == 0) return 0;                    // subnormal: y < 0.5
    const int hk = (int)((__double_as_longlong(d.h) >> 52) & 0x7ff) - 1023;
    const int j = ex - 1023 - hk;
    if (j >= 10) return 1023;
    if (j <= -3) return 0;
    if (j == -2) return mant == 0xfffffffffffffll ? 1 : 0;
    const long long M = mant | (1ll << 52);
    const int sh = 52 - j;  // 43..53
    const long long m = (M + (1ll << (sh - 1))) >> sh;
    return m > 1023 ? 1023 : (int)m;
}

// FP32 offset of coordinate x from its grid point g = m*h (exact in FP32 and
// FP64), continuous across the periodic wrap: one FP64 subtract; the wrap
// correction (|x - g| > L/2, a particle just across the box edge) in FP64
// only when the FP32 offset is not clearly inside
__device__ __forceinline__ float grid_offset(double x, float g, const RepDesc& d)
{
    double o = dsub(x, f2d(g));
    const float of = d2f_rn(o);
    if (fabsf(of) < d.halfLf * 0.9f) return of;
    o = (o > d.halfL) ? o - d.L : o;
    o = (o < -d.halfL) ? o + d.L : o;
    return (float)o;
}

__device__ __forceinline__ int grid_axis(int g, int axis) { return (g >> (10 * axis)) & 1023; }

// minimum-image difference x_i - x_j of two split-precision coordinates:
// ((o_i - o_j) - s*L_lo) + ((m_i - m_j)*h - s*L_hi) with the integer grid
// shift and L_hi = floor(L/h)*h exact in FP32, so only the small offset
// terms and the final sum round
__device__ __forceinline__ float split_dx(float oi, float oj, int mi, int mj, const RepDesc& d)
{
    const float a = oi - oj;
    const float G0 = (float)(mi - mj) * d.hf;
    const float dx0 = a + G0;
    const float s = (dx0 > d.halfLf) ? 1.0f : ((dx0 < -d.halfLf) ? -1.0f : 0.0f);
    return (a - s * d.Llo_f) + (G0 - s * d.Lhi_f);
}

// one 256-bit read-only load of a neighbour's record (sm_100 and later):
// the record is one sector, so a warp's gather costs one request per lane
// instead of two
#ifndef SIMMD_REC_V8
#define SIMMD_REC_V8 1
#endif
__device__ __forceinline__ void rec_get(const SplitRec* __restrict__ r, float4& o, float4& g)
{
#if SIMMD_REC_V8
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(o.x), "=f"(o.y), "=f"(o.z), "=f"(o.w), "=f"(g.x), "=f"(g.y), "=f"(g.z), "=f"(g.w)
        : "l"(r));
#else
    o = __ldg(&r->o);
    g = __ldg(&r->g);
#endif
}

__device__ __forceinline__ void rec_put(SplitRec* r, float4 o, float4 g)
{
    r->o = o;
    r->g = g;
}

// minimum-image x_i - x_j from split records: (o_i - o_j) + (g_i - g_j) with
// the grid difference exact; across the periodic boundary (rare) the box is
// removed as L_hi (a grid multiple, exact) plus L_lo
__device__ __forceinline__ float split_dx_g(float oi, float oj, float gi, float gj, const RepDesc& d)
{
    const float a = oi - oj;
    const float G0 = gi - gj;
    const float dx0 = a + G0;
    if (fabsf(dx0) <= d.halfLf) return dx0;
    const float s = dx0 > 0.0f ? 1.0f : -1.0f;
    return (a - s * d.Llo_f) + (G0 - s * d.Lhi_f);
}

__device__ __forceinline__ bool need_rebuild(const RepState& st, const RepDesc& d)
{
    return st.force_rebuild || (__longlong_as_double((long long)st.maxdisp2) > d.skin_half2);
}

// List layout, tile-major: the TILE slots of a tile own TILE*K consecutive
// entries (K = entries per particle, a multiple of T).  Row q of the tile
// holds entries q*T .. q*T+T-1 of every particle of the tile, so the T
// threads of one particle and the particles of one warp read one contiguous
// run per row.  The address does not depend on the slot capacity, so a
// capacity grow keeps the lists (a copy of the old prefix).
__device__ __forceinline__ size_t nbr_addr(int n, long long slot, int T, int K)
{
    return (size_t)(slot / TILE) * ((size_t)TILE * (size_t)K) + (size_t)(n / T) * (size_t)(TILE * T) +
           (size_t)(slot % TILE) * (size_t)T + (size_t)(n % T);
}

// the same address for a runtime T = 1 << tsh (no integer division)
__device__ __forceinline__ size_t nbr_addr_sh(int n, long long slot, int tsh, int K)
{
    return (size_t)(slot / TILE) * ((size_t)TILE * (size_t)K) + (size_t)(n >> tsh) * (size_t)(TILE << tsh) +
           ((size_t)(slot % TILE) << tsh) + (size_t)(n & ((1 << tsh) - 1));
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and Box-Muller normals
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        unsigned hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        unsigned hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// two N(0,1) deviates for (seed, step, particle, pair); FP64 version matches
// the oracle's orc_philox_normals to a few ulp
__device__ __forceinline__ void normal_pair_f64(unsigned long long seed, long long step, int particle,
                                                int pair, double& z0, double& z1)
{
    uint4 o = philox4x32_10(make_uint4((unsigned)particle, (unsigned)pair, (unsigned)step,
                                       (unsigned)((unsigned long long)step >> 32)),
                            make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    unsigned long long a = ((unsigned long long)o.x << 21) | (o.y >> 11);
    unsigned long long b = ((unsigned long long)o.z << 21) | (o.w >> 11);
    double u = ((double)a + 1.0) * 0x1.0p-53;
    double w = (double)b * 0x1.0p-53;
    double rad = sqrt(-2.0 * log(u));
    double s, c;
    sincospi(2.0 * w, &s, &c);
    z0 = rad * c;
    z1 = rad * s;
}

// four FP32 deviates from one Philox call (split-precision path): 24-bit
// uniforms from each 32-bit word, two Box-Muller pairs
__device__ __forceinline__ void normal_quad_f32(unsigned long long seed, long long step, int particle, float& z0,
                                                float& z1, float& z2, float& z3)
{
    uint4 o = philox4x32_10(make_uint4((unsigned)particle, 0u, (unsigned)step,
                                       (unsigned)((unsigned long long)step >> 32)),
                            make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    const float u0 = ((float)(o.x >> 8) + 1.0f) * 0x1.0p-24f, w0 = (float)(o.y >> 8) * 0x1.0p-24f;
    const float u1 = ((float)(o.z >> 8) + 1.0f) * 0x1.0p-24f, w1 = (float)(o.w >> 8) * 0x1.0p-24f;
    const float r0 = sqrtf(-2.0f * __logf(u0)), r1 = sqrtf(-2.0f * __logf(u1));
    float s0, c0, s1, c1;
    sincospif(2.0f * w0, &s0, &c0);
    sincospif(2.0f * w1, &s1, &c1);
    z0 = r0 * c0;
    z1 = r0 * s0;
    z2 = r1 * c1;
    z3 = r1 * s1;
}

// FP32 deviates (split-precision path): 24-bit uniforms, |z| <= 5.8
__device__ __forceinline__ void normal_pair_f32(unsigned long long seed, long long step, int particle,
                                                int pair, float& z0, float& z1)
{
    uint4 o = philox4x32_10(make_uint4((unsigned)particle, (unsigned)pair, (unsigned)step,
                                       (unsigned)((unsigned long long)step >> 32)),
                            make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    float u = ((float)(o.x >> 8) + 1.0f) * 0x1.0p-24f;
    float w = (float)(o.z >> 8) * 0x1.0p-24f;
    float rad = sqrtf(-2.0f * logf(u));
    float s, c;
    sincospif(2.0f * w, &s, &c);
    z0 = rad * c;
    z1 = rad * s;
}

// ---------------------------------------------------------------------------
// kernel launchers (host side, defined in the .cu files)
// ---------------------------------------------------------------------------
struct LaunchCfg {
    cudaStream_t stream;
    int grid_stream;      // blocks for streaming kernels
    int grid_force64;     // blocks for the persistent force kernel, FP64 replicas
    int grid_force32;     // ... split-precision replicas
    long long* launches;  // launch counter
};

void launch_load_aos(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, const double* r,
                     const double* v, const double* F, const double* D, const double* disp);
void launch_store_aos(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, double* r,
                      double* v, double* F, double* disp, double* epp);
void launch_rebuild(const Batch& b, const LaunchCfg& lc, int full_list_mode);
void launch_kick_drift(const Batch& b, const LaunchCfg& lc, int has_rescale);
void launch_force(const Batch& b, const LaunchCfg& lc, int mode);
void launch_brownian_update(const Batch& b, const LaunchCfg& lc);
void launch_finalize(const Batch& b, const LaunchCfg& lc, int has_rescale);
void launch_kinetic(const Batch& b, const LaunchCfg& lc);
void launch_load_all(const Batch& b, const LaunchCfg& lc, const double* r, const double* v, const double* F,
                     const double* D, const double* disp);
void launch_store_all(const Batch& b, const LaunchCfg& lc, double* r, double* v, double* F, double* disp);
void launch_export_list(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd,
                        long long* counts, long long* list, long long maxK, int half_only);

enum { FMODE_STEP = 0, FMODE_FORCES = 1, FMODE_ENERGY = 2, FMODE_STEP_ENERGY = 3 };

}  // namespace simmd
