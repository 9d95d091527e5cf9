// simmd_internal.cuh -- device-side data model of libsimmd.
//
// Layout in HBM (one engine = one CUDA stream, many replicas):
//   * a flat SLOT space; replica r owns slots [slot0, slot0 + npad), npad a
//     multiple of TILE; slots hold particles in cell-sorted order after each
//     rebuild, padding slots (orig < 0) never appear in a cell or a list;
//   * per-slot SoA FP64 arrays v, F, displacement; an AoS double4_32a (x,y,z,D)
//     gathered by neighbours; a 16-byte split-precision record (the position
//     as 32-bit box-periodic fixed point per axis, D in FP32); packed
//     rebuild-time cell coordinates; the original particle id;
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
    // split precision: positions as 32-bit fixed point of the periodic box,
    // X = round(x * 2^32 / L) mod 2^32, so x_i - x_j (minimum image) is the
    // int32 difference X_i - X_j times u = L / 2^32
    double fix_scale;          // 2^32 / L
    unsigned long long fix_mul;  // round(2^(32 + fix_sh) / L) < 2^64
    int fix_sh;
    float fix_u, fix_u2;       // u and u^2 rounded to FP32
    float zeta_lo;             // zeta - RN32(zeta)
    float rv2f;
    float Lf, halfLf, csf, rc2f, rcutf, skinf, sigma2f, sigma4f, cut2f, epsf, Ucf, c0f, c2f, c4f, zetaf;
    float noisef, gammaf;      // noise_factor, gamma rounded to FP32
    unsigned long long seed;
    long long xfer_off;        // batched host transfers: offset of this replica's dims x N block
    long long xfer_soff;       // ... and of its N-element block (D)
    const double* host_noise;  // [noise_nsteps][n][dims], original order
    long long noise_step0;
    int noise_nsteps;
    float dmaxf;               // max(D) rounded to FP32: bounds every pair threshold of the build
    double fix_ud;             // u = L / 2^32 (exact)
    // split precision: the skin trigger on the fixed-point displacement
    // since the last rebuild, |X - X_rebuild|^2 > skin_thr (units^2)
    unsigned long long skin_thr;
    // pruned (inner) list of the force pass: the outer-list pairs within
    // rc_ij + prune_skin at the last prune, valid while no particle has moved
    // prune_skin / 2 since (the pairs it drops add exactly zero to the sums)
    int prune;                 // the context keeps inner lists (every replica)
    float prune_rcut_f;        // (1 + 1e-4) sqrt(rc2) (Berthier: times s_ij; LJ: the larger of the force and
                               // energy cutoff radii) in FP32: the inner test's cutoff, with slack
    float prune_skin_f;        // inner skin (FP32)
    unsigned long long prune_thr;  // prune when max |dX|^2 since the last prune exceeds this (fixed-point units^2)
};

struct RepState {
    unsigned long long maxdisp2;  // max |disp|^2: FP64 replicas its bits (a non-negative double), split
                                  // replicas the fixed-point |X - X_rebuild|^2
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
    // swap Monte Carlo
    long long mc_sweep;           // sweeps done (counter of the MC random stream)
    long long mc_target;          // sweep count to reach in this call
    long long mc_counts[4];       // translations accepted, tried; swaps accepted, tried
    double mc_dE;                 // sum of the accepted moves' energy changes
    int mc_next;                  // next particle of the current sweep
    int mc_active;                // replica takes part in the MC call
    // inner list
    unsigned long long maxdisp_in;  // max |X - X_prune|^2 (fixed-point units^2) since the last prune
    int force_prune;              // prune before the next force pass (rebuild, host request)
    int pad_prune;
    long long prunes;             // prunes done
    long long list_entries_in;    // inner-list entries at the last prune
    unsigned long long entries_in_acc;  // ... summed by the prune in progress
};

// split-precision gather record (16 bytes, one 128-bit load): the FP64
// position quantised to 32-bit box-periodic fixed point per axis (z = 0 in
// 2D) and the diameter in FP32
struct __align__(16) FixRec {
    unsigned x, y, z;
    float d;
};

struct Slots {
    double4_32a* posD;                // x, y, z, D
    double *vx, *vy, *vz;
    double *fx, *fy, *fz;
    double *ux, *uy, *uz;         // displacement since the last rebuild
    FixRec* rec;                  // split precision: fixed-point position + D
    int* cellc;                   // packed rebuild-time cell coords (10 bits each)
    int* orig;                    // original id, -1 for padding
    int* inv;                     // slot of original id k of a replica at inv[slot0 + k]
    unsigned* nbr;                // ELL neighbour list
    int* ncnt;                    // neighbours per slot
    unsigned* nbr_in;             // inner (pruned) list, the same layout; null when not kept
    int* ncnt_in;
    FixRec* recp;                 // the record at the last prune (displacement since)
    FixRec* recb;                 // split precision: the record at the last rebuild (displacement since)
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

// sets simmd_last_error's message and returns code (host code)
int record_error(int code, const char* msg);

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
    int defer;                    // stepping force pass: replica sums reduced after the pass
    Slots s;
    double* red_val;              // [RED_LEVELS][ntiles][RED_REC] reduction tree values (sum, error)
    int* red_cnt;                 // [RED_LEVELS][ntiles] members of a tree group done (reset by the last)
    double* warp_part;            // [ntiles][WARP_SLOTS][NPART] warp partials of split tiles
    int* tile_cnt;                // [ntiles] parts of a split tile done (reset by the last)
    int* queue;                   // work-queue heads [4]
    // rebuild plan: tiles and cells of the replicas rebuilding this step
    int* plan_tiles;              // [ntiles]
    int2* plan_cells;             // [cell capacity] (replica, cell)
    int* plan_cnt;                // [0] tiles, [1] cells, [2..3] bodies run (64-bit), [4] copy-back blocks done
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

// split precision: the fixed-point coordinate X = round(x * 2^32 / L) mod
// 2^32 of a position, on the integer pipes only (GB300's FP64 pipe is the
// scarce unit of the position updates): the 53-bit mantissa of x times 2^32/L
// held as a 64-bit fixed-point integer (fix_mul = 2^32/L * 2^fix_sh, top bit
// set), the exact 117-bit product cut at the binary point and rounded half
// up.  Any finite x with |x * 2^32 / L| < 2^84 (else 0); periodic by
// construction (x and x + L give the same X).
__device__ __forceinline__ unsigned fix32(double x, const RepDesc& d)
{
    const long long b = __double_as_longlong(x);
    const long long a = b & 0x7fffffffffffffffll;
    const int ex = (int)(a >> 52) - 1023;
    // x * 2^32 / L = M * fix_mul * 2^(ex - 52 - fix_sh): the integer part
    // starts at bit sh of the product
    const int sh = 52 + d.fix_sh - ex;
    if (ex < -1022 || ex > 1023 || sh >= 128 || sh < 33) return 0u;  // zero/subnormal, inf/nan, < 2^-11, huge
    const unsigned long long M = (unsigned long long)(a & 0xfffffffffffffll) | (1ull << 52);
    const unsigned long long hi = __umul64hi(M, d.fix_mul), lo = M * d.fix_mul;
    unsigned long long v;
    if (sh >= 64) {
        const int s2 = sh - 64;  // 0 .. 63
        v = s2 ? ((hi >> s2) + ((hi >> (s2 - 1)) & 1ull)) : (hi + (lo >> 63));
    } else {
        v = (hi << (64 - sh)) | (lo >> sh);
        v += (lo >> (sh - 1)) & 1ull;
    }
    return (unsigned)((b < 0) ? (0ull - v) : v);
}

__device__ __forceinline__ FixRec fix_rec(double x, double y, double z, double D, const RepDesc& d)
{
    FixRec r;
    r.x = fix32(x, d);
    r.y = fix32(y, d);
    r.z = d.dims == 3 ? fix32(z, d) : 0u;
    r.d = d2f_rn(D);
    return r;
}

__device__ __forceinline__ FixRec rec_get(const FixRec* __restrict__ r)
{
    const uint4 q = __ldg(reinterpret_cast<const uint4*>(r));
    FixRec o;
    o.x = q.x;
    o.y = q.y;
    o.z = q.z;
    o.d = __uint_as_float(q.w);
    return o;
}

__device__ __forceinline__ bool need_rebuild(const RepState& st, const RepDesc& d)
{
    if (st.force_rebuild) return true;
    if (d.prec == PREC_FP32) return st.maxdisp2 > d.skin_thr;
    return __longlong_as_double((long long)st.maxdisp2) > d.skin_half2;
}

__device__ __forceinline__ bool need_prune(const RepState& st, const RepDesc& d)
{
    return d.prune && (st.force_prune || st.maxdisp_in > d.prune_thr);
}

// |X - X0|^2 of two fixed-point records in fixed-point units^2 (exact; the
// int32 wraparound is the minimum image)
__device__ __forceinline__ unsigned long long fix_dist2(const FixRec& a, const FixRec& b)
{
    const long long ex = (int)(a.x - b.x), ey = (int)(a.y - b.y), ez = (int)(a.z - b.z);
    return (unsigned long long)(ex * ex) + (unsigned long long)(ey * ey) + (unsigned long long)(ez * ez);
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
    int grid_copy;        // blocks for the rebuild's copy-back (4 per SM)
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
void launch_set_state_all(const Batch& b, const LaunchCfg& lc, const double* r, const double* v, const double* F,
                          const double* disp);
void launch_export_list(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd,
                        long long* counts, long long* list, long long maxK, int half_only);

// FMODE_STEP_DEFER: FMODE_STEP whose replica sums are reduced after the pass
// (k_replica_means), chosen by the launch for batches of many small replicas
enum { FMODE_STEP = 0, FMODE_FORCES = 1, FMODE_ENERGY = 2, FMODE_STEP_ENERGY = 3, FMODE_STEP_DEFER = 4 };

}  // namespace simmd
