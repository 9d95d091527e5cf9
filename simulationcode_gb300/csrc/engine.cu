// engine.cu -- host runtime of libsimmd and its C ABI (include/simmd.h).
//
// One context = one CUDA device + one stream + a slot space shared by any
// number of replicas (independent systems).  The host keeps the replica
// table (slot / cell ranges from first-fit free lists), launches the kernels
// of k_neighbor.cu, k_force.cu and k_integrate.cu in the order of the
// reference's do_time_step, captures the step loop in a CUDA graph, and
// turns device status flags into the ABI's status codes.
//
// Step sequence (all replicas of the context advance together):
//   Newtonian/Langevin (src/MD.jl:499-554): kick1+drift -> rebuild if the
//     skin trigger fired -> forces + random force + kick2 (+COM sum)
//     [-> kinetic energy / rescale factor when rescale_temperature]
//   Brownian (src/MD.jl:429-471 as intended): forces + random force (+mean
//     force) -> position update -> rebuild if the skin trigger fired
// The COM velocity is subtracted lazily at the next kick1 or by a finalize
// pass at the end of each simmd_step call.
#include "../../include/simmd.h"
#include "simmd_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace simmd {
void launch_rebuild_plan_impl(const Batch& b, const LaunchCfg& lc, cudaGraphConditionalHandle cond, int use_cond);
void launch_rebuild_body_impl(const Batch& b, const LaunchCfg& lc, unsigned* nbr_full, int* ncnt_full, int Kfull);
void launch_mark_rebuild_impl(const int* reps, int n, RepState* state, cudaStream_t s);
void launch_rep_dmax_impl(const Batch& b, const LaunchCfg& lc, const double* D, double* out);
void launch_export_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, const unsigned* lst,
                        const int* cnt, int T, long long* counts, long long* list, long long maxK, int half_only,
                        int* overflow);
void launch_force_impl(const Batch& b, const LaunchCfg& lc, int mode, int prec_mask, double* epp);
int force_blocks_per_sm(int T, int mode, int prec, int parts);
void launch_kick_drift_impl(const Batch& b, const LaunchCfg& lc);
void launch_brownian_update_impl(const Batch& b, const LaunchCfg& lc);
void launch_rescale_impl(const Batch& b, const LaunchCfg& lc);
void launch_kinetic_impl(const Batch& b, const LaunchCfg& lc);
void launch_finalize_impl(const Batch& b, const LaunchCfg& lc);
void launch_load_aos_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, const double* r,
                          const double* v, const double* F, const double* D, const double* disp);
void launch_min_iteration_impl(const Batch& b, const LaunchCfg& lc, double dt, double max_step, double tol,
                               long long max_iters);
void launch_store_aos_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, double* r,
                           double* v, double* F, double* disp, const double* epp_src, double* epp);
void launch_set_state_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, const double* r,
                           const double* v, const double* F, const double* disp);
void launch_check_conversions_impl(long long n, unsigned long long seed, unsigned long long* bad, cudaStream_t s);
void launch_mc_sweeps_impl(const Batch& b, const LaunchCfg& lc, const unsigned* nbr_full, const int* ncnt_full,
                           double max_disp, double swap_prob);
void launch_store_diameters_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd, double* D);
}  // namespace simmd

using namespace simmd;

static thread_local std::string g_last_error;

static int set_err(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

// the same record for entry points defined in other translation units
int simmd::record_error(int code, const char* msg) { return set_err(code, msg); }

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return set_err(e_ == cudaErrorMemoryAllocation ? SIMMD_ERR_OOM : SIMMD_ERR_CUDA,       \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                  \
    } while (0)

struct Range {
    long long start, len;
};

struct HostRep {
    bool active = false;
    simmd_params p{};
    RepDesc d{};
    double smax = 0.0;  // max(D): sets the Verlet radius
    long long steps_done = 0;
    long long noise_draws = 0;
    bool pending_rebuild = false;
    bool pending_prune = false;  // positions set without a rebuild: re-prune before the next force pass
    double inner_skin = 0.0;     // inner-list skin (0: the outer skin, nothing pruned by distance)
};

struct ProfileAcc {
    double force_ms = 0, kick_ms = 0, rebuild_ms = 0, update_ms = 0;
    long long force_n = 0, steps = 0;
};

struct simmd_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t pev[8] = {};
    int sm_count = 1;
    long long S_cap = 0;
    long long C_cap = 0;
    int R_cap = 0;
    int K = 0;
    int T = 1;
    int use_graphs = 1;
    int graph_steps = 16;
    int min_parts = 1;  // force pass: at least this many work items per tile (tile shape)
    int keep_full = 0;
    int Kfull = 0;
    int profile = 0;
    ProfileAcc prof;
    std::vector<HostRep> reps;
    std::vector<Range> free_slots, free_cells;
    Slots s{};
    unsigned* nbr_full = nullptr;
    int* ncnt_full = nullptr;
    double* epp = nullptr;
    RepDesc* d_desc = nullptr;
    RepState* d_state = nullptr;
    int* d_tile_rep = nullptr;
    double* d_red_val = nullptr;
    int* d_red_cnt = nullptr;
    double* d_warp_part = nullptr;
    int* d_tile_cnt = nullptr;
    int* d_queue = nullptr;
    int* d_plan_tiles = nullptr;
    int2* d_plan_cells = nullptr;
    int* d_plan_cnt = nullptr;
    int* d_mark = nullptr;  // replica ids whose rebuild the host requests
    double* d_dmax = nullptr;  // per replica max(D) of a batched upload
    bool xfer_dirty = false;  // host descriptors hold transfer offsets the device copies lack
    int prune_on = 0;         // the force pass reads inner (pruned) lists
    std::vector<int> h_tile_rep;
    std::vector<RepState> h_state;
    double* d_stage = nullptr;  // AoS staging, 5 arrays of stage_cap doubles
    long long stage_cap = 0;
    // asynchronous dump feed: its own staging (r, v, F), side stream, events
    double* d_dump = nullptr;
    long long dump_cap = 0;
    cudaStream_t dump_stream = nullptr;
    cudaEvent_t ev_dump_ready = nullptr, ev_dump_done = nullptr;
    bool dump_pending = false;
    // step-loop capture: rebuild bodies as conditional nodes
    cudaStream_t body_stream = nullptr;
    bool capturing = false;
    cudaError_t capture_error = cudaSuccess;
    double* d_noise = nullptr;
    long long noise_cap = 0;
    long long bytes = 0;
    long long budget = 0;  // 0: no limit on capacity grows
    long long launches = 0;
    long long n_force = 0, n_rebuild = 0;  // force kernel launches, rebuild sequences
    long long max_count_seen = 0;
    // graph cache
    cudaGraphExec_t gexec = nullptr;
    int gkey = -1;
    long long g_launches_per_replay = 0;
    long long g_force_per_replay = 0, g_rebuild_per_replay = 0;
};

// ---------------------------------------------------------------------------
// allocation helpers
// ---------------------------------------------------------------------------
template <typename Tp>
static int dalloc(simmd_ctx* c, Tp** p, size_t count)
{
    *p = nullptr;
    if (count == 0) return SIMMD_OK;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(Tp));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_err(SIMMD_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    c->bytes += (long long)(count * sizeof(Tp));
    return SIMMD_OK;
}

template <typename Tp>
static void dfree(simmd_ctx* c, Tp** p, size_t count)
{
    if (*p) {
        cudaFree(*p);
        c->bytes -= (long long)(count * sizeof(Tp));
    }
    *p = nullptr;
}

#define TRY(x)                        \
    do {                              \
        int st_ = (x);                \
        if (st_ != SIMMD_OK) return st_; \
    } while (0)

static void invalidate_graph(simmd_ctx* c)
{
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
    c->gkey = -1;
}

// grow a per-slot array preserving [0, old)
template <typename Tp>
static int grow_keep(simmd_ctx* c, Tp** p, long long old_n, long long new_n)
{
    Tp* np = nullptr;
    TRY(dalloc(c, &np, (size_t)new_n));
    CK(cudaMemsetAsync(np, 0, (size_t)new_n * sizeof(Tp), c->stream));
    if (*p && old_n > 0) CK(cudaMemcpyAsync(np, *p, (size_t)old_n * sizeof(Tp), cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    dfree(c, p, (size_t)old_n);
    *p = np;
    return SIMMD_OK;
}

template <typename Tp>
static int grow_fresh(simmd_ctx* c, Tp** p, long long old_n, long long new_n)
{
    CK(cudaStreamSynchronize(c->stream));
    dfree(c, p, (size_t)old_n);
    TRY(dalloc(c, p, (size_t)new_n));
    CK(cudaMemsetAsync(*p, 0, (size_t)new_n * sizeof(Tp), c->stream));
    return SIMMD_OK;
}

static int force_rebuild_all(simmd_ctx* c)
{
    for (size_t r = 0; r < c->reps.size(); r++)
        if (c->reps[r].active) c->reps[r].pending_rebuild = true;
    return SIMMD_OK;
}

// device bytes of the capacity-sized arrays: per slot the state (posD 32,
// v/F/u 72), the fixed-point record and its rebuild-time copy 16 + 16, cellc/orig/inv/ncnt 16, rebuild scratch
// (bin/rank/src 12, staged posD/v/F/orig 84), per-particle energy 8 and the
// list 4K; per tile the partial sums, plan and owner; per cell count, start
// and plan entry; per replica its descriptor and state
constexpr long long SLOT_BYTES = 32 + 72 + 16 + 16 + 16 + 12 + 84 + 8;
constexpr long long TILE_BYTES = RED_LEVELS * (RED_REC * 8 + 4) + NPART * 8 * WARP_SLOTS + 4 + 4 + 4;
constexpr long long CELL_BYTES = 4 + 4 + 8;
constexpr long long REP_BYTES = sizeof(RepDesc) + sizeof(RepState) + 4 + 8;

static long long capacity_bytes(const simmd_ctx* c, long long S, long long C, int R, int K)
{
    long long b = S * (SLOT_BYTES + 4LL * K) + (S / TILE) * TILE_BYTES + C * CELL_BYTES +
                  (long long)R * REP_BYTES;
    if (c->keep_full) b += S * (4LL * std::max(K, c->Kfull) + 4);
    if (c->prune_on) b += S * (4LL * K + 4 + 16);
    return b;
}

// (re)size everything that depends on slot capacity S, list rows K, T
static int ensure_capacity(simmd_ctx* c, long long S_need, long long C_need, int R_need, int K_need)
{
    S_need = (S_need + TILE - 1) / TILE * TILE;
    if (K_need < 1) K_need = 1;
    K_need = (K_need + c->T - 1) / c->T * c->T;
    bool grow_s = S_need > c->S_cap;
    bool grow_c = C_need > c->C_cap;
    bool grow_r = R_need > c->R_cap;
    bool grow_k = K_need > c->K;
    if (!grow_s && !grow_c && !grow_r && !grow_k) return SIMMD_OK;
    const long long S_old = c->S_cap, C_old = c->C_cap;
    const int R_old = c->R_cap;
    // geometric growth, or exactly the need when that would break the budget
    long long S_new = grow_s ? std::max(S_need, S_old + S_old / 2) : S_old;
    S_new = (S_new + TILE - 1) / TILE * TILE;
    long long C_new = grow_c ? std::max(C_need, C_old + C_old / 2) : C_old;
    int R_new = grow_r ? std::max(R_need, R_old + R_old / 2 + 1) : R_old;
    const int K_proj = grow_k ? K_need : c->K;
    if (c->budget > 0) {
        const long long now = capacity_bytes(c, S_old, C_old, R_old, c->K);
        auto projected = [&](long long S, long long C, int R) {
            return c->bytes - now + capacity_bytes(c, S, C, R, K_proj);
        };
        if (projected(S_new, C_new, R_new) > c->budget) {
            if (grow_s) S_new = S_need;
            if (grow_c) C_new = C_need;
            if (grow_r) R_new = R_need;
        }
        if (projected(S_new, C_new, R_new) > c->budget)
            return set_err(SIMMD_ERR_BUDGET, "device memory budget exceeded");
    }
    invalidate_graph(c);
    if (grow_s) {
        Slots& s = c->s;
        TRY(grow_keep(c, &s.posD, S_old, S_new));
        TRY(grow_keep(c, &s.vx, S_old, S_new));
        TRY(grow_keep(c, &s.vy, S_old, S_new));
        TRY(grow_keep(c, &s.vz, S_old, S_new));
        TRY(grow_keep(c, &s.fx, S_old, S_new));
        TRY(grow_keep(c, &s.fy, S_old, S_new));
        TRY(grow_keep(c, &s.fz, S_old, S_new));
        TRY(grow_keep(c, &s.ux, S_old, S_new));
        TRY(grow_keep(c, &s.uy, S_old, S_new));
        TRY(grow_keep(c, &s.uz, S_old, S_new));
        TRY(grow_keep(c, &s.rec, S_old, S_new));
        TRY(grow_keep(c, &s.recb, S_old, S_new));
        TRY(grow_keep(c, &s.cellc, S_old, S_new));
        TRY(grow_keep(c, &s.orig, S_old, S_new));
        TRY(grow_keep(c, &s.inv, S_old, S_new));
        TRY(grow_keep(c, &s.ncnt, S_old, S_new));
        TRY(grow_fresh(c, &s.bin_cell, S_old, S_new));
        TRY(grow_fresh(c, &s.bin_rank, S_old, S_new));
        TRY(grow_fresh(c, &s.src, S_old, S_new));
        TRY(grow_fresh(c, &s.t_posD, S_old, S_new));
        TRY(grow_fresh(c, &s.t_vx, S_old, S_new));
        TRY(grow_fresh(c, &s.t_vy, S_old, S_new));
        TRY(grow_fresh(c, &s.t_vz, S_old, S_new));
        TRY(grow_fresh(c, &s.t_fx, S_old, S_new));
        TRY(grow_fresh(c, &s.t_fy, S_old, S_new));
        TRY(grow_fresh(c, &s.t_fz, S_old, S_new));
        TRY(grow_fresh(c, &s.t_orig, S_old, S_new));
        TRY(grow_fresh(c, &c->epp, S_old, S_new));
        long long nt_old = S_old / TILE, nt_new = S_new / TILE;
        TRY(grow_fresh(c, &c->d_red_val, RED_LEVELS * nt_old * RED_REC, RED_LEVELS * nt_new * RED_REC));
        TRY(grow_fresh(c, &c->d_red_cnt, RED_LEVELS * nt_old, RED_LEVELS * nt_new));
        TRY(grow_fresh(c, &c->d_warp_part, nt_old * NPART * WARP_SLOTS, nt_new * NPART * WARP_SLOTS));
        TRY(grow_fresh(c, &c->d_tile_cnt, nt_old, nt_new));
        TRY(grow_fresh(c, &c->d_plan_tiles, nt_old, nt_new));
        TRY(grow_keep(c, &c->d_tile_rep, nt_old, nt_new));
        c->h_tile_rep.resize((size_t)nt_new, -1);
        CK(cudaMemcpyAsync(c->d_tile_rep, c->h_tile_rep.data(), sizeof(int) * nt_new, cudaMemcpyHostToDevice,
                           c->stream));
        // free-list: the new tail
        c->free_slots.push_back({S_old, S_new - S_old});
        c->S_cap = S_new;
    }
    int K_new = grow_k ? K_need : c->K;
    if (grow_s && !grow_k) {
        // tile-major lists: the old tiles keep their addresses, so resident
        // replicas keep their lists and their rebuild schedule
        TRY(grow_keep(c, &c->s.nbr, S_old * (long long)c->K, c->S_cap * (long long)c->K));
        if (c->prune_on) {
            TRY(grow_keep(c, &c->s.nbr_in, S_old * (long long)c->K, c->S_cap * (long long)c->K));
            TRY(grow_keep(c, &c->s.ncnt_in, S_old, c->S_cap));
            TRY(grow_keep(c, &c->s.recp, S_old, c->S_cap));
        }
    }
    if (grow_k) {
        dfree(c, &c->s.nbr, (size_t)S_old * (size_t)c->K);
        TRY(dalloc(c, &c->s.nbr, (size_t)c->S_cap * (size_t)K_new));
        if (c->prune_on) {  // rebuilt, then pruned, before the next force pass
            dfree(c, &c->s.nbr_in, (size_t)S_old * (size_t)c->K);
            TRY(dalloc(c, &c->s.nbr_in, (size_t)c->S_cap * (size_t)K_new));
            if (grow_s) {
                TRY(grow_fresh(c, &c->s.ncnt_in, S_old, c->S_cap));
                TRY(grow_fresh(c, &c->s.recp, S_old, c->S_cap));
            }
        }
        c->K = K_new;
        force_rebuild_all(c);
    }
    if ((grow_s || grow_k) && c->keep_full) {
        // the full list (parity export only) is slot-major: rebuild it
        dfree(c, &c->nbr_full, (size_t)S_old * (size_t)c->Kfull);
        dfree(c, &c->ncnt_full, (size_t)S_old);
        c->Kfull = std::max(c->K, c->Kfull);
        TRY(dalloc(c, &c->nbr_full, (size_t)c->S_cap * (size_t)c->Kfull));
        TRY(dalloc(c, &c->ncnt_full, (size_t)c->S_cap));
        force_rebuild_all(c);
    }
    if (grow_c) {
        TRY(grow_fresh(c, &c->s.cell_count, C_old, C_new));
        TRY(grow_fresh(c, &c->s.cell_start, C_old, C_new));
        TRY(grow_fresh(c, &c->d_plan_cells, C_old, C_new));
        c->free_cells.push_back({C_old, C_new - C_old});
        c->C_cap = C_new;
        // cell counts and starts are scratch of each rebuild: nothing to keep
    }
    if (grow_r) {
        TRY(grow_keep(c, &c->d_desc, R_old, R_new));
        TRY(grow_keep(c, &c->d_state, R_old, R_new));
        TRY(grow_fresh(c, &c->d_mark, R_old, R_new));
        TRY(grow_fresh(c, &c->d_dmax, R_old, R_new));
        c->reps.resize(R_new);
        c->h_state.resize(R_new);
        c->R_cap = R_new;
    }
    // merge adjacent free ranges
    for (auto* fl : {&c->free_slots, &c->free_cells}) {
        std::sort(fl->begin(), fl->end(), [](const Range& a, const Range& b) { return a.start < b.start; });
        std::vector<Range> m;
        for (auto& r : *fl) {
            if (r.len <= 0) continue;
            if (!m.empty() && m.back().start + m.back().len == r.start) m.back().len += r.len;
            else m.push_back(r);
        }
        *fl = m;
    }
    return SIMMD_OK;
}

static bool take_range(std::vector<Range>& fl, long long len, long long* start)
{
    for (size_t k = 0; k < fl.size(); k++) {
        if (fl[k].len >= len) {
            *start = fl[k].start;
            fl[k].start += len;
            fl[k].len -= len;
            if (fl[k].len == 0) fl.erase(fl.begin() + (long)k);
            return true;
        }
    }
    return false;
}

static void give_range(std::vector<Range>& fl, long long start, long long len)
{
    fl.push_back({start, len});
    std::sort(fl.begin(), fl.end(), [](const Range& a, const Range& b) { return a.start < b.start; });
    std::vector<Range> m;
    for (auto& r : fl) {
        if (!m.empty() && m.back().start + m.back().len == r.start) m.back().len += r.len;
        else m.push_back(r);
    }
    fl = m;
}

// work items per tile in the force pass: a batch with fewer tiles than SMs
// splits its tiles until every SM has an item (each block keeps at least one
// full warp); larger batches keep whole tiles, whose particles share their
// neighbours' records in one SM's L1
static int force_parts(const simmd_ctx* c)
{
    long long tiles = 0;
    for (const auto& h : c->reps)
        if (h.active) tiles += h.d.ntiles;
    int parts = 1;
    while (parts < c->min_parts && (TILE / (2 * parts)) * c->T >= 32) parts *= 2;
    while (parts < MAX_PARTS && tiles * parts < c->sm_count && (TILE / (2 * parts)) * c->T >= 32) parts *= 2;
    return parts;
}

// the stepping force pass leaves its replica sums to a pass of their own
// (k_replica_means) when the batch has many tiles in small replicas: the
// pass then runs no block barrier or reduction tree inside its persistent
// loop.  Small batches (an extra launch would show) and large replicas (one
// block reduces each replica's tiles) keep the reduction in the pass
static int force_defer(const simmd_ctx* c)
{
    long long tiles = 0;
    int maxt = 0;
    for (const auto& h : c->reps)
        if (h.active) {
            tiles += h.d.ntiles;
            maxt = std::max(maxt, h.d.ntiles);
        }
    return (tiles >= 4LL * c->sm_count && maxt <= 1024 && force_parts(c) == 1) ? 1 : 0;
}

static Batch make_batch(simmd_ctx* c)
{
    Batch b{};
    b.desc = c->d_desc;
    b.state = c->d_state;
    b.tile_rep = c->d_tile_rep;
    b.ntiles = (int)(c->S_cap / TILE);
    b.nreps = c->R_cap;
    b.S = c->S_cap;
    b.K = c->K;
    b.tpp = c->T;
    b.parts = force_parts(c);
    b.defer = force_defer(c);
    b.s = c->s;
    b.red_val = c->d_red_val;
    b.red_cnt = c->d_red_cnt;
    b.warp_part = c->d_warp_part;
    b.tile_cnt = c->d_tile_cnt;
    b.queue = c->d_queue;
    b.plan_tiles = c->d_plan_tiles;
    b.plan_cells = c->d_plan_cells;
    b.plan_cnt = c->d_plan_cnt;
    return b;
}

static LaunchCfg make_lc(simmd_ctx* c, int mode)
{
    LaunchCfg lc{};
    lc.stream = c->stream;
    long long nt = c->S_cap / TILE;
    lc.grid_stream = (int)std::max(1LL, std::min(nt, (long long)c->sm_count * 16));
    lc.grid_copy = std::max(1, c->sm_count * 4);
    const int parts = force_parts(c);
    lc.grid_force64 = c->sm_count * force_blocks_per_sm(c->T, mode, PREC_FP64, parts);
    lc.grid_force32 = c->sm_count * force_blocks_per_sm(c->T, mode, PREC_FP32, parts);
    lc.launches = &c->launches;
    return lc;
}

// ---------------------------------------------------------------------------
// replica descriptors
// ---------------------------------------------------------------------------
static int validate(const simmd_params* p)
{
    if (!p) return set_err(SIMMD_ERR_BAD_ARG, "params is NULL");
    if (p->dims != 2 && p->dims != 3) return set_err(SIMMD_ERR_BAD_ARG, "dims must be 2 or 3 (To be implemented)");
    if (p->N < 1 || p->N > (1LL << 24)) return set_err(SIMMD_ERR_BAD_ARG, "N out of range [1, 2^24]");
    if (p->potential != SIMMD_POT_LJ && p->potential != SIMMD_POT_BERTHIER)
        return set_err(SIMMD_ERR_BAD_ARG, "unknown potential");
    if (p->dynamics < SIMMD_NEWTONIAN || p->dynamics > SIMMD_BROWNIAN)
        return set_err(SIMMD_ERR_BAD_ARG, "unknown dynamics");
    if (p->precision != SIMMD_FP64 && p->precision != SIMMD_FP32_SPLIT)
        return set_err(SIMMD_ERR_BAD_ARG, "unknown precision");
    if (!(p->box_size > 0) || !(p->force_cutoff2 > 0) || !(p->skin >= 0) || !(p->dt > 0))
        return set_err(SIMMD_ERR_BAD_ARG, "box_size, force_cutoff2, dt must be > 0 and skin >= 0");
    if (p->dynamics != SIMMD_NEWTONIAN && !(p->gamma > 0)) return set_err(SIMMD_ERR_BAD_ARG, "gamma must be > 0");
    if (p->dynamics != SIMMD_BROWNIAN && !(p->m > 0)) return set_err(SIMMD_ERR_BAD_ARG, "m must be > 0");
    return SIMMD_OK;
}

static double max_diameter(const double* D, long long N)
{
    double smax = D[0];
    for (long long i = 1; i < N; i++) smax = std::max(smax, D[i]);
    return smax;
}

static int fill_desc_smax(const simmd_params* p, double smax, RepDesc& d);

static int fill_desc(const simmd_params* p, const double* D, RepDesc& d)
{
    return fill_desc_smax(p, max_diameter(D, p->N), d);
}

static int fill_desc_smax(const simmd_params* p, double smax, RepDesc& d)
{
    if (!(smax > 0)) return set_err(SIMMD_ERR_BAD_ARG, "diameters must be positive");
    double rc_v = p->verlet_force_cutoff > 0 ? p->verlet_force_cutoff : std::sqrt(p->force_cutoff2);
    double rv = p->skin + rc_v * smax;  // verlet_sphere_size, src/DataStructs.jl:351-352
    double L = p->box_size;
    if (!(rv < 0.5 * L)) return set_err(SIMMD_ERR_BAD_ARG, "Verlet sphere (skin + rc*max(D)) must be < box/2");
    long long nc = (long long)std::floor(L / rv);
    if (nc < 3) nc = 1;
    if (nc > MAX_CELLS_AXIS) nc = MAX_CELLS_AXIS;
    memset(&d, 0, sizeof(d));
    d.n = (int)p->N;
    d.npad = (int)((p->N + TILE - 1) / TILE * TILE);
    d.ntiles = d.npad / TILE;
    d.dims = p->dims;
    d.pot = p->potential;
    d.dyn = p->dynamics;
    d.prec = p->precision;
    d.nc = (int)nc;
    d.ncell = (int)(p->dims == 3 ? nc * nc * nc : nc * nc);
    d.rescale = (p->dynamics == SIMMD_NEWTONIAN && p->rescale_temperature) ? 1 : 0;
    d.noise_mode = NOISE_PHILOX;
    d.active = 1;
    d.L = L;
    d.halfL = L * 0.5;
    d.cs = L / (double)nc;
    d.inv_cs = (double)nc / L;
    d.rc2 = p->force_cutoff2;
    d.rcut = std::sqrt(p->force_cutoff2);
    d.skin = p->skin;
    d.rv2 = rv * rv;
    double h = p->skin / 2.0;
    d.skin_half2 = h * h;
    d.sigma2 = p->lj_sigma * p->lj_sigma;
    d.sigma4 = d.sigma2 * d.sigma2;
    d.lj_cut2 = (p->dims == 3) ? d.rc2 * d.sigma2 : d.rc2 * d.sigma4;
    d.eps = p->lj_eps;
    d.Uc = p->lj_Uc;
    d.c0 = p->b_c0;
    d.c2 = p->b_c2;
    d.c4 = p->b_c4;
    d.zeta = p->b_zeta;
    d.kBT = p->kBT;
    d.gamma = p->gamma;
    d.dt = p->dt;
    d.m = p->m;
    d.noise_factor = (p->dynamics == SIMMD_NEWTONIAN) ? 0.0 : std::sqrt(2.0 * p->kBT * p->gamma / p->dt);
    d.dt_over_gamma = (p->dynamics == SIMMD_BROWNIAN) ? p->dt / p->gamma : 0.0;
    d.two_m = 2.0 * p->m;
    d.m_half = p->m / 2.0;
    d.Lf = (float)L;
    d.halfLf = (float)(L * 0.5);
    d.csf = (float)d.cs;
    d.rc2f = (float)d.rc2;
    d.rcutf = (float)d.rcut;
    d.skinf = (float)d.skin;
    d.sigma2f = (float)d.sigma2;
    d.sigma4f = (float)d.sigma4;
    d.cut2f = (float)d.lj_cut2;
    d.epsf = (float)d.eps;
    d.Ucf = (float)d.Uc;
    d.c0f = (float)d.c0;
    d.c2f = (float)d.c2;
    d.c4f = (float)d.c4;
    d.zetaf = (float)d.zeta;
    d.noisef = (float)d.noise_factor;
    d.gammaf = (float)d.gamma;
    d.seed = p->seed;
    // floor(rnew/L) of the wrap (src/MD.jl:520) without a divide: RN(x/L) >= 1
    // exactly when x >= wrap_hi (found with IEEE host division)
    double wx = L;
    for (int k = 0; k < 64; k++) {
        double q = std::nextafter(wx, 0.0);
        if (q / L >= 1.0) wx = q;
        else break;
    }
    d.wrap_hi = wx;
    int ex = 0;
    double mant = std::frexp(d.two_m, &ex);
    d.two_m_pow2 = (mant == 0.5) ? 1 : 0;
    d.inv_two_m = 1.0 / d.two_m;
    d.dt_over_two_m = d.dt * d.inv_two_m;
    // split precision: 32-bit fixed point of the periodic box
    d.fix_scale = 4294967296.0 / L;
    {  // 2^32/L as a 64-bit fixed-point integer with its top bit set
        int e2 = 0;
        std::frexp(d.fix_scale, &e2);  // fix_scale in [2^(e2-1), 2^e2)
        d.fix_sh = 64 - e2;
        d.fix_mul = (unsigned long long)std::ldexp(d.fix_scale, d.fix_sh - 11) << 11;  // 53 significant bits
    }
    d.fix_u = (float)(L / 4294967296.0);
    d.fix_ud = L / 4294967296.0;
    {  // split precision's skin trigger in fixed-point units: a fixed-point
       // displacement |dX| bounds the true one by (|dX| + sqrt(3)) u (each
       // coordinate rounded to u/2 at both ends), so |dX| <= skin/(2u) -
       // sqrt(3) keeps it <= skin/2; one unit more of slack
        const double A = p->skin / (2.0 * d.fix_ud) - std::sqrt(3.0) - 1.0;
        d.skin_thr = A > 0.0 ? (unsigned long long)std::floor(A * A) : 0ull;
    }
    d.fix_u2 = (float)((L / 4294967296.0) * (L / 4294967296.0));
    d.zeta_lo = (float)(d.zeta - (double)(float)d.zeta);
    d.rv2f = (float)d.rv2;
    d.dmaxf = (float)smax;
    // build candidates are relative to the home cell centre: a home particle
    // and a stencil candidate differ by at most 2 cs per axis, which needs
    // no minimum image below L/2
    d.build_wrap = (nc >= 3 && 2.0 * d.cs + 1e-3 < 0.5 * L) ? 0 : 1;
    return SIMMD_OK;
}

// the inner-list fields of a replica's descriptor (after every fill_desc):
// the inner skin (the outer skin when none is set: the distance test then
// keeps every listed pair), the cutoff of the inner test with 1e-4 slack, and
// the displacement trigger in fixed-point units.  A fixed-point displacement
// |dX| bounds the true one by (|dX| + sqrt(3)) u (each coordinate is rounded
// to u/2 at both ends), so |dX| <= s_in/(2u) - sqrt(3) keeps it <= s_in/2;
// one unit more of slack
static void apply_prune_desc(const simmd_ctx* c, HostRep& h)
{
    RepDesc& d = h.d;
    d.prune = c->prune_on;
    const double s_in = (h.inner_skin > 0.0 && h.inner_skin < d.skin) ? h.inner_skin : d.skin;
    d.prune_skin_f = (float)s_in;
    const double rc = (d.pot == POT_BERTHIER) ? d.rcut : std::sqrt(std::max(d.rc2, d.lj_cut2));
    d.prune_rcut_f = (float)(rc * (1.0 + 1e-4));
    const double u = d.L / 4294967296.0;
    const double A = s_in / (2.0 * u) - std::sqrt(3.0) - 1.0;
    d.prune_thr = A > 0.0 ? (unsigned long long)std::floor(A * A) : 0ull;
}

static int push_desc(simmd_ctx* c, int r)
{
    CK(cudaMemcpyAsync(c->d_desc + r, &c->reps[r].d, sizeof(RepDesc), cudaMemcpyHostToDevice, c->stream));
    return SIMMD_OK;
}

static int set_tiles(simmd_ctx* c, int r, int value)
{
    const RepDesc& d = c->reps[r].d;
    for (int t = 0; t < d.ntiles; t++) c->h_tile_rep[d.tile0 + t] = value;
    CK(cudaMemcpyAsync(c->d_tile_rep + d.tile0, c->h_tile_rep.data() + d.tile0, sizeof(int) * d.ntiles,
                       cudaMemcpyHostToDevice, c->stream));
    return SIMMD_OK;
}

static int ensure_stage(simmd_ctx* c, long long n)
{
    if (n <= c->stage_cap) return SIMMD_OK;
    CK(cudaStreamSynchronize(c->stream));
    dfree(c, &c->d_stage, (size_t)(5 * c->stage_cap));
    long long cap = std::max(n, c->stage_cap * 2);
    TRY(dalloc(c, &c->d_stage, (size_t)(5 * cap)));
    c->stage_cap = cap;
    return SIMMD_OK;
}

static int reset_state(simmd_ctx* c, int r, bool keep_counters)
{
    RepState st{};
    if (keep_counters) {
        CK(cudaMemcpyAsync(&st, c->d_state + r, sizeof(RepState), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    long long step = keep_counters ? st.step : 0, rb = keep_counters ? st.rebuilds : 0;
    int mc = keep_counters ? st.maxcount : 0;
    memset(&st, 0, sizeof(st));
    st.step = step;
    st.rebuilds = rb;
    st.maxcount = mc;
    st.vscale = 1.0;
    st.force_rebuild = 1;
    st.force_prune = 1;
    CK(cudaMemcpyAsync(c->d_state + r, &st, sizeof(RepState), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->h_state[r] = st;
    c->reps[r].pending_rebuild = true;
    return SIMMD_OK;
}

static int upload_rep(simmd_ctx* c, int r, const double* rr, const double* v, const double* F, const double* D,
                      const double* disp)
{
    HostRep& h = c->reps[r];
    const long long nd = h.p.N * h.p.dims;
    TRY(ensure_stage(c, std::max<long long>(nd, (long long)h.p.N)));
    double* st = c->d_stage;
    double *dr = st, *dv = st + c->stage_cap, *dF = st + 2 * c->stage_cap, *dD = st + 3 * c->stage_cap,
           *du = st + 4 * c->stage_cap;
    CK(cudaMemcpyAsync(dr, rr, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
    if (v) CK(cudaMemcpyAsync(dv, v, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
    if (F) CK(cudaMemcpyAsync(dF, F, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dD, D, sizeof(double) * h.p.N, cudaMemcpyHostToDevice, c->stream));
    if (disp) CK(cudaMemcpyAsync(du, disp, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    launch_load_aos_impl(b, lc, r, h.d, dr, v ? dv : nullptr, F ? dF : nullptr, dD, disp ? du : nullptr);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

static int add_replica(simmd_ctx* c, const simmd_params* p, const double* r, const double* v, const double* F,
                       const double* D, int* out)
{
    TRY(validate(p));
    if (!r || !D) return set_err(SIMMD_ERR_BAD_ARG, "r and D are required");
    RepDesc d;
    TRY(fill_desc(p, D, d));
    int K_need = p->max_neighbors > 0 ? p->max_neighbors : 200;
    // find a replica id
    int rid = -1;
    for (int k = 0; k < c->R_cap; k++)
        if (!c->reps[k].active) { rid = k; break; }
    int R_need = rid < 0 ? c->R_cap + 1 : c->R_cap;
    long long start = 0, cstart = 0;
    bool have_s = take_range(c->free_slots, d.npad, &start);
    bool have_c = take_range(c->free_cells, d.ncell + 1, &cstart);
    if (have_s) give_range(c->free_slots, start, d.npad);
    if (have_c) give_range(c->free_cells, cstart, d.ncell + 1);
    long long S_need = have_s ? c->S_cap : c->S_cap + d.npad;
    long long C_need = have_c ? c->C_cap : c->C_cap + d.ncell + 1;
    TRY(ensure_capacity(c, S_need, C_need, R_need, std::max(K_need, c->K)));
    if (rid < 0)
        for (int k = 0; k < c->R_cap; k++)
            if (!c->reps[k].active) { rid = k; break; }
    if (!take_range(c->free_slots, d.npad, &start)) return set_err(SIMMD_ERR_BUDGET, "slot allocation failed");
    if (!take_range(c->free_cells, d.ncell + 1, &cstart)) {
        give_range(c->free_slots, start, d.npad);
        return set_err(SIMMD_ERR_BUDGET, "cell allocation failed");
    }
    d.slot0 = start;
    d.tile0 = (int)(start / TILE);
    d.cell0 = (int)cstart;
    HostRep& h = c->reps[rid];
    h = HostRep();
    h.active = true;
    h.p = *p;
    h.d = d;
    h.smax = max_diameter(D, p->N);
    apply_prune_desc(c, h);
    TRY(push_desc(c, rid));
    TRY(reset_state(c, rid, false));
    TRY(upload_rep(c, rid, r, v, F, D, nullptr));
    TRY(set_tiles(c, rid, rid));
    CK(cudaStreamSynchronize(c->stream));
    *out = rid;
    return SIMMD_OK;
}

static int remove_replica(simmd_ctx* c, int rid)
{
    if (rid < 0 || rid >= c->R_cap || !c->reps[rid].active) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    HostRep& h = c->reps[rid];
    TRY(set_tiles(c, rid, -1));
    h.d.active = 0;
    TRY(push_desc(c, rid));
    give_range(c->free_slots, h.d.slot0, h.d.npad);
    give_range(c->free_cells, h.d.cell0, h.d.ncell + 1);
    h.active = false;
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

// ---------------------------------------------------------------------------
// step sequencing
// ---------------------------------------------------------------------------
struct Mix {
    bool nl = false, br = false, rescale = false, noise = false;
    int prec_mask = 0;  // bit 0: FP64 replicas, bit 1: split precision
};

static Mix batch_mix(simmd_ctx* c)
{
    Mix m;
    for (auto& h : c->reps) {
        if (!h.active) continue;
        if (h.p.dynamics == SIMMD_BROWNIAN) m.br = true;
        else m.nl = true;
        if (h.d.rescale) m.rescale = true;
        if (h.p.dynamics != SIMMD_NEWTONIAN) m.noise = true;
        m.prec_mask |= (h.d.prec == PREC_FP64) ? 1 : 2;
    }
    return m;
}

// the rebuild sequence: plan, then (when some replica's trigger fired) the
// body.  Direct launches run the body always (its kernels find an empty
// plan); inside a stream capture of the step loop the body becomes a
// conditional IF node whose condition the plan kernel sets.
static void rebuild_launch(simmd_ctx* c, const Batch& b, const LaunchCfg& lc)
{
    c->n_rebuild += 1;
    unsigned* nf = c->keep_full ? c->nbr_full : nullptr;
    int* cf = c->keep_full ? c->ncnt_full : nullptr;
    if (!c->capturing) {
        launch_rebuild_plan_impl(b, lc, 0, 0);
        launch_rebuild_body_impl(b, lc, nf, cf, c->Kfull);
        return;
    }
    auto fail = [&](cudaError_t e) {
        if (e != cudaSuccess && c->capture_error == cudaSuccess) c->capture_error = e;
        return e != cudaSuccess;
    };
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t nd = 0;
    if (fail(cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, &deps, &edges, &nd))) return;
    cudaGraphConditionalHandle h;
    if (fail(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault))) return;
    launch_rebuild_plan_impl(b, lc, h, 1);
    if (fail(cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, &deps, &edges, &nd))) return;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (fail(cudaGraphAddNode(&node, g, deps, edges, nd, &np))) return;
    cudaGraph_t body = np.conditional.phGraph_out[0];
    if (fail(cudaStreamBeginCaptureToGraph(c->body_stream, body, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal)))
        return;
    LaunchCfg lb = lc;
    lb.stream = c->body_stream;
    launch_rebuild_body_impl(b, lb, nf, cf, c->Kfull);
    cudaGraph_t captured = nullptr;
    if (fail(cudaStreamEndCapture(c->body_stream, &captured))) return;
    fail(cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
}

static void enqueue_step(simmd_ctx* c, const Batch& b, const LaunchCfg& lc, const Mix& m, int fmode)
{
    const bool prof = c->profile != 0;
    if (m.nl) {
        if (prof) cudaEventRecord(c->pev[0], c->stream);
        launch_kick_drift_impl(b, lc);
        if (prof) cudaEventRecord(c->pev[1], c->stream);
        rebuild_launch(c, b, lc);
        if (prof) cudaEventRecord(c->pev[2], c->stream);
    }
    if (prof) cudaEventRecord(c->pev[3], c->stream);
    launch_force_impl(b, lc, fmode, m.prec_mask, nullptr);
    c->n_force += __builtin_popcount(m.prec_mask);
    if (prof) cudaEventRecord(c->pev[4], c->stream);
    if (m.rescale) launch_rescale_impl(b, lc);
    if (m.br) {
        if (prof) cudaEventRecord(c->pev[5], c->stream);
        launch_brownian_update_impl(b, lc);
        if (prof) cudaEventRecord(c->pev[6], c->stream);
        rebuild_launch(c, b, lc);
        if (prof) cudaEventRecord(c->pev[7], c->stream);
    }
    if (prof) {
        cudaStreamSynchronize(c->stream);
        float ms = 0;
        if (m.nl) {
            cudaEventElapsedTime(&ms, c->pev[0], c->pev[1]);
            c->prof.kick_ms += ms;
            cudaEventElapsedTime(&ms, c->pev[1], c->pev[2]);
            c->prof.rebuild_ms += ms;
        }
        cudaEventElapsedTime(&ms, c->pev[3], c->pev[4]);
        c->prof.force_ms += ms;
        c->prof.force_n += 1;
        if (m.br) {
            cudaEventElapsedTime(&ms, c->pev[5], c->pev[6]);
            c->prof.update_ms += ms;
            cudaEventElapsedTime(&ms, c->pev[6], c->pev[7]);
            c->prof.rebuild_ms += ms;
        }
        c->prof.steps += 1;
    }
}

// the host's rebuild and prune requests (a new or re-uploaded replica, a
// skin change, simmd_rebuild, positions set by the host): one copy of the
// replica ids and one marking kernel, then the rebuild sequence, which works
// only on the marked replicas (a requested prune is done by the next force
// pass)
static int pending_rebuilds(simmd_ctx* c)
{
    std::vector<int> ids;
    bool any = false;
    for (int r = 0; r < c->R_cap; r++) {
        HostRep& h = c->reps[r];
        if (h.active && (h.pending_rebuild || h.pending_prune)) {
            ids.push_back(r * 4 + (h.pending_rebuild ? 1 : 0) + (h.pending_prune ? 2 : 0));
            any = any || h.pending_rebuild;
            h.pending_rebuild = false;
            h.pending_prune = false;
        }
    }
    if (!ids.empty()) {
        CK(cudaMemcpyAsync(c->d_mark, ids.data(), sizeof(int) * ids.size(), cudaMemcpyHostToDevice, c->stream));
        launch_mark_rebuild_impl(c->d_mark, (int)ids.size(), c->d_state, c->stream);
    }
    if (any) {
        Batch b = make_batch(c);
        LaunchCfg lc = make_lc(c, FMODE_STEP);
        rebuild_launch(c, b, lc);
        CK(cudaGetLastError());
    }
    return SIMMD_OK;
}

static int read_states(simmd_ctx* c)
{
    CK(cudaMemcpyAsync(c->h_state.data(), c->d_state, sizeof(RepState) * c->R_cap, cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int st = SIMMD_OK;
    for (int r = 0; r < c->R_cap; r++) {
        if (!c->reps[r].active) continue;
        const RepState& s = c->h_state[r];
        c->max_count_seen = std::max<long long>(c->max_count_seen, s.maxcount);
        if (s.overflow && st == SIMMD_OK)
            st = set_err(SIMMD_ERR_NEIGHBOR_OVERFLOW, "neighbour list overflow: raise max_neighbors");
        if (s.nonfinite && st == SIMMD_OK) st = set_err(SIMMD_ERR_NONFINITE, "non-finite position or displacement");
        if (s.noise_range_error && st == SIMMD_OK) st = set_err(SIMMD_ERR_NOISE_RANGE, "host noise array too short");
    }
    return st;
}

static int graph_key(const simmd_ctx* c, const Mix& m, int fmode)
{
    return (m.nl ? 1 : 0) | (m.br ? 2 : 0) | (m.rescale ? 4 : 0) | (m.prec_mask << 3) | (fmode << 5) |
           (force_parts(c) << 8) | (force_defer(c) << 16);
}

static int run_steps(simmd_ctx* c, long long nsteps, const double* noise)
{
    if (nsteps < 0) return set_err(SIMMD_ERR_BAD_ARG, "nsteps < 0");
    int nact = 0, single = -1;
    for (int r = 0; r < c->R_cap; r++)
        if (c->reps[r].active) { nact++; single = r; }
    if (nact == 0) return SIMMD_OK;
    TRY(pending_rebuilds(c));
    Mix m = batch_mix(c);
    Batch b = make_batch(c);
    const int fmode = FMODE_STEP;
    LaunchCfg lc = make_lc(c, fmode);
    if (noise && m.noise) {
        if (nact != 1) return set_err(SIMMD_ERR_BAD_ARG, "host noise requires a single-replica context");
        HostRep& h = c->reps[single];
        long long nd = nsteps * h.p.N * h.p.dims;
        if (nd > c->noise_cap) {
            CK(cudaStreamSynchronize(c->stream));
            dfree(c, &c->d_noise, (size_t)c->noise_cap);
            TRY(dalloc(c, &c->d_noise, (size_t)nd));
            c->noise_cap = nd;
        }
        CK(cudaMemcpyAsync(c->d_noise, noise, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(&c->h_state[single], c->d_state + single, sizeof(RepState), cudaMemcpyDeviceToHost,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
        h.d.noise_mode = NOISE_HOST;
        h.d.host_noise = c->d_noise;
        h.d.noise_step0 = c->h_state[single].step;
        h.d.noise_nsteps = (int)nsteps;
        TRY(push_desc(c, single));
        for (long long s = 0; s < nsteps; s++) enqueue_step(c, b, lc, m, fmode);
        CK(cudaGetLastError());
        h.d.noise_mode = NOISE_PHILOX;
        h.d.host_noise = nullptr;
        TRY(push_desc(c, single));
    } else if (c->use_graphs && !c->profile && nsteps >= c->graph_steps) {
        int key = graph_key(c, m, fmode);
        if (!c->gexec || c->gkey != key) {
            invalidate_graph(c);
            cudaGraph_t g;
            long long l0 = c->launches, f0 = c->n_force, r0 = c->n_rebuild;
            CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            c->capturing = true;
            c->capture_error = cudaSuccess;
            for (int s = 0; s < c->graph_steps; s++) enqueue_step(c, b, lc, m, fmode);
            c->capturing = false;
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (e == cudaSuccess && c->capture_error != cudaSuccess) {
                cudaGraphDestroy(g);
                e = c->capture_error;
            }
            c->g_launches_per_replay = c->launches - l0;
            c->g_force_per_replay = c->n_force - f0;
            c->g_rebuild_per_replay = c->n_rebuild - r0;
            c->launches = l0;
            c->n_force = f0;
            c->n_rebuild = r0;
            CK(e);
            e = cudaGraphInstantiate(&c->gexec, g, 0);
            cudaGraphDestroy(g);
            CK(e);
            c->gkey = key;
        }
        long long reps = nsteps / c->graph_steps;
        for (long long k = 0; k < reps; k++) {
            CK(cudaGraphLaunch(c->gexec, c->stream));
            c->launches += c->g_launches_per_replay;
            c->n_force += c->g_force_per_replay;
            c->n_rebuild += c->g_rebuild_per_replay;
        }
        for (long long s = reps * c->graph_steps; s < nsteps; s++) enqueue_step(c, b, lc, m, fmode);
        CK(cudaGetLastError());
    } else {
        for (long long s = 0; s < nsteps; s++) enqueue_step(c, b, lc, m, fmode);
        CK(cudaGetLastError());
    }
    if (m.nl) launch_finalize_impl(b, lc);
    CK(cudaGetLastError());
    for (int r = 0; r < c->R_cap; r++)
        if (c->reps[r].active) c->reps[r].steps_done += nsteps;
    return read_states(c);
}

// ---------------------------------------------------------------------------
// batched host transfers: every active replica in one call, host layout =
// the replicas in id order, each its dims x N block (and N-element block)
// ---------------------------------------------------------------------------
// offsets of the active replicas in the batched layout; true when some
// replica's offsets changed (the device descriptors must be refreshed)
static bool xfer_layout(simmd_ctx* c, long long* nvec, long long* nsc)
{
    long long off = 0, soff = 0;
    bool changed = false;
    for (int r = 0; r < c->R_cap; r++) {
        HostRep& h = c->reps[r];
        if (!h.active) continue;
        if (h.d.xfer_off != off || h.d.xfer_soff != soff) changed = c->xfer_dirty = true;
        h.d.xfer_off = off;
        h.d.xfer_soff = soff;
        off += h.p.N * h.p.dims;
        soff += h.p.N;
    }
    *nvec = off;
    *nsc = soff;
    return changed;
}

// every replica's descriptor in one copy (staged in a host vector the
// asynchronous copy reads, so kept until the stream synchronises)
static int push_all_desc(simmd_ctx* c, std::vector<RepDesc>& staging)
{
    staging.resize((size_t)c->R_cap);
    for (int r = 0; r < c->R_cap; r++) staging[(size_t)r] = c->reps[r].d;
    CK(cudaMemcpyAsync(c->d_desc, staging.data(), sizeof(RepDesc) * (size_t)c->R_cap, cudaMemcpyHostToDevice,
                       c->stream));
    c->xfer_dirty = false;
    return SIMMD_OK;
}

// a replica's descriptor from its (new) diameters: the Verlet radius and
// the cell grid follow max(D); slots, tiles and transfer offsets stay
static int refresh_desc_smax(simmd_ctx* c, int rep, double smax)
{
    HostRep& h = c->reps[rep];
    RepDesc d;
    TRY(fill_desc_smax(&h.p, smax, d));
    h.smax = smax;
    if (d.ncell != h.d.ncell) {
        give_range(c->free_cells, h.d.cell0, h.d.ncell + 1);
        long long cstart;
        if (!take_range(c->free_cells, d.ncell + 1, &cstart)) {
            TRY(ensure_capacity(c, c->S_cap, c->C_cap + d.ncell + 1, c->R_cap, c->K));
            if (!take_range(c->free_cells, d.ncell + 1, &cstart)) return set_err(SIMMD_ERR_BUDGET, "cells");
        }
        d.cell0 = (int)cstart;
    } else {
        d.cell0 = h.d.cell0;
    }
    d.slot0 = h.d.slot0;
    d.tile0 = h.d.tile0;
    d.xfer_off = h.d.xfer_off;
    d.xfer_soff = h.d.xfer_soff;
    h.d = d;
    apply_prune_desc(c, h);
    return SIMMD_OK;
}

static int refresh_desc(simmd_ctx* c, int rep, const double* D)
{
    return refresh_desc_smax(c, rep, max_diameter(D, c->reps[rep].p.N));
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* simmd_version(void) { return "simmd 0.1.0 (sm_103a)"; }

const char* simmd_status_string(int status)
{
    switch (status) {
        case SIMMD_OK: return "ok";
        case SIMMD_ERR_BAD_ARG: return "bad argument";
        case SIMMD_ERR_CUDA: return "CUDA error";
        case SIMMD_ERR_OOM: return "out of device memory";
        case SIMMD_ERR_NEIGHBOR_OVERFLOW: return "neighbour list overflow";
        case SIMMD_ERR_NONFINITE: return "non-finite state";
        case SIMMD_ERR_NOISE_RANGE: return "noise array too short";
        case SIMMD_ERR_BUDGET: return "capacity or budget exceeded";
        case SIMMD_ERR_NOT_FOUND: return "replica not found";
        case SIMMD_ERR_NO_DEVICE: return "no CUDA device";
        case SIMMD_ERR_NOT_CONVERGED: return "not converged";
        default: return "unknown status";
    }
}

const char* simmd_last_error(void) { return g_last_error.c_str(); }

int simmd_device_count(int32_t* n)
{
    int k = 0;
    cudaError_t e = cudaGetDeviceCount(&k);
    if (e != cudaSuccess) {
        cudaGetLastError();
        k = 0;
    }
    if (n) *n = k;
    return SIMMD_OK;
}

int simmd_engine_create(int32_t device, simmd_ctx** out)
{
    if (!out) return set_err(SIMMD_ERR_BAD_ARG, "out is NULL");
    *out = nullptr;
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) {
        cudaGetLastError();
        return set_err(SIMMD_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= nd) return set_err(SIMMD_ERR_BAD_ARG, "bad device index");
    CK(cudaSetDevice(device));
    simmd_ctx* c = new simmd_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
        delete c;
        return set_err(SIMMD_ERR_CUDA, "stream/event creation failed");
    }
    for (auto& e : c->pev) cudaEventCreate(&e);
    if (cudaStreamCreateWithFlags(&c->body_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->dump_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_dump_ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_dump_done, cudaEventDisableTiming) != cudaSuccess) {
        delete c;
        return set_err(SIMMD_ERR_CUDA, "dump stream/event creation failed");
    }
    int st = dalloc(c, &c->d_queue, 4);
    if (st == SIMMD_OK) st = cudaMemsetAsync(c->d_queue, 0, 4 * sizeof(int), c->stream) == cudaSuccess ? 0 : SIMMD_ERR_CUDA;
    if (st == SIMMD_OK) st = dalloc(c, &c->d_plan_cnt, 8);
    if (st == SIMMD_OK)
        st = cudaMemsetAsync(c->d_plan_cnt, 0, 8 * sizeof(int), c->stream) == cudaSuccess ? 0 : SIMMD_ERR_CUDA;
    if (st != SIMMD_OK) {
        delete c;
        return st;
    }
    *out = c;
    return SIMMD_OK;
}

static void destroy_ctx(simmd_ctx* c)
{
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    invalidate_graph(c);
    Slots& s = c->s;
    void* ptrs[] = {s.posD, s.vx, s.vy, s.vz, s.fx, s.fy, s.fz, s.ux, s.uy, s.uz, s.rec, s.cellc, s.orig, s.inv, s.nbr,
                    s.ncnt, s.bin_cell, s.bin_rank, s.src, s.t_posD, s.t_vx, s.t_vy, s.t_vz, s.t_fx, s.t_fy,
                    s.t_fz, s.t_orig, s.cell_count, s.cell_start, c->nbr_full, c->ncnt_full, c->epp, c->d_desc,
                    c->d_state, c->d_tile_rep, c->d_red_val, c->d_red_cnt, c->d_warp_part, c->d_tile_cnt, c->d_queue, c->d_stage, c->d_dump, c->d_noise,
                    c->d_plan_tiles, c->d_plan_cells, c->d_plan_cnt, c->d_mark, c->d_dmax, s.nbr_in, s.ncnt_in, s.recp, s.recb};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (c->dump_stream) cudaStreamSynchronize(c->dump_stream);
    cudaEventDestroy(c->ev0);
    cudaEventDestroy(c->ev1);
    if (c->ev_dump_ready) cudaEventDestroy(c->ev_dump_ready);
    if (c->ev_dump_done) cudaEventDestroy(c->ev_dump_done);
    if (c->dump_stream) cudaStreamDestroy(c->dump_stream);
    if (c->body_stream) cudaStreamDestroy(c->body_stream);
    for (auto& e : c->pev) cudaEventDestroy(e);
    cudaStreamDestroy(c->stream);
    delete c;
}

int simmd_destroy(simmd_ctx* ctx)
{
    if (ctx) destroy_ctx(ctx);
    return SIMMD_OK;
}

int simmd_create(const simmd_params* p, simmd_ctx** out)
{
    TRY(validate(p));
    int dev = 0;
    cudaGetDevice(&dev);
    cudaGetLastError();
    TRY(simmd_engine_create(dev, out));
    simmd_ctx* c = *out;
    // reserve the single system's shape; data arrive with simmd_upload
    RepDesc d;
    std::vector<double> ones((size_t)p->N, p->potential == SIMMD_POT_LJ ? p->lj_sigma : 1.0);
    int st = fill_desc(p, ones.data(), d);
    if (st == SIMMD_OK) st = ensure_capacity(c, d.npad, (long long)d.ncell * 8 + 64, 1,
                                             p->max_neighbors > 0 ? p->max_neighbors : 200);
    if (st != SIMMD_OK) {
        destroy_ctx(c);
        *out = nullptr;
        return st;
    }
    c->reps[0].p = *p;  // placeholder until upload (inactive)
    return SIMMD_OK;
}

int simmd_upload_r(simmd_ctx* c, int32_t rep, const double* r, const double* v, const double* F, const double* D,
                   const double* disp)
{
    if (!c || !r || !D) return set_err(SIMMD_ERR_BAD_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    if (rep < 0 || rep >= c->R_cap) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    HostRep& h = c->reps[rep];
    if (!h.active) {
        // first upload of a simmd_create context: becomes replica 0
        simmd_params p = h.p;
        int rid = -1;
        TRY(add_replica(c, &p, r, v, F, D, &rid));
        if (rid != rep) return set_err(SIMMD_ERR_NOT_FOUND, "replica id mismatch");
        if (disp) TRY(upload_rep(c, rid, r, v, F, D, disp));
        return SIMMD_OK;
    }
    // the Verlet radius depends on max(D): refresh the descriptor and cells
    TRY(refresh_desc(c, rep, D));
    TRY(push_desc(c, rep));
    TRY(reset_state(c, rep, true));
    return upload_rep(c, rep, r, v, F, D, disp);
}

int simmd_upload(simmd_ctx* c, const double* r, const double* v, const double* F, const double* D,
                 const double* disp)
{
    return simmd_upload_r(c, 0, r, v, F, D, disp);
}

int simmd_download_r(simmd_ctx* c, int32_t rep, double* r, double* v, double* F, double* disp)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    if (rep < 0 || rep >= c->R_cap || !c->reps[rep].active) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    HostRep& h = c->reps[rep];
    const long long nd = h.p.N * h.p.dims;
    TRY(ensure_stage(c, std::max<long long>(nd, (long long)h.p.N)));
    double* st = c->d_stage;
    double *dr = st, *dv = st + c->stage_cap, *dF = st + 2 * c->stage_cap, *du = st + 4 * c->stage_cap;
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    launch_store_aos_impl(b, lc, rep, h.d, r ? dr : nullptr, v ? dv : nullptr, F ? dF : nullptr,
                          disp ? du : nullptr, nullptr, nullptr);
    CK(cudaGetLastError());
    if (r) CK(cudaMemcpyAsync(r, dr, sizeof(double) * nd, cudaMemcpyDeviceToHost, c->stream));
    if (v) CK(cudaMemcpyAsync(v, dv, sizeof(double) * nd, cudaMemcpyDeviceToHost, c->stream));
    if (F) CK(cudaMemcpyAsync(F, dF, sizeof(double) * nd, cudaMemcpyDeviceToHost, c->stream));
    if (disp) CK(cudaMemcpyAsync(disp, du, sizeof(double) * nd, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

// save_data's copy (src/Dump.jl:60-88) off the critical path: the state is
// converted to the host layout on the context stream (so it is the state at
// this point of the step sequence), then copied to the host on a side
// stream while later steps run.  Host arrays should be page-locked
// (simmd_host_register) for the copy to overlap.  One dump is in flight at
// a time: the next dump's conversion waits (on the device) for the previous
// copies; simmd_dump_wait blocks until the last dump's copies are done.
int simmd_dump_async(simmd_ctx* c, int32_t rep, double* r, double* v, double* F)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    if (rep < 0 || rep >= c->R_cap || !c->reps[rep].active) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    HostRep& h = c->reps[rep];
    const long long nd = h.p.N * h.p.dims;
    if (nd > c->dump_cap) {
        CK(cudaStreamSynchronize(c->dump_stream));
        CK(cudaStreamSynchronize(c->stream));
        dfree(c, &c->d_dump, (size_t)(3 * c->dump_cap));
        long long cap = std::max(nd, c->dump_cap * 2);
        TRY(dalloc(c, &c->d_dump, (size_t)(3 * cap)));
        c->dump_cap = cap;
        c->dump_pending = false;
    }
    double *dr = c->d_dump, *dv = c->d_dump + c->dump_cap, *dF = c->d_dump + 2 * c->dump_cap;
    if (c->dump_pending) CK(cudaStreamWaitEvent(c->stream, c->ev_dump_done, 0));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    launch_store_aos_impl(b, lc, rep, h.d, r ? dr : nullptr, v ? dv : nullptr, F ? dF : nullptr, nullptr, nullptr,
                          nullptr);
    CK(cudaGetLastError());
    CK(cudaEventRecord(c->ev_dump_ready, c->stream));
    CK(cudaStreamWaitEvent(c->dump_stream, c->ev_dump_ready, 0));
    if (r) CK(cudaMemcpyAsync(r, dr, sizeof(double) * nd, cudaMemcpyDeviceToHost, c->dump_stream));
    if (v) CK(cudaMemcpyAsync(v, dv, sizeof(double) * nd, cudaMemcpyDeviceToHost, c->dump_stream));
    if (F) CK(cudaMemcpyAsync(F, dF, sizeof(double) * nd, cudaMemcpyDeviceToHost, c->dump_stream));
    CK(cudaEventRecord(c->ev_dump_done, c->dump_stream));
    c->dump_pending = true;
    return SIMMD_OK;
}

int simmd_dump_wait(simmd_ctx* c)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    if (c->dump_pending) CK(cudaEventSynchronize(c->ev_dump_done));
    c->dump_pending = false;
    return SIMMD_OK;
}

int simmd_set_state_r(simmd_ctx* c, int32_t rep, const double* r, const double* v, const double* F,
                      const double* disp)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    if (rep < 0 || rep >= c->R_cap || !c->reps[rep].active) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    HostRep& h = c->reps[rep];
    const long long nd = h.p.N * h.p.dims;
    TRY(ensure_stage(c, std::max<long long>(nd, (long long)h.p.N)));
    double* st = c->d_stage;
    double *dr = st, *dv = st + c->stage_cap, *dF = st + 2 * c->stage_cap, *du = st + 4 * c->stage_cap;
    if (r) CK(cudaMemcpyAsync(dr, r, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
    if (v) CK(cudaMemcpyAsync(dv, v, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
    if (F) CK(cudaMemcpyAsync(dF, F, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
    if (disp) CK(cudaMemcpyAsync(du, disp, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    launch_set_state_impl(b, lc, rep, h.d, r ? dr : nullptr, v ? dv : nullptr, F ? dF : nullptr, disp ? du : nullptr);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    if (r) h.pending_prune = true;  // the lists are kept; the inner list is re-pruned
    return SIMMD_OK;
}

int simmd_set_state(simmd_ctx* c, const double* r, const double* v, const double* F, const double* disp)
{
    return simmd_set_state_r(c, 0, r, v, F, disp);
}

int simmd_download(simmd_ctx* c, double* r, double* v, double* F, double* disp)
{
    return simmd_download_r(c, 0, r, v, F, disp);
}

int64_t simmd_transfer_layout(simmd_ctx* c, int32_t n, int64_t* offsets)
{
    if (!c) return -1;
    long long nv = 0, ns = 0;
    xfer_layout(c, &nv, &ns);
    if (offsets)
        for (int r = 0; r < n; r++)
            offsets[r] = (r < c->R_cap && c->reps[r].active) ? c->reps[r].d.xfer_off : -1;
    return nv;
}

int simmd_upload_all(simmd_ctx* c, const double* r, const double* v, const double* F, const double* D,
                     const double* disp)
{
    if (!c || !r || !D) return set_err(SIMMD_ERR_BAD_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    long long nv = 0, ns = 0;
    xfer_layout(c, &nv, &ns);
    if (nv == 0) return set_err(SIMMD_ERR_NOT_FOUND, "no replica");
    std::vector<RepDesc> dstage;
    if (c->xfer_dirty) TRY(push_all_desc(c, dstage));  // the transfer offsets, read by the kernels below
    TRY(ensure_stage(c, nv));
    double* stg = c->d_stage;
    double *dr = stg, *dv = stg + c->stage_cap, *dF = stg + 2 * c->stage_cap, *dD = stg + 3 * c->stage_cap,
           *du = stg + 4 * c->stage_cap;
    CK(cudaMemcpyAsync(dr, r, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
    if (v) CK(cudaMemcpyAsync(dv, v, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
    if (F) CK(cudaMemcpyAsync(dF, F, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dD, D, sizeof(double) * ns, cudaMemcpyHostToDevice, c->stream));
    if (disp) CK(cudaMemcpyAsync(du, disp, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
    // max(D) per replica on the device (it sets the Verlet radius and the
    // cell grid), with every replica's state, in one round trip
    {
        Batch b = make_batch(c);
        LaunchCfg lc = make_lc(c, FMODE_STEP);
        launch_rep_dmax_impl(b, lc, dD, c->d_dmax);
        CK(cudaGetLastError());
    }
    std::vector<double> smax((size_t)c->R_cap, 0.0);
    CK(cudaMemcpyAsync(smax.data(), c->d_dmax, sizeof(double) * (size_t)c->R_cap, cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaMemcpyAsync(c->h_state.data(), c->d_state, sizeof(RepState) * (size_t)c->R_cap, cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int rep = 0; rep < c->R_cap; rep++) {
        if (!c->reps[rep].active) continue;
        // a new descriptor only when max(D) changed (a re-upload of the same
        // diameters keeps it)
        if (smax[(size_t)rep] != c->reps[rep].smax) TRY(refresh_desc_smax(c, rep, smax[(size_t)rep]));
        c->reps[rep].pending_rebuild = true;  // the rebuild runs before the next force pass
        // the state as reset_state(keep_counters) leaves it
        RepState& st = c->h_state[(size_t)rep];
        const long long step = st.step, rb = st.rebuilds;
        const int mc = st.maxcount;
        memset(&st, 0, sizeof(st));
        st.step = step;
        st.rebuilds = rb;
        st.maxcount = mc;
        st.vscale = 1.0;
        st.force_rebuild = 1;
        st.force_prune = 1;
    }
    TRY(push_all_desc(c, dstage));
    CK(cudaMemcpyAsync(c->d_state, c->h_state.data(), sizeof(RepState) * (size_t)c->R_cap, cudaMemcpyHostToDevice,
                       c->stream));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    launch_load_all(b, lc, dr, v ? dv : nullptr, F ? dF : nullptr, dD, disp ? du : nullptr);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

int simmd_set_state_all(simmd_ctx* c, const double* r, const double* v, const double* F, const double* disp)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    long long nv = 0, ns = 0;
    xfer_layout(c, &nv, &ns);
    if (nv == 0) return set_err(SIMMD_ERR_NOT_FOUND, "no replica");
    std::vector<RepDesc> dstage;
    if (c->xfer_dirty) TRY(push_all_desc(c, dstage));  // the transfer offsets, read by the kernel below
    TRY(ensure_stage(c, nv));
    double* stg = c->d_stage;
    double *dr = stg, *dv = stg + c->stage_cap, *dF = stg + 2 * c->stage_cap, *du = stg + 4 * c->stage_cap;
    if (r) CK(cudaMemcpyAsync(dr, r, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
    if (v) CK(cudaMemcpyAsync(dv, v, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
    if (F) CK(cudaMemcpyAsync(dF, F, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
    if (disp) CK(cudaMemcpyAsync(du, disp, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    launch_set_state_all(b, lc, r ? dr : nullptr, v ? dv : nullptr, F ? dF : nullptr, disp ? du : nullptr);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    if (r)  // the lists are kept; the inner lists are re-pruned
        for (int rep = 0; rep < c->R_cap; rep++)
            if (c->reps[rep].active) c->reps[rep].pending_prune = true;
    return SIMMD_OK;
}

int simmd_download_all(simmd_ctx* c, double* r, double* v, double* F, double* disp)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    long long nv = 0, ns = 0;
    std::vector<RepDesc> dstage;
    xfer_layout(c, &nv, &ns);
    // the offsets may have been laid out by an earlier call (simmd_transfer_layout)
    if (c->xfer_dirty) TRY(push_all_desc(c, dstage));
    if (nv == 0) return set_err(SIMMD_ERR_NOT_FOUND, "no replica");
    TRY(ensure_stage(c, nv));
    double* stg = c->d_stage;
    double *dr = stg, *dv = stg + c->stage_cap, *dF = stg + 2 * c->stage_cap, *du = stg + 4 * c->stage_cap;
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    launch_store_all(b, lc, r ? dr : nullptr, v ? dv : nullptr, F ? dF : nullptr, disp ? du : nullptr);
    CK(cudaGetLastError());
    if (r) CK(cudaMemcpyAsync(r, dr, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->stream));
    if (v) CK(cudaMemcpyAsync(v, dv, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->stream));
    if (F) CK(cudaMemcpyAsync(F, dF, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->stream));
    if (disp) CK(cudaMemcpyAsync(disp, du, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

int simmd_rebuild(simmd_ctx* c)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    for (int r = 0; r < c->R_cap; r++)
        if (c->reps[r].active) c->reps[r].pending_rebuild = true;
    TRY(pending_rebuilds(c));
    return read_states(c);
}

int simmd_set_full_list(simmd_ctx* c, int32_t enable)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    if (enable && !c->keep_full) {
        c->Kfull = c->K;
        TRY(dalloc(c, &c->nbr_full, (size_t)c->S_cap * (size_t)c->Kfull));
        TRY(dalloc(c, &c->ncnt_full, (size_t)c->S_cap));
        CK(cudaMemsetAsync(c->ncnt_full, 0, sizeof(int) * c->S_cap, c->stream));
        c->keep_full = 1;
        invalidate_graph(c);
    } else if (!enable && c->keep_full) {
        CK(cudaStreamSynchronize(c->stream));
        dfree(c, &c->nbr_full, (size_t)c->S_cap * (size_t)c->Kfull);
        dfree(c, &c->ncnt_full, (size_t)c->S_cap);
        c->keep_full = 0;
        invalidate_graph(c);
    }
    return SIMMD_OK;
}

int simmd_forces(simmd_ctx* c, const double* noise, double* F_out)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    TRY(pending_rebuilds(c));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_FORCES);
    Mix m = batch_mix(c);
    int single = -1, nact = 0;
    for (int r = 0; r < c->R_cap; r++)
        if (c->reps[r].active) { nact++; single = r; }
    if (nact == 0) return set_err(SIMMD_ERR_NOT_FOUND, "no replica uploaded");
    if (noise && m.noise) {
        if (nact != 1) return set_err(SIMMD_ERR_BAD_ARG, "host noise requires a single-replica context");
        HostRep& h = c->reps[single];
        long long nd = h.p.N * h.p.dims;
        if (nd > c->noise_cap) {
            CK(cudaStreamSynchronize(c->stream));
            dfree(c, &c->d_noise, (size_t)c->noise_cap);
            TRY(dalloc(c, &c->d_noise, (size_t)nd));
            c->noise_cap = nd;
        }
        CK(cudaMemcpyAsync(c->d_noise, noise, sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(&c->h_state[single], c->d_state + single, sizeof(RepState), cudaMemcpyDeviceToHost,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
        h.d.noise_mode = NOISE_HOST;
        h.d.host_noise = c->d_noise;
        h.d.noise_step0 = c->h_state[single].step;
        h.d.noise_nsteps = 1;
        TRY(push_desc(c, single));
        launch_force_impl(b, lc, FMODE_FORCES, m.prec_mask, nullptr);
        h.d.noise_mode = NOISE_PHILOX;
        h.d.host_noise = nullptr;
        TRY(push_desc(c, single));
    } else {
        launch_force_impl(b, lc, FMODE_FORCES, m.prec_mask, nullptr);
    }
    CK(cudaGetLastError());
    TRY(read_states(c));
    if (F_out) return simmd_download_r(c, single, nullptr, nullptr, F_out, nullptr);
    return SIMMD_OK;
}

int simmd_step(simmd_ctx* c, int64_t nsteps, const double* noise)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    return run_steps(c, nsteps, noise);
}

int simmd_energy_all(simmd_ctx* c)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    TRY(pending_rebuilds(c));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_ENERGY);
    launch_force_impl(b, lc, FMODE_ENERGY, batch_mix(c).prec_mask, c->epp);
    launch_kinetic_impl(b, lc);
    CK(cudaGetLastError());
    return read_states(c);
}

int simmd_energy(simmd_ctx* c, double* epot, double* virial, double* ekin)
{
    TRY(simmd_energy_all(c));
    int r0 = -1;
    for (int r = 0; r < c->R_cap; r++)
        if (c->reps[r].active) { r0 = r; break; }
    if (r0 < 0) return set_err(SIMMD_ERR_NOT_FOUND, "no replica");
    const RepState& s = c->h_state[r0];
    if (epot) *epot = s.epot;
    if (virial) *virial = s.virial;
    if (ekin) *ekin = c->reps[r0].p.dynamics == SIMMD_BROWNIAN ? 0.0 : s.ekin;
    return SIMMD_OK;
}

int simmd_potential_energy_array(simmd_ctx* c, double* e)
{
    if (!c || !e) return set_err(SIMMD_ERR_BAD_ARG, "NULL argument");
    TRY(simmd_energy_all(c));
    HostRep& h = c->reps[0];
    if (!h.active) return set_err(SIMMD_ERR_NOT_FOUND, "no replica");
    TRY(ensure_stage(c, h.p.N * h.p.dims));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    launch_store_aos_impl(b, lc, 0, h.d, nullptr, nullptr, nullptr, nullptr, c->epp, c->d_stage);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(e, c->d_stage, sizeof(double) * h.p.N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

int simmd_export_pairs(simmd_ctx* c, int32_t which, int64_t maxK, int64_t* counts, int64_t* list)
{
    if (!c || !counts || !list || maxK < 1) return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    CK(cudaSetDevice(c->device));
    HostRep& h = c->reps[0];
    if (!h.active) return set_err(SIMMD_ERR_NOT_FOUND, "no replica");
    if (which == 1 && !c->keep_full) return set_err(SIMMD_ERR_BAD_ARG, "full list not kept: simmd_set_full_list");
    TRY(pending_rebuilds(c));
    long long N = h.p.N;
    long long *dcnt = nullptr, *dlist = nullptr;
    int* dovf = nullptr;
    TRY(dalloc(c, &dcnt, (size_t)N));
    TRY(dalloc(c, &dlist, (size_t)(N * maxK)));
    TRY(dalloc(c, &dovf, 1));
    CK(cudaMemsetAsync(dovf, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(dlist, 0, sizeof(long long) * N * maxK, c->stream));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    if (which == 0) launch_export_impl(b, lc, 0, h.d, c->s.nbr, c->s.ncnt, c->T, dcnt, dlist, maxK, 1, dovf);
    else launch_export_impl(b, lc, 0, h.d, c->nbr_full, c->ncnt_full, 1, dcnt, dlist, maxK, 0, dovf);
    CK(cudaGetLastError());
    int ovf = 0;
    CK(cudaMemcpyAsync(counts, dcnt, sizeof(long long) * N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(list, dlist, sizeof(long long) * N * maxK, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&ovf, dovf, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    dfree(c, &dcnt, (size_t)N);
    dfree(c, &dlist, (size_t)(N * maxK));
    dfree(c, &dovf, 1);
    if (ovf) return set_err(SIMMD_ERR_NEIGHBOR_OVERFLOW, "export maxK too small");
    return SIMMD_OK;
}

static void fill_stats(simmd_ctx* c, int r, simmd_stats* out)
{
    const RepState& s = c->h_state[r];
    memset(out, 0, sizeof(*out));
    out->steps_done = c->reps[r].steps_done;
    out->rebuilds = s.rebuilds;
    out->noise_draws = s.step;
    out->max_neighbors = c->K;
    out->max_count = s.maxcount;
    out->overflow = s.overflow;
    out->nonfinite = s.nonfinite;
    out->epot = s.epot;
    out->virial = s.virial;
    out->ekin = s.ekin;
    out->list_entries = s.list_entries;
}

int simmd_stats_r(simmd_ctx* c, int32_t rep, simmd_stats* out)
{
    if (!c || !out) return set_err(SIMMD_ERR_BAD_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    if (rep < 0 || rep >= c->R_cap || !c->reps[rep].active) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    CK(cudaMemcpyAsync(&c->h_state[rep], c->d_state + rep, sizeof(RepState), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    fill_stats(c, rep, out);
    return SIMMD_OK;
}

int simmd_stats_get(simmd_ctx* c, simmd_stats* out) { return simmd_stats_r(c, 0, out); }

int simmd_reserve(simmd_ctx* c, int64_t slots, int64_t cells, int32_t replicas, int32_t max_neighbors)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    return ensure_capacity(c, std::max<long long>(slots, c->S_cap), std::max<long long>(cells, c->C_cap),
                           std::max<int>(replicas, c->R_cap), std::max<int>(max_neighbors, c->K));
}

int simmd_add_replica(simmd_ctx* c, const simmd_params* p, const double* r, const double* v, const double* F,
                      const double* D, int32_t* rep_out)
{
    if (!c || !rep_out) return set_err(SIMMD_ERR_BAD_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    int rid = -1;
    TRY(add_replica(c, p, r, v, F, D, &rid));
    *rep_out = rid;
    return SIMMD_OK;
}

int simmd_remove_replica(simmd_ctx* c, int32_t rep)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    return remove_replica(c, rep);
}

int64_t simmd_replica_bytes(const simmd_params* p, int32_t max_neighbors)
{
    if (!p || p->N < 1) return 0;
    long long npad = (p->N + TILE - 1) / TILE * TILE;
    long long K = max_neighbors > 0 ? max_neighbors : 200;
    RepDesc d;
    long long cells = npad;  // upper bound without the geometry
    if (validate(p) == SIMMD_OK && fill_desc_smax(p, 1.0, d) == SIMMD_OK) cells = d.ncell + 1;
    return npad * (SLOT_BYTES + 4 * K) + (npad / TILE) * TILE_BYTES + cells * CELL_BYTES +
           (long long)(sizeof(RepDesc) + sizeof(RepState));
}

int simmd_set_tuning(simmd_ctx* c, int32_t tpp, int32_t use_graphs, int32_t graph_steps)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    if (tpp != 1 && tpp != 2 && tpp != 4 && tpp != 8) return set_err(SIMMD_ERR_BAD_ARG, "tpp must be 1, 2, 4 or 8");
    if (tpp != 1 && c->prune_on)
        return set_err(SIMMD_ERR_BAD_ARG, "inner lists need one thread per particle (tpp = 1): simmd_set_prune 0 first");
    CK(cudaSetDevice(c->device));
    if (tpp != c->T) {
        CK(cudaStreamSynchronize(c->stream));
        c->T = tpp;
        int K = (c->K + tpp - 1) / tpp * tpp;
        if (K != c->K) {
            dfree(c, &c->s.nbr, (size_t)c->S_cap * (size_t)c->K);
            TRY(dalloc(c, &c->s.nbr, (size_t)c->S_cap * (size_t)K));
            if (c->prune_on) {
                dfree(c, &c->s.nbr_in, (size_t)c->S_cap * (size_t)c->K);
                TRY(dalloc(c, &c->s.nbr_in, (size_t)c->S_cap * (size_t)K));
            }
            c->K = K;
        }
        force_rebuild_all(c);
        invalidate_graph(c);
    }
    c->use_graphs = use_graphs ? 1 : 0;
    if (graph_steps > 0 && graph_steps != c->graph_steps) {
        c->graph_steps = graph_steps;
        invalidate_graph(c);
    }
    return SIMMD_OK;
}

int simmd_set_work_item(simmd_ctx* c, int32_t particles)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    if (particles != 0 && particles != TILE && particles != TILE / 2 && particles != TILE / 4)
        return set_err(SIMMD_ERR_BAD_ARG, "work item must be 0 (automatic), 128, 64 or 32 particles");
    const int mp = particles == 0 ? 1 : TILE / particles;
    if (mp != c->min_parts) {
        c->min_parts = mp;
        invalidate_graph(c);
    }
    return SIMMD_OK;
}

int simmd_sync(simmd_ctx* c)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

void* simmd_stream(simmd_ctx* c) { return c ? (void*)c->stream : nullptr; }

int simmd_timer_start(simmd_ctx* c)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaEventRecord(c->ev0, c->stream));
    return SIMMD_OK;
}

int simmd_timer_stop(simmd_ctx* c, float* ms)
{
    if (!c || !ms) return set_err(SIMMD_ERR_BAD_ARG, "NULL argument");
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    CK(cudaEventElapsedTime(ms, c->ev0, c->ev1));
    return SIMMD_OK;
}

// rebuild bodies executed so far (device counter of k_rb_copyback); bodies that a
// conditional graph node skipped are enqueued but not run
static long long bodies_executed(simmd_ctx* c)
{
    unsigned long long n = 0;
    cudaSetDevice(c->device);
    if (cudaMemcpyAsync(&n, c->d_plan_cnt + 2, sizeof(n), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
        cudaGetLastError();
        return c->n_rebuild;
    }
    return (long long)n;
}

static const int REBUILD_BODY_LAUNCHES = 7;  // the launches of launch_rebuild_body_impl

// kernels run: enqueued launches less the bodies that were skipped
int64_t simmd_launch_count(simmd_ctx* c)
{
    if (!c) return 0;
    return c->launches - REBUILD_BODY_LAUNCHES * (c->n_rebuild - bodies_executed(c));
}

int simmd_kernel_counts(simmd_ctx* c, int64_t* force_launches, int64_t* rebuild_sequences)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    if (force_launches) *force_launches = c->n_force;
    if (rebuild_sequences) *rebuild_sequences = bodies_executed(c);
    return SIMMD_OK;
}
int64_t simmd_device_bytes(simmd_ctx* c) { return c ? c->bytes : 0; }

int simmd_set_budget(simmd_ctx* c, int64_t bytes)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    if (bytes < 0) return set_err(SIMMD_ERR_BAD_ARG, "budget < 0");
    c->budget = bytes;
    return SIMMD_OK;
}

int simmd_time_force(simmd_ctx* c, int32_t nrep, float* ms_per_launch)
{
    if (!c || !ms_per_launch || nrep < 1) return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    CK(cudaSetDevice(c->device));
    TRY(pending_rebuilds(c));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_ENERGY);
    CK(cudaEventRecord(c->ev0, c->stream));
    const int pm = batch_mix(c).prec_mask;
    for (int k = 0; k < nrep; k++) launch_force_impl(b, lc, FMODE_ENERGY, pm, nullptr);
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    *ms_per_launch = ms / (float)nrep;
    return SIMMD_OK;
}

int simmd_inherent_structure(simmd_ctx* c, double tolerance, int64_t max_iterations, double max_step_size,
                             double dt, int64_t* iterations)
{
    if (!c || !(tolerance > 0) || max_iterations < 1 || !(max_step_size > 0) || !(dt > 0))
        return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    CK(cudaSetDevice(c->device));
    // every replica: pair forces only (a Newtonian system's random force is a
    // no-op) in the reference's FP64 arithmetic; the lists are rebuilt first
    // (src/InherentStructure.jl:9)
    std::vector<RepDesc> saved;
    for (int r = 0; r < c->R_cap; r++) {
        saved.push_back(c->reps[r].d);
        if (!c->reps[r].active) continue;
        RepDesc& d = c->reps[r].d;
        d.dyn = DYN_NEWTONIAN;
        d.prec = PREC_FP64;
        d.rescale = 0;
        TRY(push_desc(c, r));
        c->reps[r].pending_rebuild = true;
    }
    CK(cudaMemcpyAsync(c->h_state.data(), c->d_state, sizeof(RepState) * c->R_cap, cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int r = 0; r < c->R_cap; r++) {
        RepState& st = c->h_state[r];
        st.min_active = c->reps[r].active ? 1 : 0;
        st.min_done = 0;
        st.min_iters = 0;
        st.min_fmax = st.min_step = 0ull;
    }
    CK(cudaMemcpyAsync(c->d_state, c->h_state.data(), sizeof(RepState) * c->R_cap, cudaMemcpyHostToDevice,
                       c->stream));
    TRY(pending_rebuilds(c));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_FORCES);
    int status = SIMMD_OK;
    for (;;) {
        for (int k = 0; k < 32; k++) {
            launch_force_impl(b, lc, FMODE_FORCES, 1, nullptr);
            c->n_force += 1;
            launch_min_iteration_impl(b, lc, dt, max_step_size, tolerance, max_iterations);
            rebuild_launch(c, b, lc);
        }
        CK(cudaGetLastError());
        status = read_states(c);
        bool all = true;
        for (int r = 0; r < c->R_cap; r++)
            if (c->reps[r].active && !c->h_state[r].min_done && !c->h_state[r].nonfinite) all = false;
        if (all || status != SIMMD_OK) break;
    }
    for (int r = 0; r < c->R_cap; r++) {
        if (!c->reps[r].active) continue;
        if (iterations) iterations[r] = c->h_state[r].min_iters;
        if (c->h_state[r].min_done == 2 && status == SIMMD_OK)
            status = set_err(SIMMD_ERR_NOT_CONVERGED, "inherent structure: max_iterations reached");
    }
    // back to the replicas' own dynamics and precision
    for (int r = 0; r < c->R_cap; r++) {
        RepState& st = c->h_state[r];
        st.min_active = st.min_done = 0;
        st.min_fmax = st.min_step = 0ull;
        st.fmean_pending = 0;
        if (!c->reps[r].active) continue;
        c->reps[r].d = saved[r];
        TRY(push_desc(c, r));
        c->reps[r].pending_rebuild = true;
    }
    CK(cudaMemcpyAsync(c->d_state, c->h_state.data(), sizeof(RepState) * c->R_cap, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return status;
}

int simmd_relax(simmd_ctx* c, int64_t nsteps, double step_size, double max_disp)
{
    if (!c || nsteps < 0 || !(max_disp > 0) || !(step_size > 0)) return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    CK(cudaSetDevice(c->device));
    // split replicas keep no FP64 displacement: rebuilt first, so the FP64
    // relaxation starts from a zero displacement
    for (int r = 0; r < c->R_cap; r++)
        if (c->reps[r].active && c->reps[r].d.prec == PREC_FP32) c->reps[r].pending_rebuild = true;
    TRY(pending_rebuilds(c));
    std::vector<RepDesc> saved;
    for (int r = 0; r < c->R_cap; r++) {
        saved.push_back(c->reps[r].d);
        if (!c->reps[r].active) continue;
        RepDesc& d = c->reps[r].d;
        d.dyn = DYN_BROWNIAN;
        d.dt_over_gamma = step_size;
        d.relax_cap = max_disp;
        d.prec = PREC_FP64;
        TRY(push_desc(c, r));
    }
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    Mix m;
    m.br = true;
    m.prec_mask = 1;  // the relaxation runs every replica in FP64
    for (long long s = 0; s < nsteps; s++) enqueue_step(c, b, lc, m, FMODE_STEP);
    CK(cudaGetLastError());
    for (int r = 0; r < c->R_cap; r++) {
        if (!c->reps[r].active) continue;
        c->reps[r].d = saved[r];
        TRY(push_desc(c, r));
        c->reps[r].pending_rebuild = true;  // FP32 offsets / lists for the restored mode
    }
    // the relaxation's mean-force state must not leak into the dynamics
    TRY(read_states(c));
    for (int r = 0; r < c->R_cap; r++) {
        if (!c->reps[r].active) continue;
        RepState& st = c->h_state[r];
        st.fmean[0] = st.fmean[1] = st.fmean[2] = 0.0;
        st.cfmean[0] = st.cfmean[1] = st.cfmean[2] = 0.0;
        st.vmean[0] = st.vmean[1] = st.vmean[2] = 0.0;
        st.vscale = 1.0;
        st.nonfinite = 0;
        st.fmean_pending = 0;
        CK(cudaMemcpyAsync(c->d_state + r, &st, sizeof(RepState), cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

int simmd_mc_sweeps(simmd_ctx* c, int64_t nsweeps, double max_displacement, double swap_probability)
{
    if (!c || nsweeps < 0 || !(max_displacement >= 0) || !(swap_probability >= 0))
        return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    CK(cudaSetDevice(c->device));
    if (nsweeps == 0) return SIMMD_OK;
    // find_energy runs over the full Verlet list, as in the reference
    if (!c->keep_full) {
        TRY(simmd_set_full_list(c, 1));
        force_rebuild_all(c);
    }
    TRY(pending_rebuilds(c));
    CK(cudaMemcpyAsync(c->h_state.data(), c->d_state, sizeof(RepState) * (size_t)c->R_cap, cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int r = 0; r < c->R_cap; r++) {
        RepState& st = c->h_state[(size_t)r];
        st.mc_active = c->reps[r].active ? 1 : 0;
        st.mc_target = st.mc_sweep + nsweeps;
        st.mc_next = 0;
    }
    CK(cudaMemcpyAsync(c->d_state, c->h_state.data(), sizeof(RepState) * (size_t)c->R_cap, cudaMemcpyHostToDevice,
                       c->stream));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    int status = SIMMD_OK;
    // the chains run until a replica needs a list rebuild (or finishes); the
    // rebuild sequence serves those replicas, and the chains continue
    for (long long round = 0;; round++) {
        launch_mc_sweeps_impl(b, lc, c->nbr_full, c->ncnt_full, max_displacement, swap_probability);
        rebuild_launch(c, b, lc);
        CK(cudaGetLastError());
        status = read_states(c);
        bool done = true;
        for (int r = 0; r < c->R_cap; r++) {
            const RepState& st = c->h_state[(size_t)r];
            if (st.mc_active && !st.nonfinite && st.mc_sweep < st.mc_target) done = false;
        }
        if (done || status != SIMMD_OK) break;
    }
    for (int r = 0; r < c->R_cap; r++) c->h_state[(size_t)r].mc_active = 0;
    CK(cudaMemcpyAsync(c->d_state, c->h_state.data(), sizeof(RepState) * (size_t)c->R_cap, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    // the moves' displacements are not in the MD skin bookkeeping: fresh
    // lists before the next force evaluation
    force_rebuild_all(c);
    return status;
}

int simmd_mc_stats(simmd_ctx* c, int32_t rep, int64_t* counts4, double* dE)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    if (rep < 0 || rep >= c->R_cap || !c->reps[rep].active) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    RepState st;
    CK(cudaMemcpyAsync(&st, c->d_state + rep, sizeof(RepState), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (counts4)
        for (int k = 0; k < 4; k++) counts4[k] = st.mc_counts[k];
    if (dE) *dE = st.mc_dE;
    return SIMMD_OK;
}

int simmd_download_diameters(simmd_ctx* c, int32_t rep, double* D)
{
    if (!c || !D) return set_err(SIMMD_ERR_BAD_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    if (rep < 0 || rep >= c->R_cap || !c->reps[rep].active) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    HostRep& h = c->reps[rep];
    TRY(ensure_stage(c, std::max<long long>(h.p.N * h.p.dims, (long long)h.p.N)));
    Batch b = make_batch(c);
    LaunchCfg lc = make_lc(c, FMODE_STEP);
    launch_store_diameters_impl(b, lc, rep, h.d, c->d_stage);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(D, c->d_stage, sizeof(double) * h.p.N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

int simmd_set_skin(simmd_ctx* c, int32_t rep, double skin)
{
    if (!c || !(skin >= 0)) return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    CK(cudaSetDevice(c->device));
    for (int r = 0; r < c->R_cap; r++) {
        HostRep& h = c->reps[r];
        if (!h.active || (rep >= 0 && r != rep)) continue;
        simmd_params p = h.p;
        p.skin = skin;
        RepDesc d;
        TRY(fill_desc_smax(&p, h.smax, d));
        d.slot0 = h.d.slot0;
        d.tile0 = h.d.tile0;
        d.cell0 = h.d.cell0;
        if (d.ncell != h.d.ncell) {
            give_range(c->free_cells, h.d.cell0, h.d.ncell + 1);
            long long cstart;
            if (!take_range(c->free_cells, d.ncell + 1, &cstart)) {
                TRY(ensure_capacity(c, c->S_cap, c->C_cap + d.ncell + 1, c->R_cap, c->K));
                if (!take_range(c->free_cells, d.ncell + 1, &cstart)) return set_err(SIMMD_ERR_BUDGET, "cells");
            }
            d.cell0 = (int)cstart;
        }
        d.noise_mode = h.d.noise_mode;
        d.host_noise = h.d.host_noise;
        d.noise_step0 = h.d.noise_step0;
        d.noise_nsteps = h.d.noise_nsteps;
        d.xfer_off = h.d.xfer_off;
        d.xfer_soff = h.d.xfer_soff;
        h.p = p;
        h.d = d;
        apply_prune_desc(c, h);
        TRY(push_desc(c, r));
        h.pending_rebuild = true;
    }
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

int simmd_set_prune(simmd_ctx* c, int32_t rep, double inner_skin)
{
    if (!c || !(inner_skin >= 0.0)) return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    CK(cudaSetDevice(c->device));
    if (rep >= 0 && (rep >= c->R_cap || !c->reps[rep].active)) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    for (int r = 0; r < c->R_cap; r++) {
        HostRep& h = c->reps[r];
        if (h.active && (rep < 0 || r == rep)) h.inner_skin = inner_skin;
    }
    int on = 0;
    for (const auto& h : c->reps)
        if (h.active && h.inner_skin > 0.0) on = 1;
    if (on && c->T != 1) return set_err(SIMMD_ERR_BAD_ARG, "inner lists need one thread per particle (tpp = 1)");
    if (on && !c->prune_on) {
        // the inner list, its counts and the prune-time records; every
        // replica rebuilt (its record refreshed) and pruned before the next
        // force pass
        if (c->budget > 0 && c->bytes + c->S_cap * (4LL * c->K + 4 + 16) > c->budget)
            return set_err(SIMMD_ERR_BUDGET, "device memory budget exceeded");
        CK(cudaStreamSynchronize(c->stream));
        TRY(dalloc(c, &c->s.nbr_in, (size_t)c->S_cap * (size_t)c->K));
        TRY(dalloc(c, &c->s.ncnt_in, (size_t)c->S_cap));
        TRY(dalloc(c, &c->s.recp, (size_t)c->S_cap));
        CK(cudaMemsetAsync(c->s.ncnt_in, 0, sizeof(int) * (size_t)c->S_cap, c->stream));
        c->prune_on = 1;
        force_rebuild_all(c);
        invalidate_graph(c);
    } else if (!on && c->prune_on) {
        CK(cudaStreamSynchronize(c->stream));
        dfree(c, &c->s.nbr_in, (size_t)c->S_cap * (size_t)c->K);
        dfree(c, &c->s.ncnt_in, (size_t)c->S_cap);
        dfree(c, &c->s.recp, (size_t)c->S_cap);
        c->prune_on = 0;
        invalidate_graph(c);
    }
    for (int r = 0; r < c->R_cap; r++) {
        HostRep& h = c->reps[r];
        if (!h.active) continue;
        apply_prune_desc(c, h);
        h.pending_prune = c->prune_on != 0;
    }
    std::vector<RepDesc> dstage;
    TRY(push_all_desc(c, dstage));
    CK(cudaStreamSynchronize(c->stream));
    return SIMMD_OK;
}

int simmd_prune_stats(simmd_ctx* c, int32_t rep, int64_t* prunes, int64_t* inner_entries)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    CK(cudaSetDevice(c->device));
    if (rep < 0 || rep >= c->R_cap || !c->reps[rep].active) return set_err(SIMMD_ERR_NOT_FOUND, "no such replica");
    RepState st;
    CK(cudaMemcpyAsync(&st, c->d_state + rep, sizeof(RepState), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (prunes) *prunes = st.prunes;
    if (inner_entries) *inner_entries = st.list_entries_in;
    return SIMMD_OK;
}

int simmd_host_register(void* ptr, int64_t bytes)
{
    if (!ptr || bytes <= 0) return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    CK(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
    return SIMMD_OK;
}

int simmd_host_unregister(void* ptr)
{
    if (!ptr) return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    CK(cudaHostUnregister(ptr));
    return SIMMD_OK;
}

int simmd_set_profile(simmd_ctx* c, int32_t enable)
{
    if (!c) return set_err(SIMMD_ERR_BAD_ARG, "NULL context");
    c->profile = enable ? 1 : 0;
    c->prof = ProfileAcc();
    return SIMMD_OK;
}

int simmd_profile_get(simmd_ctx* c, double* out6)
{
    if (!c || !out6) return set_err(SIMMD_ERR_BAD_ARG, "NULL argument");
    out6[0] = c->prof.force_ms;
    out6[1] = (double)c->prof.force_n;
    out6[2] = c->prof.kick_ms;
    out6[3] = c->prof.rebuild_ms;
    out6[4] = c->prof.update_ms;
    out6[5] = (double)c->prof.steps;
    return SIMMD_OK;
}

int simmd_check_conversions(int64_t n, uint64_t seed, int64_t* mismatches)
{
    if (!mismatches || n < 0) return set_err(SIMMD_ERR_BAD_ARG, "bad argument");
    unsigned long long* d_bad = nullptr;
    CK(cudaMalloc(&d_bad, sizeof(unsigned long long)));
    unsigned long long h_bad = 0;
    cudaError_t e = cudaMemset(d_bad, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) {
        launch_check_conversions_impl(n, seed, d_bad, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&h_bad, d_bad, sizeof(h_bad), cudaMemcpyDeviceToHost);
    cudaFree(d_bad);
    if (e != cudaSuccess) return set_err(SIMMD_ERR_CUDA, std::string("conversion check: ") + cudaGetErrorString(e));
    *mismatches = (int64_t)h_bad;
    return SIMMD_OK;
}

}  // extern "C"
