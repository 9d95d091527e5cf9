// k_neighbor.cu -- neighbour-list rebuild (update_neighbor_lists!,
// src/NeighborLists.jl:24-104 of SimulationCode.jl) for every replica whose
// skin trigger fired or whose rebuild was requested by the host.
//
// Sequence:
//   plan      one block per replica: a rebuilding replica appends its tiles
//             and cells to the plan lists and zeroes its cell counters; the
//             kernels below work on those lists only, so the cost follows the
//             replicas that rebuild, not the batch size
//   bin       cell of each particle (FP64 position / cell size), rank in the
//             cell by atomicAdd
//   scan      one block per replica: exclusive scan of the counts -> starts
//   scatter   new slot = start[cell] + rank  (src[new] = old slot)
//   cellsort  one warp per cell: slots ordered by original particle id, so
//             the layout (and every later sum) is deterministic and
//             independent of the other replicas in the batch
//   gather    particle state to the new order (staging), displacement := 0,
//             packed cell coordinates and split-precision records
//   build     one block per cell: the stencil's candidates staged in shared
//             memory; FP32 classification with a margin, the exact FP64 test
//             of the reference only in the band around a threshold:
//             d2 <= verlet^2 (the pair enumeration radius) and
//             d2 < (sqrt(rc2)*mean_d + skin)^2 (add_pair!'s half-list test),
//             d2 from dx - round(dx/L)*L in the reference's operation order.
//             The list stores each pair in both directions (no atomics in
//             the force pass)
//   copyback  staging to the main arrays; its last block resets the
//             displacement max / request flags, counts the rebuild and
//             clears the plan
#include "simmd_internal.cuh"

namespace simmd {

__device__ __forceinline__ int pack_cell(int cx, int cy, int cz) { return cx | (cy << 10) | (cz << 20); }

__device__ __forceinline__ int plan_count(const Batch& b, int which)
{
    return *(volatile const int*)&b.plan_cnt[which];
}

// one block per replica: the tiles and cells of a rebuilding replica go to
// the plan lists (order of replicas arbitrary, each task independent), and
// its cell counters are zeroed
// Inside a captured step loop the rest of the sequence is the body of a
// conditional graph node: a planning block sets the node's condition, so a
// step in which no replica's trigger fired skips the seven other launches.
__global__ void k_rb_plan(Batch b, cudaGraphConditionalHandle cond, int use_cond)
{
    const int r = blockIdx.x;
    if (r >= b.nreps) return;
    const RepDesc& d = b.desc[r];
    // a replica with a non-finite state is not rebuilt (its particles would
    // all bin into one cell); the host retires it on the status
    if (!d.active || b.state[r].nonfinite || !need_rebuild(b.state[r], d)) return;
    __shared__ int s_tb, s_cb;
    if (threadIdx.x == 0) {
        if (use_cond) cudaGraphSetConditional(cond, 1u);
        b.state[r].in_plan = 1;
        s_tb = atomicAdd(&b.plan_cnt[0], d.ntiles);
        s_cb = atomicAdd(&b.plan_cnt[1], d.ncell);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < d.ntiles; k += blockDim.x) b.plan_tiles[s_tb + k] = d.tile0 + k;
    for (int c = threadIdx.x; c < d.ncell; c += blockDim.x) {
        b.plan_cells[s_cb + c] = make_int2(r, c);
        b.s.cell_count[d.cell0 + c] = 0;
    }
}

__global__ void k_rb_bin(Batch b)
{
    const int ntask = plan_count(b, 0);
    for (int k = blockIdx.x; k < ntask; k += gridDim.x) {
        const int t = b.plan_tiles[k];
        const int r = b.tile_rep[t];
        const RepDesc& d = b.desc[r];
        long long s = (long long)t * TILE + threadIdx.x;
        if (s >= d.slot0 + d.n) continue;
        double4_32a p = b.s.posD[s];
        int nc = d.nc;
        int c[3] = {0, 0, 0};
        double x[3] = {p.x, p.y, p.z};
        const bool finite = !(nonfinite_bits(p.x) || nonfinite_bits(p.y) || nonfinite_bits(p.z));
        if (!finite) b.state[r].nonfinite = 1;
        if (nc > 1 && finite) {
            for (int k2 = 0; k2 < d.dims; k2++) {
                int ci = __double2int_rd(x[k2] * d.inv_cs);  // floor, one conversion
                ci = ci < 0 ? 0 : (ci >= nc ? nc - 1 : ci);
                c[k2] = ci;
            }
        }
        int lin = c[0] + nc * (c[1] + nc * c[2]);
        b.s.bin_cell[s] = lin;
        b.s.bin_rank[s] = atomicAdd(&b.s.cell_count[d.cell0 + lin], 1);
    }
}

// one block per replica; blockDim 1024
__global__ void k_rb_scan(Batch b)
{
    int r = blockIdx.x;
    if (r >= b.nreps) return;
    const RepDesc& d = b.desc[r];
    if (!d.active || !b.state[r].in_plan) return;  // membership fixed by the plan
    __shared__ int warp_sums[32];
    const int nthr = blockDim.x;
    const int nc = d.ncell;
    const int per = (nc + nthr - 1) / nthr;
    const int lo = threadIdx.x * per;
    const int hi = min(lo + per, nc);
    const int* cnt = b.s.cell_count + d.cell0;
    int local = 0;
    for (int c = lo; c < hi; c++) local += cnt[c];
    // block exclusive scan of the per-thread totals
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[w] = incl;
    __syncthreads();
    if (w == 0) {
        int nw = nthr >> 5;
        int v = lane < nw ? warp_sums[lane] : 0;
        int inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane < nw) warp_sums[lane] = inc - v;
    }
    __syncthreads();
    int run = (int)d.slot0 + warp_sums[w] + incl - local;
    int* start = b.s.cell_start + d.cell0;
    for (int c = lo; c < hi; c++) {
        start[c] = run;
        run += cnt[c];
    }
    if (threadIdx.x == 0) {
        start[nc] = (int)(d.slot0 + d.n);
        b.state[r].list_entries = 0;
    }
}

__global__ void k_rb_scatter(Batch b)
{
    const int ntask = plan_count(b, 0);
    for (int k = blockIdx.x; k < ntask; k += gridDim.x) {
        const int t = b.plan_tiles[k];
        const int r = b.tile_rep[t];
        const RepDesc& d = b.desc[r];
        long long s = (long long)t * TILE + threadIdx.x;
        if (s >= d.slot0 + d.n) continue;
        int nw = b.s.cell_start[d.cell0 + b.s.bin_cell[s]] + b.s.bin_rank[s];
        b.s.src[nw] = (int)s;
    }
}

// one warp per cell: the cell's slots ordered by original particle id (rank
// sort through shuffles; ids are unique), so the layout is deterministic
__global__ void k_rb_cellsort(Batch b)
{
    const int ntask = plan_count(b, 1);
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    int* src = b.s.src;
    for (int k = gw; k < ntask; k += nw) {
        const int2 task = b.plan_cells[k];
        const RepDesc& d = b.desc[task.x];
        const int a = b.s.cell_start[d.cell0 + task.y], e = b.s.cell_start[d.cell0 + task.y + 1];
        const int n = e - a;
        if (n <= 32) {
            const int v = lane < n ? src[a + lane] : 0;
            const int key = lane < n ? b.s.orig[v] : 0x7fffffff;
            int rank = 0;
            for (int q = 0; q < n; q++) rank += (__shfl_sync(0xffffffffu, key, q) < key) ? 1 : 0;
            __syncwarp();
            if (lane < n) src[a + rank] = v;
            __syncwarp();
        } else {  // larger cell: rank sort by the warp (n^2/32 compares per
                  // lane), through the per-slot scratch bin_rank, which the
                  // scatter has consumed
            int* tmp = b.s.bin_rank;
            for (int q = lane; q < n; q += 32) {
                const int v = src[a + q];
                const int key = b.s.orig[v];
                int rank = 0;
                for (int u = 0; u < n; u++) rank += (b.s.orig[src[a + u]] < key) ? 1 : 0;
                tmp[a + rank] = v;
            }
            __syncwarp();
            for (int q = lane; q < n; q += 32) src[a + q] = tmp[a + q];
            __syncwarp();
        }
    }
}

__global__ void k_rb_gather(Batch b, int* ncnt_full)
{
    const int ntask = plan_count(b, 0);
    for (int k = blockIdx.x; k < ntask; k += gridDim.x) {
        const int t = b.plan_tiles[k];
        const int r = b.tile_rep[t];
        const RepDesc& d = b.desc[r];
        long long nw = (long long)t * TILE + threadIdx.x;
        Slots& S = b.s;
        S.ux[nw] = 0.0;
        S.uy[nw] = 0.0;
        S.uz[nw] = 0.0;
        S.ncnt[nw] = 0;
        if (ncnt_full) ncnt_full[nw] = 0;
        if (nw < d.slot0 + d.n) {
            int s = S.src[nw];
            double4_32a p = S.posD[s];
            S.t_posD[nw] = p;
            S.t_vx[nw] = S.vx[s];
            S.t_vy[nw] = S.vy[s];
            S.t_vz[nw] = S.vz[s];
            S.t_fx[nw] = S.fx[s];
            S.t_fy[nw] = S.fy[s];
            S.t_fz[nw] = S.fz[s];
            S.t_orig[nw] = S.orig[s];
            S.inv[d.slot0 + S.orig[s]] = (int)nw;
            int lin = S.bin_cell[s];
            int nc = d.nc;
            int cx = lin % nc, cy = (lin / nc) % nc, cz = lin / (nc * nc);
            S.cellc[nw] = pack_cell(cx, cy, cz);
            const FixRec q = fix_rec(p.x, p.y, p.z, p.w, d);
            S.rec[nw] = q;
            S.recb[nw] = q;  // displacement since this rebuild: 0
        } else {
            S.t_posD[nw] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
            S.t_vx[nw] = S.t_vy[nw] = S.t_vz[nw] = 0.0;
            S.t_fx[nw] = S.t_fy[nw] = S.t_fz[nw] = 0.0;
            S.t_orig[nw] = -1;
            S.cellc[nw] = 0;
            S.rec[nw] = FixRec{0u, 0u, 0u, 0.0f};
            S.recb[nw] = FixRec{0u, 0u, 0u, 0.0f};
        }
    }
}

// mean pair diameter of find_mean_D (src/InteractionPotential.jl:5-11), exact
__device__ __forceinline__ double mean_d_f64(const RepDesc& d, double Di, double Dj)
{
    if (d.pot == POT_LJ) return d.sigma2;
    return dmul(dmul(dadd(Di, Dj), 0.5), dsub(1.0, dmul(d.zeta, fabs(dsub(Di, Dj)))));
}

// ---------------------------------------------------------------------------
// Verlet build, one home cell at a time: the block stages the candidates of
// the home cell's stencil (27 cells in 3D, 9 in 2D; one cell along an axis
// with fewer than three cells) in shared memory, then Tb lanes per home
// particle test them, lane `sub` the candidates sub, sub + Tb, ...  Each
// candidate gets an FP32 test against the reference thresholds with a
// margin, and the exact FP64 test of the reference in the band around a
// threshold: d2 <= verlet^2 (the pair enumeration radius) and
// d2 < (sqrt(rc2)*mean_d + skin)^2 (add_pair!, src/NeighborLists.jl:82-104).
// 2D (few candidates per lane): one pass in candidate order, accepted
// entries appended through a warp ballot.  3D (hundreds of candidates, ~1 in
// 8 near enough): per window of 32 candidates per lane, first a radius
// filter alone -- FP32 d2 against a bound of every threshold the home
// particle can meet (its largest pair diameter; the Verlet radius as cap) --
// kept as a bit mask in a register, then the full test on the survivors, one
// per lane and round, appended in lane order per round.  A candidate the
// filter drops lies above every threshold's band, so the full test would
// have rejected it.  Either way the list order is a pure function of the
// replica's own state.
// ---------------------------------------------------------------------------
constexpr int BLD_THREADS = 128;
constexpr int BLD_CHUNK = 512;

struct BuildSmem {
    float4 o[BLD_CHUNK];  // position relative to the home cell's reference point (FP32), D
    int slot[BLD_CHUNK];  // slot of the candidate (-1: padding of the last round)
    int ca[27];      // first slot of each stencil cell
    int pre[28];     // candidates before each stencil cell (pre[nst]: all)
    unsigned rf[3];  // the home cell's centre in fixed point
    unsigned long long entries;
    int maxcnt;
};

template <int DIM, bool WRAP>
__device__ __forceinline__ float build_d2(const float4& oi, const float4& oj, const RepDesc& d)
{
    const float dxf = WRAP ? min_image_f32(oi.x - oj.x, d.halfLf, d.Lf) : oi.x - oj.x;
    const float dyf = WRAP ? min_image_f32(oi.y - oj.y, d.halfLf, d.Lf) : oi.y - oj.y;
    float d2f = dxf * dxf + dyf * dyf;
    if (DIM == 3) {
        const float dzf = WRAP ? min_image_f32(oi.z - oj.z, d.halfLf, d.Lf) : oi.z - oj.z;
        d2f += dzf * dzf;
    }
    return d2f;
}

// the full test of candidate q for home particle i: pred (half list),
// predf (the Verlet list)
template <int DIM, bool FULL, bool WRAP>
__device__ __forceinline__ void build_classify(const Slots& S, const RepDesc& d, const BuildSmem& sm, int q,
                                               long long i, const float4& oi, const double4_32a& pi,
                                               long long halfLb, float flo, float fhi, int& j, bool& pred,
                                               bool& predf)
{
    j = sm.slot[q];
    if (j < 0 || j == (int)i) return;
    const float4 oj = sm.o[q];
    const float d2f = build_d2<DIM, WRAP>(oi, oj, d);
    // FP32 classification against the reference thresholds with a relative
    // margin (1e-5) far above the FP32 error of d2 and of the thresholds
    // (~1e-6): clear accepts and rejects are the reference's decisions; the
    // exact FP64 test runs only in the narrow band around a threshold, so the
    // pair set stays bit-identical while the FP64 pipe stays idle
    float tf = (d.pot == POT_LJ) ? d.rcutf * d.sigma2f
                                 : d.rcutf * ((oi.w + oj.w) * 0.5f * (1.0f - d.zetaf * fabsf(oi.w - oj.w)));
    tf += d.skinf;
    const float thr = fminf(tf * tf, d.rv2f);
    const float lo = thr * (1.0f - 1e-5f), hi = thr * (1.0f + 1e-5f);
    const bool band = (d2f >= lo && d2f <= hi) || (FULL && d2f >= flo && d2f <= fhi);
    if (!band) {
        pred = d2f < lo;
        predf = d2f < flo;
        return;
    }
    // exact FP64 test in the reference's operation order
    const double4_32a pj = S.t_posD[j];
    const double ddx = min_image_f64(dsub(pi.x, pj.x), halfLb, d.L);
    const double ddy = min_image_f64(dsub(pi.y, pj.y), halfLb, d.L);
    double d2 = dadd(dmul(ddx, ddx), dmul(ddy, ddy));
    if (DIM == 3) {
        const double ddz = min_image_f64(dsub(pi.z, pj.z), halfLb, d.L);
        d2 = dadd(d2, dmul(ddz, ddz));
    }
    if (d2 <= d.rv2) {
        predf = true;
        const double tt = dadd(dmul(d.rcut, mean_d_f64(d, pi.w, pj.w)), d.skin);
        pred = d2 < dmul(tt, tt);
    }
}

template <int DIM, bool FULL, bool WRAP>
__device__ void build_cell(const Batch& b, const RepDesc& d, RepState& st, int c, BuildSmem& sm,
                           unsigned* nbr_full, int* ncnt_full, int Kfull)
{
    const Slots& S = b.s;
    const int tid = threadIdx.x;
    const int nc = d.nc;
    const int cx = c % nc, cy = (c / nc) % nc, cz = c / (nc * nc);
    const int ha = S.cell_start[d.cell0 + c], he = S.cell_start[d.cell0 + c + 1];
    const int P = he - ha;
    if (P == 0) return;  // uniform across the block
    const int rng = (nc >= 3) ? 1 : 0;
    const int w = 2 * rng + 1;
    const int nst = (DIM == 3) ? w * w * w : w * w;
    if (tid < 32) {
        // warp 0: stencil cell `tid`'s first slot and count, the candidates
        // before it by a warp scan
        int a = 0, n = 0;
        if (tid < nst) {
            const int ox = tid % w - rng, oy = (tid / w) % w - rng, oz = (DIM == 3) ? tid / (w * w) - rng : 0;
            const int x = (cx + ox + nc) % nc, y = (cy + oy + nc) % nc, z = (DIM == 3) ? (cz + oz + nc) % nc : 0;
            const int lin = x + nc * (y + nc * z);
            a = S.cell_start[d.cell0 + lin];
            n = S.cell_start[d.cell0 + lin + 1] - a;
        }
        int incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (tid >= o) incl += y;
        }
        if (tid < nst) {
            sm.ca[tid] = a;
            sm.pre[tid] = incl - n;
        }
        if (tid == 31) sm.pre[nst] = incl;  // lanes past the stencil add nothing
    } else if (tid < 35) {
        // reference point at the home cell centre (fixed point, (2c+1) 2^31 /
        // nc), one axis per lane of warp 1: candidate coordinates relative to
        // it are small, exact integer differences (minimum image by the int32
        // wraparound) turned into FP32, so a pair difference is one FP32
        // subtract
        const int k = tid - 32;
        const int cc = k == 0 ? cx : (k == 1 ? cy : cz);
        sm.rf[k] = (k < DIM) ? (unsigned)(((2ull * (unsigned long long)cc + 1ull) << 31) / (unsigned long long)nc)
                             : 0u;
    }
    __syncthreads();
    const int M = sm.pre[nst];
    const unsigned rfx = sm.rf[0], rfy = sm.rf[1], rfz = sm.rf[2];
    const float u = d.fix_u;
    // lanes per home particle: as many as keep the block's 128 threads busy
    // (a power of two dividing 32, so a particle's lanes share one warp)
    const int Tb = P <= 4 ? 32 : (P <= 8 ? 16 : (P <= 16 ? 8 : (P <= 32 ? 4 : (P <= 64 ? 2 : 1))));
    const int sub = tid % Tb;
    const int lane = tid & 31;
    const int gbase = (lane / Tb) * Tb;
    const unsigned gmask = (Tb == 32) ? 0xffffffffu : ((1u << Tb) - 1u);
    const unsigned below = (1u << sub) - 1u;
    const int K = b.K, tsh = 31 - __clz(b.tpp);  // threads per particle: a power of two
    const long long SS = b.S;
    const long long halfLb = __double_as_longlong(d.halfL);
    const float flo = d.rv2f * (1.0f - 1e-5f), fhi = d.rv2f * (1.0f + 1e-5f);
    for (int base = 0; base < P; base += BLD_THREADS / Tb) {
        const int p = base + tid / Tb;
        const bool active = p < P;
        const long long i = ha + (active ? p : 0);
        float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
        double4_32a pi = make_double4_32a(0.0, 0.0, 0.0, 0.0);
        if (active) {
            const FixRec q = S.rec[i];
            oi = make_float4((float)(int)(q.x - rfx) * u, (float)(int)(q.y - rfy) * u,
                             DIM == 3 ? (float)(int)(q.z - rfz) * u : 0.0f, q.d);
            pi = S.t_posD[i];
        }
        // the filter radius: every pair threshold of this home particle
        // (pair diameter <= (D_i + max D) / 2) and its band lie below it, with
        // 1e-4 relative slack for the FP32 roundings of both forms; nothing
        // passes for a lane without a home particle
        float r1 = -1.0f;
        if (active) {
            float tm = (d.pot == POT_LJ) ? d.rcutf * d.sigma2f : d.rcutf * ((oi.w + d.dmaxf) * 0.5f);
            tm += d.skinf;
            r1 = (FULL ? d.rv2f : fminf(tm * tm, d.rv2f)) * (1.0f + 1e-4f);
        }
        int cnt = 0, cntf = 0;
        // one accepted-or-not decision per lane -> appended in lane order
        auto append = [&](bool pred, bool predf, int j) {
            const unsigned gb = (__ballot_sync(0xffffffffu, pred) >> gbase) & gmask;
            if (pred) {
                const int pos = cnt + __popc(gb & below);
                if (pos < K) S.nbr[nbr_addr_sh(pos, i, tsh, K)] = (unsigned)j;
            }
            cnt += __popc(gb);
            if (FULL) {
                const unsigned gf = (__ballot_sync(0xffffffffu, predf) >> gbase) & gmask;
                if (predf) {
                    const int pos = cntf + __popc(gf & below);
                    if (pos < Kfull) nbr_full[(size_t)pos * SS + i] = (unsigned)j;
                }
                cntf += __popc(gf);
            }
        };
        for (int c0 = 0; c0 < M; c0 += BLD_CHUNK) {
            const int len = min(BLD_CHUNK, M - c0);
            // candidates of this chunk, then padding up to the last round's end
            const int lenr = min(BLD_CHUNK, (len + Tb - 1) / Tb * Tb);
            __syncthreads();
            for (int q = tid; q < lenr; q += BLD_THREADS) {
                if (q >= len) {
                    sm.o[q] = make_float4(1e30f, 1e30f, 1e30f, 0.0f);
                    sm.slot[q] = -1;
                    continue;
                }
                const int idx = c0 + q;
                // the stencil cell holding candidate idx: the last k with pre[k] <= idx
                int k = 0;
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1)
                    if (k + step < nst && sm.pre[k + step] <= idx) k += step;
                const int j = sm.ca[k] + (idx - sm.pre[k]);
                const FixRec cr = S.rec[j];
                sm.o[q] = make_float4((float)(int)(cr.x - rfx) * u, (float)(int)(cr.y - rfy) * u,
                                      DIM == 3 ? (float)(int)(cr.z - rfz) * u : 0.0f, cr.d);
                sm.slot[q] = j;
            }
            __syncthreads();
            // a warp with no home particle in this pass skips the candidates
            // (warp-uniform: the ballots stay within full warps)
            const int qend = __any_sync(0xffffffffu, active) ? lenr : 0;
            if (DIM == 2) {
                for (int q0 = 0; q0 < qend; q0 += Tb) {
                    bool pred = false, predf = false;
                    int j = -1;
                    if (active) build_classify<DIM, FULL, WRAP>(S, d, sm, q0 + sub, i, oi, pi, halfLb, flo, fhi, j,
                                                                pred, predf);
                    append(pred, predf, j);
                }
            } else {
                const int win = Tb * 32;
                for (int w0 = 0; w0 < qend; w0 += win) {
                    // radius filter: bit k of mask = candidate w0 + k*Tb + sub
                    const int nr = min(32, (qend - w0) / Tb);
                    unsigned mask = 0u;
                    {
                        int q = w0 + sub;
#pragma unroll 8
                        for (int k = 0; k < nr; k++, q += Tb)
                            mask |= (build_d2<DIM, WRAP>(oi, sm.o[q], d) <= r1) ? (1u << k) : 0u;
                    }
                    // the survivors: one per lane and round
                    const int rounds = __reduce_max_sync(0xffffffffu, __popc(mask));
                    for (int rr = 0; rr < rounds; rr++) {
                        bool pred = false, predf = false;
                        int j = -1;
                        if (mask) {
                            const int k = __ffs(mask) - 1;
                            mask &= mask - 1u;
                            build_classify<DIM, FULL, WRAP>(S, d, sm, w0 + k * Tb + sub, i, oi, pi, halfLb, flo,
                                                            fhi, j, pred, predf);
                        }
                        append(pred, predf, j);
                    }
                }
            }
        }
        if (active && sub == 0) {
            if (cnt > K) st.overflow = 1;
            S.ncnt[i] = min(cnt, K);
            if (FULL) {
                if (cntf > Kfull) st.overflow = 1;
                ncnt_full[i] = min(cntf, Kfull);
            }
            atomicMax(&sm.maxcnt, cnt);
            atomicAdd(&sm.entries, (unsigned long long)min(cnt, K));
        }
    }
    __syncthreads();
}

// one block per cell task of the plan; FULL: the full (Verlet) list as well
// (parity tests), kept in its own kernel so the production kernel's register
// budget is that of the half list alone.  8 blocks per SM (64 registers):
// the latency of the staging loads and barriers is hidden by more cells in
// flight
template <bool FULL>
__global__ void __launch_bounds__(BLD_THREADS, 8) k_rb_build(Batch b, unsigned* nbr_full, int* ncnt_full, int Kfull)
{
    __shared__ BuildSmem sm;
    const int ntask = plan_count(b, 1);
    for (int k = blockIdx.x; k < ntask; k += gridDim.x) {
        const int2 task = b.plan_cells[k];
        const RepDesc& d = b.desc[task.x];
        RepState& st = b.state[task.x];
        if (threadIdx.x == 0) {
            sm.entries = 0ull;
            sm.maxcnt = 0;
        }
        __syncthreads();
        if (FULL) {
            if (d.dims == 3) build_cell<3, true, true>(b, d, st, task.y, sm, nbr_full, ncnt_full, Kfull);
            else build_cell<2, true, true>(b, d, st, task.y, sm, nbr_full, ncnt_full, Kfull);
        } else if (d.build_wrap) {
            if (d.dims == 3) build_cell<3, false, true>(b, d, st, task.y, sm, nbr_full, ncnt_full, Kfull);
            else build_cell<2, false, true>(b, d, st, task.y, sm, nbr_full, ncnt_full, Kfull);
        } else {
            if (d.dims == 3) build_cell<3, false, false>(b, d, st, task.y, sm, nbr_full, ncnt_full, Kfull);
            else build_cell<2, false, false>(b, d, st, task.y, sm, nbr_full, ncnt_full, Kfull);
        }
        __syncthreads();
        if (threadIdx.x == 0 && sm.entries) {
            atomicMax(&st.maxcount, sm.maxcnt);
            atomicAdd((unsigned long long*)&st.list_entries, sm.entries);
        }
        __syncthreads();
    }
}

// copy the staged (re-ordered) state back; separate kernel because the build
// reads neighbours' staged positions
// the end of the sequence: the staged (re-ordered) state copied back
// (a separate kernel because the build reads neighbours' staged positions);
// the last block to finish then closes the rebuild of every planned replica
// (displacement max, request flags, counters) and clears the plan
__global__ void k_rb_copyback(Batch b)
{
    const int ntask = plan_count(b, 0);
    for (int k = blockIdx.x; k < ntask; k += gridDim.x) {
        const int t = b.plan_tiles[k];
        long long i = (long long)t * TILE + threadIdx.x;
        Slots& S = b.s;
        S.posD[i] = S.t_posD[i];
        S.vx[i] = S.t_vx[i];
        S.vy[i] = S.t_vy[i];
        S.vz[i] = S.t_vz[i];
        S.fx[i] = S.t_fx[i];
        S.fy[i] = S.t_fy[i];
        S.fz[i] = S.t_fz[i];
        S.orig[i] = S.t_orig[i];
    }
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&b.plan_cnt[4], 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (threadIdx.x == 0) {  // every block has read the plan: it is spent
        b.plan_cnt[4] = 0;
        b.plan_cnt[0] = 0;
        b.plan_cnt[1] = 0;
        *reinterpret_cast<unsigned long long*>(b.plan_cnt + 2) += 1ull;  // bodies executed
    }
    for (int r = threadIdx.x; r < b.nreps; r += blockDim.x) {
        const RepDesc& d = b.desc[r];
        RepState& st = b.state[r];
        if (!d.active || !st.in_plan) continue;
        st.in_plan = 0;
        st.maxdisp2 = 0ull;
        st.force_rebuild = 0;
        st.rebuilds += 1;
        st.force_prune = 1;  // the slots were re-ordered: the inner list follows
    }
}

// the host's requests: one thread per entry rep * 4 + flags (1 rebuild,
// 2 prune)
__global__ void k_mark_rebuild(const int* reps, int n, RepState* state)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int e = reps[k];
    if (e & 1) state[e >> 2].force_rebuild = 1;
    if (e & 2) state[e >> 2].force_prune = 1;
}

void launch_mark_rebuild_impl(const int* reps, int n, RepState* state, cudaStream_t s)
{
    k_mark_rebuild<<<(n + 127) / 128, 128, 0, s>>>(reps, n, state);
}

void launch_rebuild_plan_impl(const Batch& b, const LaunchCfg& lc, cudaGraphConditionalHandle cond, int use_cond)
{
    k_rb_plan<<<b.nreps, 128, 0, lc.stream>>>(b, cond, use_cond);
    if (lc.launches) *lc.launches += 1;
}

// the sequence after the plan (on lc.stream)
void launch_rebuild_body_impl(const Batch& b, const LaunchCfg& lc, unsigned* nbr_full, int* ncnt_full, int Kfull)
{
    int g = lc.grid_stream;
    k_rb_bin<<<g, TILE, 0, lc.stream>>>(b);
    k_rb_scan<<<b.nreps, 1024, 0, lc.stream>>>(b);
    k_rb_scatter<<<g, TILE, 0, lc.stream>>>(b);
    k_rb_cellsort<<<g, TILE, 0, lc.stream>>>(b);
    k_rb_gather<<<g, TILE, 0, lc.stream>>>(b, ncnt_full);
    if (nbr_full) k_rb_build<true><<<g, BLD_THREADS, 0, lc.stream>>>(b, nbr_full, ncnt_full, Kfull);
    else k_rb_build<false><<<g, BLD_THREADS, 0, lc.stream>>>(b, nullptr, nullptr, 0);
    // fewer blocks for the copy-back: each block's completion is one atomic on
    // the closing counter
    k_rb_copyback<<<min(g, lc.grid_copy), TILE, 0, lc.stream>>>(b);
    if (lc.launches) *lc.launches += 7;
}

// ---------------------------------------------------------------------------
// export of the lists in the reference layout: column-major (maxK, N),
// 1-based ids, counts per particle.  half_only: the force list, each pair
// once (owner = lower original id); otherwise the full Verlet list.
// ---------------------------------------------------------------------------
__global__ void k_export(Batch b, int rep, const unsigned* lst, const int* cnt, int rowstride_T,
                         long long* counts, long long* list, long long maxK, int half_only,
                         int* overflow)
{
    const RepDesc& d = b.desc[rep];
    long long s = d.slot0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.slot0 + d.n) return;
    int oi = b.s.orig[s];
    int n = cnt[s];
    long long k = 0;
    for (int q = 0; q < n; q++) {
        unsigned e = half_only ? lst[nbr_addr(q, s, rowstride_T, b.K)] : lst[(size_t)q * b.S + s];
        int oj = b.s.orig[e & IDX_MASK];
        if (half_only && oj < oi) continue;
        if (k < maxK) list[k + maxK * (long long)oi] = (long long)oj + 1;
        else *overflow = 1;
        k++;
    }
    counts[oi] = k;
}

void launch_export_impl(const Batch& b, const LaunchCfg& lc, int rep, const RepDesc& hd,
                        const unsigned* lst, const int* cnt, int T, long long* counts, long long* list,
                        long long maxK, int half_only, int* overflow)
{
    int blocks = (hd.n + 127) / 128;
    if (blocks > 0)
        k_export<<<blocks, 128, 0, lc.stream>>>(b, rep, lst, cnt, T, counts, list, maxK, half_only, overflow);
    if (lc.launches) *lc.launches += 1;
}

}  // namespace simmd
