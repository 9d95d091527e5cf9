// simmd_reduce.cuh -- deterministic per-tile / per-replica reductions.
//
// Canonical per-replica reduction: each tile's sum is its warps' partial
// sums added in warp order (when the force pass splits a tile into parts,
// the parts write warp slots and the block completing the tile's last part
// adds them in that order).  Tile sums are then combined in a fixed tree:
// groups of 32 consecutive tiles, then groups of 32 group sums, ...; the
// block that completes a group's last member reduces the group with one
// warp (a fixed shuffle tree; energies and virial compensated -- (sum,
// error) pairs combined with TwoSum -- the mean force / velocity plain) and
// climbs one level.  Every level is one round trip, so a
// replica of thousands of tiles finishes in a few, not in one warp's walk
// over all tiles.  The result depends only on the replica's own particles,
// slot layout and threads per particle -- not on the split, on which block
// ran which item, or on the other replicas in the batch.
#pragma once
#include "simmd_internal.cuh"

namespace simmd {

template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV])
{
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// s + e == a + b exactly (Knuth); e is the same whatever the operand order
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e)
{
    s = a + b;
    const double bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// compensated warp reduction of (s, c) pairs, every lane gets the total.
// The first NPLAIN values (a replica's mean force or velocity) are summed
// plainly in the same tree (their c stays 0): GB300's FP64 pipe is narrow,
// and the error-free sums are kept for the energy-like values
template <int NV, int NPLAIN = 0>
__device__ __forceinline__ void warp_sum_comp(double (&s)[NV], double (&c)[NV])
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < NV; k++) {
            const double s2 = __shfl_xor_sync(0xffffffffu, s[k], o);
            if (k < NPLAIN) {
                s[k] += s2;
                continue;
            }
            const double c2 = __shfl_xor_sync(0xffffffffu, c[k], o);
            double t, e;
            two_sum(s[k], s2, t, e);
            s[k] = t;
            c[k] = (c[k] + c2) + e;
        }
}

// Returns true in the threads of the block that must finalise the replica;
// in that case out[] (valid in thread 0) holds the replica totals.
// WARP_DONE: the caller has already reduced each warp (lane 0's v[] is
// used).  s_part: 32*NV shared doubles; s_flag: one shared int.  Must be
// called by every thread of the block (contains __syncthreads); blockDim a
// multiple of 32.
template <int NV, bool WARP_DONE = false, int NPLAIN = 0>
__device__ bool tile_reduce(const Batch& b, int item, const RepDesc& d, RepState& st, double (&v)[NV],
                            double (&out)[NV], double* s_part, int* s_flag, int parts = 1)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    const int t = item / parts, part = item - t * parts;
    if (!WARP_DONE) warp_sum<NV>(v);  // else lane 0 already holds the warp's sums
    if (lane == 0) {
        if (parts == 1) {
#pragma unroll
            for (int k = 0; k < NV; k++) s_part[wid * NV + k] = v[k];
        } else {
            double* slot = b.warp_part + ((size_t)t * WARP_SLOTS + (size_t)(part * nw + wid)) * NPART;
#pragma unroll
            for (int k = 0; k < NV; k++) slot[k] = v[k];
        }
    }
    __syncthreads();
    // ---- the tile's sum (level 0 of the tree), by warp 0 of the block that
    // completes the tile (the warp partials added in warp order)
    if (tid == 0) {
        int done = 1;
        if (parts > 1) {
            __threadfence();  // after the barrier: publishes every warp's slot
            done = atomicAdd(&b.tile_cnt[t], 1) == parts - 1;
            if (done) b.tile_cnt[t] = 0;
        }
        *s_flag = done;
    }
    __syncthreads();
    if (wid == 0 && *s_flag) {
        double ts[NV];
        if (parts == 1) {
            // whole tiles (large batches): lane k adds value k over the warps
            // in order, so the FP64 adds run on NV lanes, not on the warp
            double my = 0.0;
            if (lane < NV)
                for (int w = 0; w < nw; w++) my += s_part[w * NV + lane];
#pragma unroll
            for (int k = 0; k < NV; k++) ts[k] = __shfl_sync(0xffffffffu, my, k);
        } else {
            // split tiles (small batches): the warp slots, one per lane,
            // added in warp order through shuffles
            __threadfence();
            const int wpt = nw * parts;  // <= 32
            const double* slot = b.warp_part + (size_t)t * WARP_SLOTS * NPART;
#pragma unroll
            for (int k = 0; k < NV; k++) {
                const double x = lane < wpt ? __ldcg(slot + (size_t)lane * NPART + k) : 0.0;
                double s = 0.0;
                for (int w = 0; w < wpt; w++) s += __shfl_sync(0xffffffffu, x, w);
                ts[k] = s;
            }
        }
        if (lane == 0) {
            double* dst = b.red_val + (size_t)t * RED_REC;
#pragma unroll
            for (int k = 0; k < NV; k++) {
                dst[k] = ts[k];
                dst[NV + k] = 0.0;
            }
        }
    }
    bool last = false;
    // ---- climb the tree with warp 0
    if (wid == 0 && *s_flag) {
        __syncwarp();  // lane 0's tile sum visible to the warp
        int idx = t - d.tile0, n = d.ntiles;
        double s[NV], c[NV];
        if (n == 1) {  // a one-tile replica: its tile sum is the total
            const double* src = b.red_val + (size_t)t * RED_REC;
#pragma unroll
            for (int k = 0; k < NV; k++) { s[k] = src[k]; c[k] = 0.0; }
            last = true;
        }
        for (int level = 0; n > 1; level++) {
            const int g = idx >> 5, first = g << 5, m = min(32, n - first);
            int prev = 0;
            if (lane == 0) {
                __threadfence();
                prev = atomicAdd(&b.red_cnt[(size_t)level * b.ntiles + d.tile0 + g], 1);
            }
            prev = __shfl_sync(0xffffffffu, prev, 0);
            if (prev != m - 1) break;  // another block completes this group
            __threadfence();
            const double* src = b.red_val + ((size_t)level * b.ntiles + d.tile0 + first) * RED_REC;
#pragma unroll
            for (int k = 0; k < NV; k++) {
                s[k] = lane < m ? __ldcg(src + (size_t)lane * RED_REC + k) : 0.0;
                c[k] = lane < m ? __ldcg(src + (size_t)lane * RED_REC + NV + k) : 0.0;
            }
            warp_sum_comp<NV, NPLAIN>(s, c);
            if (lane == 0) b.red_cnt[(size_t)level * b.ntiles + d.tile0 + g] = 0;
            idx = g;
            n = (n + 31) >> 5;
            if (n == 1) {
                last = true;
            } else if (lane == 0) {
                double* dst = b.red_val + ((size_t)(level + 1) * b.ntiles + d.tile0 + g) * RED_REC;
#pragma unroll
                for (int k = 0; k < NV; k++) {
                    dst[k] = s[k];
                    dst[NV + k] = c[k];
                }
            }
        }
        if (last && lane == 0) {
#pragma unroll
            for (int k = 0; k < NV; k++) out[k] = s[k] + c[k];
        }
    }
    __syncthreads();
    if (tid == 0) *s_flag = last ? 1 : 0;
    __syncthreads();
    return *s_flag != 0;
}

}  // namespace simmd
