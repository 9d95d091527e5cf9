// simmd_reduce.cuh -- deterministic per-tile / per-replica reductions.
//
// Canonical per-replica reduction: each tile's sum is its warps' partial
// sums added in warp order; the block that completes a replica's last tile
// (atomic counter) adds the replica's tile sums in tile order
// (Neumaier-compensated per lane, then a fixed shuffle tree).  When the
// force pass splits a tile into parts, each part writes its warps' partials
// to the tile's warp slots and the block that completes the tile's last part
// (per-tile counter) forms the tile sum in the same warp order.  The result
// depends only on the replica's own particles, slot layout and threads per
// particle -- not on the split, on which block ran which item, or on the
// other replicas in the batch.
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

__device__ __forceinline__ void neumaier_add(double& s, double& c, double x)
{
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
    s = t;
}

// Returns true in the threads of the block that must finalise the replica;
// in that case out[] (valid in thread 0) holds the replica totals.
// WARP_DONE: the caller has already reduced each warp (lane 0's v[] is
// used).  s_part: 32*NV shared doubles; s_flag: one shared int.  Must be
// called by every thread of the block (contains __syncthreads); blockDim a
// multiple of 32.
template <int NV, bool WARP_DONE = false>
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
    if (tid == 0) {
        bool tile_done = true;
        double ts[NV];
        if (parts == 1) {
            for (int k = 0; k < NV; k++) {
                double s = 0.0;
                for (int w = 0; w < nw; w++) s += s_part[w * NV + k];
                ts[k] = s;
            }
        } else {
            __threadfence();  // after the barrier: publishes every warp's slot
            tile_done = atomicAdd(&b.tile_cnt[t], 1) == parts - 1;
            if (tile_done) {
                __threadfence();
                const double* slot = b.warp_part + (size_t)t * WARP_SLOTS * NPART;
                const int wpt = nw * parts;
                for (int k = 0; k < NV; k++) {
                    double s = 0.0;
                    for (int w = 0; w < wpt; w++) s += __ldcg(slot + (size_t)w * NPART + k);
                    ts[k] = s;
                }
                b.tile_cnt[t] = 0;
            }
        }
        int last = 0;
        if (tile_done) {
            for (int k = 0; k < NV; k++) b.tile_part[(size_t)t * NPART + k] = ts[k];
            __threadfence();
            last = atomicAdd(&st.done_count, 1) == d.ntiles - 1;
        }
        *s_flag = last;
    }
    __syncthreads();
    const bool last = *s_flag;
    if (last) {
        __threadfence();
        if (wid == 0) {
            double s[NV], c[NV];
#pragma unroll
            for (int k = 0; k < NV; k++) { s[k] = 0.0; c[k] = 0.0; }
            for (int q = lane; q < d.ntiles; q += 32) {
                const double* tp = b.tile_part + (size_t)(d.tile0 + q) * NPART;
#pragma unroll
                for (int k = 0; k < NV; k++) neumaier_add(s[k], c[k], __ldcg(tp + k));
            }
#pragma unroll
            for (int k = 0; k < NV; k++) s[k] += c[k];
            warp_sum<NV>(s);
#pragma unroll
            for (int k = 0; k < NV; k++) out[k] = s[k];
            if (lane == 0) st.done_count = 0;
        }
    }
    __syncthreads();
    return last;
}

}  // namespace simmd
