// simmd_reduce.cuh -- deterministic per-tile / per-replica reductions.
//
// Every warp of a work item (a tile, or one of the `parts` parts of a tile)
// writes its partial sums to its fixed slot tile_part[tile][warp of the
// tile]; the block that finishes the LAST item of a replica (atomic counter)
// sums that replica's warp partials in slot order (Neumaier-compensated per
// lane, then a fixed shuffle tree).  The result depends only on the
// replica's own particles, slot layout and threads per particle -- not on
// the parts per tile, on which block ran which item, or on the other
// replicas in the batch.
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
// used).  s_flag: one shared int.  Must be called by every thread of the
// block (contains __syncthreads); blockDim a multiple of 32.
template <int NV, bool WARP_DONE = false>
__device__ bool tile_reduce(const Batch& b, int item, const RepDesc& d, RepState& st, double (&v)[NV],
                            double (&out)[NV], int* s_flag, int parts = 1)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    const int wpt = nw * parts;  // warps per tile
    const int nitems = d.ntiles * parts;
    if (!WARP_DONE) warp_sum<NV>(v);  // else lane 0 already holds the warp's sums
    if (lane == 0) {
        const int t = item / parts, part = item - t * parts;
        double* dst = b.tile_part + ((size_t)t * wpt + (size_t)(part * nw + wid)) * NPART;
#pragma unroll
        for (int k = 0; k < NV; k++) dst[k] = v[k];
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();  // after the barrier: publishes every warp's slot (cumulative)
        const int prev = atomicAdd(&st.done_count, 1);
        *s_flag = (prev == nitems - 1);
    }
    __syncthreads();
    const bool last = *s_flag;
    if (last) {
        __threadfence();
        if (wid == 0) {
            double s[NV], c[NV];
#pragma unroll
            for (int k = 0; k < NV; k++) { s[k] = 0.0; c[k] = 0.0; }
            const int nslots = d.ntiles * wpt;
            const double* tp = b.tile_part + (size_t)d.tile0 * wpt * NPART;
            // lane-strided slots, eight loads in flight per lane (through L2:
            // other blocks wrote them), summed in slot order
            constexpr int U = 8;
            int q = lane;
            for (; q + 32 * (U - 1) < nslots; q += 32 * U) {
                double x[U][NV];
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int k = 0; k < NV; k++) x[u][k] = __ldcg(tp + (size_t)(q + 32 * u) * NPART + k);
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int k = 0; k < NV; k++) neumaier_add(s[k], c[k], x[u][k]);
            }
            for (; q < nslots; q += 32)
#pragma unroll
                for (int k = 0; k < NV; k++) neumaier_add(s[k], c[k], __ldcg(tp + (size_t)q * NPART + k));
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
