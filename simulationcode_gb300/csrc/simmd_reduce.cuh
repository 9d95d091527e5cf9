// simmd_reduce.cuh -- deterministic per-tile / per-replica reductions.
//
// Each tile writes its block-reduced partial sums to tile_part[t]; the block
// that finishes the LAST tile of a replica (atomic counter) sums that
// replica's tile partials in a fixed order (Neumaier-compensated per lane,
// then a fixed shuffle tree).  The result depends only on the replica's own
// particles and slot layout, never on which block ran which tile or on the
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

// Returns true in the threads of the block that must finalise replica r; in
// that case out[] (valid in thread 0) holds the replica totals.  WARP_DONE:
// the caller has already reduced each warp (lane 0's v[] is used).
// s_part must hold 32*NV doubles; s_flag one int.  Must be called by every
// thread of the block (contains __syncthreads).
template <int NV, bool WARP_DONE = false>
__device__ bool tile_reduce(const Batch& b, int t, const RepDesc& d, RepState& st, double (&v)[NV],
                            double (&out)[NV], double* s_part, int* s_flag)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    if (!WARP_DONE) warp_sum<NV>(v);  // else lane 0 already holds the warp's sums
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) s_part[wid * NV + k] = v[k];
    __syncthreads();
    if (tid == 0) {
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int w = 0; w < nw; w++) s += s_part[w * NV + k];
            b.tile_part[(size_t)t * NPART + k] = s;
        }
        __threadfence();
        int prev = atomicAdd(&st.done_count, 1);
        *s_flag = (prev == d.ntiles - 1);
    }
    __syncthreads();
    bool last = *s_flag;
    if (last) {
        __threadfence();
        if (wid == 0) {
            double s[NV], c[NV];
#pragma unroll
            for (int k = 0; k < NV; k++) { s[k] = 0.0; c[k] = 0.0; }
            for (int q = lane; q < d.ntiles; q += 32) {
                const volatile double* tp = b.tile_part + (size_t)(d.tile0 + q) * NPART;
#pragma unroll
                for (int k = 0; k < NV; k++) {
                    double x = tp[k];
                    double tsum = s[k] + x;
                    c[k] += (fabs(s[k]) >= fabs(x)) ? (s[k] - tsum) + x : (x - tsum) + s[k];
                    s[k] = tsum;
                }
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
