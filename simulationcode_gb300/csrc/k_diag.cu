// k_diag.cu -- device self-check (not on the simulation path): the
// bit-level float <-> double conversions of the split-precision kernels
// against the hardware converter.
#include "simmd_internal.cuh"

namespace simmd {

// self-check: f2d / d2f_rn against the converter, bit for bit
__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

__global__ void k_check_conversions(long long n, unsigned long long seed, unsigned long long* bad)
{
    unsigned long long nbad = 0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = mix64(seed + 0x9e3779b97f4a7c15ull * (unsigned long long)(k + 1));
        // widening: any float pattern
        const float f = __uint_as_float((unsigned)h);
        if (__double_as_longlong(f2d(f)) != __double_as_longlong((double)f)) nbad++;
        // narrowing: a double in the float range (exponent drawn over it and
        // a little beyond), the dropped bits often a tie or next to one
        unsigned long long b = h;
        const unsigned long long ef = 880ull + ((h >> 52) % 288ull);
        b = (b & 0x800fffffffffffffull) | (ef << 52);
        const int kind = (int)((h >> 40) & 7ull);
        if (kind == 0) b = (b & ~0x1fffffffull) | 0x10000000ull;          // exact tie
        else if (kind == 1) b = (b & ~0x1fffffffull) | 0x0fffffffull;     // just below
        else if (kind == 2) b = (b & ~0x1fffffffull) | 0x10000001ull;     // just above
        else if (kind == 3) b = (b & ~0xfffffffffffffull) | 0xfffffe0000000ull | (h & 0x1fffffffull);  // carry
        const double x = __longlong_as_double((long long)(kind == 4 ? h : b));  // kind 4: any pattern
        const float a = d2f_rn(x), c = (float)x;
        if (__float_as_uint(a) != __float_as_uint(c) && !(a != a && c != c)) nbad++;
    }
    if (nbad) atomicAdd(bad, nbad);
}

void launch_check_conversions_impl(long long n, unsigned long long seed, unsigned long long* bad, cudaStream_t s)
{
    k_check_conversions<<<1024, 256, 0, s>>>(n, seed, bad);
}

}  // namespace simmd
