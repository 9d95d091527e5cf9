// k_diag.cu -- device self-check (not on the simulation path): the
// bit-level conversions and grid index of the split-precision kernels
// against the hardware converter and the FP64 forms.
#include "simmd_internal.cuh"

namespace simmd {

// self-check: f2d / d2f_rn against the converter, bit for bit, and the
// integer grid index against its FP64 form
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
        // grid index: the FP64 form floor(x/h + 0.5) clamped to [0, 1023]
        RepDesc dd = {};
        const int hk = -(int)((h >> 20) & 7ull);  // h = 2^0 .. 2^-7
        dd.h = __longlong_as_double((long long)(1023 + hk) << 52);
        const double inv_h = __longlong_as_double((long long)(1023 - hk) << 52);
        const int gk = (int)((h >> 24) & 7ull);
        double xg;
        if (gk == 0) xg = __longlong_as_double((long long)h);  // any pattern
        else if (gk == 1) xg = ((double)(long long)((h >> 27) % 2300ull) * 0.5 - 50.0) * dd.h;  // ties
        else if (gk == 2) xg = __longlong_as_double(0x3fdfffffffffffffll) * dd.h;  // 0.5 - 2^-54
        else xg = ((double)(long long)(h >> 11) * 0x1.0p-53 * 1100.0 - 30.0) * dd.h;
        const double q = floor(xg * inv_h + 0.5);
        const int gref = (q == q) ? (int)fmax(fmin(q, 1023.0), 0.0) : 0;
        if (grid_index(xg, dd) != gref) nbad++;
    }
    if (nbad) atomicAdd(bad, nbad);
}

void launch_check_conversions_impl(long long n, unsigned long long seed, unsigned long long* bad, cudaStream_t s)
{
    k_check_conversions<<<1024, 256, 0, s>>>(n, seed, bad);
}

}  // namespace simmd
