// k_noalloc.cu -- potential energy and virial of caller-owned device arrays,
// without any device allocation.
//
// Some callers cannot call cudaMalloc: a Julia program whose GPU memory is
// owned by CUDA.jl's pool (allocating behind the pool's back can exhaust
// memory the pool believes free), a host that has to keep device memory
// under a fixed budget it manages itself, or a step loop that must not pay
// an allocation's latency or synchronisation.  simmd_energy_virial_noalloc
// serves them: it is a variant of the energy pass of k_force.cu (per-particle
// pair sums, per-block partial sums, a deterministic last-block reduction)
// that reads the caller's positions, diameters and full neighbour list
// (the reference's NeighborListStruct layout) directly, and keeps its only
// scratch -- the per-block partial sums and a completion counter -- in the
// file-scope array below.
//
// Limits and sharing: at most SIMMD_NOALLOC_MAX_N particles (the scratch
// holds one partial per block of 128 particles).  The array exists once per
// GPU that loads the library and lives until the process exits; every call
// on that GPU uses the same array, so calls whose kernels overlap on the GPU
// (different streams, no ordering between them) race and give wrong sums.
// The completion counter is cleared at the start of each call.  The first
// call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; that lookup may load the
// library's device code onto the GPU (lazy module loading), so make that
// first call before any stream capture.  The address is cached per device
// and per CUDA context: after a device reset (cudaDeviceReset, CUDA.jl's
// device_reset!) the next call runs in a new context and looks it up again.
#include "../../include/simmd.h"
#include "simmd_internal.cuh"

#include <mutex>

namespace simmd {
namespace {

constexpr int NA_BLOCK = 128;
constexpr long long NA_MAX_BLOCKS = SIMMD_NOALLOC_MAX_N / NA_BLOCK;
constexpr int NA_HEADER = 32;  // doubles reserved before the partials (256 B): counter
constexpr int NA_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_scratch[NA_HEADER + 2 * NA_MAX_BLOCKS];

static std::mutex g_na_mutex;
static double* g_na_ptr[NA_MAX_DEVICES] = {};
static unsigned long long g_na_ctx[NA_MAX_DEVICES] = {};

// unique id of the calling thread's current CUDA context (0: no context yet,
// or the driver does not report one), through the runtime's driver entry
// points so that the library needs no link to libcuda
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

static unsigned long long current_ctx_id()
{
    static CtxGetCurrentFn get_cur = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool looked = false;
    if (!looked) {
        looked = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
    }
    if (!get_cur || !get_id) return 0ull;
    void* ctx = nullptr;
    unsigned long long id = 0ull;
    if (get_cur(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0ull;
    return id;
}

struct NAParams {
    double L, rc2, sigma2, sigma4, lj_cut2, eps, Uc, c0, c2, c4, zeta;
    int dims, pot;
};

__device__ __forceinline__ double na_min_image(double dx, double L, double halfL)
{
    double sh = (dx > halfL) ? L : ((dx < -halfL) ? -L : 0.0);
    return dsub(dx, sh);
}

// energy (find_energy inner loops, src/AuxiliaryFunctions.jl:381-444, 477-507,
// 571-581) and r_ij . F_ij (force expressions of src/MD.jl:85-191, 291-309)
template <int DIM, int POT>
__device__ __forceinline__ void na_pair(const NAParams& p, double r2, double Di, double Dj, double& V, double& W)
{
    V = 0.0;
    double Fr = 0.0;
    if (POT == POT_BERTHIER) {
        const double md = dmul(dmul(dadd(Di, Dj), 0.5), dsub(1.0, dmul(p.zeta, fabs(dsub(Di, Dj)))));
        const double mds = dmul(md, md);
        if (!(dmul(p.rc2, mds) < r2)) {
            const double jx2 = ddiv(r2, mds);
            const double jx4 = dmul(jx2, jx2);
            const double xi12 = drcp(dmul(dmul(jx4, jx4), jx4));
            V = dadd(dadd(dadd(xi12, dmul(p.c4, jx4)), dmul(p.c2, jx2)), p.c0);
            const double inv = drcp(mds);
            const double ix2 = dmul(r2, inv);
            const double ix4 = dmul(ix2, ix2);
            const double xi14 = drcp(dmul(dmul(dmul(ix4, ix4), ix4), ix2));
            Fr = dmul(dmul(-2.0, inv), dsub(dadd(p.c2, dmul(dmul(2.0, p.c4), ix2)), dmul(6.0, xi14)));
        }
    } else if (DIM == 3) {
        const double xi2 = ddiv(p.sigma2, r2);
        const double xi6 = dmul(dmul(xi2, xi2), xi2);
        const double xi12 = dmul(xi6, xi6);
        if (!(p.lj_cut2 < r2)) V = dsub(dmul(dmul(4.0, p.eps), dsub(xi12, xi6)), p.Uc);
        if (!(p.rc2 < r2)) Fr = ddiv(dmul(p.eps, dsub(dmul(48.0, xi12), dmul(24.0, xi6))), r2);
    } else {
        if (p.lj_cut2 > r2) {
            const double y2 = ddiv(p.sigma4, r2);
            const double y4 = dmul(y2, y2);
            const double y6 = dmul(y2, y4);
            const double y12 = dmul(y6, y6);
            V = dsub(dmul(dmul(4.0, p.eps), dsub(y12, y6)), p.Uc);
            const double inv = drcp(r2);
            const double xi2 = dmul(p.sigma4, inv);
            const double xi6 = dmul(dmul(xi2, xi2), xi2);
            const double xi12 = dmul(xi6, xi6);
            Fr = dmul(dmul(p.eps, dsub(dmul(48.0, xi12), dmul(24.0, xi6))), inv);
        }
    }
    W = dmul(Fr, r2);
}

template <int DIM, int POT>
__global__ void __launch_bounds__(NA_BLOCK) k_energy_noalloc(NAParams p, int N, const double* __restrict__ r,
                                                             const double* __restrict__ D,
                                                             const long long* __restrict__ counts,
                                                             const long long* __restrict__ list, long long maxK,
                                                             double* scratch, double* out)
{
    __shared__ double s_e[NA_BLOCK / 32], s_w[NA_BLOCK / 32], s_b[NA_BLOCK / 32];
    __shared__ int s_last;
    const int i = blockIdx.x * NA_BLOCK + threadIdx.x;
    double e = 0.0, w = 0.0, bad = 0.0;
    if (i < N) {
        const double halfL = p.L * 0.5;
        const double xi = r[(long long)i * DIM], yi = r[(long long)i * DIM + 1];
        const double zi = DIM == 3 ? r[(long long)i * DIM + 2] : 0.0;
        const double Di = D[i];
        long long n = counts[i];
        if (n < 0 || n > maxK) {
            bad += 1.0;
            n = n < 0 ? 0 : maxK;
        }
        for (long long k = 0; k < n; k++) {
            const long long j = list[k + maxK * (long long)i] - 1;  // 1-based ids
            if (j < 0 || j >= N || j == i) {
                bad += 1.0;
                continue;
            }
            const double dx = na_min_image(dsub(xi, r[j * DIM]), p.L, halfL);
            const double dy = na_min_image(dsub(yi, r[j * DIM + 1]), p.L, halfL);
            double r2 = dadd(dmul(dx, dx), dmul(dy, dy));
            if (DIM == 3) {
                const double dz = na_min_image(dsub(zi, r[j * DIM + 2]), p.L, halfL);
                r2 = dadd(r2, dmul(dz, dz));
            }
            double V, Wp;
            na_pair<DIM, POT>(p, r2, Di, D[j], V, Wp);
            e = dadd(e, V);
            w = dadd(w, Wp);
        }
    }
    // block reduction in a fixed order
    for (int o = 16; o > 0; o >>= 1) {
        e += __shfl_xor_sync(0xffffffffu, e, o);
        w += __shfl_xor_sync(0xffffffffu, w, o);
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        s_e[wid] = e;
        s_w[wid] = w;
        s_b[wid] = bad;
    }
    __syncthreads();
    unsigned int* counter = reinterpret_cast<unsigned int*>(scratch);
    double* part = scratch + NA_HEADER;
    if (threadIdx.x == 0) {
        double te = 0.0, tw = 0.0, tb = 0.0;
        for (int k = 0; k < NA_BLOCK / 32; k++) {
            te += s_e[k];
            tw += s_w[k];
            tb += s_b[k];
        }
        part[2 * blockIdx.x] = te;
        part[2 * blockIdx.x + 1] = tw;
        if (tb != 0.0) atomicAdd(&scratch[1], tb);  // header slot 1: invalid list entries
        __threadfence();
        s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last && wid == 0) {
        __threadfence();
        double se = 0.0, sw = 0.0;
        for (int q = lane; q < (int)gridDim.x; q += 32) {
            const volatile double* pq = part + 2 * q;
            se += pq[0];
            sw += pq[1];
        }
        for (int o = 16; o > 0; o >>= 1) {
            se += __shfl_xor_sync(0xffffffffu, se, o);
            sw += __shfl_xor_sync(0xffffffffu, sw, o);
        }
        if (lane == 0) {
            out[0] = se / 2.0;
            out[1] = sw / 2.0;
            out[2] = *(volatile double*)&scratch[1];
        }
    }
}

}  // namespace
}  // namespace simmd

using simmd::NAParams;
using simmd::g_na_mutex;
using simmd::g_na_ptr;
using simmd::g_na_ctx;
using simmd::current_ctx_id;
using simmd::NA_MAX_DEVICES;
using simmd::NA_BLOCK;
using simmd::k_energy_noalloc;

extern "C" int simmd_energy_virial_noalloc(const simmd_params* prm, const double* r, const double* D,
                                           const int64_t* counts, const int64_t* list, int64_t maxK, double* out,
                                           void* stream)
{
    using simmd::record_error;
    if (!prm || !r || !D || !counts || !list || !out) return record_error(SIMMD_ERR_BAD_ARG, "NULL argument");
    if (prm->dims != 2 && prm->dims != 3) return record_error(SIMMD_ERR_BAD_ARG, "dims must be 2 or 3");
    if (prm->potential != SIMMD_POT_LJ && prm->potential != SIMMD_POT_BERTHIER)
        return record_error(SIMMD_ERR_BAD_ARG, "unknown potential");
    if (prm->N < 1) return record_error(SIMMD_ERR_BAD_ARG, "N must be >= 1");
    if (prm->N > SIMMD_NOALLOC_MAX_N)  // beyond the fixed scratch
        return record_error(SIMMD_ERR_BUDGET,
                            "N is beyond SIMMD_NOALLOC_MAX_N (1048576 particles), the size of the fixed scratch "
                            "of simmd_energy_virial_noalloc: use simmd_energy on a context instead");
    if (maxK < 1) return record_error(SIMMD_ERR_BAD_ARG, "maxK must be >= 1");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) {
        cudaGetLastError();
        return record_error(SIMMD_ERR_NO_DEVICE, "no CUDA device current");
    }
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> g(g_na_mutex);
        const unsigned long long ctx = current_ctx_id();
        if (!g_na_ptr[dev] || ctx == 0ull || ctx != g_na_ctx[dev]) {
            // set-up, once per device (and again in a new context), with that
            // device current
            void* ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, simmd::g_noalloc_scratch);
            if (e != cudaSuccess || !ptr) {
                cudaGetLastError();
                g_na_ptr[dev] = nullptr;
                return record_error(SIMMD_ERR_CUDA, "cudaGetSymbolAddress of the fixed scratch failed");
            }
            g_na_ptr[dev] = static_cast<double*>(ptr);
            g_na_ctx[dev] = current_ctx_id();  // the lookup has made the context current
        }
        scratch = g_na_ptr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // counter and invalid-entry count must start at zero for every call
    if (cudaMemsetAsync(scratch, 0, 2 * sizeof(double), s) != cudaSuccess) {
        cudaGetLastError();
        return record_error(SIMMD_ERR_CUDA, "clearing the fixed scratch failed");
    }
    NAParams p;
    p.L = prm->box_size;
    p.rc2 = prm->force_cutoff2;
    p.sigma2 = prm->lj_sigma * prm->lj_sigma;
    p.sigma4 = p.sigma2 * p.sigma2;
    p.lj_cut2 = prm->dims == 3 ? p.rc2 * p.sigma2 : p.rc2 * p.sigma4;
    p.eps = prm->lj_eps;
    p.Uc = prm->lj_Uc;
    p.c0 = prm->b_c0;
    p.c2 = prm->b_c2;
    p.c4 = prm->b_c4;
    p.zeta = prm->b_zeta;
    p.dims = prm->dims;
    p.pot = prm->potential;
    const int N = (int)prm->N;
    const int grid = (N + NA_BLOCK - 1) / NA_BLOCK;
    const long long* c = reinterpret_cast<const long long*>(counts);
    const long long* l = reinterpret_cast<const long long*>(list);
    if (p.dims == 3) {
        if (p.pot == SIMMD_POT_BERTHIER)
            k_energy_noalloc<3, simmd::POT_BERTHIER><<<grid, NA_BLOCK, 0, s>>>(p, N, r, D, c, l, maxK, scratch, out);
        else
            k_energy_noalloc<3, simmd::POT_LJ><<<grid, NA_BLOCK, 0, s>>>(p, N, r, D, c, l, maxK, scratch, out);
    } else {
        if (p.pot == SIMMD_POT_BERTHIER)
            k_energy_noalloc<2, simmd::POT_BERTHIER><<<grid, NA_BLOCK, 0, s>>>(p, N, r, D, c, l, maxK, scratch, out);
        else
            k_energy_noalloc<2, simmd::POT_LJ><<<grid, NA_BLOCK, 0, s>>>(p, N, r, D, c, l, maxK, scratch, out);
    }
    if (cudaGetLastError() != cudaSuccess) return record_error(SIMMD_ERR_CUDA, "kernel launch failed");
    return SIMMD_OK;
}
