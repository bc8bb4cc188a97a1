// CPMG walk entry point that allocates nothing (rwnmr_cpmg_run_noalloc, include/rwnmr_gb300.h).
//
// Who needs it: callers that own every byte of device memory themselves and cannot let a library
// call cudaMalloc behind their back -- a host framework whose caching allocator holds the GPU's
// memory under a fixed budget (a stray cudaMalloc can fail or fragment it), or an application that
// runs under a hard device-memory cap and pre-allocates everything at start-up. The regular entry
// points (rwnmr_cpmg_run and friends) allocate their work buffers inside the context; this one
// takes device pointers for every input and output and keeps its own scratch -- the energy tables,
// the per-echo fixed-point accumulators and a status word -- in the file-scope device array below.
//
// The energy tables are filled on the GPU by one thread per phase, as the FP64 repeated product the
// reference computes one collision at a time, so they are bit-identical to the context path's host
// tables; that serial chain adds latency in proportion to the table length (echoes x steps per echo).
//
// Limits and sharing:
//   * the scratch array is kNoallocScratchBytes (8 MiB) on every device that loads the library,
//     held until the process exits; a request whose tables plus accumulators do not fit is
//     rejected with RWNMR_ERR_UNSUPPORTED and a message giving the bytes it would need;
//   * every call on a device uses the same array and leaves its contents behind; each call
//     clears the accumulators and status word it uses before its kernels run, so results never
//     depend on an earlier call, but calls that overlap on the GPU (different streams or host
//     threads on one device) race on the array and must be serialised by the caller;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//     that device current and caches it; make that first call before any stream capture.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/rwnmr_gb300.h"
#include "walk_kernels.cuh"

namespace
{
constexpr size_t kNoallocScratchBytes = 8u << 20;
constexpr size_t kScratchWords = kNoallocScratchBytes / sizeof(unsigned long long);
constexpr size_t kTableOffsetWords = 32; // word 0 = status; tables start 256 bytes in
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned long long g_noalloc_scratch[kScratchWords];

std::mutex g_addr_mu;
unsigned long long *g_addr[kMaxDevices] = {};

// table[q][k] = round(f_q^k * 2^63) with f_q^k the FP64 repeated product, one thread per phase:
// the same values the engine's host-side table builder computes (IEEE multiply, round-to-nearest
// conversion). Unused phase slots hold 2^63 (energy factor 1).
__global__ void noalloc_tables_kernel(unsigned long long *tab, int slots, int n_phases, int64_t stride, double f0,
                                      double f1, double f2, double f3)
{
    const int q = threadIdx.x;
    if (q >= slots) return;
    const double f = q == 0 ? f0 : (q == 1 ? f1 : (q == 2 ? f2 : f3));
    unsigned long long *t = tab + (size_t)q * stride;
    double v = 1.0;
    for (int64_t k = 0; k < stride; k++)
    {
        t[k] = q < n_phases ? __double2ull_rn(v * 9223372036854775808.0) : (1ull << 63);
        v = v * f;
    }
}

// The exact 128-bit integer l0 + l1 2^21 + l2 2^42 (three u64 limb sums) rounded once to FP64
// (round to nearest, ties to even) and scaled by 2^-63: the same value the context entry point's
// host-side conversion gives. The top 64 significant bits, with a sticky bit for any nonzero bits
// below them, convert with one rounding; the power-of-two scalings are exact.
__device__ double limbs_to_double_rn(const unsigned long long *a)
{
    unsigned long long lo = a[0], hi = 0;
    const unsigned long long t1 = a[1] << 21, t2 = a[2] << 42;
    lo += t1;
    hi += (a[1] >> 43) + (lo < t1 ? 1ull : 0ull);
    lo += t2;
    hi += (a[2] >> 22) + (lo < t2 ? 1ull : 0ull);
    if (hi == 0) return ldexp(__ull2double_rn(lo), -63);
    const int sh = 64 - __clzll((long long)hi); // significant bits in hi, 1..64
    const unsigned long long top = sh == 64 ? hi : (hi << (64 - sh)) | (lo >> sh);
    const unsigned long long rest = sh == 64 ? lo : lo << (64 - sh);
    return ldexp(__ull2double_rn(top | (rest != 0 ? 1ull : 0ull)), sh - 63);
}

// Per-echo accumulator limbs -> FP64 echo sums and per-phase collision counts.
__global__ void noalloc_finish_kernel(const unsigned long long *acc, int K, int n_echoes, int n_phases, double *echo_sum,
                                      unsigned long long *echo_coll)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e <= n_echoes; e += gridDim.x * blockDim.x)
    {
        const unsigned long long *a = acc + (size_t)e * K;
        echo_sum[e] = limbs_to_double_rn(a);
        if (echo_coll && e > 0)
            for (int q = 0; q < n_phases; q++) echo_coll[(size_t)(e - 1) * n_phases + q] = a[3 + q];
    }
}

// Phase labels of a 3- or 4-phase image (W = 4 words per block: the solid mask, then bit-planes 0-2
// of the solid voxel's phase index): every solid voxel's index must be below n_phases. The walk
// reads a phase's table slot from the planes, and an index beyond the caller's phase count would
// select an unused slot (no relaxation) instead of failing, so such images are reported here.
__global__ void noalloc_check_labels_kernel(const uint32_t *__restrict__ blocks, int64_t nblocks, int n_phases,
                                            unsigned *status)
{
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblocks; b += (int64_t)gridDim.x * blockDim.x)
    {
        const uint4 lo = *reinterpret_cast<const uint4 *>(blocks + b * 8);     // words' low halves
        const uint4 hi = *reinterpret_cast<const uint4 *>(blocks + b * 8 + 4); // words' high halves
        uint32_t bad_lo = lo.w, bad_hi = hi.w;                                  // plane 2: index >= 4
        if (n_phases == 3)
        {
            bad_lo |= lo.y & lo.z; // index 3
            bad_hi |= hi.y & hi.z;
        }
        if ((bad_lo & lo.x) | (bad_hi & hi.x)) atomicOr(status, rwnmr::kStatusBadLabel);
    }
}

rwnmr_status say(char *err, int errlen, rwnmr_status s, const char *fmt, ...)
{
    if (err && errlen > 0)
    {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t)errlen, fmt, ap);
        va_end(ap);
    }
    return s;
}

// Device address of the scratch array on the current device, looked up once per device.
cudaError_t scratch_address(unsigned long long **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (!g_addr[dev])
    {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = (unsigned long long *)p;
    }
    *out = g_addr[dev];
    return cudaSuccess;
}
} // namespace

extern "C" rwnmr_status rwnmr_cpmg_run_noalloc(const rwnmr_cpmg_params *p, const rwnmr_noalloc_cpmg_args *a, char *err,
                                                int errlen)
{
    using namespace rwnmr;
    if (!p || !a) return say(err, errlen, RWNMR_ERR_INVALID, "NULL params or args");
    if (p->bc < RWNMR_BC_NOFLUX || p->bc > RWNMR_BC_MIRROR || p->shift < 0 || p->shift > 10)
        return say(err, errlen, RWNMR_ERR_INVALID, "bad boundary condition or voxel-division shift");
    if (p->n_echoes < 0 || p->steps_per_echo < 1) return say(err, errlen, RWNMR_ERR_INVALID, "bad echo count / steps per echo");
    if (a->nx < 2 || a->ny < 2 || a->nz < 2) return say(err, errlen, RWNMR_ERR_UNSUPPORTED, "3D walks need at least 2 voxels per axis");
    if ((int64_t)((a->nx + 3) / 4) * ((a->ny + 3) / 4) * ((a->nz + 3) / 4) >= (1ll << 31))
        return say(err, errlen, RWNMR_ERR_UNSUPPORTED, "images are limited to 2^31 bit-blocks");
    if (a->n_phases < 1 || a->n_phases > 4) return say(err, errlen, RWNMR_ERR_UNSUPPORTED, "1 to 4 solid phases are supported");
    if (a->n < 0 || a->n > (1ll << 31) - 1) return say(err, errlen, RWNMR_ERR_INVALID, "walker count out of range");
    if (!p->dfactor) return say(err, errlen, RWNMR_ERR_INVALID, "dfactor is NULL");
    for (int q = 0; q < a->n_phases; q++)
        if (!(p->dfactor[q] >= 0.0 && p->dfactor[q] <= 1.0))
            return say(err, errlen, RWNMR_ERR_UNSUPPORTED, "decrease factor of phase %d outside [0, 1]", q);
    if (!a->blocks || !a->echo_sum || (a->n > 0 && (!a->x0 || !a->y0 || !a->z0 || !a->seed0 || !a->x || !a->y ||
                                                     !a->z || !a->seed || !a->collisions)))
        return say(err, errlen, RWNMR_ERR_INVALID, "a required device pointer is NULL");

    if (((uintptr_t)a->blocks & (a->n_phases > 1 ? 15 : 7)) != 0)
        return say(err, errlen, RWNMR_ERR_INVALID, "blocks must be %d-byte aligned", a->n_phases > 1 ? 16 : 8);
    const int slots = a->n_phases <= 1 ? 1 : (a->n_phases == 2 ? 2 : 4);
    const int K = 3 + slots;
    const int64_t nmax = (int64_t)p->n_echoes * p->steps_per_echo;
    const size_t table_words = (size_t)slots * (size_t)(nmax + 1);
    const size_t acc_words = (size_t)(p->n_echoes + 1) * K;
    const size_t need = kTableOffsetWords + ((table_words + 31) / 32) * 32 + acc_words;
    if (nmax > (1ll << 28) || need > kScratchWords)
        return say(err, errlen, RWNMR_ERR_UNSUPPORTED,
                   "walk needs %zu bytes of scratch; the no-alloc entry point has %zu (fewer echoes or steps per echo)",
                   need * 8, kNoallocScratchBytes);

    unsigned long long *base = nullptr;
    cudaError_t ce = scratch_address(&base);
    if (ce != cudaSuccess) return say(err, errlen, RWNMR_ERR_CUDA, "scratch address: %s", cudaGetErrorString(ce));
    cudaStream_t s = (cudaStream_t)a->stream;
    unsigned *status = (unsigned *)base;
    unsigned long long *tab = base + kTableOffsetWords;
    unsigned long long *acc = tab + ((table_words + 31) / 32) * 32;

#define NA_CUDA(expr, what)                                                                                            \
    do                                                                                                                 \
    {                                                                                                                  \
        cudaError_t _e = (expr);                                                                                       \
        if (_e != cudaSuccess) return say(err, errlen, RWNMR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(_e));        \
    } while (0)

    NA_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned), s), "status reset");
    NA_CUDA(cudaMemsetAsync(acc, 0, acc_words * 8, s), "accumulator reset");
    if (slots == 4)
    {
        const int64_t nblocks = (int64_t)((a->nx + 3) / 4) * ((a->ny + 3) / 4) * ((a->nz + 3) / 4);
        const unsigned grid = (unsigned)std::min<int64_t>((nblocks + 255) / 256, 152 * 8);
        noalloc_check_labels_kernel<<<grid, 256, 0, s>>>(reinterpret_cast<const uint32_t *>(a->blocks), nblocks,
                                                         a->n_phases, status);
        NA_CUDA(cudaGetLastError(), "label check kernel");
    }
    const double *f = p->dfactor;
    noalloc_tables_kernel<<<1, 32, 0, s>>>(tab, slots, a->n_phases, nmax + 1, f[0], a->n_phases > 1 ? f[1] : 1.0,
                                           a->n_phases > 2 ? f[2] : 1.0, a->n_phases > 3 ? f[3] : 1.0);
    NA_CUDA(cudaGetLastError(), "table kernel");

    DevImage im;
    im.blocks = a->blocks;
    im.nx = a->nx;
    im.ny = a->ny;
    im.nz = a->nz;
    im.bcols = (a->nx + 3) / 4;
    im.bcr = im.bcols * ((a->ny + 3) / 4);
    im.bc = p->bc;
    im.shift = p->shift;
    WalkState st;
    st.n = a->n;
    st.x0 = a->x0;
    st.y0 = a->y0;
    st.z0 = a->z0;
    st.seed0 = a->seed0;
    st.x = a->x;
    st.y = a->y;
    st.z = a->z;
    st.seed = a->seed;
    st.coll = a->collisions;
    CpmgLaunch L{};
    L.steps_per_echo = p->steps_per_echo;
    L.record = 1;
    L.tfx = reinterpret_cast<const uint64_t *>(tab);
    L.tstride = (int)(nmax + 1);
    L.acc = acc;
    L.status = status;
    const int bc_key = p->shift > 0 ? BC_GENERIC : p->bc;
    const dim3 grid((unsigned)((a->n + kWalkThreads - 1) / kWalkThreads > 0 ? (a->n + kWalkThreads - 1) / kWalkThreads : 1));
    const int chunk = p->echoes_per_launch > 0 ? p->echoes_per_launch : std::max(32, (4096 / p->steps_per_echo) / 32 * 32);
    if (a->n > 0)
    {
        if (p->n_echoes == 0)
        {
            L.e_begin = L.e_end = 0;
            L.from_initial = 1;
            NA_CUDA(launch_cpmg_walk(bc_key, slots, im, st, L, grid, s), "walk kernel");
        }
        for (int e = 0; e < p->n_echoes; e += chunk)
        {
            L.e_begin = e;
            L.e_end = std::min(p->n_echoes, e + chunk);
            L.from_initial = e == 0;
            NA_CUDA(launch_cpmg_walk(bc_key, slots, im, st, L, grid, s), "walk kernel");
        }
    }
    noalloc_finish_kernel<<<(p->n_echoes + 256) / 256, 256, 0, s>>>(acc, K, p->n_echoes, a->n_phases, a->echo_sum,
                                                                     a->echo_coll);
    NA_CUDA(cudaGetLastError(), "finish kernel");
    unsigned h = 0;
    NA_CUDA(cudaMemcpyAsync(&h, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "status readback");
    NA_CUDA(cudaStreamSynchronize(s), "stream synchronize");
    if (h & kStatusBadLabel)
        return say(err, errlen, RWNMR_ERR_INVALID, "a solid voxel's phase index is not below n_phases = %d",
                   a->n_phases);
    if (h & kStatusBadStart) return say(err, errlen, RWNMR_ERR_INVALID, "a walker starts outside the image");
#undef NA_CUDA
    return say(err, errlen, RWNMR_OK, "");
}
