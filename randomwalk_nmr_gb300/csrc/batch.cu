// Batched multi-image CPMG with a relaxivity population per image (include/rwnmr_gb300.h,
// rwnmr_batch_*).
//
// One persistent kernel walks every image of the batch: CTAs take work items -- up to one CTA's
// worth of walkers of one image -- from a global queue (largest images first) until it is empty,
// so uneven images and walker counts share one launch without tail waste. Walk trajectories do
// not depend on the relaxivity, so each walker's walk serves all candidates of its image at once:
// after every echo the walker looks up, for each of 16 candidate decrease factors f_r, its energy
// f_r^c and its derivative c f_r^(c-1) (64-bit fixed-point tables, exact integer sums), and the warp
// reduces the 16 candidate values together with a recursive-halving shuffle transpose (16 values
// per lane -> one candidate sum per lane pair in 15 exchanges instead of 16 separate reductions).
// The echo trains M_r(e) and their derivatives dM_r(e)/df_r come out of one walk, so both the
// forward model and its vector-Jacobian product (the adjoint for one parameter per candidate) of
// all 16 candidates of all images cost one launch.
//
// The sequence table kernel -> accumulator reset -> walk -> copy-out is captured once in a CUDA
// graph and replayed for every new set of candidates (a fit iteration changes only the pinned
// decrease-factor buffer). The block size and the walkers per thread (1 or 2: two walkers share one
// transpose) are chosen by a short timed sweep (rwnmr_batch_autotune).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/rwnmr_gb300.h"
#include "walk_device.cuh"
#include "walk_kernels.cuh"

using namespace rwnmr;

namespace
{
constexpr int kCand = 16;             // candidate slots per image
constexpr int kWin = 16;              // echoes per shared-memory window
// an image gets a Morton copy (and its walkers the Morton step) when the copy takes at most this much,
// whatever the padding: only the image's own voxels are ever read, so padding costs memory, not cache
constexpr uint64_t kBatchMortonBytes = 64ull << 20;
constexpr double kEScale = 144115188075855872.0; // 2^57: energy scale (2 walkers x 32 lanes sum below 2^63)
constexpr int kScaleBits = 57;
constexpr unsigned FULLM = 0xffffffffu;

struct BatchImage
{
    const uint64_t *blocks;
    int32_t nx, ny, nz, bcols, bcr;
    int64_t walker0, n;       // walker range in the batch arrays
    int64_t acc0;             // offset of this image's accumulators (u64 words)
    int64_t tab0;             // offset of this image's tables (u64 words)
    int64_t hist0;            // offset of this image's collision histogram (u32 words)
    int32_t u_shift;          // derivative scale exponent
    MortonImage mi;           // Morton copy for the noflux histogram walk (words null: none)
};

struct WorkItem
{
    int32_t image;
    int32_t pad;
    int64_t first, last; // walker range [first, last)
};

struct BatchLaunch
{
    const BatchImage *images;
    const WorkItem *items;
    int32_t n_items;
    int32_t n_echoes, steps_per_echo, bc;
    int32_t deriv;
    int32_t tstride;             // entries per candidate table (n_echoes * steps_per_echo + 1)
    int32_t dshift;              // derivative c f^(c-1) = c * (T[c-1] >> dshift), scale 2^(57 - dshift)
    const unsigned long long *tab; // [image][cand][tstride]: energy round(f^c 2^57)
    unsigned long long *acc;       // [image][n_echoes + 1][cand][4]: energy lo/hi, derivative lo/hi
    const int32_t *x0, *y0, *z0;
    const uint64_t *seed0;
    unsigned *counter;
    unsigned *status;
    const volatile int *cancel;    // mapped host word: nonzero asks the walk to stop taking work
    unsigned long long budget_ns;  // per-CTA time budget of the walk (0: none)
    unsigned *hist;                // collision histograms (histogram walk), see hist_row
    uint2 *hist_range;             // [image][n_echoes + 1]: first and last non-zero count of each row
};

// Per-echo collision histograms: after echo e a walker has at most steps_per_echo * e collisions,
// so row e of an image's histogram holds the walker counts for c = 0 .. spe * e and starts at
// hist_row(e) = sum over earlier rows of their lengths (a triangular layout: half a dense table).
__host__ __device__ __forceinline__ int64_t hist_row(int64_t e, int spe) { return e + (int64_t)spe * e * (e - 1) / 2; }
__host__ __device__ __forceinline__ int64_t hist_words(int64_t n_echoes, int spe) { return hist_row(n_echoes + 1, spe); }

__device__ __forceinline__ DevImage dev_image(const BatchImage &img, int bc)
{
    DevImage im;
    im.blocks = img.blocks;
    im.nx = img.nx;
    im.ny = img.ny;
    im.nz = img.nz;
    im.bcols = img.bcols;
    im.bcr = img.bcr;
    im.bc = bc;
    im.shift = 0;
    return im;
}

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The next work item for the calling CTA (thread 0 calls it) -- or none, once the queue is empty,
// the batch has been cancelled or the CTA has run longer than the time budget since t0. An item
// taken and then abandoned marks the walk incomplete in the status word; the kernel ends normally,
// so a stop request never leaves a waiting kernel behind, and a walk that finished every item
// never reports a stop.
__device__ __forceinline__ int next_item(const BatchLaunch &L, unsigned long long t0)
{
    const int item = (int)atomicAdd(L.counter, 1u);
    if (item >= L.n_items) return item;
    if (*L.cancel)
    {
        atomicOr(L.status, kStatusCancelled);
        return L.n_items;
    }
    if (L.budget_ns && globaltimer_ns() - t0 > L.budget_ns)
    {
        atomicOr(L.status, kStatusBudget);
        return L.n_items;
    }
    return item;
}

// Loads the walkers of work item w that this thread walks: first + threadIdx.x + j * blockDim.x.
template <int BC, int WPT>
__device__ __forceinline__ void load_walkers(const BatchLaunch &L, const WorkItem &w, const DevImage &im,
                                             WalkerPos (&p)[WPT], uint64_t (&seed)[WPT], bool (&active)[WPT],
                                             uint32_t (&c)[WPT])
{
#pragma unroll
    for (int j = 0; j < WPT; j++)
    {
        p[j] = WalkerPos{};
        seed[j] = 0;
        c[j] = 0;
        const int64_t i = w.first + threadIdx.x + (int64_t)j * blockDim.x;
        active[j] = i < w.last;
        if (active[j])
        {
            p[j].x = L.x0[i];
            p[j].y = L.y0[i];
            p[j].z = L.z0[i];
            seed[j] = L.seed0[i];
            if (!start_ok<BC>(im, p[j]))
            {
                atomicOr(L.status, kStatusBadStart);
                active[j] = false;
            }
            init_image_coords<BC>(im, p[j]);
        }
    }
}

// Sum over the warp of v[0..15] per candidate: after the exchanges lane l holds candidate l >> 1's
// warp total (lanes 2c and 2c+1 hold the same value).
__device__ __forceinline__ unsigned long long transpose_reduce16(unsigned long long (&v)[kCand], int lane)
{
#pragma unroll
    for (int half = 8; half >= 1; half >>= 1)
    {
        const int mask = half * 2; // xor distance 16, 8, 4, 2
        const bool upper = (lane & mask) != 0;
#pragma unroll
        for (int k = 0; k < half; k++)
        {
            // keep the half of the vector this lane is responsible for, send the other half
            const unsigned long long send = upper ? v[k] : v[k + half];
            const unsigned long long keep = upper ? v[k + half] : v[k];
            const unsigned long long got = __shfl_xor_sync(FULLM, send, mask);
            v[k] = keep + got;
        }
    }
    return v[0] + __shfl_xor_sync(FULLM, v[0], 1);
}

// WPT walkers per thread: the thread walks walkers first + threadIdx.x + j * blockDim.x, j < WPT,
// and adds their table values before the warp transpose, so one transpose serves 32 * WPT walkers.
template <int BC, int WPT>
__global__ void __launch_bounds__(512, 2) batch_cpmg_kernel(BatchLaunch L)
{
    extern __shared__ unsigned long long sacc[]; // [kWin][kCand][4]
    __shared__ int s_item;
    const int lane = threadIdx.x & 31;
    const unsigned long long t0 = threadIdx.x == 0 ? globaltimer_ns() : 0;
    for (;;)
    {
        if (threadIdx.x == 0) s_item = next_item(L, t0);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= L.n_items) break;
        const WorkItem w = L.items[item];
        const BatchImage img = L.images[w.image];
        const DevImage im = dev_image(img, L.bc);
        WalkerPos p[WPT];
        uint64_t seed[WPT];
        bool active[WPT];
        uint32_t c[WPT];
        load_walkers<BC, WPT>(L, w, im, p, seed, active, c);
        // candidate pairs interleaved: entry (r, c) at ((r / 2) * tstride + c) * 2 + r % 2, so one
        // 16-byte load returns two candidates' values for a walker
        const ulonglong2 *tab2 = reinterpret_cast<const ulonglong2 *>(L.tab + img.tab0);
        unsigned long long *acc = L.acc + img.acc0;
        for (int k = threadIdx.x; k < kWin * kCand * 4; k += blockDim.x) sacc[k] = 0;
        __syncthreads();
        for (int e0 = -1; e0 < L.n_echoes; e0 += kWin)
        {
            // window covers output echoes [e0 + 1, e1]; output 0 (initial state) comes first
            const int e1 = min(e0 + kWin, L.n_echoes);
            for (int e = e0 + 1; e <= e1; e++)
            {
#pragma unroll
                for (int j = 0; j < WPT; j++)
                    if (active[j] && e > 0)
                        for (int s = 0; s < L.steps_per_echo; s++)
                        {
                            bool wall;
                            int ph;
                            walker_step<BC, 1>(im, p[j], seed[j], wall, ph);
                            c[j] += wall ? 1u : 0u;
                        }
                unsigned long long v[kCand];
#pragma unroll
                for (int r = 0; r < kCand; r++) v[r] = 0;
#pragma unroll
                for (int q = 0; q < kCand / 2; q++)
#pragma unroll
                    for (int j = 0; j < WPT; j++)
                        if (active[j])
                        {
                            const ulonglong2 t = __ldg(tab2 + (size_t)q * L.tstride + c[j]);
                            v[2 * q] += t.x;
                            v[2 * q + 1] += t.y;
                        }
                const unsigned long long sumE = transpose_reduce16(v, lane);
                const int slot = e - (e0 + 1);
                // a warp sum is below 2^63; its 32-bit halves accumulate without overflow
                unsigned long long *sa = &sacc[(slot * kCand + (lane >> 1)) * 4];
                if ((lane & 1) == 0)
                {
                    atomicAdd(&sa[0], sumE & 0xffffffffull);
                    atomicAdd(&sa[1], sumE >> 32);
                }
                if (L.deriv)
                {
#pragma unroll
                    for (int r = 0; r < kCand; r++) v[r] = 0;
#pragma unroll
                    for (int q = 0; q < kCand / 2; q++)
#pragma unroll
                        for (int j = 0; j < WPT; j++)
                            if (active[j] && c[j])
                            {
                                const ulonglong2 t = __ldg(tab2 + (size_t)q * L.tstride + c[j] - 1);
                                v[2 * q] += (unsigned long long)c[j] * (t.x >> L.dshift);
                                v[2 * q + 1] += (unsigned long long)c[j] * (t.y >> L.dshift);
                            }
                    const unsigned long long sumU = transpose_reduce16(v, lane);
                    if ((lane & 1) == 0)
                    {
                        atomicAdd(&sa[2], sumU & 0xffffffffull);
                        atomicAdd(&sa[3], sumU >> 32);
                    }
                }
            }
            __syncthreads();
            const int nslots = e1 - e0;
            for (int k = threadIdx.x; k < nslots * kCand * 4; k += blockDim.x)
            {
                const unsigned long long val = sacc[k];
                if (val) atomicAdd(&acc[(size_t)(e0 + 1) * kCand * 4 + k], val);
                sacc[k] = 0;
            }
            __syncthreads();
        }
    }
}

// Histogram walk: every walker of every image walks once and, after each echo e (and at e = 0),
// adds one to H[image][e][c] for its collision count c. Trajectories do not depend on the
// relaxivity, so these counts give every candidate's echo sums exactly:
//   sum_w f^c_w(e) = sum_c H[e][c] f^c   (batch_eval_kernel).
// The increments are fire-and-forget atomics; the rows a CTA is filling (its walkers share the
// echo) stay in L2.
// SPE: steps per echo fixed at compile time (1-3, one walker per thread, noflux), so the step loop
// unrolls; 0 reads it from the launch. (The periodic instance with 3 steps fixed gave histograms that
// differ from the candidate walk's for one image of the test batch, deterministically, while the same
// code with the count read at run time matches; the cause was not found, so the fixed-count instances
// serve the noflux walk only, where they match bit for bit.)
template <int BC, int WPT, int SPE = 0>
__global__ void __launch_bounds__(512) batch_hist_kernel(BatchLaunch L)
{
    __shared__ int s_item;
    __shared__ uint4 sdir[6]; // Morton direction table of the current item's image
    const unsigned long long t0 = threadIdx.x == 0 ? globaltimer_ns() : 0;
    for (;;)
    {
        if (threadIdx.x == 0) s_item = next_item(L, t0);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= L.n_items) break;
        const WorkItem w = L.items[item];
        const BatchImage img = L.images[w.image];
        const DevImage im = dev_image(img, L.bc);
        WalkerPos p[WPT];
        uint64_t seed[WPT];
        bool active[WPT];
        uint32_t c[WPT];
        load_walkers<BC, WPT>(L, w, im, p, seed, active, c);
        // noflux images with a Morton copy take the Morton step (uniform over the CTA's item)
        const bool mort = BC == BC_NOFLUX && img.mi.words != nullptr;
        uint32_t P[WPT];
        if (mort)
        {
            if (threadIdx.x < 6) sdir[threadIdx.x] = morton_direction(img.mi, threadIdx.x);
#pragma unroll
            for (int j = 0; j < WPT; j++)
                P[j] = dilate_bits((uint32_t)p[j].x, img.mi.mx) | dilate_bits((uint32_t)p[j].y, img.mi.my) |
                       dilate_bits((uint32_t)p[j].z, img.mi.mz);
        }
        __syncthreads();
        unsigned *H = L.hist + img.hist0;
        const int spe = SPE ? SPE : L.steps_per_echo;
        // the echo loop for one step kind, chosen once per work item
        auto walk_item = [&](auto morton) __attribute__((always_inline)) {
            constexpr bool MORT = decltype(morton)::value;
            int64_t row = 0; // hist_row(e), stepped: row(e + 1) = row(e) + spe * e + 1
            for (int e = 0; e <= L.n_echoes; row += (int64_t)spe * e + 1, e++)
            {
#pragma unroll
                for (int j = 0; j < WPT; j++)
                    if (active[j])
                    {
                        if (e > 0)
#pragma unroll(SPE ? SPE : 1)
                            for (int s = 0; s < spe; s++)
                            {
                                bool wall;
                                int ph;
                                if (MORT)
                                    morton_step<1>(img.mi, sdir, P[j], seed[j], wall, ph);
                                else
                                    walker_step<BC, 1>(im, p[j], seed[j], wall, ph);
                                c[j] += wall ? 1u : 0u;
                            }
                        atomicAdd(H + row + c[j], 1u);
                    }
            }
        };
        if (BC == BC_NOFLUX && mort) walk_item(std::true_type{});
        else walk_item(std::false_type{});
    }
}

// First and last non-zero count of every histogram row ({1, 0} for an empty row), one warp per row,
// so that the evaluation skips the stretches of counts no walker reached.
__global__ void batch_range_kernel(BatchLaunch L, int n_images)
{
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t rows_per_image = L.n_echoes + 1;
    if (row >= (int64_t)n_images * rows_per_image) return;
    const int img_i = (int)(row / rows_per_image), e = (int)(row % rows_per_image);
    const unsigned *h = L.hist + L.images[img_i].hist0 + hist_row(e, L.steps_per_echo);
    const unsigned n = (unsigned)L.steps_per_echo * e + 1;
    unsigned lo = 0xffffffffu, hi = 0;
    for (unsigned c = lane; c < n; c += 32)
        if (h[c])
        {
            lo = min(lo, c);
            hi = c;
        }
    lo = __reduce_min_sync(FULLM, lo);
    hi = __reduce_max_sync(FULLM, hi);
    if (lane == 0) L.hist_range[row] = lo == 0xffffffffu ? make_uint2(1, 0) : make_uint2(lo, hi);
}

// Echo sums from the histograms: out[e][o] = sum_c H[e][c] V_o[c] for 32 outputs o per image, the
// 16 candidates' energies V_r[c] = round(f_r^c 2^57) and their derivative terms
// V_16+r[c] = c * (round(f_r^(c-1) 2^57) >> dshift) -- the same integers the candidate walk adds up
// walker by walker, so both paths return identical sums. Exact arithmetic: V is split into 32-bit
// halves and each half's products h * V_half are summed in u64 (h * 2^32 summed over fewer than
// 2^31 walkers stays below 2^63); the two sums are stored as the accumulators' lo / hi words.
// A CTA computes kEvRows echoes x 32 outputs with kEvThreads threads: thread t owns the output pair
// 2 (t % 16), 2 (t % 16) + 1 for the 4 echoes rg .. rg + 3, rg = 4 (t / 16) -- 16 multiply-adds per
// count from one 16-byte load of its 4 counts and one of its 2 values. Histogram counts and candidate
// values are staged through shared memory kEvChunk counts at a time.
// acc += a * b (32 x 32 -> 64 bits) as one multiply-add with a 64-bit addend
__device__ __forceinline__ void mad_wide(unsigned long long &acc, unsigned a, unsigned b)
{
    asm("mad.wide.u32 %0, %1, %2, %0;" : "+l"(acc) : "r"(a), "r"(b));
}
constexpr int kEvRows = 32, kEvChunk = 64, kEvThreads = 128;
constexpr int kEvRowsPerThread = 4;

__global__ void __launch_bounds__(kEvThreads) batch_eval_kernel(BatchLaunch L, int row_blocks)
{
    // [c][echo] (rows padded to 36 words: 16-byte aligned, staging stores spread over banks) and
    // [c][output]
    __shared__ __align__(16) unsigned sh[kEvChunk][kEvRows + 4];
    __shared__ __align__(16) unsigned long long sv[kEvChunk][2 * kCand];
    const int img_i = blockIdx.x / row_blocks;
    const int e0 = (blockIdx.x % row_blocks) * kEvRows;
    const BatchImage img = L.images[img_i];
    const unsigned *H = L.hist + img.hist0;
    const ulonglong2 *tab2 = reinterpret_cast<const ulonglong2 *>(L.tab + img.tab0);
    const int spe = L.steps_per_echo;
    const int e_last = min(e0 + kEvRows - 1, L.n_echoes);
    // counts any of these rows holds: the union of their non-zero ranges
    __shared__ unsigned s_lo, s_hi;
    if (threadIdx.x < 32)
    {
        const int e = e0 + threadIdx.x;
        const uint2 r = e <= e_last ? L.hist_range[(int64_t)img_i * (L.n_echoes + 1) + e] : make_uint2(0xffffffffu, 0);
        const unsigned lo = __reduce_min_sync(FULLM, r.x), hi = __reduce_max_sync(FULLM, r.y);
        if (threadIdx.x == 0)
        {
            s_lo = lo;
            s_hi = hi;
        }
    }
    __syncthreads();
    const int64_t cmin = s_lo & ~(unsigned)(kEvChunk - 1), cmax = s_hi;
    const int op = threadIdx.x & 15;                        // outputs 2 op, 2 op + 1
    const int rg = (threadIdx.x >> 4) * kEvRowsPerThread;    // echoes e0 + rg .. + 3
    unsigned long long lo[kEvRowsPerThread][2], hi[kEvRowsPerThread][2];
#pragma unroll
    for (int k = 0; k < kEvRowsPerThread; k++)
        lo[k][0] = lo[k][1] = hi[k][0] = hi[k][1] = 0;
    for (int64_t c0 = cmin; c0 <= cmax; c0 += kEvChunk)
    {
        for (int k = threadIdx.x; k < kEvChunk * kEvRows; k += kEvThreads)
        {
            const int r = k / kEvChunk, cc = k % kEvChunk; // consecutive threads read consecutive counts
            const int e = e0 + r;
            const int64_t c = c0 + cc;
            sh[cc][r] = (e <= L.n_echoes && c <= (int64_t)spe * e) ? H[hist_row(e, spe) + c] : 0u;
        }
        for (int k = threadIdx.x; k < kEvChunk * kCand / 2; k += kEvThreads)
        {
            // candidate pair q, count c0 + cc: consecutive threads take consecutive pairs, so that a
            // warp's 16-byte stores fill whole rows of sv (no bank conflicts)
            const int q = k % (kCand / 2), cc = k / (kCand / 2);
            const int64_t c = c0 + cc;
            ulonglong2 t = make_ulonglong2(0, 0), tm = make_ulonglong2(0, 0);
            if (c < L.tstride) t = tab2[(size_t)q * L.tstride + c];
            if (c >= 1 && c < L.tstride) tm = tab2[(size_t)q * L.tstride + c - 1];
            *reinterpret_cast<ulonglong2 *>(&sv[cc][2 * q]) = t;
            *reinterpret_cast<ulonglong2 *>(&sv[cc][kCand + 2 * q]) =
                make_ulonglong2((unsigned long long)c * (tm.x >> L.dshift), (unsigned long long)c * (tm.y >> L.dshift));
        }
        __syncthreads();
#pragma unroll 4
        for (int cc = 0; cc < kEvChunk; cc++)
        {
            const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(&sv[cc][2 * op]);
            const uint4 h = *reinterpret_cast<const uint4 *>(&sh[cc][rg]);
            const unsigned vl0 = (unsigned)v.x, vh0 = (unsigned)(v.x >> 32);
            const unsigned vl1 = (unsigned)v.y, vh1 = (unsigned)(v.y >> 32);
            const unsigned hv[4] = {h.x, h.y, h.z, h.w};
#pragma unroll
            for (int k = 0; k < kEvRowsPerThread; k++)
            {
                mad_wide(lo[k][0], hv[k], vl0);
                mad_wide(hi[k][0], hv[k], vh0);
                mad_wide(lo[k][1], hv[k], vl1);
                mad_wide(hi[k][1], hv[k], vh1);
            }
        }
        __syncthreads();
    }
    if (2 * op >= kCand && !L.deriv) return;
    unsigned long long *acc = L.acc + img.acc0;
#pragma unroll
    for (int k = 0; k < kEvRowsPerThread; k++)
    {
        const int e = e0 + rg + k;
        if (e > L.n_echoes) break;
#pragma unroll
        for (int j = 0; j < 2; j++)
        {
            const int o = 2 * op + j;
            unsigned long long *a = acc + ((size_t)e * kCand + (o & (kCand - 1))) * 4 + (o >= kCand ? 2 : 0);
            a[0] = lo[k][j];
            a[1] = hi[k][j];
        }
    }
}

// Energy tables for every (image, candidate): round(f^c 2^57), f^c the FP64 repeated product. The
// walk derives the derivative c f^(c-1) from the same table (c * (T[c-1] >> dshift), exact integer
// arithmetic), so only one table per candidate competes for L2. One thread per (image, candidate).
__global__ void batch_tables_kernel(const double *__restrict__ f, int n_images, int tstride,
                                    unsigned long long *__restrict__ tab)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_images * kCand) return;
    const double fr = f[t];
    const int img = t / kCand, r = t % kCand;
    unsigned long long *te = tab + ((size_t)img * kCand + (r & ~1)) * tstride + (r & 1);
    double v = 1.0;
    for (int k = 0; k < tstride; k++)
    {
        te[2 * k] = __double2ull_rn(v * kEScale);
        v = v * fr;
    }
}

// Interleaves the low 21 bits of x, y, z (Morton / Z-order key).
uint64_t morton3(uint32_t x, uint32_t y, uint32_t z)
{
    auto spread = [](uint64_t v) {
        v &= 0x1fffff;
        v = (v | v << 32) & 0x1f00000000ffffull;
        v = (v | v << 16) & 0x1f0000ff0000ffull;
        v = (v | v << 8) & 0x100f00f00f00f00full;
        v = (v | v << 4) & 0x10c30c30c30c30c3ull;
        v = (v | v << 2) & 0x1249249249249249ull;
        return v;
    };
    return spread(x) | (spread(y) << 1) | (spread(z) << 2);
}

rwnmr_status put(std::string &s, rwnmr_status st, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    s = buf;
    return st;
}
} // namespace

struct rwnmr_batch
{
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    // host copies of the inputs until the first run uploads them
    std::vector<BatchImage> images;
    std::vector<std::vector<uint64_t>> h_blocks;
    std::vector<int32_t> hx, hy, hz;
    std::vector<uint64_t> hs;
    bool uploaded = false;
    // device
    uint64_t *d_blocks = nullptr;
    BatchImage *d_images = nullptr;
    WorkItem *d_items = nullptr;
    int32_t *d_x = nullptr, *d_y = nullptr, *d_z = nullptr;
    uint64_t *d_seed = nullptr;
    unsigned long long *d_tab = nullptr, *d_acc = nullptr;
    unsigned *d_counter = nullptr, *d_status = nullptr;
    double *d_f = nullptr;
    uint32_t *d_morton = nullptr; // Morton copies of the images that have one
    size_t tab_words = 0, acc_words = 0;
    int n_items = 0, items_block = 0; // items_block: walkers per work item
    // pinned host staging and the captured graph
    double *h_f = nullptr;
    unsigned long long *h_acc = nullptr;
    unsigned *h_status = nullptr;
    int *h_cancel = nullptr;            // mapped pinned word set by rwnmr_batch_cancel
    const int *d_cancel = nullptr;      // its device address
    unsigned long long budget_ns = 0;   // rwnmr_batch_set_time_budget
    cudaGraphExec_t graph = nullptr;
    int graph_key[7] = {0, 0, 0, 0, 0, 0, 0};
    // per-echo collision histograms of the last histogram walk, valid for hist_key
    unsigned *d_hist = nullptr;
    uint2 *d_hist_range = nullptr;
    size_t hist_alloc = 0, range_alloc = 0; // u32 words / rows allocated
    bool hist_valid = false;
    int hist_key[3] = {0, 0, 0}; // n_echoes, steps_per_echo, bc
    double hist_ms = 0.0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0, last_eval_ms = 0.0;
    int64_t launches = 0;
    int tuned_block = 0, tuned_wpt = 0;
    int sms = 0;

    void free_device()
    {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        for (void *p : {(void *)d_blocks, (void *)d_images, (void *)d_items, (void *)d_x, (void *)d_y, (void *)d_z,
                        (void *)d_seed, (void *)d_tab, (void *)d_acc, (void *)d_counter,
                        (void *)d_status, (void *)d_f, (void *)d_morton})
            if (p) cudaFree(p);
        d_blocks = nullptr;
        d_images = nullptr;
        d_items = nullptr;
        d_x = d_y = d_z = nullptr;
        d_seed = nullptr;
        d_tab = d_acc = nullptr;
        d_counter = d_status = nullptr;
        d_f = nullptr;
        d_morton = nullptr;
        if (d_hist) cudaFree(d_hist);
        if (d_hist_range) cudaFree(d_hist_range);
        d_hist = nullptr;
        d_hist_range = nullptr;
        hist_alloc = range_alloc = 0;
        hist_valid = false;
        if (h_f) cudaFreeHost(h_f);
        if (h_acc) cudaFreeHost(h_acc);
        if (h_status) cudaFreeHost(h_status);
        h_f = nullptr;
        h_acc = nullptr;
        h_status = nullptr;
        uploaded = false;
    }
};

namespace
{
#define BT_CUDA(b, expr, what)                                                                                         \
    do                                                                                                                 \
    {                                                                                                                  \
        cudaError_t _e = (expr);                                                                                       \
        if (_e != cudaSuccess)                                                                                         \
            return put((b)->err, _e == cudaErrorMemoryAllocation ? RWNMR_ERR_NOMEM : RWNMR_ERR_CUDA, "%s: %s", what,  \
                       cudaGetErrorString(_e));                                                                        \
    } while (0)

rwnmr_status upload(rwnmr_batch *b, int n_echoes, int spe)
{
    const int64_t nmax = (int64_t)n_echoes * spe;
    const int tstride = (int)(nmax + 1);
    const int ni = (int)b->images.size();
    if (b->uploaded && b->tab_words == (size_t)ni * kCand * tstride &&
        b->acc_words == (size_t)ni * (n_echoes + 1) * kCand * 4)
        return RWNMR_OK;
    b->free_device();
    size_t nb = 0;
    for (auto &h : b->h_blocks) nb += h.size();
    const size_t nw = b->hx.size();
    BT_CUDA(b, cudaMalloc(&b->d_blocks, std::max<size_t>(nb, 1) * 8), "batch image");
    BT_CUDA(b, cudaMalloc(&b->d_x, std::max<size_t>(nw, 1) * 4), "batch walkers");
    BT_CUDA(b, cudaMalloc(&b->d_y, std::max<size_t>(nw, 1) * 4), "batch walkers");
    BT_CUDA(b, cudaMalloc(&b->d_z, std::max<size_t>(nw, 1) * 4), "batch walkers");
    BT_CUDA(b, cudaMalloc(&b->d_seed, std::max<size_t>(nw, 1) * 8), "batch walkers");
    size_t off = 0;
    // derivative values c f^(c-1) <= nmax: scaled by 2^us so that they stay below 2^57 like the energies
    const int us = kScaleBits - (int)std::ceil(std::log2((double)(nmax + 2)));
    for (int k = 0; k < ni; k++)
    {
        BT_CUDA(b, cudaMemcpy(b->d_blocks + off, b->h_blocks[k].data(), b->h_blocks[k].size() * 8, cudaMemcpyHostToDevice),
                "batch image upload");
        b->images[k].blocks = b->d_blocks + off;
        off += b->h_blocks[k].size();
        b->images[k].tab0 = (int64_t)k * kCand * tstride;
        b->images[k].acc0 = (int64_t)k * (n_echoes + 1) * kCand * 4;
        b->images[k].hist0 = (int64_t)k * hist_words(n_echoes, spe);
        b->images[k].u_shift = us;
    }
    // Morton copies (single-phase: one word per 32 voxels) for the images whose box allows one
    {
        std::vector<uint32_t> words(ni, 0);
        size_t total = 0;
        for (int k = 0; k < ni; k++)
        {
            b->images[k].mi = morton_params(b->images[k].nx, b->images[k].ny, b->images[k].nz, words[k], 1, kBatchMortonBytes);
            total += words[k];
        }
        if (total)
        {
            // the block copies above ran on the default stream; the build reads them on b->stream
            BT_CUDA(b, cudaStreamSynchronize(0), "batch image upload");
            BT_CUDA(b, cudaMalloc(&b->d_morton, total * 4), "batch Morton images");
            size_t mo = 0;
            for (int k = 0; k < ni; k++)
            {
                if (!words[k]) continue;
                BatchImage &bi = b->images[k];
                bi.mi.words = b->d_morton + mo;
                DevImage im{};
                im.blocks = bi.blocks;
                im.nx = bi.nx;
                im.ny = bi.ny;
                im.nz = bi.nz;
                im.bcols = bi.bcols;
                im.bcr = bi.bcr;
                im.bc = RWNMR_BC_NOFLUX;
                im.shift = 0;
                im.mi = bi.mi;
                BT_CUDA(b, launch_morton_build(im, 1, words[k], b->d_morton + mo, b->stream), "batch Morton images");
                mo += words[k];
            }
            BT_CUDA(b, cudaStreamSynchronize(b->stream), "batch Morton images");
        }
    }
    if (nw)
    {
        BT_CUDA(b, cudaMemcpy(b->d_x, b->hx.data(), nw * 4, cudaMemcpyHostToDevice), "batch walkers upload");
        BT_CUDA(b, cudaMemcpy(b->d_y, b->hy.data(), nw * 4, cudaMemcpyHostToDevice), "batch walkers upload");
        BT_CUDA(b, cudaMemcpy(b->d_z, b->hz.data(), nw * 4, cudaMemcpyHostToDevice), "batch walkers upload");
        BT_CUDA(b, cudaMemcpy(b->d_seed, b->hs.data(), nw * 8, cudaMemcpyHostToDevice), "batch walkers upload");
    }
    BT_CUDA(b, cudaMalloc(&b->d_images, std::max(ni, 1) * sizeof(BatchImage)), "batch descriptors");
    BT_CUDA(b, cudaMemcpy(b->d_images, b->images.data(), ni * sizeof(BatchImage), cudaMemcpyHostToDevice), "batch descriptors");
    b->tab_words = (size_t)ni * kCand * tstride;
    b->acc_words = (size_t)ni * (n_echoes + 1) * kCand * 4;
    BT_CUDA(b, cudaMalloc(&b->d_tab, std::max<size_t>(b->tab_words, 1) * 8), "batch tables");
    BT_CUDA(b, cudaMalloc(&b->d_acc, std::max<size_t>(b->acc_words, 1) * 8), "batch accumulators");
    BT_CUDA(b, cudaMalloc(&b->d_counter, 4), "batch counter");
    BT_CUDA(b, cudaMalloc(&b->d_status, 4), "batch status");
    BT_CUDA(b, cudaMalloc(&b->d_f, std::max(ni, 1) * kCand * 8), "batch factors");
    BT_CUDA(b, cudaMallocHost(&b->h_f, std::max(ni, 1) * kCand * 8), "batch staging");
    BT_CUDA(b, cudaMallocHost(&b->h_acc, std::max<size_t>(b->acc_words, 1) * 8), "batch staging");
    BT_CUDA(b, cudaMallocHost(&b->h_status, 4), "batch staging");
    b->items_block = 0;
    b->uploaded = true;
    return RWNMR_OK;
}

// Work items of `block` walkers, largest images first.
rwnmr_status build_items(rwnmr_batch *b, int block)
{
    if (b->items_block == block && b->d_items) return RWNMR_OK;
    std::vector<int> order(b->images.size());
    for (size_t k = 0; k < order.size(); k++) order[k] = (int)k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->images[a].n > b->images[c].n; });
    std::vector<WorkItem> items;
    for (int k : order)
        for (int64_t s = 0; s < b->images[k].n; s += block)
            items.push_back({k, 0, b->images[k].walker0 + s, b->images[k].walker0 + std::min<int64_t>(b->images[k].n, s + block)});
    if (b->d_items) cudaFree(b->d_items);
    b->d_items = nullptr;
    BT_CUDA(b, cudaMalloc(&b->d_items, std::max<size_t>(items.size(), 1) * sizeof(WorkItem)), "work items");
    if (!items.empty())
        BT_CUDA(b, cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice), "work items");
    b->n_items = (int)items.size();
    b->items_block = block;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    return RWNMR_OK;
}

BatchLaunch launch_args(rwnmr_batch *b, const rwnmr_batch_cpmg_params *p)
{
    const int ni = (int)b->images.size();
    BatchLaunch L{};
    L.images = b->d_images;
    L.items = b->d_items;
    L.n_items = b->n_items;
    L.n_echoes = p->n_echoes;
    L.steps_per_echo = p->steps_per_echo;
    L.bc = p->bc;
    L.deriv = p->derivatives ? 1 : 0;
    L.tstride = p->n_echoes * p->steps_per_echo + 1;
    L.dshift = ni ? kScaleBits - b->images[0].u_shift : 0;
    L.tab = b->d_tab;
    L.acc = b->d_acc;
    L.x0 = b->d_x;
    L.y0 = b->d_y;
    L.z0 = b->d_z;
    L.seed0 = b->d_seed;
    L.counter = b->d_counter;
    L.status = b->d_status;
    L.cancel = b->d_cancel;
    L.budget_ns = b->budget_ns;
    L.hist = b->d_hist;
    L.hist_range = b->d_hist_range;
    return L;
}

// Launches kern over the work queue with as many resident CTAs as fit on the GPU.
template <typename K>
void launch_persistent(rwnmr_batch *b, K kern, const BatchLaunch &L, int block, size_t smem)
{
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
    const int grid = std::max(1, std::min(b->n_items, std::max(1, per_sm) * b->sms));
    kern<<<grid, block, smem, b->stream>>>(L);
}

// Candidate walk: tables -> walk (every candidate's sums, walker by walker) -> copy-out.
cudaError_t enqueue(rwnmr_batch *b, const rwnmr_batch_cpmg_params *p, int block, int wpt)
{
    const int ni = (int)b->images.size();
    const int tstride = p->n_echoes * p->steps_per_echo + 1;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b->d_f, b->h_f, (size_t)ni * kCand * 8, cudaMemcpyHostToDevice, b->stream))) return e;
    batch_tables_kernel<<<(ni * kCand + 127) / 128, 128, 0, b->stream>>>(b->d_f, ni, tstride, b->d_tab);
    if ((e = cudaGetLastError())) return e;
    if ((e = cudaMemsetAsync(b->d_acc, 0, b->acc_words * 8, b->stream))) return e;
    if ((e = cudaMemsetAsync(b->d_counter, 0, 4, b->stream))) return e;
    if ((e = cudaMemsetAsync(b->d_status, 0, 4, b->stream))) return e;
    const BatchLaunch L = launch_args(b, p);
    const size_t smem = (size_t)kWin * kCand * 4 * 8;
    auto by_wpt = [&](auto bcc) {
        constexpr int BC = decltype(bcc)::value;
        if (wpt == 2) launch_persistent(b, batch_cpmg_kernel<BC, 2>, L, block, smem);
        else launch_persistent(b, batch_cpmg_kernel<BC, 1>, L, block, smem);
    };
    if (p->bc == RWNMR_BC_PERIODIC) by_wpt(std::integral_constant<int, BC_PERIODIC>{});
    else if (p->bc == RWNMR_BC_MIRROR) by_wpt(std::integral_constant<int, BC_MIRROR>{});
    else by_wpt(std::integral_constant<int, BC_NOFLUX>{});
    if ((e = cudaGetLastError())) return e;
    if ((e = cudaMemcpyAsync(b->h_acc, b->d_acc, b->acc_words * 8, cudaMemcpyDeviceToHost, b->stream))) return e;
    return cudaMemcpyAsync(b->h_status, b->d_status, 4, cudaMemcpyDeviceToHost, b->stream);
}

// Histogram evaluation: tables -> sums from the stored histograms -> copy-out (no walk).
cudaError_t enqueue_eval(rwnmr_batch *b, const rwnmr_batch_cpmg_params *p)
{
    const int ni = (int)b->images.size();
    const int tstride = p->n_echoes * p->steps_per_echo + 1;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b->d_f, b->h_f, (size_t)ni * kCand * 8, cudaMemcpyHostToDevice, b->stream))) return e;
    batch_tables_kernel<<<(ni * kCand + 127) / 128, 128, 0, b->stream>>>(b->d_f, ni, tstride, b->d_tab);
    if ((e = cudaGetLastError())) return e;
    if ((e = cudaMemsetAsync(b->d_acc, 0, b->acc_words * 8, b->stream))) return e;
    const BatchLaunch L = launch_args(b, p);
    const int row_blocks = (p->n_echoes + 1 + kEvRows - 1) / kEvRows;
    batch_eval_kernel<<<ni * row_blocks, kEvThreads, 0, b->stream>>>(L, row_blocks);
    if ((e = cudaGetLastError())) return e;
    if ((e = cudaMemcpyAsync(b->h_acc, b->d_acc, b->acc_words * 8, cudaMemcpyDeviceToHost, b->stream))) return e;
    return cudaMemcpyAsync(b->h_status, b->d_status, 4, cudaMemcpyDeviceToHost, b->stream);
}

size_t hist_bytes(const rwnmr_batch *b, const rwnmr_batch_cpmg_params *p)
{
    return b->images.size() * (size_t)hist_words(p->n_echoes, p->steps_per_echo) * 4;
}

// Method of a call: histograms unless asked otherwise or they would take more than half the free
// device memory (then every call walks its candidates).
int resolve_method(rwnmr_batch *b, const rwnmr_batch_cpmg_params *p)
{
    if (p->method == RWNMR_BATCH_CANDIDATE_WALK) return RWNMR_BATCH_CANDIDATE_WALK;
    if (p->method == RWNMR_BATCH_HISTOGRAMS) return RWNMR_BATCH_HISTOGRAMS;
    if (b->hist_valid && b->hist_key[0] == p->n_echoes && b->hist_key[1] == p->steps_per_echo && b->hist_key[2] == p->bc)
        return RWNMR_BATCH_HISTOGRAMS;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return RWNMR_BATCH_CANDIDATE_WALK;
    const size_t need = hist_bytes(b, p);
    return need <= (free_b + b->hist_alloc * 4) / 2 ? RWNMR_BATCH_HISTOGRAMS : RWNMR_BATCH_CANDIDATE_WALK;
}

// Runs the histogram walk unless the stored histograms already belong to this walk (same echoes,
// steps per echo and boundary condition; images and walkers are fixed once uploaded).
// The status word of the last persistent walk: a walker outside its image, or a walk stopped by
// rwnmr_batch_cancel or the time budget (its sums are incomplete; a cancel request is consumed).
rwnmr_status walk_status(rwnmr_batch *b)
{
    const unsigned st = *b->h_status;
    if (st & (kStatusCancelled | kStatusBudget))
    {
        b->hist_valid = false;
        if (st & kStatusCancelled)
        {
            __atomic_store_n(b->h_cancel, 0, __ATOMIC_SEQ_CST);
            return put(b->err, RWNMR_ERR_CANCELLED, "batch walk cancelled");
        }
        return put(b->err, RWNMR_ERR_TIMEOUT, "batch walk exceeded its time budget of %g s", b->budget_ns * 1e-9);
    }
    if (st & kStatusBadStart) return put(b->err, RWNMR_ERR_INVALID, "a walker starts outside its image");
    return RWNMR_OK;
}

rwnmr_status histogram_walk(rwnmr_batch *b, const rwnmr_batch_cpmg_params *p, int block, int wpt, bool force,
                            bool *walked)
{
    *walked = false;
    if (!force && b->hist_valid && b->hist_key[0] == p->n_echoes && b->hist_key[1] == p->steps_per_echo &&
        b->hist_key[2] == p->bc)
        return RWNMR_OK;
    *walked = true;
    const size_t words = b->images.size() * (size_t)hist_words(p->n_echoes, p->steps_per_echo);
    const size_t rows = b->images.size() * (size_t)(p->n_echoes + 1);
    if (b->hist_alloc < words || b->range_alloc < rows)
    {
        if (b->d_hist) cudaFree(b->d_hist);
        if (b->d_hist_range) cudaFree(b->d_hist_range);
        b->d_hist = nullptr;
        b->d_hist_range = nullptr;
        b->hist_alloc = b->range_alloc = 0;
        BT_CUDA(b, cudaMalloc(&b->d_hist, std::max<size_t>(words, 1) * 4), "collision histograms");
        BT_CUDA(b, cudaMalloc(&b->d_hist_range, std::max<size_t>(rows, 1) * sizeof(uint2)), "collision histograms");
        b->hist_alloc = words;
        b->range_alloc = rows;
        if (b->graph) cudaGraphExecDestroy(b->graph); // the evaluation graph holds the old pointers
        b->graph = nullptr;
    }
    b->hist_valid = false;
    BT_CUDA(b, cudaMemsetAsync(b->d_hist, 0, words * 4, b->stream), "histogram reset");
    BT_CUDA(b, cudaMemsetAsync(b->d_counter, 0, 4, b->stream), "histogram walk");
    BT_CUDA(b, cudaMemsetAsync(b->d_status, 0, 4, b->stream), "histogram walk");
    BT_CUDA(b, cudaEventRecord(b->ev0, b->stream), "event");
    const BatchLaunch L = launch_args(b, p);
    auto by_wpt = [&](auto bcc) {
        constexpr int BC = decltype(bcc)::value;
        if (wpt == 2) launch_persistent(b, batch_hist_kernel<BC, 2>, L, block, 0);
        else if (BC == BC_NOFLUX && p->steps_per_echo == 3) launch_persistent(b, batch_hist_kernel<BC, 1, 3>, L, block, 0);
        else if (BC == BC_NOFLUX && p->steps_per_echo == 2) launch_persistent(b, batch_hist_kernel<BC, 1, 2>, L, block, 0);
        else if (BC == BC_NOFLUX && p->steps_per_echo == 1) launch_persistent(b, batch_hist_kernel<BC, 1, 1>, L, block, 0);
        else launch_persistent(b, batch_hist_kernel<BC, 1>, L, block, 0);
    };
    if (p->bc == RWNMR_BC_PERIODIC) by_wpt(std::integral_constant<int, BC_PERIODIC>{});
    else if (p->bc == RWNMR_BC_MIRROR) by_wpt(std::integral_constant<int, BC_MIRROR>{});
    else by_wpt(std::integral_constant<int, BC_NOFLUX>{});
    BT_CUDA(b, cudaGetLastError(), "histogram walk");
    {
        const int64_t threads = (int64_t)rows * 32;
        batch_range_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, b->stream>>>(L, (int)b->images.size());
        BT_CUDA(b, cudaGetLastError(), "histogram ranges");
    }
    BT_CUDA(b, cudaEventRecord(b->ev1, b->stream), "event");
    BT_CUDA(b, cudaMemcpyAsync(b->h_status, b->d_status, 4, cudaMemcpyDeviceToHost, b->stream), "histogram walk");
    BT_CUDA(b, cudaStreamSynchronize(b->stream), "histogram walk");
    b->launches += 2;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->hist_ms = ms;
    if (rwnmr_status ws = walk_status(b)) return ws;
    b->hist_key[0] = p->n_echoes;
    b->hist_key[1] = p->steps_per_echo;
    b->hist_key[2] = p->bc;
    b->hist_valid = true;
    return RWNMR_OK;
}

// A cancel request belongs to the batch call in flight when it is made, or to the next call if
// none is: every call consumes it when it returns, whether or not one of its walks saw it (the
// request may land after the last work item was taken, or in a call that walks nothing), so it
// never carries over into a later, unrelated call.
struct ConsumeCancel
{
    rwnmr_batch *b;
    ~ConsumeCancel()
    {
        if (b && b->h_cancel) __atomic_store_n(b->h_cancel, 0, __ATOMIC_SEQ_CST);
    }
};

rwnmr_status check_params(rwnmr_batch *b, const rwnmr_batch_cpmg_params *p)
{
    if (!p) return put(b->err, RWNMR_ERR_INVALID, "params is NULL");
    if (b->images.empty()) return put(b->err, RWNMR_ERR_STATE, "batch has no images");
    if (p->bc < RWNMR_BC_NOFLUX || p->bc > RWNMR_BC_MIRROR) return put(b->err, RWNMR_ERR_INVALID, "unknown boundary condition");
    if (p->n_echoes < 0 || p->steps_per_echo < 1) return put(b->err, RWNMR_ERR_INVALID, "bad echo count / steps per echo");
    if (p->n_candidates < 1 || p->n_candidates > kCand)
        return put(b->err, RWNMR_ERR_INVALID, "1 to %d relaxivity candidates per image", kCand);
    if ((int64_t)p->n_echoes * p->steps_per_echo > (1 << 24)) return put(b->err, RWNMR_ERR_UNSUPPORTED, "walk too long for the batch tables");
    if (p->threads_per_block != 0 && (p->threads_per_block % 32 || p->threads_per_block < 64 || p->threads_per_block > 512))
        return put(b->err, RWNMR_ERR_INVALID, "threads_per_block must be a multiple of 32 in 64..512");
    if (p->walkers_per_thread < 0 || p->walkers_per_thread > 2)
        return put(b->err, RWNMR_ERR_INVALID, "walkers_per_thread must be 0 (tuned), 1 or 2");
    if (p->method < RWNMR_BATCH_AUTO || p->method > RWNMR_BATCH_CANDIDATE_WALK)
        return put(b->err, RWNMR_ERR_INVALID, "unknown batch method");
    return RWNMR_OK;
}
} // namespace

extern "C" {

rwnmr_status rwnmr_batch_create(rwnmr_batch **out, int device)
{
    if (!out) return RWNMR_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) return RWNMR_ERR_CUDA;
    if (device < 0 || device >= count) return RWNMR_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return RWNMR_ERR_CUDA;
    rwnmr_batch *b = new rwnmr_batch();
    b->device = device;
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
    void *dc = nullptr;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaHostAlloc((void **)&b->h_cancel, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(&dc, b->h_cancel, 0) != cudaSuccess)
    {
        rwnmr_batch_destroy(b);
        return RWNMR_ERR_CUDA;
    }
    *b->h_cancel = 0;
    b->d_cancel = (const int *)dc;
    *out = b;
    return RWNMR_OK;
}

void rwnmr_batch_destroy(rwnmr_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    b->free_device();
    if (b->d_items) cudaFree(b->d_items);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->h_cancel) cudaFreeHost(b->h_cancel);
    delete b;
}

rwnmr_status rwnmr_batch_cancel(rwnmr_batch *b)
{
    if (!b || !b->h_cancel) return RWNMR_ERR_INVALID;
    __atomic_store_n(b->h_cancel, 1, __ATOMIC_SEQ_CST);
    return RWNMR_OK;
}

rwnmr_status rwnmr_batch_set_time_budget(rwnmr_batch *b, double seconds)
{
    if (!b) return RWNMR_ERR_INVALID;
    if (!(seconds >= 0.0) || seconds > 1.0e6) return put(b->err, RWNMR_ERR_INVALID, "time budget %g s", seconds);
    b->budget_ns = (unsigned long long)(seconds * 1e9);
    if (b->graph) cudaGraphExecDestroy(b->graph); // the budget is a captured launch parameter
    b->graph = nullptr;
    return RWNMR_OK;
}

const char *rwnmr_batch_last_error(const rwnmr_batch *b) { return b ? b->err.c_str() : "null batch"; }
double rwnmr_batch_last_kernel_ms(const rwnmr_batch *b) { return b ? b->last_ms : 0.0; }
int64_t rwnmr_batch_launch_count(const rwnmr_batch *b) { return b ? b->launches : 0; }

rwnmr_status rwnmr_batch_add_image(rwnmr_batch *b, const uint64_t *blocks, int32_t nx, int32_t ny, int32_t nz,
                                   int64_t n, const int32_t *x0, const int32_t *y0, const int32_t *z0,
                                   const uint64_t *seed0, int32_t *index)
{
    if (!b) return RWNMR_ERR_INVALID;
    if (!blocks || nx < 2 || ny < 2 || nz < 2) return put(b->err, RWNMR_ERR_INVALID, "bad image");
    if (n < 0 || (n > 0 && (!x0 || !y0 || !z0 || !seed0))) return put(b->err, RWNMR_ERR_INVALID, "bad walkers");
    // walkers must start inside the image (checked here so that the kernel's status word only
    // ever reports engine faults)
    for (int64_t i = 0; i < n; i++)
        if ((unsigned)x0[i] >= (unsigned)nx || (unsigned)y0[i] >= (unsigned)ny || (unsigned)z0[i] >= (unsigned)nz)
            return put(b->err, RWNMR_ERR_INVALID, "walker %lld starts outside the image", (long long)i);
    BatchImage im{};
    im.nx = nx;
    im.ny = ny;
    im.nz = nz;
    im.bcols = (nx + 3) / 4;
    im.bcr = im.bcols * ((ny + 3) / 4);
    im.walker0 = (int64_t)b->hx.size();
    im.n = n;
    const size_t nb = (size_t)im.bcr * ((nz + 3) / 4);
    b->h_blocks.emplace_back(blocks, blocks + nb);
    // Walkers are stored in Morton order of their start voxel: a warp then walks neighbouring
    // walkers, which gather neighbouring bit-blocks and, having similar collision counts, nearby
    // table entries. Only sums over walkers leave the batch, so the order changes no result.
    std::vector<std::pair<uint64_t, int64_t>> order((size_t)n);
    for (int64_t i = 0; i < n; i++) order[(size_t)i] = {morton3(x0[i], y0[i], z0[i]), i};
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<uint64_t, int64_t> &a, const std::pair<uint64_t, int64_t> &c) { return a.first < c.first; });
    for (const auto &o : order)
    {
        b->hx.push_back(x0[o.second]);
        b->hy.push_back(y0[o.second]);
        b->hz.push_back(z0[o.second]);
        b->hs.push_back(seed0[o.second]);
    }
    b->images.push_back(im);
    b->free_device();
    if (b->d_items) cudaFree(b->d_items);
    b->d_items = nullptr;
    b->items_block = 0;
    if (index) *index = (int32_t)b->images.size() - 1;
    return RWNMR_OK;
}

rwnmr_status rwnmr_batch_cpmg(rwnmr_batch *b, const rwnmr_batch_cpmg_params *p, const double *dfactor, double *echo,
                              double *decho)
{
    nvtxRangePushA("rwnmr_batch_cpmg");
    struct Pop
    {
        ~Pop() { nvtxRangePop(); }
    } pop;
    if (!b) return RWNMR_ERR_INVALID;
    ConsumeCancel consume{b};
    rwnmr_status st = check_params(b, p);
    if (st != RWNMR_OK) return st;
    if (!dfactor) return put(b->err, RWNMR_ERR_INVALID, "dfactor is NULL");
    const int ni = (int)b->images.size();
    const int R = p->n_candidates;
    for (int k = 0; k < ni * R; k++)
        if (!(dfactor[k] >= 0.0 && dfactor[k] <= 1.0))
            return put(b->err, RWNMR_ERR_UNSUPPORTED, "decrease factor %g outside [0, 1]", dfactor[k]);
    cudaSetDevice(b->device);
    if ((st = upload(b, p->n_echoes, p->steps_per_echo)) != RWNMR_OK) return st;
    const int block = p->threads_per_block ? p->threads_per_block : (b->tuned_block ? b->tuned_block : 256);
    const int wpt = p->walkers_per_thread ? p->walkers_per_thread : (b->tuned_wpt ? b->tuned_wpt : 1);
    if ((st = build_items(b, block * wpt)) != RWNMR_OK) return st;
    const int method = resolve_method(b, p);
    double walk_ms = 0.0;
    if (method == RWNMR_BATCH_HISTOGRAMS)
    {
        bool walked = false;
        if ((st = histogram_walk(b, p, block, wpt, false, &walked)) != RWNMR_OK) return st;
        walk_ms = walked ? b->hist_ms : 0.0;
    }
    for (int k = 0; k < ni; k++)
        for (int r = 0; r < kCand; r++) b->h_f[k * kCand + r] = r < R ? dfactor[k * R + r] : 1.0;
    const bool hist = method == RWNMR_BATCH_HISTOGRAMS;
    const int key[7] = {p->n_echoes, p->steps_per_echo, p->bc, p->derivatives ? 1 : 0, hist ? 0 : block,
                        hist ? 0 : wpt, method};
    BT_CUDA(b, cudaEventRecord(b->ev0, b->stream), "event");
    if (p->use_graph)
    {
        if (!b->graph || std::memcmp(key, b->graph_key, sizeof key) != 0)
        {
            if (b->graph) cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
            cudaGraph_t g;
            BT_CUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
            cudaError_t ce = hist ? enqueue_eval(b, p) : enqueue(b, p, block, wpt);
            cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
            BT_CUDA(b, ce, "graph capture");
            BT_CUDA(b, ee, "graph capture");
            ce = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            BT_CUDA(b, ce, "graph instantiate");
            std::memcpy(b->graph_key, key, sizeof key);
        }
        BT_CUDA(b, cudaGraphLaunch(b->graph, b->stream), "graph launch");
    }
    else
        BT_CUDA(b, hist ? enqueue_eval(b, p) : enqueue(b, p, block, wpt), "batch launch");
    b->launches += 2;
    BT_CUDA(b, cudaEventRecord(b->ev1, b->stream), "event");
    BT_CUDA(b, cudaStreamSynchronize(b->stream), "batch walk");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->last_ms = ms + walk_ms; // this call's GPU time, its histogram walk included
    b->last_eval_ms = hist ? ms : 0.0;
    if (rwnmr_status ws = walk_status(b)) return ws;
    const int E1 = p->n_echoes + 1;
    for (int k = 0; k < ni; k++)
    {
        const double ds = std::ldexp(1.0, -b->images[k].u_shift);
        const unsigned long long *a = b->h_acc + b->images[k].acc0;
        for (int r = 0; r < R; r++)
            for (int e = 0; e < E1; e++)
            {
                const unsigned long long *v = a + ((size_t)e * kCand + r) * 4;
                const size_t o = ((size_t)k * R + r) * E1 + e;
                const unsigned __int128 se = (unsigned __int128)v[0] + ((unsigned __int128)v[1] << 32);
                const unsigned __int128 su = (unsigned __int128)v[2] + ((unsigned __int128)v[3] << 32);
                if (echo) echo[o] = (double)se / kEScale;
                if (decho) decho[o] = p->derivatives ? (double)su * ds : 0.0;
            }
    }
    return RWNMR_OK;
}

rwnmr_status rwnmr_batch_autotune(rwnmr_batch *b, const rwnmr_batch_cpmg_params *p, int32_t *best_threads,
                                  int32_t *best_walkers_per_thread, double *best_ms)
{
    if (!b) return RWNMR_ERR_INVALID;
    ConsumeCancel consume{b};
    rwnmr_status st = check_params(b, p);
    if (st != RWNMR_OK) return st;
    const int ni = (int)b->images.size();
    std::vector<double> f((size_t)ni * p->n_candidates, 0.999);
    cudaSetDevice(b->device);
    if ((st = upload(b, p->n_echoes, p->steps_per_echo)) != RWNMR_OK) return st;
    const bool hist = resolve_method(b, p) == RWNMR_BATCH_HISTOGRAMS;
    double best = 1e30;
    int arg = 256, arg_w = 1;
    for (int w : {1, 2})
        for (int t : {128, 256, 512})
        {
            if (hist)
            {
                // the walk the method runs: the histogram walk (timed twice, the faster kept)
                bool walked = false;
                double ms = 1e30;
                for (int rep = 0; rep < 2; rep++)
                {
                    if ((st = build_items(b, t * w)) != RWNMR_OK) return st;
                    if ((st = histogram_walk(b, p, t, w, true, &walked)) != RWNMR_OK) return st;
                    ms = std::min(ms, b->hist_ms);
                }
                if (ms < best)
                {
                    best = ms;
                    arg = t;
                    arg_w = w;
                }
                continue;
            }
            rwnmr_batch_cpmg_params q = *p;
            q.threads_per_block = t;
            q.walkers_per_thread = w;
            q.use_graph = 0;
            q.method = RWNMR_BATCH_CANDIDATE_WALK;
            if ((st = rwnmr_batch_cpmg(b, &q, f.data(), nullptr, nullptr)) != RWNMR_OK) return st;
            if ((st = rwnmr_batch_cpmg(b, &q, f.data(), nullptr, nullptr)) != RWNMR_OK) return st;
            if (b->last_ms < best)
            {
                best = b->last_ms;
                arg = t;
                arg_w = w;
            }
        }
    // the sweep's histograms are dropped: the next call walks (and times) its own
    b->hist_valid = false;
    b->tuned_block = arg;
    b->tuned_wpt = arg_w;
    if (best_threads) *best_threads = arg;
    if (best_walkers_per_thread) *best_walkers_per_thread = arg_w;
    if (best_ms) *best_ms = best;
    return RWNMR_OK;
}

rwnmr_status rwnmr_batch_collision_histogram(rwnmr_batch *b, int32_t image, int32_t echo, uint32_t *counts,
                                             int32_t *n_counts)
{
    if (!b) return RWNMR_ERR_INVALID;
    if (!b->hist_valid) return put(b->err, RWNMR_ERR_STATE, "no histogram walk has run");
    if (image < 0 || image >= (int)b->images.size() || echo < 0 || echo > b->hist_key[0])
        return put(b->err, RWNMR_ERR_INVALID, "image or echo out of range");
    const int spe = b->hist_key[1];
    const int64_t n = (int64_t)spe * echo + 1;
    if (n_counts) *n_counts = (int32_t)n;
    if (!counts) return RWNMR_OK;
    cudaSetDevice(b->device);
    BT_CUDA(b, cudaMemcpy(counts, b->d_hist + b->images[image].hist0 + hist_row(echo, spe), (size_t)n * 4,
                          cudaMemcpyDeviceToHost), "histogram download");
    return RWNMR_OK;
}

double rwnmr_batch_histogram_walk_ms(const rwnmr_batch *b) { return b ? b->hist_ms : 0.0; }

} // extern "C"
