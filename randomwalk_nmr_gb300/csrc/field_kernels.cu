// CPMG walk in an internal magnetic field (sm_103a).
//
// Reference semantics (NMR_cpmg_cuda.cpp:146-293 noflux, 409-567 periodic, 683-838 mirror; the
// field itself NMR_Simulation/InternalField.cpp):
//   * an echo is two inversions of steps_per_echo / 2 steps (an odd step count loses a step);
//   * an inversion negates the walker's phase;
//   * every step adds gammatau * B at the walker's image voxel before and after the move, each
//     addition a fused multiply-add (nvcc contracts the reference's `phase += gammatau * B`);
//   * a rejected move multiplies the survival probability pAlive by the decrease factor;
//   * after each echo the walker's energy is pAlive * cos(phase).
// GB300 formulation:
//   * pAlive is the FP64 table T[c] of the collision count, the reference's repeated product bit
//     for bit (a product over phases for multi-phase images);
//   * B at the walker's voxel lives in a register and is refreshed only after a move; the
//     uniform field (coord * dG in pore voxels, 0 in solid ones) is evaluated in place rather
//     than gathered from an 8-byte-per-voxel array;
//   * energies are signed: each walker adds E * 2^61 + 2^61, in [0, 2^62], as three 21-bit limbs
//     through redux.sync (the same echo-transposed accumulation as the plain CPMG walk), and the host
//     subtracts n * 2^61. Sums are exact integers, identical run to run;
//   * the only FP64 arithmetic per echo is the reference's phase updates (two FMAs per step, kept bit
//     for bit). E = pAlive * cos(phase) is evaluated in 64-bit integer arithmetic, since FP64 is the
//     slow pipe of this GPU and its integer pipes are nearly idle here: pAlive from the fixed-point
//     survival tables (or the per-walker FP64 product converted exactly), cos(phase) by the
//     fixed-point cosine of fixed_cos.cuh (a Payne-Hanek-style reduction to turns, a 1024-entry
//     quadrant table and Taylor terms). The absolute error of E is below 2^-59.5 for |phase| < 2^40
//     (the reference's FP64 cos itself rounds at up to 2^-53); larger or non-finite phases take
//     CUDA's cos.
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "fixed_cos.cuh"
#include "walk_device.cuh"
#include "walk_kernels.cuh"

namespace rwnmr
{

namespace
{
constexpr unsigned FULL = 0xffffffffu;
constexpr uint64_t M21 = (1ull << 21) - 1;

template <int BC, int W, bool UNIFORM>
__device__ __forceinline__ double field_at(const DevImage &im, const WalkerPos &p, const FieldLaunch &L,
                                           bool may_be_solid)
{
    int ix, iy, iz;
    current_voxel<BC>(im, p, ix, iy, iz);
    if (UNIFORM)
    {
        // a walker only ever moves into pore voxels; only its start voxel can be solid
        if (may_be_solid && voxel_solid<W>(im, ix, iy, iz)) return 0.0;
        const int coord = L.axis == 0 ? ix : (L.axis == 1 ? iy : iz);
        return __ldg(L.btab + coord); // (double)coord * dg, tabulated: a load instead of FP64 work
    }
    return __ldg(L.field + ((int64_t)ix + (int64_t)iy * im.nx + (int64_t)iz * im.nx * im.ny));
}

// round(e * 2^61) + 2^61 for |e| <= 1, round half to even, in integer arithmetic: the mantissa shifted
// by the exponent (the FP64 pipe is this kernel's bound; its integer ALU is nearly idle).
__device__ __forceinline__ uint64_t energy_offset_fx(double e)
{
    const long long bits = __double_as_longlong(e);
    const int ex = (int)((bits >> 52) & 0x7ff);
    uint64_t mag = 0;
    if (ex != 0)
    {
        const uint64_t mant = ((uint64_t)bits & ((1ull << 52) - 1)) | (1ull << 52);
        const int sh = ex - 1014; // e * 2^61 = mant * 2^(ex - 1075 + 61)
        if (sh >= 0)
            mag = mant << sh;
        else if (sh > -64)
        {
            const int r = -sh;
            const uint64_t q = mant >> r, rem = mant & ((1ull << r) - 1), half = 1ull << (r - 1);
            mag = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
        }
    }
    const long long v = bits < 0 ? -(long long)mag : (long long)mag;
    return (uint64_t)(v + (1ll << 61));
}

// The echo term E * 2^61 + 2^61 of a walker with survival probability pal63 / 2^63 and phase `phase`.
// pal_fp64() is the same probability as an FP64 number, used only when cos_q62 declines the phase.
template <typename PalFp64>
__device__ __forceinline__ uint64_t echo_term(double phase, uint64_t pal63, PalFp64 &&pal_fp64,
                                              const ulonglong2 *__restrict__ quad)
{
    long long c62;
    if (!fxcos::cos_q62(phase, quad, c62)) return energy_offset_fx(pal_fp64() * cos(phase));
    const uint64_t m = __umul64hi(pal63, (uint64_t)(c62 < 0 ? -c62 : c62)); // pal |cos| 2^61
    return (uint64_t)((c62 < 0 ? -(long long)m : (long long)m) + (1ll << 61));
}

__global__ void field_table_kernel(double dg, int n, double *__restrict__ btab)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) btab[k] = (double)k * dg;
}
} // namespace

// WF (single phase): per-walker decrease factors; pAlive is then the walker's own running FP64
// product, one multiply per collision, exactly the reference's `local_pAlive *= local_dFactor`.
// MORTON (noflux, no voxel division, uniform field): steps on the image's Morton copy (see
// cpmg_walk_kernel) with the coordinate along the gradient carried beside the Morton index: a move
// changes it by one exactly when it changes the index's bits of that axis, in the direction those
// bits moved (dilated integers keep their order).
template <int BC, int NP, bool UNIFORM, bool WF, bool MORTON = false>
__global__ void __launch_bounds__(kWalkThreads, MORTON ? 6 : 4) cpmg_field_kernel(DevImage im, WalkState st, FieldLaunch L)
{
    static_assert(!WF || NP == 1, "per-walker decrease factors are for single-phase images");
    static_assert(!MORTON || (BC == BC_NOFLUX && UNIFORM), "the Morton field walk is the noflux uniform-field walk");
    constexpr int W = WordsPerBlock<NP>::value;
    constexpr int K = 3;
    __shared__ unsigned long long sacc[32 * K];
    __shared__ ulonglong2 quad[fxcos::kQuadrant]; // 16 KB: cos / sin of the first quadrant
    __shared__ uint4 sdir[6];              // MORTON: direction table
    if (MORTON && threadIdx.x < 6) sdir[threadIdx.x] = morton_direction(im.mi, threadIdx.x);

    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool active = i < st.n;

    WalkerPos p{};
    uint64_t seed = 0;
    uint32_t c[NP];
#pragma unroll
    for (int q = 0; q < NP; q++) c[q] = 0;
    double phase = 0.0;
    double fw = 1.0, pa = 1.0; // WF: decrease factor and survival probability
    if (active)
    {
        if (WF)
        {
            fw = L.wf[i];
            pa = L.from_initial ? 1.0 : L.palive[i];
        }
        if (L.from_initial)
        {
            p.x = st.x0[i];
            p.y = st.y0[i];
            p.z = st.z0[i];
            seed = st.seed0[i];
        }
        else
        {
            p.x = st.x[i];
            p.y = st.y[i];
            p.z = st.z[i];
            seed = st.seed[i];
#pragma unroll
            for (int q = 0; q < NP; q++) c[q] = st.coll[(size_t)q * st.n + i];
            phase = L.phase[i];
        }
        if (!start_ok<BC>(im, p))
        {
            atomicOr(L.status, kStatusBadStart);
            active = false;
        }
        init_image_coords<BC>(im, p);
    }
    const double B0 = active ? field_at<BC, W, UNIFORM>(im, p, L, true) : 0.0;
    double B = B0;
    uint32_t P = 0, gm = 0; // MORTON: Morton index, its bits of the gradient axis
    int gc = 0;             // MORTON: coordinate along the gradient axis
    if (MORTON)
    {
        gm = L.axis == 0 ? im.mi.mx : (L.axis == 1 ? im.mi.my : im.mi.mz);
        gc = L.axis == 0 ? p.x : (L.axis == 1 ? p.y : p.z);
        if (active)
            P = dilate_bits((uint32_t)p.x, im.mi.mx) | dilate_bits((uint32_t)p.y, im.mi.my) |
                dilate_bits((uint32_t)p.z, im.mi.mz);
    }

    for (int k = threadIdx.x; k < 32 * K; k += blockDim.x) sacc[k] = 0;
    fxcos::load_quadrant_table(quad);
    __syncthreads();
    // pAlive as 2^63 fixed point: the survival tables, or the walker's own FP64 product converted
    auto pal_q63 = [&]() { return WF ? fxcos::prob_q63(pa) : energy_fx<NP>(L.tfx, L.tstride, c); };
    auto pal_fp64 = [&]() { return WF ? pa : ldexp((double)energy_fx<NP>(L.tfx, L.tstride, c), -63); };
    if (L.e_begin == 0)
    {
        // initial energy sum (output index 0)
        const uint64_t u = active ? echo_term(phase, pal_q63(), pal_fp64, quad) : 0;
        const uint32_t r0 = __reduce_add_sync(FULL, (uint32_t)(u & M21));
        const uint32_t r1 = __reduce_add_sync(FULL, (uint32_t)((u >> 21) & M21));
        const uint32_t r2 = __reduce_add_sync(FULL, (uint32_t)(u >> 42));
        if (lane == 0)
        {
            atomicAdd(&L.acc[0], (unsigned long long)r0);
            atomicAdd(&L.acc[1], (unsigned long long)r1);
            atomicAdd(&L.acc[2], (unsigned long long)r2);
        }
    }
    __syncthreads();

    for (int e0 = L.e_begin; e0 < L.e_end; e0 += 32)
    {
        const int e1 = min(e0 + 32, L.e_end);
        uint32_t keep[K] = {0, 0, 0};
        for (int e = e0; e < e1; e++)
        {
            uint64_t u = 0;
            if (active)
            {
#pragma unroll 1
                for (int inv = 0; inv < 2; inv++)
                {
                    // the inversion: an exact sign flip, on the integer pipe (FP64 is this kernel's
                    // scarce pipe)
                    phase = __longlong_as_double(__double_as_longlong(phase) ^ (long long)(1ull << 63));
                    for (int s = 0; s < L.steps_per_inversion; s++)
                    {
                        phase = __fma_rn(L.gammatau, B, phase);
                        bool wall;
                        int ph;
                        if (MORTON)
                        {
                            const uint32_t f0 = P & gm;
                            morton_step<W>(im.mi, sdir, P, seed, wall, ph);
                            const uint32_t f1 = P & gm;
                            gc += (f1 > f0 ? 1 : 0) - (f1 < f0 ? 1 : 0);
                        }
                        else
                            walker_step<BC, W>(im, p, seed, wall, ph);
                        if (wall)
                        {
#pragma unroll
                            for (int q = 0; q < NP; q++) c[q] += (ph == q) ? 1u : 0u;
                            if (WF) pa = pa * fw;
                        }
                        else
                        {
                            B = MORTON ? __ldg(L.btab + gc) : field_at<BC, W, UNIFORM>(im, p, L, false);
                        }
                        phase = __fma_rn(L.gammatau, B, phase);
                    }
                }
                u = echo_term(phase, pal_q63(), pal_fp64, quad);
            }
            const uint32_t r0 = __reduce_add_sync(FULL, (uint32_t)(u & M21));
            const uint32_t r1 = __reduce_add_sync(FULL, (uint32_t)((u >> 21) & M21));
            const uint32_t r2 = __reduce_add_sync(FULL, (uint32_t)(u >> 42));
            const bool mine = lane == (e - e0);
            keep[0] = mine ? r0 : keep[0];
            keep[1] = mine ? r1 : keep[1];
            keep[2] = mine ? r2 : keep[2];
        }
        // lane l holds this warp's sums for echo e0 + l
        if (lane < e1 - e0)
        {
#pragma unroll
            for (int k = 0; k < K; k++)
                if (keep[k]) atomicAdd(&sacc[lane * K + k], (unsigned long long)keep[k]);
        }
        __syncthreads();
        for (int k = threadIdx.x; k < (e1 - e0) * K; k += blockDim.x)
        {
            unsigned long long v = sacc[k];
            if (v) atomicAdd(&L.acc[(size_t)(e0 + 1 + k / K) * K + (k % K)], v);
            sacc[k] = 0;
        }
        __syncthreads();
    }

    if (active)
    {
        if (MORTON)
        {
            p.x = (int)undilate_bits(P, im.mi.mx);
            p.y = (int)undilate_bits(P, im.mi.my);
            p.z = (int)undilate_bits(P, im.mi.mz);
        }
        st.x[i] = p.x;
        st.y[i] = p.y;
        st.z[i] = p.z;
        st.seed[i] = seed;
#pragma unroll
        for (int q = 0; q < NP; q++) st.coll[(size_t)q * st.n + i] = c[q];
        L.phase[i] = phase;
        if (WF) L.palive[i] = pa;
    }
}

namespace
{
template <typename F>
void with_bc_field(int bc_key, F &&f)
{
    switch (bc_key)
    {
    case BC_NOFLUX: f(std::integral_constant<int, BC_NOFLUX>{}); break;
    case BC_PERIODIC: f(std::integral_constant<int, BC_PERIODIC>{}); break;
    case BC_MIRROR: f(std::integral_constant<int, BC_MIRROR>{}); break;
    default: f(std::integral_constant<int, BC_GENERIC>{}); break;
    }
}
} // namespace

cudaError_t launch_field_table(double dg, int n, double *btab, cudaStream_t s)
{
    field_table_kernel<<<(n + 255) / 256, 256, 0, s>>>(dg, n, btab);
    return cudaGetLastError();
}

cudaError_t launch_cpmg_field(int bc_key, int np, bool uniform, const DevImage &im, const WalkState &st,
                              const FieldLaunch &L, dim3 grid, cudaStream_t s)
{
    auto go = [&](auto npc) {
        constexpr int NP = decltype(npc)::value;
        with_bc_field(bc_key, [&](auto bcc) {
            constexpr int BC = decltype(bcc)::value;
            if constexpr (NP == 1)
            {
                if (L.wf)
                {
                    if constexpr (BC == BC_NOFLUX)
                    {
                        if (uniform && im.mi.words)
                        {
                            cpmg_field_kernel<BC, 1, true, true, true><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                            return;
                        }
                    }
                    if (uniform)
                        cpmg_field_kernel<BC, 1, true, true><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                    else
                        cpmg_field_kernel<BC, 1, false, true><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                    return;
                }
            }
            if constexpr (BC == BC_NOFLUX)
            {
                if (uniform && im.mi.words)
                {
                    cpmg_field_kernel<BC, NP, true, false, true><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                    return;
                }
            }
            if (uniform)
                cpmg_field_kernel<BC, NP, true, false><<<grid, kWalkThreads, 0, s>>>(im, st, L);
            else
                cpmg_field_kernel<BC, NP, false, false><<<grid, kWalkThreads, 0, s>>>(im, st, L);
        });
    };
    if (np == 1) go(std::integral_constant<int, 1>{});
    else if (np == 2) go(std::integral_constant<int, 2>{});
    else go(std::integral_constant<int, 4>{});
    return cudaGetLastError();
}

} // namespace rwnmr
