// Walk kernels of the GB300 walker engine (sm_103a).
//
// Design (the reference's kernels, NMR_cpmg_cuda.cpp / NMR_pfgse_cuda.cpp, are one thread per
// walker with FP64 energy per collision, a [16][walkers] FP64 energy buffer in HBM per launch and
// host-finished reductions):
//   * the hot loop is integer-only: position, xorshift64 state and per-phase collision counters
//     live in registers; a walker's energy is never multiplied per collision. After each echo it
//     is looked up as table[c] = round(f^c * 2^63) (the reference's FP64 repeated product f^c,
//     rounded once to 64-bit fixed point). GB300 runs FP64 at a small fraction of its integer
//     rate, so FP64 stays out of the per-step and per-echo paths;
//   * per-echo sums are exact integers: each walker's 64-bit energy is split into three limbs
//     (21/21/22 bits) and summed with warp-wide redux.sync, one lane per echo keeps the warp sum,
//     warps combine in shared memory every 32 echoes and CTAs add into global 64-bit counters.
//     Integer addition is associative, so results are bit-identical run to run and across launch
//     shapes, and exact to 2^-63 per walker. At one or two steps per echo (about 6 % of walkers
//     collide per step) the walk instead records each lane's collisions of a 32-step window as
//     bits and replays them after the window, adding the limb changes into per-echo shared
//     counters: the same integers without a reduction per echo;
//   * walker state is read once per launch and written once at its end; a launch covers a
//     bounded number of echoes so that no single kernel runs for long on a shared GPU.
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

// The 96-bit product e * cq as four 24-bit limbs (the last holds bits 72-95).
__device__ __forceinline__ void product_limbs24(uint64_t e, uint32_t cq, uint32_t *l)
{
    constexpr uint32_t M24 = (1u << 24) - 1;
    const uint64_t lo = e * (uint64_t)cq;                     // bits 0-63
    const uint32_t hi = (uint32_t)__umul64hi(e, (uint64_t)cq); // bits 64-95
    l[0] = (uint32_t)lo & M24;
    l[1] = (uint32_t)(lo >> 24) & M24;
    l[2] = ((uint32_t)(lo >> 48) | (hi << 16)) & M24;
    l[3] = hi >> 8;
}

// 2^63 fixed point of an energy in [0, 1]: round(e * 2^63), the rounding of the energy tables.
__device__ __forceinline__ uint64_t walker_fx(double e) { return __double2ull_rn(e * 0x1p63); }

__device__ __forceinline__ void load_pos(const WalkState &s, int64_t i, WalkerPos &p, uint64_t &seed)
{
    p.x = s.x[i];
    p.y = s.y[i];
    p.z = s.z[i];
    seed = s.seed[i];
}
} // namespace

// ---------------------------------------------------------------------------------------------
// CPMG / collision-mapping walk over echoes [e_begin, e_end).
// acc layout: [(n_echoes+1)][K], K = 3 + NP: limbs of the energy sum after echo e (index e+1;
// index 0 = initial state) and, for k = 3 + p, collisions on phase p gained during echo e.
// PACK (two phases; at most 2047 steps per recorded echo, 65535 per unrecorded one): a lane
// counts both phases' collisions of the echo in the 16-bit halves of one word, and one
// redux.sync sums both halves over the warp (at most 32 * 2047 < 2^16 each).
// WF (single phase): every walker has its own decrease factor f_w (the reference's per-walker
// Walker::decreaseFactor, e.g. from a sigmoid of its collision rate) and its energy is the FP64
// repeated product f_w * f_w * ..., one multiply per collision as in Walker::walk_3D, applied after
// each echo for the collisions the echo gained and rounded to the same 2^63 fixed point.
// Occupancy: at 256 threads, 8 resident blocks per SM need <= 32 registers a thread, 6 need <= 40,
// 5 need <= 48. The minimum-block bounds below were chosen by measurement: 8 blocks for the bit-block
// walks (+4 % two-phase, +6 % one-phase walker-steps/s over the unbounded build; a few instances spill
// up to 16 bytes); for the Morton walks 5 blocks (48 registers; the collision replay 3.77e11 -> 4.34e11
// on the two-phase 400^3 walk, the mapping walk +6.7 %), 6 for the three-step fast echo loop (+13 %),
// where 32 registers spilled 70-140 bytes.
template <int BC, int NP, bool PACK, bool WF, bool SENS = false, int SPE = 0, bool MORTON = false>
constexpr int cpmg_min_blocks()
{
    // the sensitivity sums need more than 32 registers; their collision replay (one or two steps per
    // echo) at four phases 64 (48 spilled 68 bytes: 35.7 vs 33.5 ms per 4-phase 200^3 walk)
    if (SENS) return NP == 4 ? (MORTON && SPE >= 1 && SPE <= 2 ? 4 : 5) : 6;
    if (MORTON && !WF && (NP == 1 || PACK)) return SPE == 3 ? 6 : 5;
    if (SPE >= 1 && SPE <= 2 && !WF && (NP == 1 || PACK)) return 5; // the bit-block collision replay
    return NP == 4 ? 5 : ((BC == BC_NOFLUX || BC == BC_GENERIC) && !WF && (NP == 1 || PACK) ? 8 : 6);
}

// SPE: steps per echo known at compile time (1, 2 or 3, the common cases; 0 = read from the launch),
// so the step loop unrolls away.
// MORTON (noflux, no voxel division): the walk runs on the image's Morton copy with the position held
// as one Morton index (morton_step), converted from and back to x, y, z once per launch.
// SENS (per-phase tables): after each echo also the exact sums over walkers of E * c_q, the walker's
// 2^-63 fixed-point energy times its collision count with phase q -- the forward sensitivities,
// d(echo sum)/d f_q = sum E c_q / f_q. Each 96-bit product is summed as four 24-bit limbs.
template <int BC, int NP, bool PACK, bool WF, int SPE, bool MORTON = false, bool SENS = false>
__global__ void __launch_bounds__(kWalkThreads, (cpmg_min_blocks<BC, NP, PACK, WF, SENS, SPE, MORTON>()))
    cpmg_walk_kernel(DevImage im, WalkState st, CpmgLaunch L)
{
    static_assert(!PACK || NP == 2, "packed collision counts are for two phases");
    static_assert(!WF || NP == 1, "per-walker decrease factors are for single-phase images");
    static_assert(!MORTON || BC == BC_NOFLUX, "the Morton walk is the noflux walk");
    static_assert(!SENS || (!PACK && !WF), "sensitivities use unpacked counts and the per-phase tables");
    constexpr int W = WordsPerBlock<NP>::value;
    constexpr int NG = PACK ? 1 : NP;    // collision-count words per echo
    constexpr int KS = SENS ? 4 * NP : 0; // SENS: limbs of sum E c_q per echo
    constexpr int KK = 3 + NG + KS;       // values kept per echo
    constexpr int K = 3 + NP + KS;        // values per echo in the accumulators
    constexpr int KP = (KK + 3) / 4 * 4;  // KK padded to whole 16-byte stores
    // each warp's sums of the current 32-echo window, [warp][echo][value]: lane 0 stores them after
    // the reductions, the CTA adds the warps up when the window is flushed
    __shared__ __align__(16) uint32_t wsum[kWalkThreads / 32][32][KP];
    __shared__ uint4 sdir[6]; // MORTON: direction table
    if (MORTON && threadIdx.x < 6) sdir[threadIdx.x] = morton_direction(im.mi, threadIdx.x);

    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool active = i < st.n;
    const bool rec = SPE > 0 || L.record; // the fixed-step instances only run recorded walks

    WalkerPos p{};
    uint64_t seed = 0;
    uint32_t c[NP];
#pragma unroll
    for (int q = 0; q < NP; q++) c[q] = 0;
    if (active)
    {
        if (L.from_initial)
        {
            p.x = st.x0[i];
            p.y = st.y0[i];
            p.z = st.z0[i];
            seed = st.seed0[i];
        }
        else
        {
            load_pos(st, i, p, seed);
#pragma unroll
            for (int q = 0; q < NP; q++) c[q] = st.coll[(size_t)q * st.n + i];
        }
        if (!start_ok<BC>(im, p))
        {
            atomicOr(L.status, kStatusBadStart);
            active = false;
        }
        init_image_coords<BC>(im, p);
    }
    uint32_t P = 0; // MORTON: Morton index of the position
    if (MORTON && active)
        P = dilate_bits((uint32_t)p.x, im.mi.mx) | dilate_bits((uint32_t)p.y, im.mi.my) | dilate_bits((uint32_t)p.z, im.mi.mz);

    double fw = 1.0, ew = 1.0; // WF: decrease factor and energy of this walker
    if (WF && active)
    {
        fw = L.wf[i];
        ew = L.from_initial ? 1.0 : L.wenergy[i];
    }


    uint64_t efx = 0;
    if (active && L.record) efx = WF ? walker_fx(ew) : energy_fx<NP>(L.tfx, L.tstride, c);
    if (L.record && L.e_begin == 0)
    {
        // initial energy sum (output index 0)
        const uint32_t r0 = __reduce_add_sync(FULL, (uint32_t)(efx & M21));
        const uint32_t r1 = __reduce_add_sync(FULL, (uint32_t)((efx >> 21) & M21));
        const uint32_t r2 = __reduce_add_sync(FULL, (uint32_t)(efx >> 42));
        if (lane == 0)
        {
            atomicAdd(&L.acc[0], (unsigned long long)r0);
            atomicAdd(&L.acc[1], (unsigned long long)r1);
            atomicAdd(&L.acc[2], (unsigned long long)r2);
        }
    }
    __syncthreads();

    // The Morton walks with a fixed step count per echo and per-phase tables take, when every walker of
    // the CTA is live (every CTA but a partial last one, unless a walker started outside the image), one
    // of two loops without the per-lane liveness branch; the choice is CTA-uniform, so every loop reaches
    // the same barriers. At one or two steps per echo (one phase, packed two phases, or the sensitivity
    // walks) the collision replay below; otherwise the fast echo loop: the echo loop unrolled 8 echoes
    // deep at one step per echo (4 at two or three) so that the loop and window bookkeeping is shared
    // (+5 % on the one-step-per-echo walk before the replay). Its per-lane `changed` test stays: only
    // lanes whose counts changed look up their energy, which keeps the table gathers -- scattered over
    // the lanes' counts late in a walk -- to a few lanes per warp (every lane every echo: 25 % slower).
    constexpr bool FAST = MORTON && SPE > 0 && !SENS && !WF;
    // the collision replay at one or two steps per echo, for the plain and the sensitivity walks, Morton
    // or bit-block steps (at three the per-echo work is shared by three steps: the fast loop below
    // measured faster for the plain walk, and the per-echo reductions as fast for the sensitivity walk)
    constexpr bool REPLAY = SPE > 0 && SPE <= 2 && !WF && (SENS || NP == 1 || PACK);
    constexpr int NE = SPE > 0 ? 32 / SPE : 1;          // REPLAY: echoes per window (n SPE <= 32 steps)
    constexpr int NB = NP == 1 ? 0 : (NP == 2 ? 1 : 2); // REPLAY: phase bit-planes of a window's collisions
    constexpr int KC = PACK ? 4 : K;                    // REPLAY: per-echo counters (PACK: one count word)
    constexpr int NW = kWalkThreads / 32;
    constexpr int KF = (KC + NW - 1) / NW; // counters flushed per warp
    bool done = false;
    if constexpr (REPLAY)
    {
        if (__syncthreads_and(active))
        {
            done = true;
            // During a window of n <= NE echoes (n SPE <= 32 steps) a lane only shifts its collisions
            // into bit masks: step k of the window is bit n SPE - 1 - k of m, and of mb[0..NB) the bits of
            // the colliding phase. After the window the warp replays its collisions, spread evenly over
            // its lanes (walkers in narrow pores collide far more often than the average 2 per window),
            // and adds each one's change of the walker's three energy limbs (SENS: and of the four
            // limbs of each E c_q), and the collision, into the window's per-echo counters dsum (shared
            // 32-bit atomics). The flush turns the changes into the CTA's sums after each echo with a
            // prefix sum over the window, starting from the sums after the previous window. A CTA's
            // limb sums stay below 2^32 (256 lanes x 2^24), so the 32-bit modular arithmetic is exact
            // and the global counters receive the same integers as from per-echo warp reductions.
            __shared__ uint32_t dsum[2][32][KC]; // [buffer][echo of the window][counter]
            __shared__ uint32_t lsum0[NW][3 + KS];
            const int wp = threadIdx.x >> 5;
            // level counters (energy limbs; SENS: limbs of E c_q) carry the CTA's sums from window to
            // window; the collision counters are per echo
            auto is_level = [](int col) { return col < 3 || col >= 3 + NG; };
            uint32_t lk[KF]; // the CTA's sums of this warp's level counters after the last flushed echo
            {
                const uint64_t es = energy_fx<NP>(L.tfx, L.tstride, c);
                uint32_t r[3 + KS];
                r[0] = __reduce_add_sync(FULL, (uint32_t)(es & M21));
                r[1] = __reduce_add_sync(FULL, (uint32_t)((es >> 21) & M21));
                r[2] = __reduce_add_sync(FULL, (uint32_t)(es >> 42));
                if constexpr (SENS)
                {
#pragma unroll
                    for (int q = 0; q < NP; q++)
                    {
                        uint32_t l[4];
                        product_limbs24(es, c[q], l);
#pragma unroll
                        for (int k = 0; k < 4; k++) r[3 + 4 * q + k] = __reduce_add_sync(FULL, l[k]);
                    }
                }
                if (lane == 0)
#pragma unroll
                    for (int k = 0; k < 3 + KS; k++) lsum0[wp][k] = r[k];
                for (int k = threadIdx.x; k < 2 * 32 * KC; k += blockDim.x) (&dsum[0][0][0])[k] = 0;
                __syncthreads();
#pragma unroll
                for (int t = 0; t < KF; t++)
                {
                    const int col = wp + t * NW;
                    lk[t] = 0;
                    if (col < KC && is_level(col))
                        for (int w = 0; w < NW; w++) lk[t] += lsum0[w][col < 3 ? col : col - NG];
                }
            }
            int buf = 0;
            for (int e0 = L.e_begin; e0 < L.e_end; e0 += NE)
            {
                const int n = min(NE, L.e_end - e0);
                uint32_t m = 0, mb[NB > 0 ? NB : 1];
#pragma unroll
                for (int k = 0; k < NB; k++) mb[k] = 0;
#pragma unroll(SPE == 1 ? (SENS ? 8 : 16) : 4)
                for (int j = 0; j < n; j++)
                {
#pragma unroll
                    for (int s = 0; s < SPE; s++)
                    {
                        bool wall;
                        int ph;
                        if constexpr (MORTON)
                            morton_step<W>(im.mi, sdir, P, seed, wall, ph);
                        else
                            walker_step<BC, W>(im, p, seed, wall, ph);
                        m = 2 * m + (wall ? 1u : 0u);
#pragma unroll
                        // the Morton copy holds phase bits only at solid voxels, so there a phase bit
                        // implies the collision; the bit-blocks may come from the caller
                        for (int k = 0; k < NB; k++)
                            mb[k] = 2 * mb[k] + ((MORTON || wall) ? ((uint32_t)ph >> k & 1u) : 0u);
                    }
                }
                // the warp's collisions of the window, spread evenly over its lanes: lane l takes
                // collisions 32 r + l in (lane, echo) order; the owner lane and the collision's bit
                // come from binary searches, its counts before and after from popcounts
                m <<= 32 - n * SPE; // step k of the window at bit 31 - k
#pragma unroll
                for (int k = 0; k < NB; k++) mb[k] <<= 32 - n * SPE;
                const uint32_t kc = __popc(m);
                uint32_t pre = kc; // inclusive prefix over lanes
#pragma unroll
                for (int o = 1; o < 32; o <<= 1)
                {
                    const uint32_t t = __shfl_up_sync(FULL, pre, o);
                    if (lane >= o) pre += t;
                }
                const uint32_t total = __shfl_sync(FULL, pre, 31);
                pre -= kc; // exclusive
                for (uint32_t base = 0; base < total; base += 32)
                {
                    const uint32_t ix = base + lane;
                    int o = 0; // the last lane whose first collision index is <= ix
#pragma unroll
                    for (int st2 = 16; st2 >= 1; st2 >>= 1)
                        if (__shfl_sync(FULL, pre, o + st2) <= ix) o += st2;
                    const uint32_t mo = __shfl_sync(FULL, m, o);
                    uint32_t mbo[NB > 0 ? NB : 1], co[NP];
#pragma unroll
                    for (int k = 0; k < NB; k++) mbo[k] = __shfl_sync(FULL, mb[k], o);
#pragma unroll
                    for (int q = 0; q < NP; q++) co[q] = __shfl_sync(FULL, c[q], o);
                    const uint32_t qr = ix - __shfl_sync(FULL, pre, o); // collisions of lane o before this one
                    if (ix < total)
                    {
                        int b = 0; // bit of the collision: the last b with more than qr bits of mo at >= b
#pragma unroll
                        for (int st2 = 16; st2 >= 1; st2 >>= 1)
                            if ((uint32_t)__popc(mo >> (b + st2)) > qr) b += st2;
                        const int jj = SPE == 1 ? 31 - b : (31 - b) / SPE; // the collision's echo
                        // the collision's phase and the walker's counts before it
                        uint32_t ph = 0, cb[NP];
                        if constexpr (NB == 0)
                            cb[0] = co[0] + qr;
                        else if constexpr (NB == 1)
                        {
                            const uint32_t n1 = __popc((mbo[0] >> b) >> 1); // phase-1 collisions before
                            ph = (mbo[0] >> b) & 1u;
                            cb[0] = co[0] + (qr - n1);
                            cb[1] = co[1] + n1;
                        }
                        else
                        {
                            const uint32_t a0 = (mbo[0] >> b) >> 1, a1 = (mbo[1] >> b) >> 1;
                            const uint32_t nq[4] = {0u, (uint32_t)__popc(a0 & ~a1), (uint32_t)__popc(a1 & ~a0),
                                                    (uint32_t)__popc(a0 & a1)};
                            ph = ((mbo[0] >> b) & 1u) | (((mbo[1] >> b) & 1u) << 1);
                            cb[0] = co[0] + (qr - nq[1] - nq[2] - nq[3]);
#pragma unroll
                            for (int q = 1; q < NP; q++) cb[q] = co[q] + nq[q];
                        }
                        // energies before and after: the tables' product in energy_fx's order, the
                        // colliding phase's entry advanced by one
                        uint64_t t[NP];
                        uint32_t cph = cb[0];
#pragma unroll
                        for (int q = 0; q < NP; q++)
                        {
                            t[q] = __ldg(L.tfx + (size_t)q * L.tstride + cb[q]);
                            if (q > 0 && ph == (uint32_t)q) cph = cb[q];
                        }
                        const uint64_t tx = __ldg(L.tfx + (size_t)ph * L.tstride + cph + 1);
                        uint64_t eo = t[0], en = ph == 0 ? tx : t[0];
#pragma unroll
                        for (int q = 1; q < NP; q++)
                        {
                            eo = fx_mul(eo, t[q]);
                            en = fx_mul(en, ph == (uint32_t)q ? tx : t[q]);
                        }
                        uint32_t *d = dsum[buf][jj];
                        atomicAdd(d + 0, (uint32_t)(en & M21) - (uint32_t)(eo & M21));
                        atomicAdd(d + 1, (uint32_t)((en >> 21) & M21) - (uint32_t)((eo >> 21) & M21));
                        atomicAdd(d + 2, (uint32_t)(en >> 42) - (uint32_t)(eo >> 42));
                        if (PACK) atomicAdd(d + 3, 1u << (16 * ph));
                        else atomicAdd(d + 3 + ph, 1u);
                        if constexpr (SENS)
                        {
#pragma unroll
                            for (int q = 0; q < NP; q++)
                            {
                                uint32_t lo4[4], ln4[4];
                                product_limbs24(eo, cb[q], lo4);
                                product_limbs24(en, cb[q] + (ph == (uint32_t)q ? 1u : 0u), ln4);
#pragma unroll
                                for (int k = 0; k < 4; k++) atomicAdd(d + 3 + NP + 4 * q + k, ln4[k] - lo4[k]);
                            }
                        }
                    }
                }
                if constexpr (NB == 0)
                    c[0] += kc;
                else if constexpr (NB == 1)
                {
                    const uint32_t k1 = __popc(mb[0]);
                    c[0] += kc - k1;
                    c[1] += k1;
                }
                else
                {
                    const uint32_t nq[4] = {0u, (uint32_t)__popc(mb[0] & ~mb[1]), (uint32_t)__popc(mb[1] & ~mb[0]),
                                            (uint32_t)__popc(mb[0] & mb[1])};
                    c[0] += kc - nq[1] - nq[2] - nq[3];
#pragma unroll
                    for (int q = 1; q < NP; q++) c[q] += nq[q];
                }
                // every replay of this window is in dsum[buf]; the next window writes the other buffer,
                // which the flush of the previous window emptied before this barrier
                __syncthreads();
#pragma unroll
                for (int t = 0; t < KF; t++)
                {
                    const int col = wp + t * NW; // warp-uniform
                    if (col < KC)
                    {
                        uint32_t v = dsum[buf][lane][col];
                        dsum[buf][lane][col] = 0;
                        unsigned long long *a = L.acc + (size_t)(e0 + 1 + lane) * K;
                        if (is_level(col))
                        {
#pragma unroll
                            for (int o = 1; o < 32; o <<= 1)
                            {
                                const uint32_t u = __shfl_up_sync(FULL, v, o);
                                if (lane >= o) v += u;
                            }
                            v += lk[t];
                            lk[t] = __shfl_sync(FULL, v, 31);
                            if (lane < n && v) atomicAdd(a + col, (unsigned long long)v);
                        }
                        else if (lane < n && v)
                        {
                            if (PACK)
                            {
                                if (v & 0xffffu) atomicAdd(a + 3, (unsigned long long)(v & 0xffffu));
                                if (v >> 16) atomicAdd(a + 4, (unsigned long long)(v >> 16));
                            }
                            else
                                atomicAdd(a + col, (unsigned long long)v);
                        }
                    }
                }
                buf ^= 1;
            }
        }
    }
    else if constexpr (FAST)
    {
        if (__syncthreads_and(active))
        {
            done = true;
            for (int e0 = L.e_begin; e0 < L.e_end; e0 += 32)
            {
                const int e1 = min(e0 + 32, L.e_end);
#pragma unroll(SPE == 1 ? 8 : 4)
                for (int e = e0; e < e1; e++)
                {
                    uint32_t g[NG];
#pragma unroll
                    for (int k = 0; k < NG; k++) g[k] = 0;
#pragma unroll
                    for (int s = 0; s < SPE; s++)
                    {
                        bool wall;
                        int ph;
                        morton_step<W>(im.mi, sdir, P, seed, wall, ph);
                        // Morton copy: a phase bit implies the collision, so phase 1 adds 1 + 0xffff
                        if (PACK) g[0] += MORTON ? (wall ? 1u : 0u) + (uint32_t)ph * 0xffffu : (wall ? 1u : 0u) << (ph << 4);
                        else
                        {
#pragma unroll
                            for (int q = 0; q < NP; q++) g[q] += (wall && ph == q) ? 1u : 0u;
                        }
                    }
                    bool changed = false;
                    if (PACK)
                    {
                        c[0] += g[0] & 0xffffu;
                        c[1] += g[0] >> 16;
                        changed = g[0] != 0;
                    }
                    else
                    {
#pragma unroll
                        for (int q = 0; q < NP; q++)
                        {
                            c[q] += g[q];
                            changed |= g[q] != 0;
                        }
                    }
                    if (changed) efx = energy_fx<NP>(L.tfx, L.tstride, c);
                    uint32_t r[KP];
                    r[0] = __reduce_add_sync(FULL, (uint32_t)(efx & M21));
                    r[1] = __reduce_add_sync(FULL, (uint32_t)((efx >> 21) & M21));
                    r[2] = __reduce_add_sync(FULL, (uint32_t)(efx >> 42));
#pragma unroll
                    for (int k = 0; k < NG; k++) r[3 + k] = __reduce_add_sync(FULL, g[k]);
#pragma unroll
                    for (int k = 3 + NG; k < KP; k++) r[k] = 0;
                    if (lane == 0)
                    {
                        uint4 *slot = reinterpret_cast<uint4 *>(&wsum[threadIdx.x >> 5][e - e0][0]);
#pragma unroll
                        for (int v = 0; v < KP / 4; v++)
                            slot[v] = make_uint4(r[4 * v], r[4 * v + 1], r[4 * v + 2], r[4 * v + 3]);
                    }
                }
                __syncthreads();
                for (int k = threadIdx.x; k < (e1 - e0) * K; k += blockDim.x)
                {
                    const int er = k / K, kk = k % K;
                    unsigned long long v = 0;
#pragma unroll
                    for (int w = 0; w < kWalkThreads / 32; w++)
                    {
                        const uint32_t x = kk < 3 ? wsum[w][er][kk]
                                                  : (PACK ? (wsum[w][er][3] >> (16 * (kk - 3))) & 0xffffu : wsum[w][er][kk]);
                        v += x;
                    }
                    if (v) atomicAdd(&L.acc[(size_t)(e0 + 1 + er) * K + kk], v);
                }
                __syncthreads();
            }
        }
    }

    // the general echo loop
    if (!done)
    {
        for (int e0 = L.e_begin; e0 < L.e_end; e0 += 32)
        {
            const int e1 = min(e0 + 32, L.e_end);
            for (int e = e0; e < e1; e++)
            {
                uint32_t g[NG]; // collisions gained this echo, per phase (PACK: 16 bits per phase)
#pragma unroll
                for (int k = 0; k < NG; k++) g[k] = 0;
                if (active)
                {
                    const int spe = SPE ? SPE : L.steps_per_echo;
#pragma unroll(SPE ? SPE : 4)
                    for (int s = 0; s < spe; s++)
                    {
                        bool wall;
                        int ph;
                        if (MORTON)
                            morton_step<W>(im.mi, sdir, P, seed, wall, ph);
                        else
                            walker_step<BC, W>(im, p, seed, wall, ph);
                        // Morton copy: a phase bit implies the collision, so phase 1 adds 1 + 0xffff
                        if (PACK) g[0] += MORTON ? (wall ? 1u : 0u) + (uint32_t)ph * 0xffffu : (wall ? 1u : 0u) << (ph << 4);
                        else
                        {
#pragma unroll
                            for (int q = 0; q < NP; q++) g[q] += (wall && ph == q) ? 1u : 0u;
                        }
                    }
                    bool changed = false;
                    if (PACK)
                    {
                        c[0] += g[0] & 0xffffu;
                        c[1] += g[0] >> 16;
                        changed = g[0] != 0;
                    }
                    else
                    {
#pragma unroll
                        for (int q = 0; q < NP; q++)
                        {
                            c[q] += g[q];
                            changed |= g[q] != 0;
                        }
                    }
                    if (changed && rec)
                    {
                        if (WF)
                        {
                            for (uint32_t k = 0; k < g[0]; k++) ew = ew * fw;
                            efx = walker_fx(ew);
                        }
                        else
                        {
                            efx = energy_fx<NP>(L.tfx, L.tstride, c);
                        }
                    }
                }
                if (rec)
                {
                    uint32_t r[KP];
                    r[0] = __reduce_add_sync(FULL, (uint32_t)(efx & M21));
                    r[1] = __reduce_add_sync(FULL, (uint32_t)((efx >> 21) & M21));
                    r[2] = __reduce_add_sync(FULL, (uint32_t)(efx >> 42));
#pragma unroll
                    for (int k = 0; k < NG; k++) r[3 + k] = __reduce_add_sync(FULL, g[k]);
                    if (SENS)
                    {
                        constexpr uint32_t M24 = (1u << 24) - 1;
#pragma unroll
                        for (int q = 0; q < NP; q++)
                        {
                            const uint64_t lo = efx * (uint64_t)c[q];                     // bits 0-63 of E c_q
                            const uint32_t hi = (uint32_t)__umul64hi(efx, (uint64_t)c[q]); // bits 64-95
                            uint32_t *rq = r + 3 + NG + 4 * q;
                            rq[0] = __reduce_add_sync(FULL, (uint32_t)lo & M24);
                            rq[1] = __reduce_add_sync(FULL, (uint32_t)(lo >> 24) & M24);
                            rq[2] = __reduce_add_sync(FULL, ((uint32_t)(lo >> 48) | (hi << 16)) & M24);
                            rq[3] = __reduce_add_sync(FULL, hi >> 8);
                        }
                    }
#pragma unroll
                    for (int k = 3 + NG + KS; k < KP; k++) r[k] = 0;
                    if (lane == 0)
                    {
                        uint4 *slot = reinterpret_cast<uint4 *>(&wsum[threadIdx.x >> 5][e - e0][0]);
#pragma unroll
                        for (int v = 0; v < KP / 4; v++) slot[v] = make_uint4(r[4 * v], r[4 * v + 1], r[4 * v + 2], r[4 * v + 3]);
                    }
                }
            }
            if (rec)
            {
                __syncthreads();
                for (int k = threadIdx.x; k < (e1 - e0) * K; k += blockDim.x)
                {
                    const int er = k / K, kk = k % K;
                    unsigned long long v = 0;
#pragma unroll
                    for (int w = 0; w < kWalkThreads / 32; w++)
                    {
                        const uint32_t x = kk < 3 ? wsum[w][er][kk]
                                                  : (PACK ? (wsum[w][er][3] >> (16 * (kk - 3))) & 0xffffu : wsum[w][er][kk]);
                        v += x;
                    }
                    if (v) atomicAdd(&L.acc[(size_t)(e0 + 1 + er) * K + kk], v);
                }
                __syncthreads();
            }
        }
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
        if (WF) L.wenergy[i] = ew;
    }
}

// ---------------------------------------------------------------------------------------------
// Seed-replay adjoint of the CPMG echo sums with respect to the per-phase decrease factors.
// A walker's energy is E = prod_q f_q^c_q, so dE/df_q = c_q f_q^(c_q - 1) prod_{r != q} f_r^c_r.
// L.t holds [2][NP][tstride]: the energy tables f^k, then the derivative tables k f^(k-1). Each
// walker replays its trajectory from its stored seed and accumulates sum_e g[e] dE(e)/df_q in FP64
// (a few multiply-adds per walker-echo, no cross-lane FP64), then reduces once at the end.
// partial: [gridDim.x][NP], summed on the host in block order (deterministic).
// MORTON (noflux, no voxel division): the replay steps on the image's Morton copy.
// This direct form serves decrease factors that include zero; with every f_q > 0 the host takes the
// gradient from the forward walk's exact sensitivity sums instead (cpmg_walk_kernel, SENS).
template <int BC, int NP, bool MORTON = false>
__global__ void __launch_bounds__(kWalkThreads) cpmg_adjoint_kernel(DevImage im, WalkState st, AdjointLaunch L)
{
    static_assert(!MORTON || BC == BC_NOFLUX, "the Morton walk is the noflux walk");
    constexpr int W = WordsPerBlock<NP>::value;
    __shared__ double sred[kWalkThreads / 32][NP];
    __shared__ uint4 sdir[6]; // MORTON: direction table
    if (MORTON && threadIdx.x < 6) sdir[threadIdx.x] = morton_direction(im.mi, threadIdx.x);
    if (MORTON) __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool active = i < st.n;
    WalkerPos p{};
    uint64_t seed = 0;
    uint32_t c[NP];
    double acc[NP];
#pragma unroll
    for (int q = 0; q < NP; q++)
    {
        c[q] = 0;
        acc[q] = 0.0;
    }
    if (active)
    {
        p.x = st.x0[i];
        p.y = st.y0[i];
        p.z = st.z0[i];
        seed = st.seed0[i];
        if (!start_ok<BC>(im, p))
        {
            atomicOr(L.status, kStatusBadStart);
            active = false;
        }
        init_image_coords<BC>(im, p);
    }
    uint32_t P = 0; // MORTON: Morton index of the position
    if (MORTON && active)
        P = dilate_bits((uint32_t)p.x, im.mi.mx) | dilate_bits((uint32_t)p.y, im.mi.my) | dilate_bits((uint32_t)p.z, im.mi.mz);
    if (active)
    {
        const double *T = L.t;
        const double *dT = L.t + (size_t)NP * L.tstride;
        for (int e = 0; e < L.n_echoes; e++)
        {
            for (int s = 0; s < L.steps_per_echo; s++)
            {
                bool wall;
                int ph;
                if (MORTON)
                    morton_step<W>(im.mi, sdir, P, seed, wall, ph);
                else
                    walker_step<BC, W>(im, p, seed, wall, ph);
#pragma unroll
                for (int q = 0; q < NP; q++) c[q] += (wall && ph == q) ? 1u : 0u;
            }
            const double g = __ldg(L.grad + e + 1);
            if (g != 0.0)
            {
                double tv[NP], dv[NP];
#pragma unroll
                for (int q = 0; q < NP; q++)
                {
                    tv[q] = __ldg(T + (size_t)q * L.tstride + c[q]);
                    dv[q] = __ldg(dT + (size_t)q * L.tstride + c[q]);
                }
#pragma unroll
                for (int q = 0; q < NP; q++)
                {
                    double term = dv[q];
#pragma unroll
                    for (int r = 0; r < NP; r++)
                        if (r != q) term *= tv[r];
                    acc[q] = fma(g, term, acc[q]);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < NP; q++)
    {
        double v = acc[q];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
        if (lane == 0) sred[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < NP)
    {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += sred[w][threadIdx.x];
        L.partial[(size_t)blockIdx.x * NP + threadIdx.x] = v;
    }
}

// ---------------------------------------------------------------------------------------------
// PFGSE walk: walkers walk cumulatively to each exposure time. At each one the kernel adds
//   * the exact fixed-point energy sum (3 limbs) and the integer squared displacements per axis;
//   * for a gradient along one axis (the usual case), each walker's fixed-point energy into a
//     displacement histogram H_i[d] (two 32-bit-split limbs per bin), so the phase sums
//     M_ij = sum_d H_i[d] cos(k_j d res) need one cosine per distinct displacement rather than
//     one per walker (pfgse_phase_kernel);
//   * for any other gradient direction, each walker's displacement and FP64 energy, measured by
//     pfgse_direct_kernel.
// WF: per-walker decrease factors, energies as FP64 repeated products (see cpmg_walk_kernel).
// MORTON (noflux, no voxel division): steps on the image's Morton copy (see cpmg_walk_kernel); the
// position is converted back to x, y, z at each exposure time.
template <int BC, int NP, bool WF, bool MORTON = false>
__global__ void __launch_bounds__(kWalkThreads) pfgse_walk_kernel(DevImage im, WalkState st, PfgseLaunch L)
{
    static_assert(!WF || NP == 1, "per-walker decrease factors are for single-phase images");
    static_assert(!MORTON || BC == BC_NOFLUX, "the Morton walk is the noflux walk");
    constexpr int W = WordsPerBlock<NP>::value;
    __shared__ uint4 sdir[6]; // MORTON: direction table
    if (MORTON && threadIdx.x < 6) sdir[threadIdx.x] = morton_direction(im.mi, threadIdx.x);
    if (MORTON) __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool active = i < st.n;
    WalkerPos p{};
    uint64_t seed = 0;
    int x0 = 0, y0 = 0, z0 = 0;
    uint32_t c[NP];
#pragma unroll
    for (int q = 0; q < NP; q++) c[q] = 0;
    if (active)
    {
        x0 = st.x0[i];
        y0 = st.y0[i];
        z0 = st.z0[i];
        p.x = x0;
        p.y = y0;
        p.z = z0;
        seed = st.seed0[i];
        if (!start_ok<BC>(im, p))
        {
            atomicOr(L.status, kStatusBadStart);
            active = false;
        }
        init_image_coords<BC>(im, p);
    }
    const double fw = (WF && active) ? L.wf[i] : 1.0;
    double ew = 1.0;
    uint32_t c_done = 0; // WF: collisions already folded into ew
    uint32_t P = 0;      // MORTON: Morton index of the position
    if (MORTON && active)
        P = dilate_bits((uint32_t)p.x, im.mi.mx) | dilate_bits((uint32_t)p.y, im.mi.my) | dilate_bits((uint32_t)p.z, im.mi.mz);
    int done = 0;
    for (int d = 0; d < L.n_delta; d++)
    {
        const int target = L.steps[d];
        if (active)
        {
#pragma unroll 4
            for (; done < target; done++)
            {
                bool wall;
                int ph;
                if (MORTON)
                    morton_step<W>(im.mi, sdir, P, seed, wall, ph);
                else
                    walker_step<BC, W>(im, p, seed, wall, ph);
#pragma unroll
                for (int q = 0; q < NP; q++) c[q] += (wall && ph == q) ? 1u : 0u;
            }
            if (MORTON)
            {
                p.x = (int)undilate_bits(P, im.mi.mx);
                p.y = (int)undilate_bits(P, im.mi.my);
                p.z = (int)undilate_bits(P, im.mi.mz);
            }
        }
        if (WF)
        {
            for (; c_done < c[0]; c_done++) ew = ew * fw;
        }
        uint64_t efx = 0;
        if (active) efx = WF ? walker_fx(ew) : energy_fx<NP>(L.tfx, L.tstride, c);
        const int ddx = p.x - x0, ddy = p.y - y0, ddz = p.z - z0;
        unsigned long long *acc = L.acc + (size_t)d * 6;
        uint32_t r;
        r = __reduce_add_sync(FULL, (uint32_t)(efx & M21));
        if (lane == 0 && r) atomicAdd(&acc[0], (unsigned long long)r);
        r = __reduce_add_sync(FULL, (uint32_t)((efx >> 21) & M21));
        if (lane == 0 && r) atomicAdd(&acc[1], (unsigned long long)r);
        r = __reduce_add_sync(FULL, (uint32_t)(efx >> 42));
        if (lane == 0 && r) atomicAdd(&acc[2], (unsigned long long)r);
        // squared displacements: |d| <= steps, so split at 16 bits to keep redux sums in 32 bits
        const int dd[3] = {ddx, ddy, ddz};
#pragma unroll
        for (int a = 0; a < 3; a++)
        {
            uint64_t sq = active ? (uint64_t)((int64_t)dd[a] * dd[a]) : 0ull;
            uint32_t lo = __reduce_add_sync(FULL, (uint32_t)(sq & 0xffffull));
            uint32_t hi = __reduce_add_sync(FULL, (uint32_t)(sq >> 16));
            if (lane == 0 && (lo | hi)) atomicAdd(&acc[3 + a], (unsigned long long)lo + ((unsigned long long)hi << 16));
        }
        if (active)
        {
            if (L.axis >= 0)
            {
                const int dv = L.axis == 0 ? ddx : (L.axis == 1 ? ddy : ddz);
                const int bin = dv + L.hist_half;
                if ((unsigned)bin < (unsigned)(2 * L.hist_half + 1))
                {
                    unsigned long long *h = L.hist + ((size_t)d * (2 * L.hist_half + 1) + bin) * 2;
                    atomicAdd(&h[0], (unsigned long long)(efx & 0xffffffffull));
                    atomicAdd(&h[1], (unsigned long long)(efx >> 32));
                }
                else
                {
                    atomicOr(L.status, kStatusHistRange);
                }
            }
            else
            {
                const size_t o = (size_t)d * st.n + i;
                L.disp[o * 3 + 0] = ddx;
                L.disp[o * 3 + 1] = ddy;
                L.disp[o * 3 + 2] = ddz;
                L.energy[o] = WF ? ew : energy_fp64<NP>(L.t, L.tstride, c);
            }
        }
    }
    if (active)
    {
        st.x[i] = p.x;
        st.y[i] = p.y;
        st.z[i] = p.z;
        st.seed[i] = seed;
#pragma unroll
        for (int q = 0; q < NP; q++) st.coll[(size_t)q * st.n + i] = c[q];
    }
}

// M[i][j] (and optionally dM/dg) from the displacement histograms; one block per (i, j), bins in a
// fixed order, so the result is deterministic.
__global__ void pfgse_phase_kernel(PhaseLaunch L)
{
    const int i = blockIdx.y, j = blockIdx.x;
    const int nb = 2 * L.hist_half + 1;
    const double k = L.kaxis[j];
    const unsigned long long *h = L.hist + (size_t)i * nb * 2;
    double s = 0.0, g = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
    {
        const unsigned long long lo = h[2 * b], hi = h[2 * b + 1];
        if ((lo | hi) == 0) continue;
        // exact value hi * 2^32 + lo, scaled by 2^-63
        const double e = ((double)hi * 4294967296.0 + (double)lo) * 1.0842021724855044e-19;
        const double dd = (double)(b - L.hist_half);
        const double arg = (k * dd) * L.res;
        double sn, cs;
        sincos(arg, &sn, &cs);
        s += e * cs;
        if (L.dMdg) g -= e * sn * (L.kscale_axis * dd * L.res);
    }
    __shared__ double red[2][256];
    red[0][threadIdx.x] = s;
    red[1][threadIdx.x] = g;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1)
    {
        if (threadIdx.x < o)
        {
            red[0][threadIdx.x] += red[0][threadIdx.x + o];
            red[1][threadIdx.x] += red[1][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        L.M[(size_t)i * gridDim.x + j] = red[0][0];
        if (L.dMdg) L.dMdg[(size_t)i * gridDim.x + j] = red[1][0];
    }
}

// PFGSE phase sums for a general gradient direction: M_ij = sum_w E_w cos(k_j . dR_w res) for every
// walker w (its displacement dR and energy at exposure time i, stored by the walk), and with grad_on
// dM_ij/dg = -sum_w E_w sin(k_j . dR_w res) kscale (dir . dR_w) res. The angle is formed in turns from
// the host's kappa_ja = k_ja res / (2 pi) mod 1 (2^-64 turns): theta = sum_a dR_a kappa_ja modulo one
// turn, exact integer arithmetic with no reduction step; cos and sin come from the fixed-point
// cosine (fixed_cos.cuh). Each walker adds E cos * 2^61 + 2^61 (E as round(E 2^63)), summed exactly as
// three 21-bit limbs through redux.sync; lane l keeps the sums of gradient points j = 32 s + l. The
// gradient sums stay FP64 (E sin times the walker's projection), reduced in a fixed order.
// grid (blocks, n_delta) x 256 threads; each warp takes 32 walkers at a time.
__global__ void __launch_bounds__(256) pfgse_direct_kernel(DirectLaunch L)
{
    __shared__ ulonglong2 quad[fxcos::kQuadrant];
    __shared__ uint64_t skap[kDirectMaxG][3];
    __shared__ unsigned long long sacc[kDirectMaxG][3];
    __shared__ double sgw[8][kDirectMaxG];
    fxcos::load_quadrant_table(quad);
    const int ng = L.n_g;
    for (int k = threadIdx.x; k < ng * 3; k += blockDim.x)
    {
        skap[k / 3][k % 3] = L.kappa[k];
        sacc[k / 3][k % 3] = 0;
    }
    __syncthreads();
    const int i = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int NS = kDirectMaxG / 32;
    unsigned long long acc[NS][3];
    double gacc[NS];
#pragma unroll
    for (int s = 0; s < NS; s++)
    {
        acc[s][0] = acc[s][1] = acc[s][2] = 0;
        gacc[s] = 0.0;
    }
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + warp * 32; base < L.n; base += stride)
    {
        const int64_t w = base + lane;
        const bool active = w < L.n;
        int32_t d0 = 0, d1 = 0, d2 = 0;
        uint64_t e63 = 0;
        double pr = 0.0; // grad_on: kscale (dir . dR) res 2^-61
        if (active)
        {
            const size_t o = (size_t)i * L.n + w;
            d0 = L.disp[o * 3 + 0];
            d1 = L.disp[o * 3 + 1];
            d2 = L.disp[o * 3 + 2];
            e63 = fxcos::prob_q63(L.energy[o]);
            if (L.grad_on)
                pr = L.kscale * (L.dir[0] * (double)d0 + L.dir[1] * (double)d1 + L.dir[2] * (double)d2) * L.res *
                     0x1p-61;
        }
#pragma unroll
        for (int s = 0; s < NS; s++)
        {
            for (int jj = 0; jj < 32; jj++)
            {
                const int j = 32 * s + jj;
                if (j >= ng) break;
                const uint64_t theta = (uint64_t)(int64_t)d0 * skap[j][0] + (uint64_t)(int64_t)d1 * skap[j][1] +
                                       (uint64_t)(int64_t)d2 * skap[j][2];
                long long c62, s62 = 0;
                if (L.grad_on)
                    fxcos::sincos_turns_q62(theta, 0, quad, c62, s62);
                else
                    c62 = fxcos::cos_turns_q62(theta, 0, quad);
                const uint64_t m = __umul64hi(e63, (uint64_t)(c62 < 0 ? -c62 : c62)); // E |cos| 2^61
                const uint64_t u = active ? (uint64_t)((c62 < 0 ? -(long long)m : (long long)m) + (1ll << 61)) : 0;
                const uint32_t r0 = __reduce_add_sync(FULL, (uint32_t)(u & M21));
                const uint32_t r1 = __reduce_add_sync(FULL, (uint32_t)((u >> 21) & M21));
                const uint32_t r2 = __reduce_add_sync(FULL, (uint32_t)(u >> 42));
                if (lane == jj)
                {
                    acc[s][0] += r0;
                    acc[s][1] += r1;
                    acc[s][2] += r2;
                }
                if (L.grad_on)
                {
                    const uint64_t ms = __umul64hi(e63, (uint64_t)(s62 < 0 ? -s62 : s62)); // E |sin| 2^61
                    double v = -(double)(s62 < 0 ? -(long long)ms : (long long)ms) * pr;
                    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
                    v = __shfl_sync(FULL, v, 0);
                    if (lane == jj) gacc[s] += v;
                }
            }
        }
    }
#pragma unroll
    for (int s = 0; s < NS; s++)
    {
        const int j = 32 * s + lane;
        if (j < ng)
        {
            atomicAdd(&sacc[j][0], acc[s][0]);
            atomicAdd(&sacc[j][1], acc[s][1]);
            atomicAdd(&sacc[j][2], acc[s][2]);
            sgw[warp][j] = gacc[s];
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < ng * 3; k += blockDim.x)
        L.partial[(((size_t)i * ng + k / 3) * gridDim.x + blockIdx.x) * 3 + k % 3] = sacc[k / 3][k % 3];
    if (L.grad_on)
        for (int j = threadIdx.x; j < ng; j += blockDim.x)
        {
            double v = 0.0;
            for (int wv = 0; wv < 8; wv++) v += sgw[wv][j];
            L.partial_g[((size_t)i * ng + j) * gridDim.x + blockIdx.x] = v;
        }
}

// Packs a label volume into bit-blocks with phase planes (BitBlock/bitBlock.cpp:138-221 plus the
// multi-phase extension). One thread per block; voxels beyond the image edge stay pore.
__global__ void pack_blocks_kernel(const uint8_t *__restrict__ labels, int nx, int ny, int nz, int bcols, int brows,
                                   int64_t nblocks, int words, int n_phases, uint64_t *__restrict__ out,
                                   unsigned *status)
{
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblocks) return;
    const int bx = (int)(b % bcols);
    const int by = (int)((b / bcols) % brows);
    const int bz = (int)(b / ((int64_t)bcols * brows));
    uint64_t solid = 0, p0 = 0, p1 = 0, p2 = 0;
    for (int k = 0; k < 64; k++)
    {
        const int x = bx * 4 + (k & 3), y = by * 4 + ((k >> 2) & 3), z = bz * 4 + (k >> 4);
        if (x >= nx || y >= ny || z >= nz) continue;
        const uint8_t l = labels[((int64_t)z * ny + y) * nx + x];
        if (!l) continue;
        solid |= 1ull << k;
        const unsigned ph = (unsigned)l - 1u;
        // multi-phase images: a label must name one of the image's phases (single-phase images treat
        // every non-zero label as solid)
        if (ph >= 8u || (n_phases > 1 && ph >= (unsigned)n_phases)) atomicOr(status, kStatusBadLabel);
        p0 |= (uint64_t)(ph & 1u) << k;
        p1 |= (uint64_t)((ph >> 1) & 1u) << k;
        p2 |= (uint64_t)((ph >> 2) & 1u) << k;
    }
    // half-interleaved layout (see DevImage): the words' low halves, then their high halves
    uint32_t *o = reinterpret_cast<uint32_t *>(out) + b * 2 * words;
    const uint64_t wv[4] = {solid, p0, p1, p2};
    for (int h = 0; h < 2; h++)
        for (int w = 0; w < words; w++) o[h * words + w] = (uint32_t)(wv[w] >> (32 * h));
}

// ---------------------------------------------------------------------------------------------
// Morton copy of an image (see MortonImage): one thread per Morton word gathers its 32 voxels' solid
// and phase bits from the bit-block layout; voxels of the padding beyond the image stay 0 (no walker
// reaches them: noflux walks stay inside).
__global__ void morton_build_kernel(DevImage im, int W, uint32_t n_words, uint32_t *__restrict__ out)
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n_words) return;
    uint32_t acc[4] = {0, 0, 0, 0};
    const uint32_t *base = reinterpret_cast<const uint32_t *>(im.blocks);
    if ((im.mi.mx & 9u) == 9u && (im.mi.my & 18u) == 18u && (im.mi.mz & 4u) == 4u)
    {
        // The five lowest index bits are x0, y0, z0, x1, y1 (the box spans at least 4 x 4 x 2 voxels):
        // word w is then one half (z & 2) of one bit-block -- the 4 x 4 x 2 voxels at its base corner --
        // with its bits reordered from the block's x + 4 y + 16 z to the index's x0 y0 z0 x1 y1.
        const uint32_t P = w << 5;
        const uint32_t x = undilate_bits(P, im.mi.mx), y = undilate_bits(P, im.mi.my), z = undilate_bits(P, im.mi.mz);
        if (x < (uint32_t)im.nx && y < (uint32_t)im.ny && z < (uint32_t)im.nz)
        {
            const uint32_t blk = (x >> 2) + (y >> 2) * (uint32_t)im.bcols + (z >> 2) * (uint32_t)im.bcr;
            const uint32_t *bp = base + (size_t)blk * (2 * W) + ((z >> 1) & 1u) * W;
            for (int k = 0; k < W; k++)
            {
                const uint32_t v = bp[k];
                uint32_t r = 0;
#pragma unroll
                for (uint32_t m = 0; m < 32; m++)
                {
                    const uint32_t src = (m & 1u) | (((m >> 3) & 1u) << 1) | (((m >> 1) & 1u) << 2) |
                                         (((m >> 4) & 1u) << 3) | (((m >> 2) & 1u) << 4);
                    r |= ((v >> src) & 1u) << m;
                }
                acc[k] = r;
            }
        }
        for (int k = 1; k < W; k++) acc[k] &= acc[0]; // phase bits only at solid voxels
        for (int k = 0; k < W; k++) out[(size_t)w * W + k] = acc[k];
        return;
    }
    for (uint32_t b = 0; b < 32; b++)
    {
        const uint32_t P = (w << 5) | b;
        const uint32_t x = undilate_bits(P, im.mi.mx), y = undilate_bits(P, im.mi.my), z = undilate_bits(P, im.mi.mz);
        if (x >= (uint32_t)im.nx || y >= (uint32_t)im.ny || z >= (uint32_t)im.nz) continue;
        const uint32_t blk = (x >> 2) + (y >> 2) * (uint32_t)im.bcols + (z >> 2) * (uint32_t)im.bcr;
        const uint32_t bit = (x & 3) | ((y & 3) << 2) | ((z & 3) << 4);
        const uint32_t *bp = base + (size_t)blk * (2 * W) + (bit >> 5) * W;
        for (int k = 0; k < W; k++) acc[k] |= ((bp[k] >> (bit & 31)) & 1u) << b;
    }
    for (int k = 1; k < W; k++) acc[k] &= acc[0];
    for (int k = 0; k < W; k++) out[(size_t)w * W + k] = acc[k];
}

cudaError_t launch_morton_build(const DevImage &im, int W, uint32_t n_words, uint32_t *out, cudaStream_t s)
{
    morton_build_kernel<<<(n_words + 255) / 256, 256, 0, s>>>(im, W, n_words, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Host-side dispatch over the (boundary condition, phase count) template grid.
namespace
{
template <int NP, typename F>
void with_bc(int bc_key, F &&f)
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

cudaError_t launch_cpmg_walk(int bc_key, int np, const DevImage &im, const WalkState &st, const CpmgLaunch &L,
                             dim3 grid, cudaStream_t s)
{
    auto go = [&](auto npc) {
        constexpr int NP = decltype(npc)::value;
        with_bc<NP>(bc_key, [&](auto bcc) {
            constexpr int BC = decltype(bcc)::value;
            // packed counts: a lane's half-word holds at most steps_per_echo < 2^16 collisions, and a
            // recorded echo's warp sum of a half at most 32 * steps_per_echo < 2^16
            auto run_m = [&](auto spe, auto mort) {
                constexpr int SPE = decltype(spe)::value;
                constexpr bool M = decltype(mort)::value;
                if (L.sens)
                {
                    // sensitivity walks: the Morton instance, or the runtime-bc instance for the rest
                    if constexpr (M)
                        cpmg_walk_kernel<BC, NP, false, false, SPE, true, true><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                    else
                        cpmg_walk_kernel<BC_GENERIC, NP, false, false, 0, false, true><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                    return;
                }
                if constexpr (NP == 1)
                {
                    if (L.wf)
                        cpmg_walk_kernel<BC, 1, false, true, SPE, M><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                    else
                        cpmg_walk_kernel<BC, 1, false, false, SPE, M><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                }
                else if (NP == 2 && L.steps_per_echo <= (L.record ? 2047 : 65535))
                    cpmg_walk_kernel<BC, NP, NP == 2, false, SPE, M><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                else
                    cpmg_walk_kernel<BC, NP, false, false, SPE, M><<<grid, kWalkThreads, 0, s>>>(im, st, L);
            };
            auto run = [&](auto spe) {
                if constexpr (BC == BC_NOFLUX)
                {
                    if (im.mi.words)
                    {
                        run_m(spe, std::true_type{});
                        return;
                    }
                }
                run_m(spe, std::false_type{});
            };
            const int spe = L.record ? L.steps_per_echo : 0;
            if (spe == 1) run(std::integral_constant<int, 1>{});
            else if (spe == 2) run(std::integral_constant<int, 2>{});
            else if (spe == 3) run(std::integral_constant<int, 3>{});
            else run(std::integral_constant<int, 0>{});
        });
    };
    if (np == 1) go(std::integral_constant<int, 1>{});
    else if (np == 2) go(std::integral_constant<int, 2>{});
    else go(std::integral_constant<int, 4>{});
    return cudaGetLastError();
}

cudaError_t launch_cpmg_adjoint(int bc_key, int np, const DevImage &im, const WalkState &st, const AdjointLaunch &L,
                                dim3 grid, cudaStream_t s)
{
    auto go = [&](auto npc) {
        constexpr int NP = decltype(npc)::value;
        with_bc<NP>(bc_key, [&](auto bcc) {
            constexpr int BC = decltype(bcc)::value;
            auto run = [&](auto mort) {
                constexpr bool M = decltype(mort)::value;
                cpmg_adjoint_kernel<BC, NP, M><<<grid, kWalkThreads, 0, s>>>(im, st, L);
            };
            if constexpr (BC == BC_NOFLUX)
            {
                if (im.mi.words)
                {
                    run(std::true_type{});
                    return;
                }
            }
            run(std::false_type{});
        });
    };
    if (np == 1) go(std::integral_constant<int, 1>{});
    else if (np == 2) go(std::integral_constant<int, 2>{});
    else go(std::integral_constant<int, 4>{});
    return cudaGetLastError();
}

cudaError_t launch_pfgse_walk(int bc_key, int np, const DevImage &im, const WalkState &st, const PfgseLaunch &L,
                              dim3 grid, cudaStream_t s)
{
    auto go = [&](auto npc) {
        constexpr int NP = decltype(npc)::value;
        with_bc<NP>(bc_key, [&](auto bcc) {
            constexpr int BC = decltype(bcc)::value;
            auto run = [&](auto mort) {
                constexpr bool M = decltype(mort)::value;
                if constexpr (NP == 1)
                {
                    if (L.wf)
                        pfgse_walk_kernel<BC, 1, true, M><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                    else
                        pfgse_walk_kernel<BC, 1, false, M><<<grid, kWalkThreads, 0, s>>>(im, st, L);
                }
                else
                    pfgse_walk_kernel<BC, NP, false, M><<<grid, kWalkThreads, 0, s>>>(im, st, L);
            };
            if constexpr (BC == BC_NOFLUX)
            {
                if (im.mi.words)
                {
                    run(std::true_type{});
                    return;
                }
            }
            run(std::false_type{});
        });
    };
    if (np == 1) go(std::integral_constant<int, 1>{});
    else if (np == 2) go(std::integral_constant<int, 2>{});
    else go(std::integral_constant<int, 4>{});
    return cudaGetLastError();
}

cudaError_t launch_pfgse_phase(const PhaseLaunch &L, int n_delta, int n_g, cudaStream_t s)
{
    pfgse_phase_kernel<<<dim3(n_g, n_delta), 256, 0, s>>>(L);
    return cudaGetLastError();
}

cudaError_t launch_pfgse_direct(const DirectLaunch &L, int n_delta, int blocks, cudaStream_t s)
{
    pfgse_direct_kernel<<<dim3(blocks, n_delta), 256, 0, s>>>(L);
    return cudaGetLastError();
}

cudaError_t launch_pack_blocks(const uint8_t *labels, int nx, int ny, int nz, int bcols, int brows, int64_t nblocks,
                               int words, int n_phases, uint64_t *out, unsigned *status, cudaStream_t s)
{
    const int t = 256;
    pack_blocks_kernel<<<(unsigned)((nblocks + t - 1) / t), t, 0, s>>>(labels, nx, ny, nz, bcols, brows, nblocks,
                                                                       words, n_phases, out, status);
    return cudaGetLastError();
}

} // namespace rwnmr
