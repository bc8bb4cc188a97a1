// Launch-argument structs and launchers shared by walk_kernels.cu and engine.cu.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "walk_device.cuh"

namespace rwnmr
{

constexpr int kWalkThreads = 256;
constexpr int kDirectMaxG = 128; // gradient points handled by the general-direction PFGSE path

// Device status word bits (the kernels never trap; they report through this word).
constexpr unsigned kStatusBadStart = 1u;  // a walker started outside the image (noflux)
constexpr unsigned kStatusHistRange = 2u; // a displacement fell outside the histogram
constexpr unsigned kStatusBadLabel = 4u;  // a label exceeded the supported phase count
constexpr unsigned kStatusCancelled = 8u; // a persistent batch walk stopped taking work: cancelled
constexpr unsigned kStatusBudget = 16u;   // a persistent batch walk stopped taking work: time budget spent

// Walker state, structure of arrays. coll is [n_phases][n].
struct WalkState
{
    int64_t n;
    const int32_t *__restrict__ x0;
    const int32_t *__restrict__ y0;
    const int32_t *__restrict__ z0;
    const uint64_t *__restrict__ seed0;
    int32_t *x, *y, *z;
    uint64_t *seed;
    uint32_t *coll;
};

struct CpmgLaunch
{
    int e_begin, e_end;    // echoes walked by this launch
    int steps_per_echo;
    int from_initial;      // 1: start from (x0, seed0) with zero collisions; 0: continue (x, seed, coll)
    int record;            // accumulate per-echo sums into acc
    int sens;              // with record and the tables: also the sensitivity sums sum E c_q (4 limbs per phase)
    const uint64_t *tfx;   // [n_phases][tstride] fixed-point energy tables
    int tstride;
    const double *wf;      // per-walker decrease factors [n] (single phase), or null for the tables
    double *wenergy;       // per-walker FP64 energies [n], carried across launches (with wf)
    unsigned long long *acc; // [(n_echoes+1)][3 + NP (+ 4 NP with sens)]
    unsigned *status;
};

struct FieldLaunch
{
    int e_begin, e_end;      // echoes walked by this launch
    int steps_per_inversion; // steps_per_echo / 2
    int from_initial;        // 1: start from (x0, seed0), no collisions, phase 0; 0: continue
    const uint64_t *tfx;     // [n_phases][tstride] survival tables, round(f^n * 2^63)
    int tstride;
    double gammatau;         // 0.5 * gamma * time interval
    const double *field;     // array field [nz][ny][nx]
    double dg;               // uniform field: value per voxel along `axis` (0 in solid voxels)
    const double *btab;      // uniform field: btab[k] = k * dg for the image coordinates k along `axis`
    int axis;
    double *phase;           // [n] walker phases, carried across launches
    const double *wf;        // per-walker decrease factors [n] (single phase), or null for the tables
    double *palive;          // with wf: per-walker survival probabilities [n], carried across launches
    unsigned long long *acc; // [(n_echoes+1)][3] limbs of sum(round(E * 2^61) + 2^61)
    unsigned *status;
};

struct AdjointLaunch
{
    int n_echoes, steps_per_echo;
    const double *t;     // [n_phases][tstride] FP64 energy tables
    int tstride;
    const double *grad;  // [n_echoes + 1]
    double *partial;     // [gridDim.x][NP]
    unsigned *status;
};

struct PfgseLaunch
{
    int n_delta;
    const int32_t *steps;    // device [n_delta]
    const uint64_t *tfx;
    const double *t;
    int tstride;
    unsigned long long *acc; // [n_delta][6]: energy limbs x3, sum dx^2, dy^2, dz^2
    int axis;                // gradient axis 0/1/2, or -1 for the general path
    int hist_half;
    unsigned long long *hist; // [n_delta][2*hist_half+1][2]
    int32_t *disp;            // general path: [n_delta][n][3]
    double *energy;           // general path: [n_delta][n]
    const double *wf;         // per-walker decrease factors [n] (single phase), or null for the tables
    unsigned *status;
};

struct PhaseLaunch
{
    const unsigned long long *hist;
    int hist_half;
    const double *kaxis; // device [n_g]
    double res;
    double kscale_axis;  // dk/dg along the axis (for dM/dg), 0 if unused
    double *M;           // device [n_delta][n_g]
    double *dMdg;        // device [n_delta][n_g] or null
};

struct DirectLaunch
{
    int64_t n;
    int n_g;
    const int32_t *disp;
    const double *energy;
    const uint64_t *kappa; // device [n_g][3]: k_ja res / (2 pi) mod 1, in 2^-64 turns
    double res;
    int grad_on;
    double kscale;
    double dir[3];
    unsigned long long *partial; // [n_delta][n_g][blocks][3]: limbs of sum (E cos 2^61 + 2^61)
    double *partial_g;           // [n_delta][n_g][blocks]
};

cudaError_t launch_cpmg_walk(int bc_key, int np, const DevImage &im, const WalkState &st, const CpmgLaunch &L,
                             dim3 grid, cudaStream_t s);
cudaError_t launch_cpmg_field(int bc_key, int np, bool uniform, const DevImage &im, const WalkState &st,
                              const FieldLaunch &L, dim3 grid, cudaStream_t s);
// btab[k] = (double)k * dg, k < n (the uniform field along one axis, as cpmg_field_kernel evaluates it)
cudaError_t launch_field_table(double dg, int n, double *btab, cudaStream_t s);
cudaError_t launch_cpmg_adjoint(int bc_key, int np, const DevImage &im, const WalkState &st, const AdjointLaunch &L,
                                dim3 grid, cudaStream_t s);
cudaError_t launch_pfgse_walk(int bc_key, int np, const DevImage &im, const WalkState &st, const PfgseLaunch &L,
                              dim3 grid, cudaStream_t s);
cudaError_t launch_pfgse_phase(const PhaseLaunch &L, int n_delta, int n_g, cudaStream_t s);
cudaError_t launch_pfgse_direct(const DirectLaunch &L, int n_delta, int blocks, cudaStream_t s);
// Spatial walker order (walker_order.cu): perm[k] = upload index of the walker stored at k, sorted
// stably by a coarse Morton key of (x, y, z) >> shift. scratch: walker_order_scratch_words(n) uint32.
size_t walker_order_scratch_words(int64_t n);
cudaError_t walker_order(const int32_t *x, const int32_t *y, const int32_t *z, int64_t n, int shift, uint32_t *scratch,
                         int32_t *perm, cudaStream_t s);
// dst[k] = src[perm[k]], k < n
cudaError_t permute_u32(const int32_t *perm, int64_t n, const uint32_t *src, uint32_t *dst, cudaStream_t s);
cudaError_t permute_u64(const int32_t *perm, int64_t n, const uint64_t *src, uint64_t *dst, cudaStream_t s);
// x0[k] = ux[perm[k]] (and y, z, seeds)
cudaError_t gather_walkers(const int32_t *perm, int64_t n, const int32_t *ux, const int32_t *uy, const int32_t *uz,
                           const uint64_t *us, int32_t *x0, int32_t *y0, int32_t *z0, uint64_t *s0, cudaStream_t s);
// Morton parameters of an nx x ny x nz image (words = 0: no Morton copy). A copy is made when its
// index fits 32 bits and the power-of-two box around the image holds at most four times its voxels
// or, with max_bytes > 0, when the copy (W words per 32 voxels) takes at most max_bytes; the lowest
// index bits cycle x, y, z.
inline MortonImage morton_params(int nx, int ny, int nz, uint32_t &n_words, int W = 1, uint64_t max_bytes = 0)
{
    MortonImage m;
    n_words = 0;
    auto bits = [](int n) {
        int b = 0;
        while ((1ll << b) < n) b++;
        return b;
    };
    const int bx = bits(nx), by = bits(ny), bz = bits(nz);
    const int total = bx + by + bz;
    if (total > 32) return m;
    const uint64_t padded = 1ull << total;
    const bool small = max_bytes > 0 && (padded / 32) * 4 * (uint64_t)W <= max_bytes;
    if (padded > 4ull * (uint64_t)nx * ny * nz && !small) return m;
    int pos = 0;
    for (int i = 0; i < std::max(bx, std::max(by, bz)); i++)
    {
        if (i < bx) m.mx |= 1u << pos++;
        if (i < by) m.my |= 1u << pos++;
        if (i < bz) m.mz |= 1u << pos++;
    }
    m.ex = dilate_bits((uint32_t)nx - 1, m.mx);
    m.ey = dilate_bits((uint32_t)ny - 1, m.my);
    m.ez = dilate_bits((uint32_t)nz - 1, m.mz);
    n_words = (uint32_t)std::max<uint64_t>(1, padded >> 5);
    return m;
}

// Builds the Morton copy im.mi describes (n_words x W uint32) from im's bit-blocks.
cudaError_t launch_morton_build(const DevImage &im, int W, uint32_t n_words, uint32_t *out, cudaStream_t s);
// labels above n_phases (multi-phase images) set kStatusBadLabel
cudaError_t launch_pack_blocks(const uint8_t *labels, int nx, int ny, int nz, int bcols, int brows, int64_t nblocks,
                               int words, int n_phases, uint64_t *out, unsigned *status, cudaStream_t s);

} // namespace rwnmr
