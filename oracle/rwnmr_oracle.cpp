// CPU restatement of RandomWalk_NMR's walker hot path -- TEST ORACLE ONLY (see rwnmr_oracle.h).
//
// Each function names the reference code it restates (paths relative to the reference's
// src/backend/). Built with -ffp-contract=off so x86 and Arm give identical FP64 results.

#include "rwnmr_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>
#include <omp.h>

namespace
{
typedef unsigned __int128 u128;

const int kNorth = 1, kWest = 2, kSouth = 3, kEast = 4, kUp = 5, kDown = 6; // Walker/walker_defs.h:6-15

// xorshift64 (RNG/xorshift.cpp:17-24, Walker/walker.h:557-564): the state is the output.
inline uint64_t xs64(uint64_t x)
{
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return x;
}

// Digit-sum reduction modulo 6 exactly as Walker/walker.h:566-582 writes it.
inline uint32_t mod6_digits(uint64_t a)
{
    while (a > 11)
    {
        int s = 0;
        while (a != 0)
        {
            s = s + (int)(a & 7);
            a = (a >> 2) & (uint64_t)-2;
        }
        a = (uint64_t)s;
    }
    if (a > 5) a = a - 6;
    return (uint32_t)a;
}

// Periodic image index (NMR_cpmg_cuda.cpp:1991-1999).
inline int map_periodic(int local, int shift, int dim)
{
    int g = local >> shift;
    g = g % dim;
    return g < 0 ? g + dim : g;
}

// Mirrored-tiling image index (NMR_cpmg_cuda.cpp:2001-2015).
inline int map_mirror(int local, int shift, int dim)
{
    int g = local >> shift;
    int img = g % dim;
    if (img < 0) img += dim;
    int mirror = (g > 0) ? (g / dim) % 2 : ((-g - 1 + dim) / dim) % 2;
    int anti = (mirror + 1) % 2;
    return anti * img + mirror * (dim - 1 - img);
}

struct Walk
{
    int32_t x, y, z;
    uint64_t seed;
};

// One walker step. Returns -1 if the walker moved, else the phase index of the solid voxel it
// hit. Restates Walker::walk_3D/map_3D (Walker/walker.cpp:197-231): direction from xorshift64 and
// mod 6 (walker.h:346-358); for noflux a move off the image is reversed, comparing the voxel
// coordinate pos >> shift with the image edge (walker.h:444-491, NMR_cpmg_cuda.cpp:1847-1902);
// next position (walker.h:360-391); image-space lookup per boundary condition
// (NMR_cpmg_cuda.cpp:1986-2015) and the bit test (BitBlock/bitBlock.h:113-139).
inline int step(const orc_image &im, int bc, int shift, Walk &w)
{
    w.seed = xs64(w.seed);
    int dir = (int)mod6_digits(w.seed) + 1;
    if (bc == ORC_BC_NOFLUX)
    {
        int gx = w.x >> shift, gy = w.y >> shift, gz = w.z >> shift;
        switch (dir)
        {
        case kNorth: if (gy == 0) dir = kSouth; break;
        case kSouth: if (gy == im.ny - 1) dir = kNorth; break;
        case kWest: if (gx == 0) dir = kEast; break;
        case kEast: if (gx == im.nx - 1) dir = kWest; break;
        case kUp: if (gz == im.nz - 1) dir = kDown; break;
        case kDown: if (gz == 0) dir = kUp; break;
        }
    }
    int nx = w.x, ny = w.y, nz = w.z;
    switch (dir)
    {
    case kNorth: ny -= 1; break;
    case kWest: nx -= 1; break;
    case kSouth: ny += 1; break;
    case kEast: nx += 1; break;
    case kUp: nz += 1; break;
    case kDown: nz -= 1; break;
    }
    int ix, iy, iz;
    if (bc == ORC_BC_PERIODIC)
    {
        ix = map_periodic(nx, shift, im.nx);
        iy = map_periodic(ny, shift, im.ny);
        iz = map_periodic(nz, shift, im.nz);
    }
    else if (bc == ORC_BC_MIRROR)
    {
        ix = map_mirror(nx, shift, im.nx);
        iy = map_mirror(ny, shift, im.ny);
        iz = map_mirror(nz, shift, im.nz);
    }
    else
    {
        ix = nx >> shift;
        iy = ny >> shift;
        iz = nz >> shift;
    }
    int64_t block = (int64_t)(ix >> 2) + (int64_t)(iy >> 2) * im.bcols + (int64_t)(iz >> 2) * im.bcols * im.brows;
    int bit = (ix & 3) + ((iy & 3) << 2) + ((iz & 3) << 4);
    if (((im.blocks[block] >> bit) & 1ull) == 0)
    {
        w.x = nx;
        w.y = ny;
        w.z = nz;
        return -1;
    }
    if (!im.labels) return 0;
    return (int)im.labels[((int64_t)iz * im.ny + iy) * im.nx + ix] - 1;
}

// Image voxel of a walk-grid position: pos >> shift for noflux (convertLocalToGlobal_CPMG), the
// periodic / mirrored maps otherwise (NMR_cpmg_cuda.cpp:470-474, 749-751).
inline void image_voxel(const orc_image &im, int bc, int shift, const Walk &w, int &ix, int &iy, int &iz)
{
    if (bc == ORC_BC_PERIODIC)
    {
        ix = map_periodic(w.x, shift, im.nx);
        iy = map_periodic(w.y, shift, im.ny);
        iz = map_periodic(w.z, shift, im.nz);
    }
    else if (bc == ORC_BC_MIRROR)
    {
        ix = map_mirror(w.x, shift, im.nx);
        iy = map_mirror(w.y, shift, im.ny);
        iz = map_mirror(w.z, shift, im.nz);
    }
    else
    {
        ix = w.x >> shift;
        iy = w.y >> shift;
        iz = w.z >> shift;
    }
}

inline bool voxel_solid(const orc_image &im, int ix, int iy, int iz)
{
    int64_t block = (int64_t)(ix >> 2) + (int64_t)(iy >> 2) * im.bcols + (int64_t)(iz >> 2) * im.bcols * im.brows;
    int bit = (ix & 3) + ((iy & 3) << 2) + ((iz & 3) << 4);
    return ((im.blocks[block] >> bit) & 1ull) != 0;
}

inline uint64_t fxmul(uint64_t a, uint64_t b) { return (uint64_t)(((u128)a * (u128)b) >> 63); }

struct Tables
{
    int P = 1;
    int32_t n_max = 0;
    std::vector<double> t;   // [P][n_max+1]
    std::vector<uint64_t> fx; // [P][n_max+1]
    void build(const double *dfactor, int p, int32_t nmax)
    {
        P = p;
        n_max = nmax;
        t.assign((size_t)P * (nmax + 1), 0.0);
        fx.assign((size_t)P * (nmax + 1), 0);
        for (int q = 0; q < P; q++) orc_energy_table(dfactor[q], nmax, &t[(size_t)q * (nmax + 1)], &fx[(size_t)q * (nmax + 1)]);
    }
    // Multi-phase energy E = T_0[c_0] * T_1[c_1] * ... (left to right); for one phase this is
    // the reference's repeated product energy *= decreaseFactor (Walker/walker.cpp:229).
    double energy(const uint32_t *c) const
    {
        double e = t[c[0]];
        for (int q = 1; q < P; q++) e = e * t[(size_t)q * (n_max + 1) + c[q]];
        return e;
    }
    uint64_t energy_fx(const uint32_t *c) const
    {
        uint64_t e = fx[c[0]];
        for (int q = 1; q < P; q++) e = fxmul(e, fx[(size_t)q * (n_max + 1) + c[q]]);
        return e;
    }
};

inline void add_limbs(uint64_t *acc, uint64_t e)
{
    acc[0] += e & ((1ull << 21) - 1);
    acc[1] += (e >> 21) & ((1ull << 21) - 1);
    acc[2] += e >> 42;
}

bool image_ok(const orc_image *im)
{
    return im && im->blocks && im->nx > 0 && im->ny > 0 && im->nz > 0 && im->n_phases >= 1 &&
           (im->labels || im->n_phases == 1);
}
} // namespace

extern "C" {

// BitBlock::setBlockMapDimensions_3D + createBitBlocksArray_3D (BitBlock/bitBlock.cpp:138-221):
// block dims rounded up; bit = x%4 + 4*(y%4) + 16*(z%4); voxels past the image edge stay 0 (pore).
int64_t orc_pack_blocks(const uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, uint64_t *blocks, int32_t *bdims)
{
    int32_t bc = (nx + 3) / 4, br = (ny + 3) / 4, bd = (nz + 3) / 4;
    if (bdims)
    {
        bdims[0] = bc;
        bdims[1] = br;
        bdims[2] = bd;
    }
    int64_t nb = (int64_t)bc * br * bd;
    if (!blocks) return nb;
    std::memset(blocks, 0, sizeof(uint64_t) * (size_t)nb);
    for (int32_t z = 0; z < nz; z++)
        for (int32_t y = 0; y < ny; y++)
            for (int32_t x = 0; x < nx; x++)
                if (labels[((int64_t)z * ny + y) * nx + x])
                {
                    int64_t b = (int64_t)(x / 4) + (int64_t)(y / 4) * bc + (int64_t)(z / 4) * bc * br;
                    blocks[b] |= 1ull << ((x % 4) + 4 * (y % 4) + 16 * (z % 4));
                }
    return nb;
}

uint64_t orc_xorshift64(uint64_t state) { return xs64(state); }
uint32_t orc_mod6(uint64_t a) { return mod6_digits(a); }

void orc_energy_table(double f, int32_t n_max, double *t_fp64, uint64_t *t_fx)
{
    double t = 1.0; // WALKER_INITIAL_ENERGY (Walker/walker_defs.h)
    for (int32_t n = 0; n <= n_max; n++)
    {
        if (t_fp64) t_fp64[n] = t;
        if (t_fx) t_fx[n] = (uint64_t)std::nearbyint(std::ldexp(t, 63));
        t = t * f;
    }
}

int orc_cpmg(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0, const int32_t *y0,
             const int32_t *z0, const uint64_t *seed0, int32_t n_echoes, int32_t steps_per_echo,
             const double *dfactor, double *echo_fp64, uint64_t *echo_fx, uint64_t *echo_coll, int32_t *xf,
             int32_t *yf, int32_t *zf, uint64_t *seedf, uint32_t *collf, int32_t threads)
{
    if (!image_ok(img) || n < 0 || n_echoes < 0 || steps_per_echo < 1 || shift < 0 || !dfactor) return -1;
    const int P = img->n_phases;
    Tables tab;
    tab.build(dfactor, P, n_echoes * steps_per_echo);
    const int nt = threads > 1 ? threads : 1;
    const size_t E1 = (size_t)n_echoes + 1;
    std::vector<double> acc_fp((size_t)nt * E1, 0.0);
    std::vector<uint64_t> acc_fx((size_t)nt * E1 * 3, 0);
    std::vector<uint64_t> acc_c((size_t)nt * n_echoes * P, 0);

#pragma omp parallel num_threads(nt)
    {
        int t = omp_get_thread_num();
        int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        double *afp = &acc_fp[(size_t)t * E1];
        uint64_t *afx = &acc_fx[(size_t)t * E1 * 3];
        uint64_t *ac = &acc_c[(size_t)t * n_echoes * P];
        std::vector<uint32_t> c(P);
        for (int64_t i = lo; i < hi; i++)
        {
            Walk w{x0[i], y0[i], z0[i], seed0[i]};
            std::fill(c.begin(), c.end(), 0u);
            afp[0] += tab.energy(c.data());
            add_limbs(afx, tab.energy_fx(c.data()));
            for (int32_t e = 0; e < n_echoes; e++)
            {
                for (int32_t s = 0; s < steps_per_echo; s++)
                {
                    int ph = step(*img, bc, shift, w);
                    if (ph >= 0)
                    {
                        c[ph]++;
                        ac[(size_t)e * P + ph]++;
                    }
                }
                afp[e + 1] += tab.energy(c.data());
                add_limbs(&afx[(size_t)(e + 1) * 3], tab.energy_fx(c.data()));
            }
            if (xf) xf[i] = w.x;
            if (yf) yf[i] = w.y;
            if (zf) zf[i] = w.z;
            if (seedf) seedf[i] = w.seed;
            if (collf)
                for (int q = 0; q < P; q++) collf[(size_t)i * P + q] = c[q];
        }
    }
    for (size_t e = 0; e < E1; e++)
    {
        double s = 0.0;
        uint64_t f0 = 0, f1 = 0, f2 = 0;
        for (int t = 0; t < nt; t++)
        {
            s += acc_fp[(size_t)t * E1 + e];
            f0 += acc_fx[((size_t)t * E1 + e) * 3 + 0];
            f1 += acc_fx[((size_t)t * E1 + e) * 3 + 1];
            f2 += acc_fx[((size_t)t * E1 + e) * 3 + 2];
        }
        if (echo_fp64) echo_fp64[e] = s;
        if (echo_fx)
        {
            echo_fx[e * 3 + 0] = f0;
            echo_fx[e * 3 + 1] = f1;
            echo_fx[e * 3 + 2] = f2;
        }
    }
    if (echo_coll)
        for (size_t k = 0; k < (size_t)n_echoes * P; k++)
        {
            uint64_t s = 0;
            for (int t = 0; t < nt; t++) s += acc_c[(size_t)t * n_echoes * P + k];
            echo_coll[k] = s;
        }
    return 0;
}

void orc_uniform_field(const orc_image *img, double resolution, double gradient, int32_t direction, double *out)
{
    const double dg = gradient * (1.0e-6) * resolution; // InternalField.cpp: _gValue * (1.0e-6) * _resolution
    for (int32_t z = 0; z < img->nz; z++)
        for (int32_t y = 0; y < img->ny; y++)
            for (int32_t x = 0; x < img->nx; x++)
            {
                const int coord = direction == 0 ? x : (direction == 1 ? y : z);
                out[((int64_t)z * img->ny + y) * img->nx + x] = voxel_solid(*img, x, y, z) ? 0.0 : coord * dg;
            }
}

int orc_cpmg_field(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0, const int32_t *y0,
                   const int32_t *z0, const uint64_t *seed0, int32_t n_echoes, int32_t steps_per_echo,
                   const double *dfactor, const double *walker_dfactor, double gammatau, const double *field,
                   double dg, int32_t axis, double *echo_fp64, uint64_t *echo_fx, int32_t *xf, int32_t *yf,
                   int32_t *zf, uint64_t *seedf, uint32_t *collf, double *phasef, int32_t threads)
{
    if (!image_ok(img) || n < 0 || n_echoes < 0 || steps_per_echo < 1 || shift < 0 || axis < 0 || axis > 2)
        return -1;
    if (!dfactor && !(walker_dfactor && img->n_phases == 1)) return -1;
    const double one = 1.0;
    if (!dfactor) dfactor = &one; // tables unused
    const int P = img->n_phases;
    const int32_t spi = steps_per_echo / 2; // stepsPerInversion
    Tables tab;
    tab.build(dfactor, P, n_echoes * 2 * spi);
    const int nt = threads > 1 ? threads : 1;
    const size_t E1 = (size_t)n_echoes + 1;
    std::vector<double> acc_fp((size_t)nt * E1, 0.0);
    std::vector<uint64_t> acc_fx((size_t)nt * E1 * 3, 0);
    // field value at the walker's voxel (the array, or the uniform field evaluated in place)
    auto field_at = [&](const Walk &w) {
        int ix, iy, iz;
        image_voxel(*img, bc, shift, w, ix, iy, iz);
        if (field) return field[((int64_t)iz * img->ny + iy) * img->nx + ix];
        const int coord = axis == 0 ? ix : (axis == 1 ? iy : iz);
        return voxel_solid(*img, ix, iy, iz) ? 0.0 : coord * dg;
    };
    auto energy_fx = [](double e) { return (uint64_t)((int64_t)std::nearbyint(std::ldexp(e, 61)) + (1ll << 61)); };

#pragma omp parallel num_threads(nt)
    {
        int t = omp_get_thread_num();
        int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        double *afp = &acc_fp[(size_t)t * E1];
        uint64_t *afx = &acc_fx[(size_t)t * E1 * 3];
        std::vector<uint32_t> c(P);
        for (int64_t i = lo; i < hi; i++)
        {
            Walk w{x0[i], y0[i], z0[i], seed0[i]};
            std::fill(c.begin(), c.end(), 0u);
            double phase = 0.0;
            double palive = 1.0; // per-walker factors: the reference's running product
            const double fw = walker_dfactor ? walker_dfactor[i] : 1.0;
            auto survival = [&]() { return walker_dfactor ? palive : tab.energy(c.data()); };
            double e0 = survival() * std::cos(phase);
            afp[0] += e0;
            add_limbs(afx, energy_fx(e0));
            for (int32_t e = 0; e < n_echoes; e++)
            {
                for (int inv = 0; inv < 2; inv++)
                {
                    phase = -phase;
                    for (int32_t s = 0; s < spi; s++)
                    {
                        phase = std::fma(gammatau, field_at(w), phase);
                        int ph = step(*img, bc, shift, w);
                        if (ph >= 0)
                        {
                            c[ph]++;
                            palive = palive * fw;
                        }
                        phase = std::fma(gammatau, field_at(w), phase);
                    }
                }
                const double en = survival() * std::cos(phase);
                afp[e + 1] += en;
                add_limbs(&afx[(size_t)(e + 1) * 3], energy_fx(en));
            }
            if (xf) xf[i] = w.x;
            if (yf) yf[i] = w.y;
            if (zf) zf[i] = w.z;
            if (seedf) seedf[i] = w.seed;
            if (collf)
                for (int q = 0; q < P; q++) collf[(size_t)i * P + q] = c[q];
            if (phasef) phasef[i] = phase;
        }
    }
    for (size_t e = 0; e < E1; e++)
    {
        double s = 0.0;
        uint64_t f[3] = {0, 0, 0};
        for (int t = 0; t < nt; t++)
        {
            s += acc_fp[(size_t)t * E1 + e];
            for (int k = 0; k < 3; k++) f[k] += acc_fx[((size_t)t * E1 + e) * 3 + k];
        }
        if (echo_fp64) echo_fp64[e] = s;
        if (echo_fx)
            for (int k = 0; k < 3; k++) echo_fx[e * 3 + k] = f[k];
    }
    return 0;
}

int orc_pfgse(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0, const int32_t *y0,
              const int32_t *z0, const uint64_t *seed0, const double *dfactor, int32_t n_delta, const int32_t *steps,
              int32_t n_g, const double *kvec, double res, double *M, double *esum, uint64_t *msd, uint64_t *esum_fx,
              int32_t threads)
{
    if (!image_ok(img) || n < 0 || n_delta < 0 || n_g < 0 || shift < 0 || !dfactor || (n_delta > 0 && !steps))
        return -1;
    for (int32_t i = 1; i < n_delta; i++)
        if (steps[i] < steps[i - 1]) return -1;
    const int P = img->n_phases;
    Tables tab;
    tab.build(dfactor, P, n_delta ? steps[n_delta - 1] : 0);
    const int nt = threads > 1 ? threads : 1;
    std::vector<double> accd((size_t)nt * n_delta * (n_g + 1), 0.0);
    std::vector<uint64_t> accu((size_t)nt * n_delta * 6, 0);
#pragma omp parallel num_threads(nt)
    {
        int t = omp_get_thread_num();
        int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        double *ad = &accd[(size_t)t * n_delta * (n_g + 1)];
        uint64_t *au = &accu[(size_t)t * n_delta * 6];
        std::vector<uint32_t> c(P);
        for (int64_t i = lo; i < hi; i++)
        {
            Walk w{x0[i], y0[i], z0[i], seed0[i]};
            std::fill(c.begin(), c.end(), 0u);
            int32_t done = 0;
            for (int32_t d = 0; d < n_delta; d++)
            {
                for (; done < steps[d]; done++)
                {
                    int ph = step(*img, bc, shift, w);
                    if (ph >= 0) c[ph]++;
                }
                // NMR_pfgse.cpp:1747-1765: phase = E * cos((k . dR) * res), dR in doubles
                double e = tab.energy(c.data());
                double dX = (double)w.x - (double)x0[i];
                double dY = (double)w.y - (double)y0[i];
                double dZ = (double)w.z - (double)z0[i];
                for (int32_t j = 0; j < n_g; j++)
                {
                    double kd = kvec[3 * j + 0] * dX + kvec[3 * j + 1] * dY + kvec[3 * j + 2] * dZ;
                    ad[(size_t)d * (n_g + 1) + j] += e * std::cos(kd * res);
                }
                ad[(size_t)d * (n_g + 1) + n_g] += e;
                int64_t ix = w.x - x0[i], iy = w.y - y0[i], iz = w.z - z0[i];
                au[(size_t)d * 6 + 0] += (uint64_t)(ix * ix);
                au[(size_t)d * 6 + 1] += (uint64_t)(iy * iy);
                au[(size_t)d * 6 + 2] += (uint64_t)(iz * iz);
                uint64_t lim[3] = {0, 0, 0};
                add_limbs(lim, tab.energy_fx(c.data()));
                au[(size_t)d * 6 + 3] += lim[0];
                au[(size_t)d * 6 + 4] += lim[1];
                au[(size_t)d * 6 + 5] += lim[2];
            }
        }
    }
    for (int32_t d = 0; d < n_delta; d++)
    {
        for (int32_t j = 0; j <= n_g; j++)
        {
            double s = 0.0;
            for (int t = 0; t < nt; t++) s += accd[((size_t)t * n_delta + d) * (n_g + 1) + j];
            if (j < n_g && M) M[(size_t)d * n_g + j] = s;
            if (j == n_g && esum) esum[d] = s;
        }
        for (int k = 0; k < 6; k++)
        {
            uint64_t s = 0;
            for (int t = 0; t < nt; t++) s += accu[((size_t)t * n_delta + d) * 6 + k];
            if (k < 3 && msd) msd[(size_t)d * 3 + k] = s;
            if (k >= 3 && esum_fx) esum_fx[(size_t)d * 3 + (k - 3)] = s;
        }
    }
    return 0;
}

// Pathwise FP64 derivative of the PFGSE phase sums with respect to the gradient strength g, for a
// gradient ramp k_j = kscale * g_j * dir (kscale = dk/dg, NMR_pfgse.cpp:483-486; dir a unit
// vector). For fixed trajectories M_j = sum_w E_w cos((k_j . dR_w) res), so
//   dM_j/dg = -sum_w E_w sin((k_j . dR_w) res) * (kscale dir . dR_w) res,
// evaluated per walker in FP64 (the same walks, energies and k . dR as orc_pfgse) and summed in
// the walker order of each thread's contiguous range, then over threads in order.
int orc_pfgse_grad_g(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0,
                     const int32_t *y0, const int32_t *z0, const uint64_t *seed0, const double *dfactor,
                     int32_t n_delta, const int32_t *steps, int32_t n_g, const double *kvec, double res, double kscale,
                     const double *dir, double *dMdg, int32_t threads)
{
    if (!image_ok(img) || n < 0 || n_delta < 0 || n_g < 0 || shift < 0 || !dfactor || !dir || !dMdg ||
        (n_delta > 0 && !steps))
        return -1;
    for (int32_t i = 1; i < n_delta; i++)
        if (steps[i] < steps[i - 1]) return -1;
    const int P = img->n_phases;
    Tables tab;
    tab.build(dfactor, P, n_delta ? steps[n_delta - 1] : 0);
    const int nt = threads > 1 ? threads : 1;
    std::vector<double> acc((size_t)nt * n_delta * n_g, 0.0);
#pragma omp parallel num_threads(nt)
    {
        int t = omp_get_thread_num();
        int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        double *a = &acc[(size_t)t * n_delta * n_g];
        std::vector<uint32_t> c(P);
        for (int64_t i = lo; i < hi; i++)
        {
            Walk w{x0[i], y0[i], z0[i], seed0[i]};
            std::fill(c.begin(), c.end(), 0u);
            int32_t done = 0;
            for (int32_t d = 0; d < n_delta; d++)
            {
                for (; done < steps[d]; done++)
                {
                    int ph = step(*img, bc, shift, w);
                    if (ph >= 0) c[ph]++;
                }
                const double e = tab.energy(c.data());
                const double dX = (double)w.x - (double)x0[i];
                const double dY = (double)w.y - (double)y0[i];
                const double dZ = (double)w.z - (double)z0[i];
                const double proj = kscale * (dir[0] * dX + dir[1] * dY + dir[2] * dZ) * res;
                for (int32_t j = 0; j < n_g; j++)
                {
                    const double kd = kvec[3 * j + 0] * dX + kvec[3 * j + 1] * dY + kvec[3 * j + 2] * dZ;
                    a[(size_t)d * n_g + j] -= e * std::sin(kd * res) * proj;
                }
            }
        }
    }
    for (int32_t d = 0; d < n_delta; d++)
        for (int32_t j = 0; j < n_g; j++)
        {
            double s = 0.0;
            for (int t = 0; t < nt; t++) s += acc[((size_t)t * n_delta + d) * n_g + j];
            dMdg[(size_t)d * n_g + j] = s;
        }
    return 0;
}

int orc_displacements(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0,
                      const int32_t *y0, const int32_t *z0, const uint64_t *seed0, int32_t steps, int32_t *dx,
                      int32_t *dy, int32_t *dz, uint32_t *collf, int32_t threads)
{
    if (!image_ok(img) || n < 0 || steps < 0 || shift < 0) return -1;
    const int nt = threads > 1 ? threads : 1;
    const int P = img->n_phases;
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int64_t i = 0; i < n; i++)
    {
        Walk w{x0[i], y0[i], z0[i], seed0[i]};
        uint32_t total = 0;
        std::vector<uint32_t> c(P, 0);
        for (int32_t s = 0; s < steps; s++)
        {
            int ph = step(*img, bc, shift, w);
            if (ph >= 0)
            {
                c[ph]++;
                total++;
            }
        }
        if (dx) dx[i] = w.x - x0[i];
        if (dy) dy[i] = w.y - y0[i];
        if (dz) dz[i] = w.z - z0[i];
        if (collf)
            for (int q = 0; q < P; q++) collf[(size_t)i * P + q] = c[q];
    }
    return 0;
}

// ---------------------------------------------------------------------------------------------
// Synthetic inputs for the CPU reference arm of the benchmark, so that it needs no product code.

// The benchmark's overlapping-sphere packs: centre uniform in the box, radius uniform in
// [rmin, rmax], label uniform in 1..n_phases, spheres added until at most floor(porosity * volume)
// voxels are pore. Draws are splitmix64 outputs (Steele, Lea & Flood 2014) turned into doubles in
// [0, 1) from their top 53 bits, four per sphere in the order cx, cy, cz, r, label; a voxel is in a
// sphere when its squared distance from the centre is at most r^2 (later spheres relabel).
int64_t orc_synth_spheres(uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, double rmin, double rmax,
                          double porosity, int32_t n_phases, uint64_t seed, double *porosity_out)
{
    if (!labels || nx <= 0 || ny <= 0 || nz <= 0 || rmin < 0 || rmax < rmin || n_phases < 1 || n_phases > 255)
        return -1;
    uint64_t state = seed;
    auto draw = [&state]() {
        uint64_t v = (state += 0x9E3779B97F4A7C15ull);
        v = (v ^ (v >> 30)) * 0xBF58476D1CE4E5B9ull;
        v = (v ^ (v >> 27)) * 0x94D049BB133111EBull;
        v ^= v >> 31;
        return (double)(v >> 11) / 9007199254740992.0;
    };
    const int64_t volume = (int64_t)nx * ny * nz;
    std::fill(labels, labels + volume, (uint8_t)0);
    int64_t pore = volume, spheres = 0;
    const int64_t goal = (int64_t)std::floor(porosity * (double)volume);
    while (pore > goal)
    {
        const double cx = draw() * nx, cy = draw() * ny, cz = draw() * nz;
        const double r = rmin + (rmax - rmin) * draw();
        int lab = 1 + (int)(draw() * n_phases);
        if (lab > n_phases) lab = n_phases;
        for (int z = std::max(0, (int)std::ceil(cz - r)); z <= std::min(nz - 1, (int)std::floor(cz + r)); z++)
            for (int y = std::max(0, (int)std::ceil(cy - r)); y <= std::min(ny - 1, (int)std::floor(cy + r)); y++)
            {
                const double d2 = (z - cz) * (z - cz) + (y - cy) * (y - cy);
                if (d2 > r * r) continue;
                for (int x = std::max(0, (int)std::ceil(cx - r)); x <= std::min(nx - 1, (int)std::floor(cx + r)); x++)
                {
                    if (d2 + (x - cx) * (x - cx) > r * r) continue;
                    uint8_t &v = labels[((int64_t)z * ny + y) * nx + x];
                    pore -= v == 0;
                    v = (uint8_t)lab;
                }
            }
        spheres++;
    }
    if (porosity_out) *porosity_out = (double)pore / (double)volume;
    return spheres;
}

// The reference's uniformly random walker placement with its seeds, draw for draw
// (NMR_Simulation/NMR_Simulation.cpp): std::mt19937 seeded with SEED then discard(4096)
// (:86-95); one uniform_int_distribution<uint64_t> seed per walker (createWalkers, :1139-1204);
// pore voxels listed in z, y, x order (createPoreList, :930-980); the pore count re-derived as
// (uint)(porosity * volume) and n pore ids drawn from uniform_int_distribution(0, that count), which
// includes one past the end (updateNumberOfPores, createWalkersIDList, :904-907, 1086-1136) -- an id
// past the list is clamped to its last pore and counted in *clamped; with every pore occupied the
// walkers take the pores in order (placeWalkersUniformly, :1271-1333); voxel division then draws x,
// y, z offsets per walker (applyVoxelDivision, :192-268). labels: [nz][ny][nx], non-zero = solid.
int orc_place_walkers_random(const uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, uint64_t seed, int64_t n,
                             int32_t shift, int32_t *x0, int32_t *y0, int32_t *z0, uint64_t *seed0, int64_t *clamped)
{
    if (!labels || nx <= 0 || ny <= 0 || nz <= 0 || seed == 0 || n < 0 || n > 0xffffffffll || shift < 0 || shift > 10)
        return -1;
    std::mt19937 mt((std::mt19937::result_type)seed);
    mt.discard(4096);
    std::vector<int32_t> px, py, pz;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++)
                if (!labels[((int64_t)z * ny + y) * nx + x])
                {
                    px.push_back(x);
                    py.push_back(y);
                    pz.push_back(z);
                }
    if (px.empty()) return -2;
    const double volume = (double)nx * ny * nz;
    const double occupancy = (double)n / (double)px.size();
    std::uniform_int_distribution<uint64_t> seeds;
    for (int64_t i = 0; i < n; i++) seed0[i] = seeds(mt);
    std::uniform_int_distribution<std::mt19937::result_type> pick(
        0, (std::mt19937::result_type)((double)px.size() / volume * volume));
    std::vector<uint64_t> ids((size_t)n);
    for (int64_t i = 0; i < n; i++) ids[i] = pick(mt);
    int64_t clamp = 0;
    for (int64_t i = 0; i < n; i++)
    {
        uint64_t id = occupancy != 1.0 ? ids[i] : (uint64_t)i;
        if (id >= px.size())
        {
            id = px.size() - 1;
            clamp++;
        }
        x0[i] = px[id];
        y0[i] = py[id];
        z0[i] = pz[id];
    }
    if (shift > 0)
    {
        const std::mt19937::result_type factor = 1u << shift;
        std::uniform_int_distribution<std::mt19937::result_type> sub(0, factor - 1);
        for (int64_t i = 0; i < n; i++)
        {
            x0[i] = (int32_t)((double)x0[i] * factor + (double)sub(mt));
            y0[i] = (int32_t)((double)y0[i] * factor + (double)sub(mt));
            z0[i] = (int32_t)((double)z0[i] * factor + (double)sub(mt));
        }
    }
    if (clamped) *clamped = clamp;
    return 0;
}

} // extern "C"
