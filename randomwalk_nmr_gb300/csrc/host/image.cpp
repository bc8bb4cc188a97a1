// Host image utilities: synthetic sphere packs and the bit-block packer.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "rwnmr_host.h"

namespace
{
// splitmix64 (Steele, Lea & Flood 2014): a fixed, documented generator so images are identical
// on every platform.
struct SplitMix64
{
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); } // [0, 1)
};
} // namespace

extern "C" {

int64_t rwnmr_synth_spheres(uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, double rmin, double rmax,
                            double porosity_target, int32_t n_phases, uint64_t seed, double *porosity)
{
    if (!labels || nx <= 0 || ny <= 0 || nz <= 0 || rmin < 0 || rmax < rmin || n_phases < 1 || n_phases > 255)
        return -1;
    const int64_t total = (int64_t)nx * ny * nz;
    std::memset(labels, 0, (size_t)total);
    int64_t pores = total;
    const int64_t target = (int64_t)std::floor(porosity_target * (double)total);
    SplitMix64 rng{seed};
    int64_t spheres = 0;
    while (pores > target)
    {
        const double cx = rng.uniform() * nx, cy = rng.uniform() * ny, cz = rng.uniform() * nz;
        const double r = rmin + (rmax - rmin) * rng.uniform();
        const uint8_t lab = (uint8_t)(1 + std::min<int32_t>(n_phases - 1, (int32_t)(rng.uniform() * n_phases)));
        const double r2 = r * r;
        const int x0 = std::max(0, (int)std::ceil(cx - r)), x1 = std::min(nx - 1, (int)std::floor(cx + r));
        const int y0 = std::max(0, (int)std::ceil(cy - r)), y1 = std::min(ny - 1, (int)std::floor(cy + r));
        const int z0 = std::max(0, (int)std::ceil(cz - r)), z1 = std::min(nz - 1, (int)std::floor(cz + r));
        for (int z = z0; z <= z1; z++)
        {
            const double dz2 = (z - cz) * (z - cz);
            for (int y = y0; y <= y1; y++)
            {
                const double dyz = dz2 + (y - cy) * (y - cy);
                if (dyz > r2) continue;
                uint8_t *row = labels + ((int64_t)z * ny + y) * nx;
                for (int x = x0; x <= x1; x++)
                {
                    if (dyz + (x - cx) * (x - cx) > r2) continue;
                    if (row[x] == 0) pores--;
                    row[x] = lab;
                }
            }
        }
        spheres++;
    }
    if (porosity) *porosity = (double)pores / (double)total;
    return spheres;
}

int64_t rwnmr_pack_blocks(const uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, uint64_t *blocks, int32_t *bdims)
{
    if (nx <= 0 || ny <= 0 || nz <= 0) return -1;
    const int32_t bc = (nx + 3) / 4, br = (ny + 3) / 4, bd = (nz + 3) / 4;
    if (bdims)
    {
        bdims[0] = bc;
        bdims[1] = br;
        bdims[2] = bd;
    }
    const int64_t nb = (int64_t)bc * br * bd;
    if (!blocks || !labels) return nb;
    std::memset(blocks, 0, sizeof(uint64_t) * (size_t)nb);
    for (int32_t z = 0; z < nz; z++)
        for (int32_t y = 0; y < ny; y++)
        {
            const uint8_t *row = labels + ((int64_t)z * ny + y) * nx;
            const int64_t base = (int64_t)(y >> 2) * bc + (int64_t)(z >> 2) * bc * br;
            const int bityz = ((y & 3) << 2) | ((z & 3) << 4);
            for (int32_t x = 0; x < nx; x++)
                if (row[x]) blocks[base + (x >> 2)] |= 1ull << (bityz | (x & 3));
        }
    return nb;
}

} // extern "C"
