// Walker creation and placement, draw-for-draw with the reference's NMR_Simulation setup:
//   ctor:            mt19937 seeded with SEED, then discard(4096)          (NMR_Simulation.cpp:86-95)
//   createWalkers:   one seed per walker, uniform_int_distribution<uint64_t> (NMR_Simulation.cpp:1139-1204)
//   createPoreList:  pore voxels in z, y, x order; numberOfPores re-derived from the porosity
//                    as (uint)(porosity * volume)                          (NMR_Simulation.cpp:930-980, 904-907)
//   createWalkersIDList: uniform_int_distribution<mt19937::result_type>(0, numberOfPores), which
//                    includes numberOfPores itself                         (NMR_Simulation.cpp:1086-1136)
//   placeWalkersUniformly / InSamePoint / InCubicSpace                     (NMR_Simulation.cpp:1271-1454)
//   applyVoxelDivision: three draws per walker, x then y then z            (NMR_Simulation.cpp:192-268)
// The same C++ standard library distributions are used, so the draws are identical.
// Deviation: a pore index equal to the pore count (one past the end; the reference reads past its
// vector there) is clamped to the last pore and counted in info->clamped.
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "rwnmr_host.h"
#include "host_internal.h"

namespace rwnmr_host
{

static inline bool is_solid(const uint64_t *blocks, int bcols, int brows, int x, int y, int z)
{
    int64_t b = (int64_t)(x >> 2) + (int64_t)(y >> 2) * bcols + (int64_t)(z >> 2) * bcols * brows;
    int bit = (x & 3) + ((y & 3) << 2) + ((z & 3) << 4);
    return (blocks[b] >> bit) & 1ull;
}

int place_walkers(std::mt19937 &rng, const uint64_t *blocks, int nx, int ny, int nz, const PlacementRequest &req,
                  std::vector<int32_t> &x0, std::vector<int32_t> &y0, std::vector<int32_t> &z0,
                  std::vector<uint64_t> &seed0, PlacementInfo &info, std::string &err)
{
    const int bcols = (nx + 3) / 4, brows = (ny + 3) / 4;
    const uint32_t n = (uint32_t)req.n;
    info = PlacementInfo();
    // countPoresInBitBlock (NMR_Simulation.cpp:675-726)
    uint32_t pores_total = 0;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++)
                if (!is_solid(blocks, bcols, brows, x, y, z)) pores_total++;
    const double volume = (double)nx * ny * nz;
    const double porosity = (double)pores_total / volume;
    info.pores = pores_total;
    info.porosity = porosity;

    x0.assign(n, 0);
    y0.assign(n, 0);
    z0.assign(n, 0);
    seed0.assign(n, 0);
    auto create_walkers = [&]() {
        std::uniform_int_distribution<uint64_t> d64;
        for (uint32_t i = 0; i < n; i++) seed0[i] = d64(rng);
    };
    struct P3
    {
        int x, y, z;
    };
    std::vector<P3> pores;

    if (req.mode == "point")
    {
        const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
        create_walkers();
        if (is_solid(blocks, bcols, brows, cx, cy, cz))
        {
            err = "could not place walkers: point is not pore";
            return -1;
        }
        for (uint32_t i = 0; i < n; i++)
        {
            x0[i] = cx;
            y0[i] = cy;
            z0[i] = cz;
        }
        info.occupancy = n / (double)pores_total;
    }
    else if (req.mode == "cubic")
    {
        const int cx = (nx - 1) / 2, cy = (ny - 1) / 2, cz = (nz - 1) / 2, dv = req.deviation;
        int x_lo = std::max(0, cx - dv), y_lo = std::max(0, cy - dv), z_lo = std::max(0, cz - dv);
        int x_hi = std::min(nx, cx + dv), y_hi = std::min(ny, cy + dv), z_hi = std::min(nz, cz + dv);
        // countPoresInCubicSpace / createPoreList(p1, p2): half-open box [p1, p2)
        for (int z = z_lo; z < z_hi; z++)
            for (int y = y_lo; y < y_hi; y++)
                for (int x = x_lo; x < x_hi; x++)
                    if (!is_solid(blocks, bcols, brows, x, y, z)) pores.push_back({x, y, z});
        info.pores = (uint32_t)pores.size();
        create_walkers();
        if (pores.empty())
        {
            err = "no pores in the selected cubic space";
            return -1;
        }
        std::uniform_int_distribution<std::mt19937::result_type> dist(0, pores.size());
        for (uint32_t i = 0; i < n; i++)
        {
            size_t id = dist(rng);
            if (id >= pores.size())
            {
                id = pores.size() - 1;
                info.clamped++;
            }
            x0[i] = pores[id].x;
            y0[i] = pores[id].y;
            z0[i] = pores[id].z;
        }
        info.occupancy = n / (double)pores.size();
    }
    else
    {
        if (pores_total == 0)
        {
            err = "image has no pore voxels";
            return -1;
        }
        const double occupancy = n / (double)pores_total; // updateWalkerOccupancy, before the recount
        create_walkers();
        for (int z = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++)
                    if (!is_solid(blocks, bcols, brows, x, y, z)) pores.push_back({x, y, z});
        const uint32_t recount = (uint32_t)(porosity * volume); // updateNumberOfPores
        std::uniform_int_distribution<std::mt19937::result_type> dist(0, recount);
        std::vector<uint32_t> ids(n);
        for (uint32_t i = 0; i < n; i++) ids[i] = (uint32_t)dist(rng);
        for (uint32_t i = 0; i < n; i++)
        {
            size_t id = occupancy != 1.0 ? ids[i] : i;
            if (id >= pores.size())
            {
                id = pores.size() - 1;
                info.clamped++;
            }
            x0[i] = pores[id].x;
            y0[i] = pores[id].y;
            z0[i] = pores[id].z;
        }
        info.occupancy = occupancy;
    }

    if (req.shift > 0)
    {
        // applyVoxelDivision: each walker moves to a random sub-voxel of its voxel
        const uint32_t factor = 1u << req.shift;
        std::uniform_int_distribution<std::mt19937::result_type> d(0, factor - 1);
        for (uint32_t i = 0; i < n; i++)
        {
            int sx = (int)((double)x0[i] * (double)factor + (double)d(rng));
            int sy = (int)((double)y0[i] * (double)factor + (double)d(rng));
            int sz = (int)((double)z0[i] * (double)factor + (double)d(rng));
            x0[i] = sx;
            y0[i] = sy;
            z0[i] = sz;
        }
    }
    return 0;
}

} // namespace rwnmr_host

extern "C" {

int rwnmr_place_walkers(const uint64_t *blocks, int32_t nx, int32_t ny, int32_t nz, const char *mode,
                        int32_t deviation, int32_t shift, uint64_t seed, int64_t n, int32_t *x0, int32_t *y0,
                        int32_t *z0, uint64_t *seed0, rwnmr_placement_info *info)
{
    if (!blocks || nx <= 0 || ny <= 0 || nz <= 0 || n < 0 || n > 0xffffffffll || shift < 0 || shift > 10) return -1;
    std::mt19937 rng;
    rwnmr_host::seed_rng(rng, seed);
    rwnmr_host::PlacementRequest req;
    req.mode = mode ? mode : "random";
    req.deviation = deviation;
    req.shift = shift;
    req.n = n;
    std::vector<int32_t> x, y, z;
    std::vector<uint64_t> s;
    rwnmr_host::PlacementInfo pi;
    std::string err;
    int rc = rwnmr_host::place_walkers(rng, blocks, nx, ny, nz, req, x, y, z, s, pi, err);
    if (info)
    {
        info->pores = pi.pores;
        info->porosity = pi.porosity;
        info->occupancy = pi.occupancy;
        info->clamped = pi.clamped;
    }
    if (rc != 0) return -2;
    if (n > 0)
    {
        std::memcpy(x0, x.data(), (size_t)n * 4);
        std::memcpy(y0, y.data(), (size_t)n * 4);
        std::memcpy(z0, z.data(), (size_t)n * 4);
        std::memcpy(seed0, s.data(), (size_t)n * 8);
    }
    return 0;
}

} // extern "C"
