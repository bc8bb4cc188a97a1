// Internal C++ interfaces of the host frontend (not part of the C ABI).
#pragma once
#include <cstdint>
#include <random>
#include <string>
#include <vector>

namespace rwnmr_host
{

// The reference seeds its static std::mt19937 with SEED (a random value when SEED is 0) and
// discards 4096 outputs (NMR_Simulation.cpp:86-95).
inline void seed_rng(std::mt19937 &rng, uint64_t seed)
{
    if (seed == 0)
    {
        std::random_device dev;
        seed = ((uint64_t)dev() << 32) | dev();
    }
    rng.seed((std::mt19937::result_type)seed);
    rng.discard(4096);
}

struct PlacementRequest
{
    std::string mode = "random"; // WALKERS_PLACEMENT: random | point | cubic
    int deviation = 0;           // PLACEMENT_DEVIATION
    int shift = 0;               // log2(VOXEL_DIVISION factor)
    int64_t n = 0;
};

struct PlacementInfo
{
    uint32_t pores = 0;
    double porosity = 0.0;
    double occupancy = 0.0;
    uint32_t clamped = 0;
};

int place_walkers(std::mt19937 &rng, const uint64_t *blocks, int nx, int ny, int nz, const PlacementRequest &req,
                  std::vector<int32_t> &x0, std::vector<int32_t> &y0, std::vector<int32_t> &z0,
                  std::vector<uint64_t> &seed0, PlacementInfo &info, std::string &err);

} // namespace rwnmr_host
