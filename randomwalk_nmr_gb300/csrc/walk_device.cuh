// Device-side walker step for the GB300 walker engine.
//
// One walker step is the reference's Walker::walk_3D / map_3D (Walker/walker.cpp:197-231) and the
// CUDA CPMG_walk_* / map_3D_* / PFG_map_* kernels (NMR_cpmg_cuda.cpp:37-139, 300-402, 574-676):
//   xorshift64 -> direction (state mod 6) -> [noflux: reverse a move off the image] -> next
//   position -> image-space lookup -> bit test in the 4x4x4 bit-block -> move, or count a
//   collision on the solid voxel's phase.
// The formulation here is branch-free integer code:
//   * the direction (the reference's digit-sum mod6 of the state, walker.h:566-582) is drawn as the
//     slot 2 ((-a) mod 3) + (a mod 2) (dir_slot): the same six outcomes, one slot per direction, with
//     the remainder by 3 on the multiplier.
//   * periodic and mirror boundaries keep the image-space coordinate incrementally (wrap, or
//     stay-and-flip the tile orientation) instead of the per-step modulo of
//     NMR_cpmg_cuda.cpp:1991-2015; positions stay unwrapped like the reference's.
//   * voxel division (shift > 0) takes the general path that applies the reference's formulas.
#pragma once
#include <cstdint>

namespace rwnmr
{

enum
{
    BC_NOFLUX = 0,
    BC_PERIODIC = 1,
    BC_MIRROR = 2,
    BC_GENERIC = 3 // any bc with voxel division: runtime bc, reference formulas
};

// Bit-block image on the device, read as 32-bit halves: block b occupies 2W uint32 at 2W*b, half h
// (bits 32h..32h+31 of the 4x4x4 block) at 2W*b + W*h, as W words: the solid mask, then (multi-
// phase images, W = 2 or 4) bit-planes of the solid voxel's phase index. For W = 1 this is the
// reference's uint64 block array itself (little-endian halves); for W > 1 one aligned 8- or
// 16-byte load returns the solid bit and the phase bits of a voxel. Blocks are indexed in 32 bits
// (images of fewer than 2^31 blocks, checked on the host).
// Morton (bit-interleaved) copy of the image for the noflux walk without voxel division. A voxel's
// index P interleaves the bits of x, y and z (each axis padded to a power of two; masks mx, my, mz
// give each axis' bit positions). Word w holds the solid bits of voxels P = 32w .. 32w + 31, followed
// by W - 1 phase bit-planes, so a step's gather address is P >> 5 and its bit P & 31. A move along one
// axis is an increment or decrement of that axis' bit field alone ("dilated" arithmetic:
// ((P | ~m) + 1) & m steps the field up, ((P & m) - 1) & m down), and the noflux edge test compares
// the field with the dilated coordinate of the last voxel (dilation preserves order).
struct MortonImage
{
    const uint32_t *__restrict__ words = nullptr; // null: no Morton copy
    uint32_t mx = 0, my = 0, mz = 0;              // bit masks of each axis in P
    uint32_t ex = 0, ey = 0, ez = 0;              // dilated coordinate n - 1 along each axis
};

struct DevImage
{
    const uint64_t *__restrict__ blocks;
    int32_t nx, ny, nz;
    int32_t bcols;
    int32_t bcr; // bcols * brows
    int32_t bc;  // runtime boundary condition (BC_GENERIC path)
    int32_t shift;
    MortonImage mi;
};

// Scatters the low bits of v onto the set bits of mask (lowest first), and gathers them back.
__host__ __device__ inline uint32_t dilate_bits(uint32_t v, uint32_t mask)
{
    uint32_t r = 0;
    for (uint32_t m = mask; m; m &= m - 1)
    {
        if (v & 1u) r |= m & (~m + 1u);
        v >>= 1;
    }
    return r;
}
__host__ __device__ inline uint32_t undilate_bits(uint32_t p, uint32_t mask)
{
    uint32_t r = 0, bit = 1;
    for (uint32_t m = mask; m; m &= m - 1, bit <<= 1)
        if (p & m & (~m + 1u)) r |= bit;
    return r;
}

// 64-bit words per bit-block for NP phase slots (1, 2 or 4).
template <int NP>
struct WordsPerBlock
{
    static constexpr int value = NP == 1 ? 1 : (NP == 2 ? 2 : 4);
};

__device__ __forceinline__ uint64_t xorshift64(uint64_t x)
{
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return x;
}

// Direction slot of the xorshift state a: 2 ((-a) mod 3) + (a mod 2). The 32-bit fold t = lo + hi (+ carry)
// keeps a mod 3 (2^32 = 1 mod 3), and for t = 3k + r the product t * 0xAAAAAAAB (the inverse of 3 mod 2^32)
// is k + r * 0xAAAAAAAB mod 2^32, which lies in [0, 0x55555555] for r = 0, in [0x55555556, 0xAAAAAAAA] for
// r = 2 and in [0xAAAAAAAB, 2^32) for r = 1 (k <= 0x55555554 for r > 0): its high product by 3 is (-r) mod 3.
// Slot s stands for the direction a mod 6 = r6 with r6 = -(s >> 1) (mod 3) and r6 = s (mod 2):
// 0:N(-y) 1:E(+x) 2:S(+y) 3:Down(-z) 4:Up(+z) 5:W(-x) (reference numbering 0:N 1:W 2:S 3:E 4:Up 5:Down).
__device__ __forceinline__ uint32_t dir_slot(uint64_t a)
{
    const uint32_t lo = (uint32_t)a, hi = (uint32_t)(a >> 32);
    uint32_t t = lo + hi;
    t += (t < lo) ? 1u : 0u;
    return 2u * __umulhi(t * 0xAAAAAAABu, 3u) + (lo & 1u);
}

// Reference periodic / mirror image index for the generic path (NMR_cpmg_cuda.cpp:1991-2015).
__device__ __forceinline__ int map_periodic(int local, int shift, int dim)
{
    int g = (local >> shift) % dim;
    return g < 0 ? g + dim : g;
}
__device__ __forceinline__ int map_mirror(int local, int shift, int dim)
{
    int g = local >> shift;
    int img = g % dim;
    if (img < 0) img += dim;
    int mirror = (g > 0) ? (g / dim) % 2 : ((-g - 1 + dim) / dim) % 2;
    return mirror ? (dim - 1 - img) : img;
}
// Tile orientation (+1 / -1) of a mirrored coordinate, used to seed the incremental mirror path.
__device__ __forceinline__ int mirror_orientation(int g, int dim)
{
    int mirror = (g > 0) ? (g / dim) % 2 : ((-g - 1 + dim) / dim) % 2;
    return mirror ? -1 : 1;
}

// Walker position: real (unwrapped) walk-grid coordinates plus, for periodic/mirror without
// voxel division, the image coordinates and mirror orientations carried incrementally.
struct WalkerPos
{
    int x, y, z;
    int ix, iy, iz;
    int ox, oy, oz;
};

template <int BC>
__device__ __forceinline__ void init_image_coords(const DevImage &im, WalkerPos &p)
{
    if (BC == BC_PERIODIC)
    {
        p.ix = map_periodic(p.x, 0, im.nx);
        p.iy = map_periodic(p.y, 0, im.ny);
        p.iz = map_periodic(p.z, 0, im.nz);
    }
    else if (BC == BC_MIRROR)
    {
        p.ix = map_mirror(p.x, 0, im.nx);
        p.iy = map_mirror(p.y, 0, im.ny);
        p.iz = map_mirror(p.z, 0, im.nz);
        p.ox = mirror_orientation(p.x, im.nx);
        p.oy = mirror_orientation(p.y, im.ny);
        p.oz = mirror_orientation(p.z, im.nz);
    }
    else
    {
        p.ix = p.x;
        p.iy = p.y;
        p.iz = p.z;
    }
}

// Image voxel of the walker's current position: pos >> shift (noflux), the periodic / mirrored
// image index otherwise (NMR_cpmg_cuda.cpp:1986-2015).
template <int BC>
__device__ __forceinline__ void current_voxel(const DevImage &im, const WalkerPos &p, int &ix, int &iy, int &iz)
{
    if (BC == BC_NOFLUX)
    {
        ix = p.x;
        iy = p.y;
        iz = p.z;
    }
    else if (BC == BC_PERIODIC || BC == BC_MIRROR)
    {
        ix = p.ix;
        iy = p.iy;
        iz = p.iz;
    }
    else
    {
        const int s = im.shift;
        if (im.bc == BC_PERIODIC)
        {
            ix = map_periodic(p.x, s, im.nx);
            iy = map_periodic(p.y, s, im.ny);
            iz = map_periodic(p.z, s, im.nz);
        }
        else if (im.bc == BC_MIRROR)
        {
            ix = map_mirror(p.x, s, im.nx);
            iy = map_mirror(p.y, s, im.ny);
            iz = map_mirror(p.z, s, im.nz);
        }
        else
        {
            ix = p.x >> s;
            iy = p.y >> s;
            iz = p.z >> s;
        }
    }
}

// Solid bit of an image voxel (solid word of its block half).
template <int W>
__device__ __forceinline__ bool voxel_solid(const DevImage &im, int ix, int iy, int iz)
{
    const uint32_t blk = (uint32_t)(ix >> 2) + (uint32_t)(iy >> 2) * (uint32_t)im.bcols + (uint32_t)(iz >> 2) * (uint32_t)im.bcr;
    const uint32_t bit = (uint32_t)((ix & 3) | ((iy & 3) << 2) | ((iz & 3) << 4));
    const uint32_t *bp = reinterpret_cast<const uint32_t *>(im.blocks) + (size_t)blk * (2 * W) + (bit >> 5) * W;
    return ((__ldg(bp) >> (bit & 31u)) & 1u) != 0;
}

// Returns true if a walker may start at p: inside the image for noflux (in walk units).
template <int BC>
__device__ __forceinline__ bool start_ok(const DevImage &im, const WalkerPos &p)
{
    if (BC == BC_NOFLUX || (BC == BC_GENERIC && im.bc == BC_NOFLUX))
    {
        int s = (BC == BC_GENERIC) ? im.shift : 0;
        return (unsigned)(p.x >> s) < (unsigned)im.nx && (unsigned)(p.y >> s) < (unsigned)im.ny &&
               (unsigned)(p.z >> s) < (unsigned)im.nz && p.x >= 0 && p.y >= 0 && p.z >= 0;
    }
    return true;
}

// One step. On return `wall` tells whether the move was rejected; if so `phase` is the solid
// voxel's phase index (0 for single-phase images). W = words per block.
template <int BC, int W>
__device__ __forceinline__ void walker_step(const DevImage &im, WalkerPos &p, uint64_t &seed, bool &wall, int &phase)
{
    seed = xorshift64(seed);
    const uint32_t r = dir_slot(seed); // 0:N(-y) 1:E(+x) 2:S(+y) 3:Down(-z) 4:Up(+z) 5:W(-x)
    int dx = (r == 1u) - (r == 5u);
    int dy = (r == 2u) - (r == 0u);
    int dz = (r == 4u) - (r == 3u);

    int tx, ty, tz;    // candidate real position
    int cix, ciy, ciz; // candidate image position
    int cox = 0, coy = 0, coz = 0;
    if (BC == BC_NOFLUX)
    {
        // A move off the image is reversed (walker.h:444-491): the walker steps inward.
        if ((unsigned)(p.x + dx) >= (unsigned)im.nx) dx = -dx;
        if ((unsigned)(p.y + dy) >= (unsigned)im.ny) dy = -dy;
        if ((unsigned)(p.z + dz) >= (unsigned)im.nz) dz = -dz;
        tx = p.x + dx;
        ty = p.y + dy;
        tz = p.z + dz;
        cix = tx;
        ciy = ty;
        ciz = tz;
    }
    else if (BC == BC_PERIODIC)
    {
        tx = p.x + dx;
        ty = p.y + dy;
        tz = p.z + dz;
        cix = p.ix + dx;
        ciy = p.iy + dy;
        ciz = p.iz + dz;
        cix = cix < 0 ? im.nx - 1 : (cix >= im.nx ? 0 : cix);
        ciy = ciy < 0 ? im.ny - 1 : (ciy >= im.ny ? 0 : ciy);
        ciz = ciz < 0 ? im.nz - 1 : (ciz >= im.nz ? 0 : ciz);
    }
    else if (BC == BC_MIRROR)
    {
        tx = p.x + dx;
        ty = p.y + dy;
        tz = p.z + dz;
        // Crossing a tile edge keeps the image index and flips the tile orientation.
        cix = p.ix + p.ox * dx;
        ciy = p.iy + p.oy * dy;
        ciz = p.iz + p.oz * dz;
        cox = p.ox;
        coy = p.oy;
        coz = p.oz;
        if ((unsigned)cix >= (unsigned)im.nx) { cix = p.ix; cox = -p.ox; }
        if ((unsigned)ciy >= (unsigned)im.ny) { ciy = p.iy; coy = -p.oy; }
        if ((unsigned)ciz >= (unsigned)im.nz) { ciz = p.iz; coz = -p.oz; }
    }
    else // BC_GENERIC: voxel division, reference formulas (NMR_cpmg_cuda.cpp:1847-2015)
    {
        const int s = im.shift;
        if (im.bc == BC_NOFLUX)
        {
            if ((unsigned)((p.x >> s) + dx) >= (unsigned)im.nx) dx = -dx;
            if ((unsigned)((p.y >> s) + dy) >= (unsigned)im.ny) dy = -dy;
            if ((unsigned)((p.z >> s) + dz) >= (unsigned)im.nz) dz = -dz;
        }
        tx = p.x + dx;
        ty = p.y + dy;
        tz = p.z + dz;
        if (im.bc == BC_PERIODIC)
        {
            cix = map_periodic(tx, s, im.nx);
            ciy = map_periodic(ty, s, im.ny);
            ciz = map_periodic(tz, s, im.nz);
        }
        else if (im.bc == BC_MIRROR)
        {
            cix = map_mirror(tx, s, im.nx);
            ciy = map_mirror(ty, s, im.ny);
            ciz = map_mirror(tz, s, im.nz);
        }
        else
        {
            cix = tx >> s;
            ciy = ty >> s;
            ciz = tz >> s;
        }
    }

    const uint32_t blk = (uint32_t)(cix >> 2) + (uint32_t)(ciy >> 2) * (uint32_t)im.bcols + (uint32_t)(ciz >> 2) * (uint32_t)im.bcr;
    const uint32_t bit = (uint32_t)((cix & 3) | ((ciy & 3) << 2) | ((ciz & 3) << 4));
    const uint32_t sh = bit & 31u;
    const uint32_t *bp = reinterpret_cast<const uint32_t *>(im.blocks) + (size_t)blk * (2 * W) + (bit >> 5) * W;
    uint32_t solid;
    phase = 0;
    if (W == 1)
    {
        solid = __ldg(bp);
    }
    else if (W == 2)
    {
        const uint2 v = __ldg(reinterpret_cast<const uint2 *>(bp));
        solid = v.x;
        phase = (int)((v.y >> sh) & 1u);
    }
    else
    {
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(bp));
        solid = v.x;
        phase = (int)(((v.y >> sh) & 1u) | (((v.z >> sh) & 1u) << 1) | (((v.w >> sh) & 1u) << 2));
    }
    wall = ((solid >> sh) & 1u) != 0;
    if (!wall)
    {
        p.x = tx;
        p.y = ty;
        p.z = tz;
        if (BC == BC_PERIODIC || BC == BC_MIRROR)
        {
            p.ix = cix;
            p.iy = ciy;
            p.iz = ciz;
        }
        if (BC == BC_MIRROR)
        {
            p.ox = cox;
            p.oy = coy;
            p.oz = coz;
        }
    }
}

// Per direction r (0:N(-y) 1:W(-x) 2:S(+y) 3:E(+x) 4:Up(+z) 5:Down(-z)) of the Morton walk: the moving
// axis' bit mask m, the field value at which the move is reversed (the last voxel for a move up, 0 for
// a move down), and the steps to subtract from the axis field f = P & m for the move and for its
// reversal: in dilated arithmetic (f - m) & m is f + 1 and (f - 1) & m is f - 1. Kept in shared
// memory, so that decoding a direction is one lookup instead of integer compares and selects.
// The Morton walks index this table by the direction slot of the state (dir_slot); slot s stands for
// the direction r with r = -(s >> 1) (mod 3) and r = s (mod 2).
__host__ __device__ inline int morton_slot_direction(int slot)
{
    const int r3 = (3 - (slot >> 1)) % 3;
    return r3 + 3 * ((r3 ^ slot) & 1);
}

__host__ __device__ inline uint4 morton_direction(const MortonImage &mi, int slot)
{
    const int r = morton_slot_direction(slot);
    const uint32_t m = r >= 4 ? mi.mz : ((r & 1) ? mi.mx : mi.my);
    const bool up = r == 2 || r == 3 || r == 4;
    const uint32_t edge = up ? (r >= 4 ? mi.ez : ((r & 1) ? mi.ex : mi.ey)) : 0u;
    return make_uint4(m, edge, up ? m : 1u, up ? 1u : m);
}

// One noflux step on the Morton copy (see MortonImage): the same xorshift64 draw, direction and
// reversal rule as walker_step<BC_NOFLUX>, with the position held as the Morton index P. dirs: the
// six morton_direction entries, by slot.
template <int W>
__device__ __forceinline__ void morton_step(const MortonImage &mi, const uint4 *dirs, uint32_t &P, uint64_t &seed,
                                            bool &wall, int &phase)
{
    seed = xorshift64(seed);
    const uint4 d = dirs[dir_slot(seed)];
    const uint32_t f = P & d.x;
    // a move off the image is reversed (walker.h:444-491): a move up at the last voxel goes down, a
    // move down at voxel 0 goes up (every axis has at least two voxels)
    const uint32_t step = f == d.y ? d.w : d.z;
    const uint32_t Pn = ((f - step) & d.x) | (P & ~d.x);
    const uint32_t *wp = mi.words + (size_t)(Pn >> 5) * W;
    // bit Pn & 31 of each word: funnel shifts use the low five bits of the shift
    uint32_t solid;
    phase = 0;
    if (W == 1)
    {
        solid = __ldg(wp);
    }
    else if (W == 2)
    {
        const uint2 v = __ldg(reinterpret_cast<const uint2 *>(wp));
        solid = v.x;
        phase = (int)(__funnelshift_r(v.y, v.y, Pn) & 1u);
    }
    else
    {
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(wp));
        solid = v.x;
        phase = (int)((__funnelshift_r(v.y, v.y, Pn) & 1u) | ((__funnelshift_r(v.z, v.z, Pn) & 1u) << 1) |
                      ((__funnelshift_r(v.w, v.w, Pn) & 1u) << 2));
    }
    wall = (__funnelshift_r(solid, solid, Pn) & 1u) != 0;
    if (!wall) P = Pn;
}

// Fixed-point energy (scale 2^63) of a walker with per-phase collision counts c[]: the product of
// the per-phase tables, each table[n] = round(f^n * 2^63) with f^n the FP64 repeated product.
__device__ __forceinline__ uint64_t fx_mul(uint64_t a, uint64_t b)
{
    // floor(a b / 2^63) = floor(2a b / 2^64) for a < 2^63; a = 2^63 (the value 1) returns b
    return a >> 63 ? b : __umul64hi(a << 1, b);
}

template <int NP>
__device__ __forceinline__ uint64_t energy_fx(const uint64_t *__restrict__ tfx, int tstride, const uint32_t *c)
{
    uint64_t e = __ldg(tfx + c[0]);
#pragma unroll
    for (int q = 1; q < NP; q++) e = fx_mul(e, __ldg(tfx + (size_t)q * tstride + c[q]));
    return e;
}

template <int NP>
__device__ __forceinline__ double energy_fp64(const double *__restrict__ t, int tstride, const uint32_t *c)
{
    double e = __ldg(t + c[0]);
#pragma unroll
    for (int q = 1; q < NP; q++) e = e * __ldg(t + (size_t)q * tstride + c[q]);
    return e;
}

} // namespace rwnmr
