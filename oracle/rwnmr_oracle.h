/* CPU restatement of RandomWalk_NMR's walker hot path -- TEST ORACLE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline/reference legs may load
 * this library, and only as the checker or the timed CPU baseline. The product path
 * (randomwalk_nmr_gb300) never calls it.
 *
 * Parity is pinned: tests/test_oracle_vs_reference.py checks this restatement against the
 * reference's own CPU code compiled by this directory's Makefile (oracle/_ref), and
 * tests/test_oracle_golden.py against fixtures generated from that build
 * (tests/golden/make_golden.py). Periodic/mirror boundaries and voxel division exist only in
 * the reference's CUDA kernels; those are restated from NMR_cpmg_cuda.cpp:1986-2015 and are
 * pinned by the bit-exact GPU parity tests, not by a CPU run of the reference.
 */
#ifndef RWNMR_ORACLE_H
#define RWNMR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BC_NOFLUX = 0, ORC_BC_PERIODIC = 1, ORC_BC_MIRROR = 2 };

/* Pore image: bit-blocks (solid = 1) plus an optional uint8 label volume [nz][ny][nx]
 * (0 = pore, p >= 1 = solid of phase p-1) for the multi-phase extension. */
typedef struct orc_image
{
    const uint64_t *blocks;
    const uint8_t *labels; /* NULL: single phase */
    int32_t nx, ny, nz;
    int32_t bcols, brows, bdepth;
    int32_t n_phases;
} orc_image;

/* Packs labels (non-zero = solid) into 4x4x4 bit-blocks; returns the block count and writes
 * bdims[3] = {blockColumns, blockRows, blockDepth}. blocks may be NULL to query the size. */
int64_t orc_pack_blocks(const uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, uint64_t *blocks, int32_t *bdims);

uint64_t orc_xorshift64(uint64_t state);
uint32_t orc_mod6(uint64_t a);

/* Fixed-point energy tables: table[n] = round(T[n] * 2^63), T[0] = 1, T[n] = T[n-1] * f (FP64). */
void orc_energy_table(double f, int32_t n_max, double *t_fp64, uint64_t *t_fx);

/* CPMG / mapping walk of n walkers for n_echoes * steps_per_echo steps from the given state.
 *   dfactor[p]     per-phase decrease factor f_p
 *   echo_fp64      [n_echoes+1] serial FP64 sum of walker energies (index 0 = initial state)
 *   echo_fx        [(n_echoes+1)*3] exact fixed-point sums, three limbs per echo (bits 0-20,
 *                  21-41, 42-63 of each walker's 2^63-scaled energy, summed separately)
 *   echo_coll      [n_echoes*n_phases] collisions gained during each echo, per phase
 *   final state    positions, current seeds, per-walker per-phase collision totals [n*n_phases]
 * Any output pointer may be NULL. threads > 1 splits walkers across OpenMP threads (the FP64
 * sum is then no longer in serial walker order). Returns 0, or -1 on bad arguments. */
int orc_cpmg(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0, const int32_t *y0,
             const int32_t *z0, const uint64_t *seed0, int32_t n_echoes, int32_t steps_per_echo,
             const double *dfactor, double *echo_fp64, uint64_t *echo_fx, uint64_t *echo_coll, int32_t *xf,
             int32_t *yf, int32_t *zf, uint64_t *seedf, uint32_t *collf, int32_t threads);

/* PFGSE walk: walkers walk cumulatively to steps[i] (non-decreasing) and, at each exposure time,
 * every gradient point j gets M[i*n_g+j] = sum_w E_w cos((k_j . dR_w) * res) with E_w = prod_p T_p[c_p]
 * and dR the displacement from the start (NMR_pfgse.cpp:1747-1765). Also per exposure time:
 * esum[i] = sum_w E_w; msd[i*3+a] = sum_w dR_a^2 (integer, per axis);
 * esum_fx[i*3..] the fixed-point energy sum limbs. Any output may be NULL. */
int orc_pfgse(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0, const int32_t *y0,
              const int32_t *z0, const uint64_t *seed0, const double *dfactor, int32_t n_delta, const int32_t *steps,
              int32_t n_g, const double *kvec, double res, double *M, double *esum, uint64_t *msd, uint64_t *esum_fx,
              int32_t threads);

// dM/dg of the PFGSE phase sums along a gradient ramp k_j = kscale g_j dir (FP64, pathwise).
int orc_pfgse_grad_g(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0,
                     const int32_t *y0, const int32_t *z0, const uint64_t *seed0, const double *dfactor,
                     int32_t n_delta, const int32_t *steps, int32_t n_g, const double *kvec, double res, double kscale,
                     const double *dir, double *dMdg, int32_t threads);

/* The reference's uniform internal field (NMR_Simulation/InternalField.cpp, fillDataArray):
 * out[(z*ny + y)*nx + x] = coord * dG in pore voxels and 0 in solid ones, coord the voxel's
 * x, y or z (direction 0/1/2) and dG = gradient * 1e-6 * resolution. */
void orc_uniform_field(const orc_image *img, double resolution, double gradient, int32_t direction, double *out);

/* CPMG walk in an internal magnetic field (NMR_cpmg_cuda.cpp:146-293 noflux, 409-567 periodic,
 * 683-838 mirror). Each echo is two inversions of steps_per_echo/2 steps; an inversion negates
 * the phase, and every step adds gammatau * field at the walker's voxel before and after the
 * move, each addition one fused multiply-add (nvcc's contraction of `phase += gammatau *
 * field[i]`). A rejected move counts a collision on the solid's phase; the walker's energy after
 * an echo is prod_p T_p[c_p] * cos(phase).
 *   field        [nz][ny][nx] values at image voxels, or NULL for the uniform field of
 *                orc_uniform_field with dG = dg along axis `axis`, evaluated voxel by voxel
 *   walker_dfactor  [n] per-walker decrease factors (single phase: pAlive *= f_w per collision,
 *                the reference's own update), or NULL for the per-phase tables of dfactor
 *   echo_fp64    [n_echoes+1] serial FP64 sum of walker energies
 *   echo_fx      [(n_echoes+1)*3] limb sums (bits 0-20, 21-41, 42-62) of round(E * 2^61) + 2^61
 *   final state  positions, seeds, collisions [n*n_phases], phases [n]
 * Any output may be NULL. Returns 0, or -1 on bad arguments. */
int orc_cpmg_field(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0, const int32_t *y0,
                   const int32_t *z0, const uint64_t *seed0, int32_t n_echoes, int32_t steps_per_echo,
                   const double *dfactor, const double *walker_dfactor, double gammatau, const double *field,
                   double dg, int32_t axis, double *echo_fp64, uint64_t *echo_fx, int32_t *xf, int32_t *yf,
                   int32_t *zf, uint64_t *seedf, uint32_t *collf, double *phasef, int32_t threads);

/* Per-walker displacements after a PFGSE-style walk of `steps` steps (for histogram checks). */
int orc_displacements(const orc_image *img, int32_t bc, int32_t shift, int64_t n, const int32_t *x0,
                      const int32_t *y0, const int32_t *z0, const uint64_t *seed0, int32_t steps, int32_t *dx,
                      int32_t *dy, int32_t *dz, uint32_t *collf, int32_t threads);

// Synthetic sphere-pack labels [nz][ny][nx] (0 = pore) for the CPU reference arm; returns the
// sphere count, or -1 on bad arguments.
int64_t orc_synth_spheres(uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, double rmin, double rmax,
                          double porosity, int32_t n_phases, uint64_t seed, double *porosity_out);

// The reference's random walker placement (seeds, then pore ids, then sub-voxel offsets).
// Returns 0, -1 on bad arguments, -2 for an image without pores.
int orc_place_walkers_random(const uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, uint64_t seed, int64_t n,
                             int32_t shift, int32_t *x0, int32_t *y0, int32_t *z0, uint64_t *seed0, int64_t *clamped);

#ifdef __cplusplus
}
#endif
#endif
