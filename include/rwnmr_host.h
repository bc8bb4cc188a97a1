/* rwnmr_gb300 host frontend, C ABI: synthetic images, bit-block packing, walker placement,
 * configuration files and the CPMG / PFGSE sequences that drive the GPU engine
 * (include/rwnmr_gb300.h). Host-only code; no function here launches GPU work except the
 * sequence drivers, which call the engine.
 */
#ifndef RWNMR_HOST_H
#define RWNMR_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Overlapping-sphere pore image (the synthetic stand-in for micro-CT images): labels
 * [nz][ny][nx] start as pore (0); solid spheres with uniform centres and radii uniform in
 * [rmin, rmax] are painted until the porosity drops to porosity_target or below. Each sphere
 * gets phase 1..n_phases uniformly (later spheres overwrite earlier ones). Deterministic in
 * `seed` (splitmix64 stream). Returns the number of spheres; *porosity gets the final value. */
int64_t rwnmr_synth_spheres(uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, double rmin, double rmax,
                            double porosity_target, int32_t n_phases, uint64_t seed, double *porosity);

/* Host bit-block packer (BitBlock/bitBlock.cpp:138-221): solid = label != 0. Returns the block
 * count; bdims = {blockColumns, blockRows, blockDepth}; blocks may be NULL to size the output. */
int64_t rwnmr_pack_blocks(const uint8_t *labels, int32_t nx, int32_t ny, int32_t nz, uint64_t *blocks,
                          int32_t *bdims);


/* Walker placement statistics. */
typedef struct rwnmr_placement_info
{
    uint32_t pores;    /* pore voxels considered */
    double porosity;   /* image porosity */
    double occupancy;  /* walkers / pores */
    uint32_t clamped;  /* pore draws one past the end, clamped to the last pore */
} rwnmr_placement_info;

/* Creates n walkers the way NMR_Simulation::setWalkers does (NMR_Simulation.cpp:324-409,
 * 1086-1454): RNG = std::mt19937 seeded with `seed` then discard(4096); one uint64 RNG seed per
 * walker; positions by mode "random" (uniform over pore voxels), "point" (image centre) or
 * "cubic" (centre +- deviation); then voxel division by 2^shift. Positions are in walk units.
 * Returns 0, -1 on bad arguments, -2 if placement is impossible (no pores / point is solid). */
int rwnmr_place_walkers(const uint64_t *blocks, int32_t nx, int32_t ny, int32_t nz, const char *mode,
                        int32_t deviation, int32_t shift, uint64_t seed, int64_t n, int32_t *x0, int32_t *y0,
                        int32_t *z0, uint64_t *seed0, rwnmr_placement_info *info);

/* Configuration files (rwnmr / uct / cpmg / pfgse / multitau) read with the reference's rules (default file
 * under <config_root>default/, then the user file; "KEY: value" lines) and returned as JSON in out
 * (cap bytes). Returns the JSON length, or -1 with the error message in out. */
int rwnmr_config_json(const char *kind, const char *config_root, const char *user_path, char *out, int cap);

/* The command-line driver, the reference's RWNMR (App/rwnmrApp.cpp, Utils/ArgsParser.cpp):
 *   -rwconfig FILE -uctconfig FILE cpmg [-config FILE] pfgse [-config FILE]
 *   multitau [-config MTFILE CPMGFILE | -mtconfig MTFILE | -cpmgconfig CPMGFILE]
 * plus --config-root, --synthetic, --labels/--shape, --device, --quiet. Writes the reference's
 * output files under ./db/<NAME>/. Returns the process exit code. */
int rwnmr_cli_main(int argc, const char *const *argv);

/* Decodes one PNG slice into a solid mask (1 = solid: any colour channel non-zero, as the
 * reference's createBinaryMap treats a colour-loaded slice; NMR_Simulation.cpp:577-617). Call with
 * mask = NULL to get the size. Returns width*height, or -1 with the message in err (errlen bytes). */
int64_t rwnmr_png_solid_mask(const char *path, int32_t *width, int32_t *height, uint8_t *mask, char *err,
                             int32_t errlen);

/* T2 distribution of a CPMG decay (Tikhonov-regularised non-negative inverse Laplace transform),
 * replacing the reference's NMRInverter as NMR_cpmg::applyLaplace runs it
 * (NMR_Simulation/NMR_cpmg.cpp:387-453; Laplace/src/nmrinv_core.cpp, TikhonovSolver.cpp,
 * Laplace/include/NNLS.hpp). Fields are the cpmg config keys of the same names. */
typedef struct rwnmr_t2_config
{
    double min_t2, max_t2;         /* MIN_T2, MAX_T2 (ms) */
    int32_t use_logspace;          /* USE_T2_LOGSPACE */
    int32_t num_t2_bins;           /* NUM_T2_BINS */
    double min_lambda, max_lambda; /* MIN_LAMBDA, MAX_LAMBDA (log10 of the Tikhonov parameter) */
    int32_t num_lambdas;           /* NUM_LAMBDAS */
    int32_t prune_num;             /* PRUNE_NUM (0: no prune-averaging) */
    double noise_amp;              /* NOISE_AMP: std of Gaussian noise added before inverting (0: none) */
    uint64_t noise_seed;           /* seed of that noise (the reference draws it from std::random_device) */
} rwnmr_t2_config;

/* Inverts the decay (times[i], amps[i]), i < n, whose first point is t = 0 (dropped, as the
 * reference does): noise, prune-averaging to prune_num points, the L-curve choice of lambda, NNLS on
 * [K; lambda I]. Writes num_t2_bins bins and amplitudes, the chosen lambda and (nullable) the noise
 * added to each of the n points (noise[0] = 0). Returns num_t2_bins, or -1 with the message in err. */
int32_t rwnmr_t2_invert(const double *times, const double *amps, int32_t n, const rwnmr_t2_config *cfg,
                        double *t2_bins, double *t2_amps, double *lambda, double *noise, char *err, int32_t errlen);

/* The steps of rwnmr_t2_invert, exported for tests and for callers that build their own kernels.
 * Prune-averaging (nmrinv_core.cpp:145-239): returns prune_num and writes prune_num points, or 0 if
 * the decay is not longer than prune_num (no pruning), -1 on bad arguments. */
int32_t rwnmr_t2_prune(const double *times, const double *amps, int32_t n, int32_t prune_num, double *out_times,
                       double *out_amps);
/* L-curve over 10^linspace(min_lambda, max_lambda, num_lambdas) for the column-major m x n kernel a
 * and data b (TikhonovSolver.cpp:14-116): writes the curvature per lambda and the non-zero singular
 * values (count in *n_singular); returns the index of the first curvature maximum, -1 on error. */
int32_t rwnmr_t2_lcurve(const double *a, int32_t m, int32_t n, const double *b, double min_lambda,
                        double max_lambda, int32_t num_lambdas, double *curvature, double *singular_values,
                        int32_t *n_singular);
/* Non-negative least squares min ||a x - b||, x >= 0, a column-major m x n (Lawson-Hanson, the
 * algorithm of Laplace/include/NNLS.hpp:289-406). max_solves <= 0: 50 (n + 1). Returns the number of
 * least-squares solves, or -1 (bad arguments or no convergence). */
int32_t rwnmr_nnls(const double *a, int32_t m, int32_t n, const double *b, double *x, int32_t max_solves);

#ifdef __cplusplus
}
#endif
#endif
