/* rwnmr_gb300 -- GB300-native random-walk NMR walker engine, C ABI.
 *
 * Drop-in boundary for the walker hot path of RandomWalk_NMR. The reference has no FFI of its
 * own: its walks sit behind three C++ dispatch points, which these entry points replace:
 *   NMR_Simulation::mapSimulation()   (NMR_Simulation/NMR_Simulation.h:264-267,
 *                                      NMR_Simulation.cpp:1522-1539)  -> rwnmr_map_run
 *   NMR_cpmg::run_simulation()        (NMR_Simulation/NMR_cpmg.cpp:149-175;
 *                                      image_simulation_cuda/_omp)     -> rwnmr_cpmg_run
 *   NMR_PFGSE::simulation()           (NMR_Simulation/NMR_pfgse.cpp:593-603;
 *                                      simulation_cuda/_omp)           -> rwnmr_pfgse_run
 * The host-side setup those methods read (NMR_Simulation::bitBlock, walkers[].initialPosition /
 * initialSeed / decreaseFactor; NMR_Simulation.cpp:619-633, 1139-1333) is passed in through
 * rwnmr_image_upload and rwnmr_walkers_upload.
 *
 * Conventions
 *  - Every call returns an rwnmr_status; on failure rwnmr_last_error() describes it. The
 *    reference prints and exit(1)s instead and checks no CUDA errors.
 *  - Host pointers are caller-owned and only read or written during the call. The context owns
 *    all device memory. No call resets the device (the reference's cudaDeviceReset() is not
 *    reproduced: it would tear down other users of the same CUDA context).
 *  - One context per host thread; calls on one context are serialised on its CUDA stream.
 *  - There is no CPU fallback: without a usable CUDA device rwnmr_ctx_create fails.
 */
#ifndef RWNMR_GB300_H
#define RWNMR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rwnmr_status
{
    RWNMR_OK = 0,
    RWNMR_ERR_INVALID = 1,     /* bad argument or size */
    RWNMR_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    RWNMR_ERR_NOMEM = 3,       /* device allocation failed */
    RWNMR_ERR_STATE = 4,       /* call out of order (e.g. no image uploaded) */
    RWNMR_ERR_UNSUPPORTED = 5, /* valid request this build does not handle */
    RWNMR_ERR_DEVICE = 6,      /* the kernel reported a fault through its status word */
    RWNMR_ERR_CANCELLED = 7,   /* a batch walk stopped on rwnmr_batch_cancel (no results) */
    RWNMR_ERR_TIMEOUT = 8      /* a batch walk stopped at its time budget (no results) */
} rwnmr_status;

/* Boundary conditions (rwnmr.config BC; ConfigFiles/rwnmr_config.cpp:228-240). */
enum
{
    RWNMR_BC_NOFLUX = 0,
    RWNMR_BC_PERIODIC = 1,
    RWNMR_BC_MIRROR = 2
};

typedef struct rwnmr_ctx rwnmr_ctx;

/* ---- context --------------------------------------------------------------------------- */
rwnmr_status rwnmr_ctx_create(rwnmr_ctx **out, int device);
void rwnmr_ctx_destroy(rwnmr_ctx *ctx);
const char *rwnmr_last_error(const rwnmr_ctx *ctx);
const char *rwnmr_version(void);
/* Runs subsequent work on an external cudaStream_t (NULL restores the context's own stream). */
rwnmr_status rwnmr_ctx_set_stream(rwnmr_ctx *ctx, void *cuda_stream);

/* Device allocator of the engine contexts' buffers (images, walkers, tables, accumulators): by
 * default cudaMalloc / cudaFree; after this call, alloc(bytes, user) / free_fn(ptr, user) for every
 * allocation made from then on by any context in the process (a buffer is always freed by the
 * allocator that made it). alloc must return device memory of the context's device, aligned to at
 * least 256 bytes and usable on the context's stream, or NULL: the call that needed it then fails
 * with RWNMR_ERR_NOMEM and the context stays usable. Both NULL restores cudaMalloc / cudaFree; one
 * NULL is RWNMR_ERR_INVALID. For frameworks that own the GPU's memory (a caching allocator) and for
 * allocation-failure tests. Batch objects allocate with cudaMalloc. */
typedef void *(*rwnmr_alloc_fn)(size_t bytes, void *user);
typedef void (*rwnmr_free_fn)(void *ptr, void *user);
rwnmr_status rwnmr_set_device_allocator(rwnmr_alloc_fn alloc, rwnmr_free_fn free_fn, void *user);
/* Kernels launched by this context so far (for launch accounting). */
int64_t rwnmr_ctx_launch_count(const rwnmr_ctx *ctx);
/* Device-side duration of the last walk kernel(s) of the last run call, in milliseconds. */
double rwnmr_ctx_last_kernel_ms(const rwnmr_ctx *ctx);

/* ---- image ----------------------------------------------------------------------------- */
/* Bit-block image (BitBlock/bitBlock.cpp:138-221): blocks[bx + by*bcols + bz*bcols*brows],
 * bit (x%4) + 4*(y%4) + 16*(z%4) set for solid voxels, bcols = ceil(nx/4) etc.
 * labels (nullable): uint8 [nz][ny][nx], 0 = pore, p = solid of material phase p (1..n_phases);
 * must agree with blocks. Multi-phase labels extend the reference (its image is binary). With
 * n_phases > 1 a label above n_phases is rejected (RWNMR_ERR_INVALID); with n_phases = 1 every
 * non-zero label is solid. */
rwnmr_status rwnmr_image_upload(rwnmr_ctx *ctx, const uint64_t *blocks, int32_t nx, int32_t ny, int32_t nz,
                                const uint8_t *labels, int32_t n_phases);
/* Same from a label volume alone; the bit-blocks are packed on the GPU. */
rwnmr_status rwnmr_image_upload_labels(rwnmr_ctx *ctx, const uint8_t *labels, int32_t nx, int32_t ny, int32_t nz,
                                       int32_t n_phases);
/* Reads back the packed bit-blocks (ceil(nx/4)*ceil(ny/4)*ceil(nz/4) words). */
rwnmr_status rwnmr_image_download_blocks(rwnmr_ctx *ctx, uint64_t *blocks);
/* 1 if the uploaded image also has a Morton (bit-interleaved) copy, which the noflux walks without
 * voxel division use (CPMG, PFGSE, the adjoint; built when the power-of-two box around the image
 * holds at most four times its voxels or the copy takes at most 48 MB); 0 otherwise. Results do not
 * depend on it. */
int32_t rwnmr_image_layout(const rwnmr_ctx *ctx);
/* allow_morton = 0: later image uploads build no Morton copy (saves its memory; the walks then use
 * the bit-blocks). Default 1. No counterpart in the reference. */
rwnmr_status rwnmr_ctx_set_image_layout(rwnmr_ctx *ctx, int32_t allow_morton);

/* ---- walkers --------------------------------------------------------------------------- */
/* Initial state (Walker::initialPosition / initialSeed). Positions are in walk units (voxels
 * << voxel-division shift). The engine stores the walkers sorted by a coarse Morton key of their
 * start voxel (a stable sort on the GPU), so that neighbouring threads walk neighbouring walkers;
 * every per-walker input and output of this API is in the upload order. */
rwnmr_status rwnmr_walkers_upload(rwnmr_ctx *ctx, int64_t n, const int32_t *x0, const int32_t *y0, const int32_t *z0,
                                  const uint64_t *seed0);
/* State after the last run: positions, current RNG state, per-phase collision totals
 * ([n][n_phases]). Any pointer may be NULL. */
rwnmr_status rwnmr_walkers_download(rwnmr_ctx *ctx, int32_t *x, int32_t *y, int32_t *z, uint64_t *seed,
                                    uint32_t *collisions);
/* Checkpoint / resume: sets the current walker state from arrays in the layout rwnmr_walkers_download
 * returns (upload order; collisions [n][n_phases]) -- typically a checkpoint of an earlier walk of
 * the same walkers, in this or another process. The initial positions and seeds stay those of
 * rwnmr_walkers_upload. rwnmr_map_continue then resumes the walk exactly where the checkpoint left
 * it (a walk is a function of this state alone). No counterpart in the reference, whose walkers
 * re-derive their state from initialSeed and initialPosition. */
rwnmr_status rwnmr_walkers_restore(rwnmr_ctx *ctx, const int32_t *x, const int32_t *y, const int32_t *z,
                                   const uint64_t *seed, const uint32_t *collisions);

/* Per-walker decrease factors [n], each in [0, 1]: the reference's Walker::decreaseFactor when it
 * differs between walkers (RHO_TYPE: sigmoid, where each walker's relaxivity follows from its
 * collision rate; NMR_Simulation.cpp:1500-1508, Walker/walker.h:162-209). A CPMG or PFGSE walk
 * whose params carry dfactor == NULL uses them; each walker's energy is then its own FP64 repeated
 * product, as in Walker::walk_3D. Single-phase images only; uploading walkers clears them. */
rwnmr_status rwnmr_walkers_set_dfactor(rwnmr_ctx *ctx, const double *dfactor);

/* ---- CPMG walk ------------------------------------------------------------------------- */
typedef struct rwnmr_cpmg_params
{
    int32_t bc;             /* RWNMR_BC_* */
    int32_t shift;          /* log2(voxel division) */
    int32_t steps_per_echo; /* STEPS_PER_ECHO */
    int32_t n_echoes;       /* NMR_Simulation::numberOfEchoes */
    const double *dfactor;  /* [n_phases] collision decrease factor per phase,
                               1 - (2/3) rho res / (D0 1e3)  (Walker/walker.h:203-209);
                               NULL: the per-walker factors of rwnmr_walkers_set_dfactor */
    int32_t echoes_per_launch; /* 0 = automatic; bounds one kernel's duration */
} rwnmr_cpmg_params;

/* Walks every walker from its initial state for n_echoes * steps_per_echo steps
 * (NMR_cpmg::image_simulation_cuda, NMR_cpmg_cuda.cpp:929-1774). Outputs (each nullable):
 *   echo_sum  [n_echoes+1]    sum over walkers of the energy after each echo (index 0 =
 *                             initial), un-normalised and without bulk relaxation, like the
 *                             reference's signal_amps before applyBulk/normalizeSignal
 *   echo_fx   [(n_echoes+1)*3] the same sums as exact fixed-point integers: each walker's
 *                             energy is rounded to a multiple of 2^-63 and split into bits
 *                             0-20, 21-41, 42-63, and each limb is summed over walkers
 *   echo_coll [n_echoes*n_phases] collisions gained during each echo, per phase */
rwnmr_status rwnmr_cpmg_run(rwnmr_ctx *ctx, const rwnmr_cpmg_params *p, double *echo_sum, uint64_t *echo_fx,
                            uint64_t *echo_coll);

/* rwnmr_cpmg_run (same walk, same echo_sum) that also returns the forward sensitivities of the echo
 * sums to the per-phase decrease factors, for gradients without a second walk:
 *   echo_sens    [(n_echoes+1)*n_phases] sum over walkers of E_w(e) * c_wq(e), the walker's energy
 *                after echo e times its collisions with phase q so far, so that
 *                d echo_sum[e] / d dfactor[q] = echo_sens[e][q] / dfactor[q] for dfactor[q] > 0
 *   echo_sens_fx [(n_echoes+1)*n_phases*4] the same sums exactly: each walker's product of its 2^-63
 *                fixed-point energy and its count (96 bits) split into bits 0-23, 24-47, 48-71,
 *                72-95, each limb summed over walkers
 * Both nullable. Per-phase decrease factors only (dfactor must not be NULL). No counterpart in the
 * reference. */
rwnmr_status rwnmr_cpmg_run_sens(rwnmr_ctx *ctx, const rwnmr_cpmg_params *p, double *echo_sum, double *echo_sens,
                                 uint64_t *echo_sens_fx);

/* Vector-Jacobian product of rwnmr_cpmg_run by replaying every trajectory from its stored seed:
 * grad_dfactor[p] = sum_e grad_echo[e] * d echo_sum[e] / d dfactor[p]. grad_echo: [n_echoes+1].
 * With every decrease factor positive the replay is one integer walk with the sensitivity sums of
 * rwnmr_cpmg_run_sens (on scratch state); with a zero factor, an FP64 replay of the direct
 * derivative. Either way the context's walkers are left as they were. */
rwnmr_status rwnmr_cpmg_adjoint(rwnmr_ctx *ctx, const rwnmr_cpmg_params *p, const double *grad_echo,
                                double *grad_dfactor);

/* ---- CPMG walk in an internal magnetic field ------------------------------------------- */
/* The reference's RESIDUAL_FIELD option (NMR_cpmg.cpp:48-64 setInternalField;
 * InternalField.cpp; CPMG_walk_{noflux,periodic,mirror}_field, NMR_cpmg_cuda.cpp:146-293,
 * 409-567, 683-838). A field belongs to the uploaded image; uploading another image clears it. */

/* Uniform field (RESIDUAL_FIELD: uniform): B = coord * gradient * 1e-6 * resolution in pore
 * voxels and 0 in solid ones, coord the voxel index along direction 0/1/2 (x/y/z). Evaluated in
 * the kernel; nothing is stored per voxel. */
rwnmr_status rwnmr_field_set_uniform(rwnmr_ctx *ctx, double gradient, int32_t direction, double resolution);

/* Arbitrary field (RESIDUAL_FIELD: import): count = nx*ny*nz doubles, x fastest, the layout of
 * the reference's PATH_TO_FIELD file (InternalField::readDataFromFile). */
rwnmr_status rwnmr_field_upload(rwnmr_ctx *ctx, const double *values, int64_t count);
rwnmr_status rwnmr_field_clear(rwnmr_ctx *ctx);

typedef struct rwnmr_field_cpmg_params
{
    int32_t bc;
    int32_t shift;
    int32_t steps_per_echo; /* each echo is two inversions of steps_per_echo / 2 steps */
    int32_t n_echoes;
    const double *dfactor;  /* [n_phases], or NULL for the per-walker factors */
    double gamma;           /* 1e6 * gyromagnetic ratio (NMR_cpmg_cuda.cpp: gamma) */
    double time_interval;   /* seconds per step (1e-3 * the walk's time step in ms) */
    int32_t echoes_per_launch; /* 0 = automatic */
} rwnmr_field_cpmg_params;

/* Walks every walker from its initial state. Per step the phase gains gammatau * B before and
 * after the move (gammatau = 0.5 * gamma * time_interval); an inversion negates it; a walker's
 * energy after an echo is (prod over phases of f_p^collisions) * cos(phase). Outputs (nullable):
 *   echo_sum  [n_echoes+1] energy sums (index 0 = initial), each walker's energy rounded to a
 *             multiple of 2^-61 and summed exactly
 *   echo_fx   [n_echoes+1][3] the exact sums behind echo_sum: limbs l0, l1, l2 of
 *             S = sum over walkers of (E * 2^61 + 2^61), S = l0 + l1 * 2^21 + l2 * 2^42
 *             (echo_sum = (S - n * 2^61) * 2^-61)
 *   phase_out [n]          final phase of every walker
 * Final positions, seeds and collision counts are left in the context (rwnmr_walkers_download).
 * Requires a field set by rwnmr_field_set_uniform or rwnmr_field_upload. */
rwnmr_status rwnmr_cpmg_field_run(rwnmr_ctx *ctx, const rwnmr_field_cpmg_params *p, double *echo_sum,
                                  uint64_t *echo_fx, double *phase_out);

/* ---- CPMG walk without allocation ------------------------------------------------------ */
/* No counterpart in the reference (its CUDA path cudaMallocs its buffers on every run).
 * For callers that cannot let a library allocate device memory -- a framework whose caching
 * allocator owns the GPU's memory under a fixed budget, or an application under a hard
 * device-memory cap that pre-allocates everything -- this entry point takes device pointers for
 * all inputs and outputs and allocates nothing: no context, no cudaMalloc/cudaFree. Its scratch
 * (energy tables, per-echo accumulators, status word) lives in one file-scope device array of
 * 8 MiB that every GPU loading the library holds until exit; walks whose tables and accumulators
 * need more than that are rejected with RWNMR_ERR_UNSUPPORTED. All calls on a device share that
 * array: each call clears what it uses, but calls that overlap on the GPU race and must be
 * serialised by the caller. The first call on a device resolves the array's address with that
 * device current; make it before any stream capture. Runs on `stream` and synchronises it before
 * returning. Results equal rwnmr_cpmg_run's (echo_sum to the last bits of FP64 rounding). */
typedef struct rwnmr_noalloc_cpmg_args
{
    const uint64_t *blocks;    /* device: bit-blocks, 1 word per block for one phase (the reference's
                                  array); for n_phases 2 (or 3-4) each block is W = 2 (or 4) words
                                  -- the solid mask, then bit-planes of the solid voxel's phase index
                                  (label - 1) -- stored as 2W uint32: the W words' low halves, then
                                  their high halves */
    int32_t nx, ny, nz, n_phases;
    int64_t n;                 /* walkers */
    const int32_t *x0, *y0, *z0; /* device: initial positions */
    const uint64_t *seed0;     /* device: initial RNG states */
    int32_t *x, *y, *z;        /* device out: final positions */
    uint64_t *seed;            /* device out: final RNG states */
    uint32_t *collisions;      /* device out: [n_phases][n] collision totals */
    double *echo_sum;          /* device out: [n_echoes+1] */
    unsigned long long *echo_coll; /* device out, nullable: [n_echoes][n_phases] */
    void *stream;              /* cudaStream_t, NULL = legacy default stream */
} rwnmr_noalloc_cpmg_args;

/* err (nullable, errlen bytes) receives a message on failure. */
rwnmr_status rwnmr_cpmg_run_noalloc(const rwnmr_cpmg_params *p, const rwnmr_noalloc_cpmg_args *args, char *err,
                                    int errlen);

/* ---- batched multi-image CPMG with a relaxivity population per image ------------------ */
/* Extends the reference (one image per process, one relaxivity per run): many images of uneven
 * size and walker count are walked by one persistent work-queue launch, and each image carries up
 * to 16 candidate decrease factors that one walk evaluates together (trajectories do not depend on
 * the relaxivity). Per image and candidate the walk returns the normalisation-free echo sums
 * M_r(e) = sum_w f_r^c_w(e) and, if asked, their exact derivatives dM_r(e)/df_r =
 * sum_w c_w f_r^(c_w - 1), from which any loss gradient (the adjoint for that candidate) follows on
 * the host. Single-phase images (labels != 0 are solid).
 * Two methods give identical sums. RWNMR_BATCH_HISTOGRAMS walks every walker once per (n_echoes,
 * steps_per_echo, bc) and keeps exact integer per-echo collision-count histograms H[image][e][c]
 * (walkers with c collisions after echo e) on the device; every call then evaluates
 * M_r(e) = sum_c H[e][c] f_r^c and its derivative from them without walking (the reference's
 * `histogram` CPMG method, NMR_cpmg.cpp:235-343, bins collision rates approximately instead).
 * RWNMR_BATCH_CANDIDATE_WALK walks on every call and adds up the candidates walker by walker. */
typedef struct rwnmr_batch rwnmr_batch;

enum
{
    RWNMR_BATCH_AUTO = 0,           /* histograms if they fit in half the free device memory */
    RWNMR_BATCH_HISTOGRAMS = 1,
    RWNMR_BATCH_CANDIDATE_WALK = 2
};

typedef struct rwnmr_batch_cpmg_params
{
    int32_t bc;                /* RWNMR_BC_* for every image */
    int32_t steps_per_echo;
    int32_t n_echoes;
    int32_t n_candidates;      /* 1..16 decrease factors per image */
    int32_t derivatives;       /* also return dM/df per candidate */
    int32_t threads_per_block; /* 0 = autotuned value (or 256 before rwnmr_batch_autotune) */
    int32_t use_graph;         /* replay the launch sequence as a captured CUDA graph */
    int32_t walkers_per_thread; /* 1 or 2; 0 = autotuned value (or 1 before rwnmr_batch_autotune).
                                   Results do not depend on it (exact integer sums). */
    int32_t method;             /* RWNMR_BATCH_*; histograms take 4 * (n_echoes + 1 + steps_per_echo *
                                   n_echoes * (n_echoes + 1) / 2) bytes per image */
} rwnmr_batch_cpmg_params;

rwnmr_status rwnmr_batch_create(rwnmr_batch **out, int device);
void rwnmr_batch_destroy(rwnmr_batch *batch);
const char *rwnmr_batch_last_error(const rwnmr_batch *batch);

/* Asks the persistent batch walk in flight on batch (or the next one to start) to stop: its CTAs take
 * no further work items, the kernel ends normally, and the call returns RWNMR_ERR_CANCELLED with no
 * results (stored histograms are dropped); later calls run normally. The request belongs to the batch
 * call (rwnmr_batch_cpmg / rwnmr_batch_autotune) in flight when it is made, or to the next one if none
 * is, and that call consumes it when it returns even if no walk saw it (it landed after the last work
 * item was taken, or the call only evaluated stored histograms): a request never carries over to a
 * later call. Safe to call from another host thread while a batch call runs. No counterpart in the
 * reference. */
rwnmr_status rwnmr_batch_cancel(rwnmr_batch *batch);

/* Time budget of each persistent batch walk launch, in seconds (0, the default: none). A CTA that has
 * run longer than the budget takes no further work items; the call then returns RWNMR_ERR_TIMEOUT
 * with no results. A bound on how long one walk can hold a shared GPU, not a precise deadline: work
 * items in progress finish first. */
rwnmr_status rwnmr_batch_set_time_budget(rwnmr_batch *batch, double seconds);
double rwnmr_batch_last_kernel_ms(const rwnmr_batch *batch);
int64_t rwnmr_batch_launch_count(const rwnmr_batch *batch);
/* Adds one image (bit-blocks as for rwnmr_image_upload) with its walkers; *index = image number. */
rwnmr_status rwnmr_batch_add_image(rwnmr_batch *batch, const uint64_t *blocks, int32_t nx, int32_t ny, int32_t nz,
                                   int64_t n, const int32_t *x0, const int32_t *y0, const int32_t *z0,
                                   const uint64_t *seed0, int32_t *index);
/* dfactor [n_images][n_candidates]; echo and decho (nullable) [n_images][n_candidates][n_echoes+1]. */
rwnmr_status rwnmr_batch_cpmg(rwnmr_batch *batch, const rwnmr_batch_cpmg_params *p, const double *dfactor,
                              double *echo, double *decho);
/* Times the walk of the method p selects (the histogram walk, or the candidate walk) for 128, 256
 * and 512 threads per block with 1 and 2 walkers per thread and keeps the fastest pair for later
 * calls (outputs nullable). */
rwnmr_status rwnmr_batch_autotune(rwnmr_batch *batch, const rwnmr_batch_cpmg_params *p, int32_t *best_threads,
                                  int32_t *best_walkers_per_thread, double *best_ms);
/* Row `echo` of image `image`'s collision histogram from the last histogram walk: counts[c] =
 * walkers with c collisions after that echo, c = 0 .. steps_per_echo * echo (*n_counts entries;
 * counts NULL: size only). */
rwnmr_status rwnmr_batch_collision_histogram(rwnmr_batch *batch, int32_t image, int32_t echo, uint32_t *counts,
                                             int32_t *n_counts);
/* GPU time of the last histogram walk (ms); rwnmr_batch_last_kernel_ms includes it in the call
 * that ran it. */
double rwnmr_batch_histogram_walk_ms(const rwnmr_batch *batch);

/* ---- collision-mapping walk ------------------------------------------------------------ */
/* NMR_Simulation::mapSimulation (NMR_Simulation.cpp:1787-1841; NMR_Simulation_cuda.cpp:726-1270):
 * walks every walker from its initial state for `steps` steps and writes its collision count. */
rwnmr_status rwnmr_map_run(rwnmr_ctx *ctx, int32_t bc, int32_t shift, int64_t steps, uint32_t *collisions);
/* Same walk continued from the state the previous walk left (positions, RNG states, collision
 * totals), as the reference's histogram windows continue one another (NMR_Simulation.cpp:1787-1841);
 * collisions receives the running totals. */
rwnmr_status rwnmr_map_continue(rwnmr_ctx *ctx, int32_t bc, int32_t shift, int64_t steps, uint32_t *collisions);

/* ---- PFGSE walk ------------------------------------------------------------------------ */
typedef struct rwnmr_pfgse_params
{
    int32_t bc;
    int32_t shift;
    int32_t n_delta;      /* exposure times */
    const int32_t *steps; /* [n_delta] walk steps to each exposure time, non-decreasing */
    int32_t n_g;          /* gradient points */
    const double *kvec;   /* [n_g][3] wave vectors k (1/um), NMR_pfgse.cpp:299-313,483-486 */
    double res;           /* voxel resolution of the walk grid (um) */
    const double *dfactor;/* [n_phases] */
} rwnmr_pfgse_params;

/* PFGSE walk (NMR_PFGSE::simulation_cuda/_omp): walkers walk cumulatively to each exposure time;
 * then M[i][j] = sum_w E_w cos((k_j . dR_w) res), esum[i] = sum_w E_w (the reference normalises
 * M by esum, NMR_pfgse.cpp:1795-1798), msd[i][a] = sum_w dR_a^2 (exact integer, walk units).
 * Each output nullable. */
rwnmr_status rwnmr_pfgse_run(rwnmr_ctx *ctx, const rwnmr_pfgse_params *p, double *M, double *esum, uint64_t *msd);

/* d M[i][j] / d g_j for a gradient ramp g_j with k_j = kscale * g_j * dir (kscale = dk/dg,
 * dir the unit gradient direction): dMdg[i][j] = -sum_w E_w sin((k_j . dR) res) (kscale dir . dR) res. */
rwnmr_status rwnmr_pfgse_grad_g(rwnmr_ctx *ctx, const rwnmr_pfgse_params *p, double kscale, const double *dir,
                                double *dMdg);

#ifdef __cplusplus
}
#endif
#endif
