// C-ABI engine of the GB300 walker path: context, device memory, launches (include/rwnmr_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rwnmr_gb300.h"
#include <nvtx3/nvToolsExt.h>

#include "fixed_cos.cuh"
#include "walk_kernels.cuh"

using namespace rwnmr;

namespace
{
typedef unsigned __int128 u128;

// NVTX range over one C-ABI call (visible in Nsight Systems / Nsight Compute timelines; inert without a tool).
struct NvtxRange
{
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Device allocator of the engine contexts' buffers: cudaMalloc / cudaFree, or the caller's pair set by
// rwnmr_set_device_allocator (for example a framework's caching allocator).
struct AllocHook
{
    rwnmr_alloc_fn alloc = nullptr;
    rwnmr_free_fn free = nullptr;
    void *user = nullptr;
};
std::mutex g_alloc_mu;
AllocHook g_alloc;

AllocHook current_alloc()
{
    std::lock_guard<std::mutex> lock(g_alloc_mu);
    return g_alloc;
}

template <typename T>
struct DevBuf
{
    T *p = nullptr;
    size_t cap = 0;
    AllocHook hook; // the allocator that made p, which also frees it
    cudaError_t ensure(size_t n)
    {
        if (n <= cap && p) return cudaSuccess;
        release();
        const size_t count = std::max<size_t>(n, 1);
        const AllocHook h = current_alloc();
        if (h.alloc)
        {
            p = (T *)h.alloc(count * sizeof(T), h.user);
            if (!p) return cudaErrorMemoryAllocation;
        }
        else
        {
            cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
            if (e != cudaSuccess)
            {
                p = nullptr;
                return e;
            }
        }
        hook = h;
        cap = count;
        return cudaSuccess;
    }
    void release()
    {
        if (p)
        {
            if (hook.alloc) hook.free(p, hook.user);
            else cudaFree(p);
        }
        p = nullptr;
        cap = 0;
        hook = AllocHook{};
    }
};

int phase_slots(int n_phases) { return n_phases <= 1 ? 1 : (n_phases == 2 ? 2 : 4); }
int words_for(int n_phases) { return phase_slots(n_phases); }

// table[n] = f^n as the FP64 repeated product (Walker/walker.cpp:229 applied n times) and its
// fixed-point copy round(table[n] * 2^63).
void build_tables(const double *f, int n_phases, int slots, int64_t nmax, std::vector<double> *t,
                  std::vector<uint64_t> *fx)
{
    const size_t stride = (size_t)nmax + 1;
    if (t) t->assign(slots * stride, 1.0);
    if (fx) fx->assign(slots * stride, 1ull << 63);
    for (int q = 0; q < n_phases; q++)
    {
        double v = 1.0;
        for (int64_t k = 0; k <= nmax; k++)
        {
            if (t) (*t)[q * stride + k] = v;
            if (fx) (*fx)[q * stride + k] = (uint64_t)std::nearbyint(std::ldexp(v, 63));
            v = v * f[q];
        }
    }
}

double limbs_to_double(const unsigned long long *l)
{
    u128 v = (u128)l[0] + ((u128)l[1] << 21) + ((u128)l[2] << 42);
    return std::ldexp((double)v, -63);
}
} // namespace

struct rwnmr_ctx
{
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t launches = 0;
    double last_ms = 0.0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    bool has_image = false;
    int nx = 0, ny = 0, nz = 0, bcols = 0, brows = 0, bdepth = 0, n_phases = 1, words = 1;
    DevBuf<uint64_t> blocks;
    DevBuf<uint8_t> labels;
    DevBuf<uint32_t> morton; // Morton copy of the image for the noflux walk (mi.words null: none)
    MortonImage mi;
    bool allow_morton = true; // build the Morton copy at upload (rwnmr_ctx_set_image_layout)

    int64_t n = 0;
    bool has_walkers = false;
    // walkers are stored in spatial order: perm[k] = upload index of the walker at k (host copy
    // fetched when a per-walker input or output needs it)
    DevBuf<int32_t> perm;
    DevBuf<uint32_t> order_scratch;
    std::vector<int32_t> h_perm;
    bool h_perm_valid = false;
    bool has_wf = false; // per-walker decrease factors uploaded
    DevBuf<double> wf, wenergy;
    DevBuf<int32_t> x0, y0, z0, x, y, z;
    DevBuf<uint64_t> seed0, seed;
    DevBuf<uint32_t> coll;
    DevBuf<int32_t> rx, ry, rz; // scratch walker state of the adjoint's sensitivity walk
    DevBuf<int32_t> sperm, ti32; // walker re-sort: the new order and per-type scratch
    DevBuf<uint64_t> tu64;
    DevBuf<uint32_t> tu32;
    DevBuf<double> tf64;
    DevBuf<uint64_t> rseed;
    DevBuf<uint32_t> rcoll;

    DevBuf<uint64_t> tfx;
    DevBuf<double> tfp;
    DevBuf<unsigned long long> acc, hist;
    DevBuf<unsigned> status;
    DevBuf<double> grad, partial, partial_g, kbuf, Mbuf, gbuf;
    DevBuf<uint64_t> kappa;                  // general-direction PFGSE: k res / (2 pi) in turns
    DevBuf<unsigned long long> dpart;        // general-direction PFGSE: exact block partials
    DevBuf<int32_t> ibuf, disp;
    DevBuf<double> energy;

    // internal field: 0 none, 1 uniform (evaluated in the kernel), 2 array
    int field_mode = 0;
    double field_dg = 0.0;
    int field_axis = 0;
    DevBuf<double> field, phase, btab;

    rwnmr_status fail(rwnmr_status s, const char *fmt, ...)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return s;
    }
    rwnmr_status cuda(cudaError_t e, const char *what)
    {
        if (e == cudaSuccess) return RWNMR_OK;
        return fail(e == cudaErrorMemoryAllocation ? RWNMR_ERR_NOMEM : RWNMR_ERR_CUDA, "%s: %s", what,
                    cudaGetErrorString(e));
    }
    DevImage image(int bc, int shift) const
    {
        DevImage im;
        im.blocks = blocks.p;
        im.nx = nx;
        im.ny = ny;
        im.nz = nz;
        im.bcols = bcols;
        im.bcr = bcols * brows;
        im.bc = bc;
        im.shift = shift;
        im.mi = mi;
        return im;
    }
    WalkState state()
    {
        WalkState s;
        s.n = n;
        s.x0 = x0.p;
        s.y0 = y0.p;
        s.z0 = z0.p;
        s.seed0 = seed0.p;
        s.x = x.p;
        s.y = y.p;
        s.z = z.p;
        s.seed = seed.p;
        s.coll = coll.p;
        return s;
    }
    rwnmr_status check_status(const char *what)
    {
        unsigned h = 0;
        rwnmr_status r = cuda(cudaMemcpyAsync(&h, status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, stream), what);
        if (r != RWNMR_OK) return r;
        r = cuda(cudaStreamSynchronize(stream), what);
        if (r != RWNMR_OK) return r;
        if (h & kStatusBadStart) return fail(RWNMR_ERR_INVALID, "%s: a walker starts outside the image", what);
        if (h & kStatusBadLabel) return fail(RWNMR_ERR_INVALID, "%s: label exceeds the phase count", what);
        if (h & kStatusHistRange) return fail(RWNMR_ERR_DEVICE, "%s: displacement histogram overflow", what);
        return RWNMR_OK;
    }
};

namespace
{
rwnmr_status need_run_state(rwnmr_ctx *ctx)
{
    if (!ctx) return RWNMR_ERR_INVALID;
    if (!ctx->has_image) return ctx->fail(RWNMR_ERR_STATE, "no image uploaded");
    if (!ctx->has_walkers) return ctx->fail(RWNMR_ERR_STATE, "no walkers uploaded");
    return RWNMR_OK;
}

rwnmr_status check_geom(rwnmr_ctx *ctx, int bc, int shift)
{
    if (bc < RWNMR_BC_NOFLUX || bc > RWNMR_BC_MIRROR) return ctx->fail(RWNMR_ERR_INVALID, "unknown boundary condition %d", bc);
    if (shift < 0 || shift > 10) return ctx->fail(RWNMR_ERR_INVALID, "voxel-division shift %d out of range 0..10", shift);
    return RWNMR_OK;
}

// dfactor == NULL selects the per-walker decrease factors (single-phase images).
rwnmr_status check_walker_dfactor(rwnmr_ctx *ctx)
{
    if (!ctx->has_wf) return ctx->fail(RWNMR_ERR_STATE, "dfactor is NULL and no per-walker decrease factors are set");
    if (ctx->n_phases != 1)
        return ctx->fail(RWNMR_ERR_UNSUPPORTED, "per-walker decrease factors need a single-phase image");
    return RWNMR_OK;
}

// Host copy of the walker order (upload index of each stored walker).
rwnmr_status host_perm(rwnmr_ctx *c)
{
    if (c->h_perm_valid) return RWNMR_OK;
    c->h_perm.resize((size_t)c->n);
    if (c->n > 0)
    {
        rwnmr_status r = c->cuda(cudaMemcpyAsync(c->h_perm.data(), c->perm.p, (size_t)c->n * 4, cudaMemcpyDeviceToHost,
                                                 c->stream), "walker order");
        if (r == RWNMR_OK) r = c->cuda(cudaStreamSynchronize(c->stream), "walker order");
        if (r != RWNMR_OK) return r;
    }
    c->h_perm_valid = true;
    return RWNMR_OK;
}

rwnmr_status check_dfactor(rwnmr_ctx *ctx, const double *f)
{
    if (!f) return ctx->fail(RWNMR_ERR_INVALID, "dfactor is NULL");
    for (int q = 0; q < ctx->n_phases; q++)
        if (!(f[q] >= 0.0 && f[q] <= 1.0))
            return ctx->fail(RWNMR_ERR_UNSUPPORTED, "decrease factor %g of phase %d outside [0, 1]", f[q], q);
    return RWNMR_OK;
}

int bc_key(int bc, int shift) { return shift > 0 ? BC_GENERIC : bc; }

dim3 walk_grid(int64_t n) { return dim3((unsigned)std::max<int64_t>(1, (n + kWalkThreads - 1) / kWalkThreads)); }
} // namespace

#define RW_TRY(expr)                                                                                                   \
    do                                                                                                                 \
    {                                                                                                                  \
        rwnmr_status _s = (expr);                                                                                      \
        if (_s != RWNMR_OK) return _s;                                                                                 \
    } while (0)
#define RW_CUDA(ctx, expr, what) RW_TRY((ctx)->cuda((expr), (what)))

extern "C" {

const char *rwnmr_version(void) { return "rwnmr_gb300 0.1 (sm_103a)"; }

rwnmr_status rwnmr_ctx_create(rwnmr_ctx **out, int device)
{
    if (!out) return RWNMR_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) return RWNMR_ERR_CUDA;
    if (device < 0 || device >= count) return RWNMR_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return RWNMR_ERR_CUDA;
    rwnmr_ctx *c = new rwnmr_ctx();
    c->device = device;
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
        c->status.ensure(1) != cudaSuccess)
    {
        rwnmr_ctx_destroy(c);
        return RWNMR_ERR_CUDA;
    }
    c->stream = c->own_stream;
    *out = c;
    return RWNMR_OK;
}

void rwnmr_ctx_destroy(rwnmr_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto *b : {&c->blocks}) b->release();
    c->labels.release();
    c->morton.release();
    c->perm.release(); c->order_scratch.release();
    c->x0.release(); c->y0.release(); c->z0.release();
    c->x.release(); c->y.release(); c->z.release();
    c->seed0.release(); c->seed.release(); c->coll.release();
    c->tfx.release(); c->tfp.release(); c->acc.release(); c->hist.release(); c->status.release();
    c->grad.release(); c->partial.release(); c->partial_g.release(); c->kbuf.release(); c->Mbuf.release();
    c->kappa.release(); c->dpart.release();
    c->gbuf.release(); c->ibuf.release(); c->disp.release(); c->energy.release();
    c->wf.release(); c->wenergy.release(); c->field.release(); c->phase.release(); c->btab.release();
    c->rx.release(); c->ry.release(); c->rz.release(); c->rseed.release(); c->rcoll.release();
    c->sperm.release(); c->ti32.release(); c->tu64.release(); c->tu32.release(); c->tf64.release();
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

const char *rwnmr_last_error(const rwnmr_ctx *c) { return c ? c->err.c_str() : "null context"; }

rwnmr_status rwnmr_ctx_set_stream(rwnmr_ctx *c, void *s)
{
    if (!c) return RWNMR_ERR_INVALID;
    c->stream = s ? (cudaStream_t)s : c->own_stream;
    return RWNMR_OK;
}

int64_t rwnmr_ctx_launch_count(const rwnmr_ctx *c) { return c ? c->launches : 0; }
double rwnmr_ctx_last_kernel_ms(const rwnmr_ctx *c) { return c ? c->last_ms : 0.0; }

rwnmr_status rwnmr_set_device_allocator(rwnmr_alloc_fn alloc, rwnmr_free_fn free_fn, void *user)
{
    if ((alloc == nullptr) != (free_fn == nullptr)) return RWNMR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_alloc_mu);
    g_alloc.alloc = alloc;
    g_alloc.free = free_fn;
    g_alloc.user = alloc ? user : nullptr;
    return RWNMR_OK;
}

// ---- image ------------------------------------------------------------------------------------
static rwnmr_status set_dims(rwnmr_ctx *c, int32_t nx, int32_t ny, int32_t nz, int32_t n_phases)
{
    if (nx <= 0 || ny <= 0 || nz <= 0) return c->fail(RWNMR_ERR_INVALID, "image dims must be positive");
    // The reference walks images with one slice on a separate 2D walker (Walker::walk_2D); this
    // engine is the 3D walk, and its noflux reversal needs at least two voxels per axis.
    if (nx < 2 || ny < 2 || nz < 2) return c->fail(RWNMR_ERR_UNSUPPORTED, "3D walks need at least 2 voxels per axis");
    if ((int64_t)nx * ny * nz > (1ll << 40)) return c->fail(RWNMR_ERR_INVALID, "image too large");
    // the kernels index bit-blocks in 32 bits
    if ((int64_t)((nx + 3) / 4) * ((ny + 3) / 4) * ((nz + 3) / 4) >= (1ll << 31))
        return c->fail(RWNMR_ERR_UNSUPPORTED, "images are limited to 2^31 bit-blocks");
    if (n_phases < 1) return c->fail(RWNMR_ERR_INVALID, "n_phases must be >= 1");
    if (n_phases > 4) return c->fail(RWNMR_ERR_UNSUPPORTED, "at most 4 solid phases are supported");
    c->nx = nx;
    c->ny = ny;
    c->nz = nz;
    c->bcols = (nx + 3) / 4;
    c->brows = (ny + 3) / 4;
    c->bdepth = (nz + 3) / 4;
    c->n_phases = n_phases;
    c->words = words_for(n_phases);
    c->field_mode = 0; // a field belongs to the image it was set for
    return RWNMR_OK;
}

// Builds the Morton copy of the uploaded image when the power-of-two box around it holds at most
// four times its voxels and fits 32-bit indices; otherwise the walks use the bit-block layout.
static rwnmr_status build_morton(rwnmr_ctx *c)
{
    c->mi = MortonImage{};
    if (!c->allow_morton)
    {
        c->morton.release();
        return RWNMR_OK;
    }
    uint32_t n_words = 0;
    // padded copies of up to 48 MB stay L2-resident on GB300 (the padding is never touched)
    MortonImage m = morton_params(c->nx, c->ny, c->nz, n_words, c->words, 48ull << 20);
    if (!n_words) return RWNMR_OK;
    if (c->morton.ensure((size_t)n_words * c->words) != cudaSuccess)
    {
        cudaGetLastError(); // no room for the copy: the walks use the bit-block layout
        c->morton.release();
        return RWNMR_OK;
    }
    m.words = c->morton.p;
    DevImage im = c->image(RWNMR_BC_NOFLUX, 0);
    im.mi = m;
    RW_CUDA(c, launch_morton_build(im, c->words, n_words, c->morton.p, c->stream), "Morton image");
    c->launches++;
    c->mi = m;
    return RWNMR_OK;
}

int32_t rwnmr_image_layout(const rwnmr_ctx *c) { return c && c->has_image && c->mi.words ? 1 : 0; }

rwnmr_status rwnmr_ctx_set_image_layout(rwnmr_ctx *c, int32_t allow_morton)
{
    if (!c) return RWNMR_ERR_INVALID;
    c->allow_morton = allow_morton != 0;
    return RWNMR_OK;
}

rwnmr_status rwnmr_image_upload_labels(rwnmr_ctx *c, const uint8_t *labels, int32_t nx, int32_t ny, int32_t nz,
                                       int32_t n_phases)
{
    if (!c) return RWNMR_ERR_INVALID;
    if (!labels) return c->fail(RWNMR_ERR_INVALID, "labels is NULL");
    c->has_image = false;
    RW_TRY(set_dims(c, nx, ny, nz, n_phases));
    cudaSetDevice(c->device);
    const int64_t nb = (int64_t)c->bcols * c->brows * c->bdepth;
    const size_t nvox = (size_t)nx * ny * nz;
    RW_CUDA(c, c->labels.ensure(nvox), "image labels");
    RW_CUDA(c, c->blocks.ensure((size_t)nb * c->words), "image blocks");
    RW_CUDA(c, cudaMemcpyAsync(c->labels.p, labels, nvox, cudaMemcpyHostToDevice, c->stream), "labels upload");
    RW_CUDA(c, cudaMemsetAsync(c->status.p, 0, sizeof(unsigned), c->stream), "status reset");
    RW_CUDA(c, launch_pack_blocks(c->labels.p, nx, ny, nz, c->bcols, c->brows, nb, c->words, c->n_phases, c->blocks.p,
                                  c->status.p, c->stream), "pack kernel");
    c->launches++;
    RW_TRY(c->check_status("image packing"));
    if (c->n_phases == 1) c->labels.release();
    RW_TRY(build_morton(c));
    RW_CUDA(c, cudaStreamSynchronize(c->stream), "Morton image");
    c->has_image = true;
    return RWNMR_OK;
}

rwnmr_status rwnmr_image_upload(rwnmr_ctx *c, const uint64_t *blocks, int32_t nx, int32_t ny, int32_t nz,
                                const uint8_t *labels, int32_t n_phases)
{
    if (!c) return RWNMR_ERR_INVALID;
    if (!blocks) return c->fail(RWNMR_ERR_INVALID, "blocks is NULL");
    if (labels)
    {
        RW_TRY(rwnmr_image_upload_labels(c, labels, nx, ny, nz, n_phases));
        // the labels must describe the same solid voxels as the given bit-blocks
        const int64_t nb = (int64_t)c->bcols * c->brows * c->bdepth;
        std::vector<uint64_t> packed((size_t)nb);
        RW_TRY(rwnmr_image_download_blocks(c, packed.data()));
        for (int64_t b = 0; b < nb; b++)
            if (packed[(size_t)b] != blocks[b])
            {
                c->has_image = false;
                return c->fail(RWNMR_ERR_INVALID, "labels disagree with bit-block %lld", (long long)b);
            }
        return RWNMR_OK;
    }
    if (n_phases != 1) return c->fail(RWNMR_ERR_INVALID, "multi-phase images need labels");
    c->has_image = false;
    RW_TRY(set_dims(c, nx, ny, nz, 1));
    cudaSetDevice(c->device);
    const int64_t nb = (int64_t)c->bcols * c->brows * c->bdepth;
    RW_CUDA(c, c->blocks.ensure((size_t)nb), "image blocks");
    RW_CUDA(c, cudaMemcpyAsync(c->blocks.p, blocks, (size_t)nb * 8, cudaMemcpyHostToDevice, c->stream), "blocks upload");
    RW_TRY(build_morton(c));
    RW_CUDA(c, cudaStreamSynchronize(c->stream), "blocks upload");
    c->has_image = true;
    return RWNMR_OK;
}

rwnmr_status rwnmr_image_download_blocks(rwnmr_ctx *c, uint64_t *out)
{
    if (!c || !out) return RWNMR_ERR_INVALID;
    if (!c->has_image) return c->fail(RWNMR_ERR_STATE, "no image uploaded");
    const int64_t nb = (int64_t)c->bcols * c->brows * c->bdepth;
    if (c->words == 1)
    {
        RW_CUDA(c, cudaMemcpyAsync(out, c->blocks.p, (size_t)nb * 8, cudaMemcpyDeviceToHost, c->stream), "blocks download");
        RW_CUDA(c, cudaStreamSynchronize(c->stream), "blocks download");
        return RWNMR_OK;
    }
    // multi-phase blocks: the solid word's halves sit at uint32 2W*b and 2W*b + W
    const int W = c->words;
    std::vector<uint32_t> lo((size_t)nb), hi((size_t)nb);
    const uint32_t *dev = reinterpret_cast<const uint32_t *>(c->blocks.p);
    RW_CUDA(c, cudaMemcpy2DAsync(lo.data(), 4, dev, (size_t)8 * W, 4, (size_t)nb, cudaMemcpyDeviceToHost, c->stream),
            "blocks download");
    RW_CUDA(c, cudaMemcpy2DAsync(hi.data(), 4, dev + W, (size_t)8 * W, 4, (size_t)nb, cudaMemcpyDeviceToHost, c->stream),
            "blocks download");
    RW_CUDA(c, cudaStreamSynchronize(c->stream), "blocks download");
    for (int64_t b = 0; b < nb; b++) out[b] = (uint64_t)lo[(size_t)b] | ((uint64_t)hi[(size_t)b] << 32);
    return RWNMR_OK;
}

// ---- walkers ----------------------------------------------------------------------------------
rwnmr_status rwnmr_walkers_upload(rwnmr_ctx *c, int64_t n, const int32_t *x0, const int32_t *y0, const int32_t *z0,
                                  const uint64_t *seed0)
{
    NvtxRange nvtx("rwnmr_walkers_upload");
    if (!c) return RWNMR_ERR_INVALID;
    if (n < 0 || n > (1ll << 31) - 1) return c->fail(RWNMR_ERR_INVALID, "walker count %lld out of range", (long long)n);
    if (n > 0 && (!x0 || !y0 || !z0 || !seed0)) return c->fail(RWNMR_ERR_INVALID, "walker arrays must not be NULL");
    c->has_walkers = false;
    c->has_wf = false;
    cudaSetDevice(c->device);
    const size_t m = (size_t)std::max<int64_t>(n, 1);
    RW_CUDA(c, c->x0.ensure(m), "walkers"); RW_CUDA(c, c->y0.ensure(m), "walkers"); RW_CUDA(c, c->z0.ensure(m), "walkers");
    RW_CUDA(c, c->x.ensure(m), "walkers"); RW_CUDA(c, c->y.ensure(m), "walkers"); RW_CUDA(c, c->z.ensure(m), "walkers");
    RW_CUDA(c, c->seed0.ensure(m), "walkers"); RW_CUDA(c, c->seed.ensure(m), "walkers");
    RW_CUDA(c, c->coll.ensure(m * 4), "walkers");
    RW_CUDA(c, c->perm.ensure(m), "walker order");
    RW_CUDA(c, c->order_scratch.ensure(walker_order_scratch_words((int64_t)m)), "walker order");
    c->h_perm_valid = false;
    if (n > 0)
    {
        const size_t b4 = (size_t)n * 4, b8 = (size_t)n * 8;
        // stage in upload order, sort by start voxel, gather into the stored order
        RW_CUDA(c, cudaMemcpyAsync(c->x.p, x0, b4, cudaMemcpyHostToDevice, c->stream), "walkers upload");
        RW_CUDA(c, cudaMemcpyAsync(c->y.p, y0, b4, cudaMemcpyHostToDevice, c->stream), "walkers upload");
        RW_CUDA(c, cudaMemcpyAsync(c->z.p, z0, b4, cudaMemcpyHostToDevice, c->stream), "walkers upload");
        RW_CUDA(c, cudaMemcpyAsync(c->seed.p, seed0, b8, cudaMemcpyHostToDevice, c->stream), "walkers upload");
        int shift = 0; // keep 10 bits per axis of the image's coordinates
        if (c->has_image)
            while ((std::max(c->nx, std::max(c->ny, c->nz)) - 1) >> (10 + shift)) shift++;
        RW_CUDA(c, walker_order(c->x.p, c->y.p, c->z.p, n, shift, c->order_scratch.p, c->perm.p, c->stream), "walker order");
        RW_CUDA(c, gather_walkers(c->perm.p, n, c->x.p, c->y.p, c->z.p, c->seed.p, c->x0.p, c->y0.p, c->z0.p,
                                  c->seed0.p, c->stream), "walker order");
        c->launches += 8;
        RW_CUDA(c, cudaMemcpyAsync(c->x.p, c->x0.p, b4, cudaMemcpyDeviceToDevice, c->stream), "walkers init");
        RW_CUDA(c, cudaMemcpyAsync(c->y.p, c->y0.p, b4, cudaMemcpyDeviceToDevice, c->stream), "walkers init");
        RW_CUDA(c, cudaMemcpyAsync(c->z.p, c->z0.p, b4, cudaMemcpyDeviceToDevice, c->stream), "walkers init");
        RW_CUDA(c, cudaMemcpyAsync(c->seed.p, c->seed0.p, b8, cudaMemcpyDeviceToDevice, c->stream), "walkers init");
        RW_CUDA(c, cudaMemsetAsync(c->coll.p, 0, b4 * 4, c->stream), "walkers init");
    }
    RW_CUDA(c, cudaStreamSynchronize(c->stream), "walkers upload");
    c->n = n;
    c->has_walkers = true;
    return RWNMR_OK;
}

rwnmr_status rwnmr_walkers_restore(rwnmr_ctx *c, const int32_t *x, const int32_t *y, const int32_t *z,
                                   const uint64_t *seed, const uint32_t *coll)
{
    if (!c) return RWNMR_ERR_INVALID;
    if (!c->has_walkers) return c->fail(RWNMR_ERR_STATE, "no walkers uploaded");
    const int64_t n = c->n;
    if (n == 0) return RWNMR_OK;
    if (!x || !y || !z || !seed || !coll) return c->fail(RWNMR_ERR_INVALID, "NULL walker state");
    RW_TRY(host_perm(c));
    const std::vector<int32_t> &pm = c->h_perm;
    const int P = c->n_phases, slots = phase_slots(P);
    std::vector<int32_t> tx((size_t)n), ty((size_t)n), tz((size_t)n);
    std::vector<uint64_t> ts((size_t)n);
    std::vector<uint32_t> tc((size_t)n * slots, 0u);
    for (int64_t k = 0; k < n; k++) // to the stored order
    {
        const size_t u = (size_t)pm[(size_t)k];
        tx[(size_t)k] = x[u];
        ty[(size_t)k] = y[u];
        tz[(size_t)k] = z[u];
        ts[(size_t)k] = seed[u];
        for (int q = 0; q < P; q++) tc[(size_t)q * n + k] = coll[u * P + q];
    }
    const size_t b4 = (size_t)n * 4;
    RW_CUDA(c, cudaMemcpyAsync(c->x.p, tx.data(), b4, cudaMemcpyHostToDevice, c->stream), "walkers restore");
    RW_CUDA(c, cudaMemcpyAsync(c->y.p, ty.data(), b4, cudaMemcpyHostToDevice, c->stream), "walkers restore");
    RW_CUDA(c, cudaMemcpyAsync(c->z.p, tz.data(), b4, cudaMemcpyHostToDevice, c->stream), "walkers restore");
    RW_CUDA(c, cudaMemcpyAsync(c->seed.p, ts.data(), b4 * 2, cudaMemcpyHostToDevice, c->stream), "walkers restore");
    RW_CUDA(c, cudaMemcpyAsync(c->coll.p, tc.data(), b4 * slots, cudaMemcpyHostToDevice, c->stream), "walkers restore");
    RW_CUDA(c, cudaStreamSynchronize(c->stream), "walkers restore");
    return RWNMR_OK;
}

rwnmr_status rwnmr_walkers_download(rwnmr_ctx *c, int32_t *x, int32_t *y, int32_t *z, uint64_t *seed, uint32_t *coll)
{
    if (!c) return RWNMR_ERR_INVALID;
    if (!c->has_walkers) return c->fail(RWNMR_ERR_STATE, "no walkers uploaded");
    const int64_t n = c->n;
    if (n == 0) return RWNMR_OK;
    RW_TRY(host_perm(c));
    const std::vector<int32_t> &pm = c->h_perm;
    const size_t b4 = (size_t)n * 4;
    std::vector<int32_t> tx(x ? n : 0), ty(y ? n : 0), tz(z ? n : 0);
    std::vector<uint64_t> ts(seed ? n : 0);
    std::vector<uint32_t> tmp;
    const int P = c->n_phases;
    if (x) RW_CUDA(c, cudaMemcpyAsync(tx.data(), c->x.p, b4, cudaMemcpyDeviceToHost, c->stream), "walkers download");
    if (y) RW_CUDA(c, cudaMemcpyAsync(ty.data(), c->y.p, b4, cudaMemcpyDeviceToHost, c->stream), "walkers download");
    if (z) RW_CUDA(c, cudaMemcpyAsync(tz.data(), c->z.p, b4, cudaMemcpyDeviceToHost, c->stream), "walkers download");
    if (seed) RW_CUDA(c, cudaMemcpyAsync(ts.data(), c->seed.p, b4 * 2, cudaMemcpyDeviceToHost, c->stream), "walkers download");
    if (coll)
    {
        tmp.resize((size_t)n * P);
        RW_CUDA(c, cudaMemcpyAsync(tmp.data(), c->coll.p, b4 * P, cudaMemcpyDeviceToHost, c->stream), "walkers download");
    }
    RW_CUDA(c, cudaStreamSynchronize(c->stream), "walkers download");
    // back to upload order
    for (int64_t k = 0; k < n; k++)
    {
        const size_t u = (size_t)pm[(size_t)k];
        if (x) x[u] = tx[(size_t)k];
        if (y) y[u] = ty[(size_t)k];
        if (z) z[u] = tz[(size_t)k];
        if (seed) seed[u] = ts[(size_t)k];
        if (coll)
            for (int q = 0; q < P; q++) coll[u * P + q] = tmp[(size_t)q * n + k];
    }
    return RWNMR_OK;
}

rwnmr_status rwnmr_walkers_set_dfactor(rwnmr_ctx *c, const double *dfactor)
{
    if (!c) return RWNMR_ERR_INVALID;
    if (!c->has_walkers) return c->fail(RWNMR_ERR_STATE, "no walkers uploaded");
    if (c->n > 0 && !dfactor) return c->fail(RWNMR_ERR_INVALID, "dfactor is NULL");
    for (int64_t i = 0; i < c->n; i++)
        if (!(dfactor[i] >= 0.0 && dfactor[i] <= 1.0))
            return c->fail(RWNMR_ERR_UNSUPPORTED, "decrease factor %g of walker %lld outside [0, 1]", dfactor[i], (long long)i);
    cudaSetDevice(c->device);
    RW_CUDA(c, c->wf.ensure((size_t)std::max<int64_t>(c->n, 1)), "walker decrease factors");
    RW_TRY(host_perm(c));
    std::vector<double> stored((size_t)c->n); // in the stored walker order
    for (int64_t k = 0; k < c->n; k++) stored[(size_t)k] = dfactor[c->h_perm[(size_t)k]];
    if (c->n > 0)
        RW_CUDA(c, cudaMemcpyAsync(c->wf.p, stored.data(), (size_t)c->n * 8, cudaMemcpyHostToDevice, c->stream),
                "walker decrease factors");
    RW_CUDA(c, cudaStreamSynchronize(c->stream), "walker decrease factors");
    c->has_wf = true;
    return RWNMR_OK;
}

// ---- CPMG -------------------------------------------------------------------------------------
namespace
{
// rwnmr_cpmg_run, and with sens the sensitivity sums of rwnmr_cpmg_run_sens; with scratch the walk
// carries its state in scratch buffers and leaves the context's walkers as they were
rwnmr_status cpmg_impl(rwnmr_ctx *c, const rwnmr_cpmg_params *p, bool sens, bool scratch, double *echo_sum,
                       uint64_t *echo_fx, uint64_t *echo_coll, double *echo_sens, uint64_t *echo_sens_fx)
{
    NvtxRange nvtx(sens ? "rwnmr_cpmg_run_sens" : "rwnmr_cpmg_run");
    RW_TRY(need_run_state(c));
    if (!p) return c->fail(RWNMR_ERR_INVALID, "params is NULL");
    RW_TRY(check_geom(c, p->bc, p->shift));
    if (sens && !p->dfactor) return c->fail(RWNMR_ERR_UNSUPPORTED, "sensitivities are for per-phase decrease factors");
    const bool per_walker = p->dfactor == nullptr;
    RW_TRY(per_walker ? check_walker_dfactor(c) : check_dfactor(c, p->dfactor));
    if (p->n_echoes < 0 || p->steps_per_echo < 1) return c->fail(RWNMR_ERR_INVALID, "bad echo count / steps per echo");
    const int64_t nmax = (int64_t)p->n_echoes * p->steps_per_echo;
    if (nmax > (1ll << 28)) return c->fail(RWNMR_ERR_UNSUPPORTED, "walk of %lld steps too long", (long long)nmax);
    cudaSetDevice(c->device);
    const int slots = phase_slots(c->n_phases);
    const int K = 3 + slots + (sens ? 4 * slots : 0);
    if (per_walker)
        RW_CUDA(c, c->wenergy.ensure((size_t)std::max<int64_t>(c->n, 1)), "walker energies");
    else
    {
        std::vector<uint64_t> fx;
        build_tables(p->dfactor, c->n_phases, slots, nmax, nullptr, &fx);
        RW_CUDA(c, c->tfx.ensure(fx.size()), "tables");
        RW_CUDA(c, cudaMemcpyAsync(c->tfx.p, fx.data(), fx.size() * 8, cudaMemcpyHostToDevice, c->stream), "tables upload");
    }
    RW_CUDA(c, c->acc.ensure((size_t)(p->n_echoes + 1) * K), "echo accumulators");
    RW_CUDA(c, cudaMemsetAsync(c->acc.p, 0, (size_t)(p->n_echoes + 1) * K * 8, c->stream), "accumulator reset");
    RW_CUDA(c, cudaMemsetAsync(c->status.p, 0, sizeof(unsigned), c->stream), "status reset");

    int chunk = p->echoes_per_launch > 0 ? p->echoes_per_launch : std::max(32, (4096 / p->steps_per_echo) / 32 * 32);
    const DevImage im = c->image(p->bc, p->shift);
    WalkState st = c->state();
    if (scratch)
    {
        const size_t n1 = (size_t)std::max<int64_t>(c->n, 1);
        RW_CUDA(c, c->rx.ensure(n1), "scratch state");
        RW_CUDA(c, c->ry.ensure(n1), "scratch state");
        RW_CUDA(c, c->rz.ensure(n1), "scratch state");
        RW_CUDA(c, c->rseed.ensure(n1), "scratch state");
        RW_CUDA(c, c->rcoll.ensure(n1 * slots), "scratch state");
        st.x = c->rx.p;
        st.y = c->ry.p;
        st.z = c->rz.p;
        st.seed = c->rseed.p;
        st.coll = c->rcoll.p;
    }
    CpmgLaunch L{};
    L.steps_per_echo = p->steps_per_echo;
    L.record = 1;
    L.sens = sens ? 1 : 0;
    L.tfx = per_walker ? nullptr : c->tfx.p;
    L.tstride = (int)(nmax + 1);
    L.wf = per_walker ? c->wf.p : nullptr;
    L.wenergy = per_walker ? c->wenergy.p : nullptr;
    L.acc = c->acc.p;
    L.status = c->status.p;
    RW_CUDA(c, cudaEventRecord(c->ev0, c->stream), "event");
    if (c->n > 0)
    {
        if (p->n_echoes == 0)
        {
            L.e_begin = 0;
            L.e_end = 0;
            L.from_initial = 1;
            RW_CUDA(c, launch_cpmg_walk(bc_key(p->bc, p->shift), slots, im, st, L, walk_grid(c->n), c->stream), "cpmg kernel");
            c->launches++;
        }
        for (int e = 0; e < p->n_echoes; e += chunk)
        {
            L.e_begin = e;
            L.e_end = std::min(p->n_echoes, e + chunk);
            L.from_initial = e == 0;
            RW_CUDA(c, launch_cpmg_walk(bc_key(p->bc, p->shift), slots, im, st, L, walk_grid(c->n), c->stream), "cpmg kernel");
            c->launches++;
        }
    }
    RW_CUDA(c, cudaEventRecord(c->ev1, c->stream), "event");
    std::vector<unsigned long long> acc((size_t)(p->n_echoes + 1) * K);
    RW_CUDA(c, cudaMemcpyAsync(acc.data(), c->acc.p, acc.size() * 8, cudaMemcpyDeviceToHost, c->stream), "echo readback");
    RW_TRY(c->check_status("cpmg walk"));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->last_ms = ms;
    for (int e = 0; e <= p->n_echoes; e++)
    {
        const unsigned long long *a = &acc[(size_t)e * K];
        if (echo_sum) echo_sum[e] = limbs_to_double(a);
        if (echo_fx)
            for (int k = 0; k < 3; k++) echo_fx[(size_t)e * 3 + k] = a[k];
        if (echo_coll && e > 0)
            for (int q = 0; q < c->n_phases; q++) echo_coll[(size_t)(e - 1) * c->n_phases + q] = a[3 + q];
        if (sens)
            for (int q = 0; q < c->n_phases; q++)
            {
                const unsigned long long *l = a + 3 + slots + 4 * q; // 24-bit limbs of sum E c_q
                if (echo_sens_fx)
                    for (int k = 0; k < 4; k++) echo_sens_fx[((size_t)e * c->n_phases + q) * 4 + k] = l[k];
                if (echo_sens)
                {
                    const u128 v = (u128)l[0] + ((u128)l[1] << 24) + ((u128)l[2] << 48) + ((u128)l[3] << 72);
                    echo_sens[(size_t)e * c->n_phases + q] = std::ldexp((double)v, -63);
                }
            }
    }
    return RWNMR_OK;
}
} // namespace

rwnmr_status rwnmr_cpmg_run(rwnmr_ctx *c, const rwnmr_cpmg_params *p, double *echo_sum, uint64_t *echo_fx,
                            uint64_t *echo_coll)
{
    return cpmg_impl(c, p, false, false, echo_sum, echo_fx, echo_coll, nullptr, nullptr);
}

rwnmr_status rwnmr_cpmg_run_sens(rwnmr_ctx *c, const rwnmr_cpmg_params *p, double *echo_sum, double *echo_sens,
                                 uint64_t *echo_sens_fx)
{
    return cpmg_impl(c, p, true, false, echo_sum, nullptr, nullptr, echo_sens, echo_sens_fx);
}

// ---- internal field ---------------------------------------------------------------------------
rwnmr_status rwnmr_field_set_uniform(rwnmr_ctx *c, double gradient, int32_t direction, double resolution)
{
    if (!c) return RWNMR_ERR_INVALID;
    if (!c->has_image) return c->fail(RWNMR_ERR_STATE, "no image uploaded");
    if (direction < 0 || direction > 2) return c->fail(RWNMR_ERR_INVALID, "gradient direction %d not in 0..2", direction);
    if (!std::isfinite(gradient) || !std::isfinite(resolution))
        return c->fail(RWNMR_ERR_INVALID, "gradient and resolution must be finite");
    c->field_dg = gradient * (1.0e-6) * resolution; // InternalField::fillDataArray
    c->field_axis = direction;
    c->field_mode = 1;
    return RWNMR_OK;
}

rwnmr_status rwnmr_field_upload(rwnmr_ctx *c, const double *values, int64_t count)
{
    if (!c) return RWNMR_ERR_INVALID;
    if (!c->has_image) return c->fail(RWNMR_ERR_STATE, "no image uploaded");
    const int64_t vol = (int64_t)c->nx * c->ny * c->nz;
    if (!values || count != vol)
        return c->fail(RWNMR_ERR_INVALID, "field has %lld values, the image %lld voxels", (long long)count, (long long)vol);
    cudaSetDevice(c->device);
    RW_CUDA(c, c->field.ensure((size_t)vol), "field");
    RW_CUDA(c, cudaMemcpyAsync(c->field.p, values, (size_t)vol * 8, cudaMemcpyHostToDevice, c->stream), "field upload");
    RW_CUDA(c, cudaStreamSynchronize(c->stream), "field upload");
    c->field_mode = 2;
    return RWNMR_OK;
}

rwnmr_status rwnmr_field_clear(rwnmr_ctx *c)
{
    if (!c) return RWNMR_ERR_INVALID;
    c->field_mode = 0;
    c->field.release();
    return RWNMR_OK;
}

rwnmr_status rwnmr_cpmg_field_run(rwnmr_ctx *c, const rwnmr_field_cpmg_params *p, double *echo_sum, uint64_t *echo_fx,
                                  double *phase_out)
{
    NvtxRange nvtx("rwnmr_cpmg_field_run");
    RW_TRY(need_run_state(c));
    if (!p) return c->fail(RWNMR_ERR_INVALID, "params is NULL");
    if (c->field_mode == 0) return c->fail(RWNMR_ERR_STATE, "no internal field set");
    RW_TRY(check_geom(c, p->bc, p->shift));
    const bool per_walker = p->dfactor == nullptr;
    RW_TRY(per_walker ? check_walker_dfactor(c) : check_dfactor(c, p->dfactor));
    if (p->n_echoes < 0 || p->steps_per_echo < 1) return c->fail(RWNMR_ERR_INVALID, "bad echo count / steps per echo");
    if (!std::isfinite(p->gamma) || !std::isfinite(p->time_interval))
        return c->fail(RWNMR_ERR_INVALID, "gamma and time interval must be finite");
    const int spi = p->steps_per_echo / 2;
    const int64_t nmax = (int64_t)p->n_echoes * 2 * spi;
    if (nmax > (1ll << 28)) return c->fail(RWNMR_ERR_UNSUPPORTED, "walk of %lld steps too long", (long long)nmax);
    cudaSetDevice(c->device);
    const int slots = phase_slots(c->n_phases);
    constexpr int K = 3;
    if (per_walker)
        RW_CUDA(c, c->wenergy.ensure((size_t)std::max<int64_t>(c->n, 1)), "walker survival probabilities");
    else
    {
        std::vector<uint64_t> fx;
        build_tables(p->dfactor, c->n_phases, slots, nmax, nullptr, &fx);
        RW_CUDA(c, c->tfx.ensure(fx.size()), "tables");
        RW_CUDA(c, cudaMemcpyAsync(c->tfx.p, fx.data(), fx.size() * 8, cudaMemcpyHostToDevice, c->stream), "tables upload");
    }
    RW_CUDA(c, c->acc.ensure((size_t)(p->n_echoes + 1) * K), "echo accumulators");
    RW_CUDA(c, c->phase.ensure((size_t)std::max<int64_t>(c->n, 1)), "walker phases");
    RW_CUDA(c, cudaMemsetAsync(c->acc.p, 0, (size_t)(p->n_echoes + 1) * K * 8, c->stream), "accumulator reset");
    RW_CUDA(c, cudaMemsetAsync(c->status.p, 0, sizeof(unsigned), c->stream), "status reset");

    const int chunk = p->echoes_per_launch > 0 ? p->echoes_per_launch
                                               : std::max(32, (4096 / std::max(1, 2 * spi)) / 32 * 32);
    const DevImage im = c->image(p->bc, p->shift);
    const WalkState st = c->state();
    FieldLaunch L{};
    L.steps_per_inversion = spi;
    L.tfx = per_walker ? nullptr : c->tfx.p;
    L.tstride = (int)(nmax + 1);
    L.wf = per_walker ? c->wf.p : nullptr;
    L.palive = per_walker ? c->wenergy.p : nullptr;
    L.gammatau = 0.5 * p->gamma * p->time_interval; // NMR_cpmg_cuda.cpp: gammatau = 0.5*gamma*timeInterval
    L.field = c->field_mode == 2 ? c->field.p : nullptr;
    L.dg = c->field_dg;
    L.axis = c->field_axis;
    if (c->field_mode == 1)
    {
        const int na = c->field_axis == 0 ? c->nx : (c->field_axis == 1 ? c->ny : c->nz);
        RW_CUDA(c, c->btab.ensure((size_t)na), "field table");
        RW_CUDA(c, launch_field_table(c->field_dg, na, c->btab.p, c->stream), "field table");
        c->launches++;
        L.btab = c->btab.p;
    }
    L.phase = c->phase.p;
    L.acc = c->acc.p;
    L.status = c->status.p;
    const bool uniform = c->field_mode == 1;
    RW_CUDA(c, cudaEventRecord(c->ev0, c->stream), "event");
    if (c->n > 0)
    {
        for (int e = 0; e < std::max(p->n_echoes, 1); e += chunk)
        {
            L.e_begin = e;
            L.e_end = std::min(p->n_echoes, e + chunk);
            L.from_initial = e == 0;
            RW_CUDA(c, launch_cpmg_field(bc_key(p->bc, p->shift), slots, uniform, im, st, L, walk_grid(c->n), c->stream),
                    "field cpmg kernel");
            c->launches++;
        }
    }
    RW_CUDA(c, cudaEventRecord(c->ev1, c->stream), "event");
    std::vector<unsigned long long> acc((size_t)(p->n_echoes + 1) * K);
    RW_CUDA(c, cudaMemcpyAsync(acc.data(), c->acc.p, acc.size() * 8, cudaMemcpyDeviceToHost, c->stream), "echo readback");
    std::vector<double> ph;
    if (phase_out && c->n > 0)
    {
        ph.resize((size_t)c->n);
        RW_CUDA(c, cudaMemcpyAsync(ph.data(), c->phase.p, (size_t)c->n * 8, cudaMemcpyDeviceToHost, c->stream),
                "phase readback");
    }
    RW_TRY(c->check_status("field cpmg walk"));
    if (!ph.empty())
    {
        RW_TRY(host_perm(c));
        for (int64_t k = 0; k < c->n; k++) phase_out[c->h_perm[(size_t)k]] = ph[(size_t)k];
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->last_ms = ms;
    if (echo_fx)
        for (size_t k = 0; k < acc.size(); k++) echo_fx[k] = acc[k];
    if (echo_sum)
    {
        // every walker added E * 2^61 + 2^61
        const __int128 offset = (__int128)c->n << 61;
        for (int e = 0; e <= p->n_echoes; e++)
        {
            const unsigned long long *a = &acc[(size_t)e * K];
            const __int128 v = (__int128)a[0] + ((__int128)a[1] << 21) + ((__int128)a[2] << 42) - offset;
            echo_sum[e] = std::ldexp((double)v, -61);
        }
    }
    return RWNMR_OK;
}

rwnmr_status rwnmr_cpmg_adjoint(rwnmr_ctx *c, const rwnmr_cpmg_params *p, const double *grad_echo, double *grad_dfactor)
{
    NvtxRange nvtx("rwnmr_cpmg_adjoint");
    RW_TRY(need_run_state(c));
    if (!p || !grad_echo || !grad_dfactor) return c->fail(RWNMR_ERR_INVALID, "NULL argument");
    if (!p->dfactor) return c->fail(RWNMR_ERR_UNSUPPORTED, "the adjoint differentiates per-phase decrease factors");
    RW_TRY(check_geom(c, p->bc, p->shift));
    RW_TRY(check_dfactor(c, p->dfactor));
    if (p->n_echoes < 0 || p->steps_per_echo < 1) return c->fail(RWNMR_ERR_INVALID, "bad echo count / steps per echo");
    const int64_t nmax = (int64_t)p->n_echoes * p->steps_per_echo;
    if (nmax > (1ll << 28)) return c->fail(RWNMR_ERR_UNSUPPORTED, "walk too long");
    bool positive = true;
    for (int q = 0; q < c->n_phases; q++) positive = positive && p->dfactor[q] > 0.0;
    if (positive)
    {
        // d echo_sum[e] / d f_q = (sum over walkers of E c_q) / f_q: one integer walk with the exact
        // sensitivity sums, on scratch state; the FP64 replay below is for a zero factor
        std::vector<double> sens((size_t)(p->n_echoes + 1) * c->n_phases);
        RW_TRY(cpmg_impl(c, p, true, true, nullptr, nullptr, nullptr, sens.data(), nullptr));
        for (int q = 0; q < c->n_phases; q++)
        {
            double s = 0.0;
            for (int e = 1; e <= p->n_echoes; e++) s += grad_echo[e] * sens[(size_t)e * c->n_phases + q];
            grad_dfactor[q] = s / p->dfactor[q];
        }
        return RWNMR_OK;
    }
    cudaSetDevice(c->device);
    const int slots = phase_slots(c->n_phases);
    // derivative tables: dt[q][k] = k * f_q^(k-1) (so d/df_q of walker energy is dt[q][c_q] * prod_{r != q} t[r][c_r])
    std::vector<double> t;
    build_tables(p->dfactor, c->n_phases, slots, nmax, &t, nullptr);
    const size_t stride = (size_t)nmax + 1;
    std::vector<double> tab(2 * slots * stride);
    for (int q = 0; q < slots; q++)
        for (size_t k = 0; k < stride; k++)
        {
            tab[q * stride + k] = t[q * stride + k];
            tab[(slots + q) * stride + k] = k == 0 ? 0.0 : (double)k * t[q * stride + k - 1];
        }
    const dim3 grid = walk_grid(c->n);
    RW_CUDA(c, c->tfp.ensure(tab.size()), "tables");
    RW_CUDA(c, c->grad.ensure((size_t)p->n_echoes + 1), "grad");
    RW_CUDA(c, c->partial.ensure((size_t)grid.x * slots), "partials");
    RW_CUDA(c, cudaMemcpyAsync(c->tfp.p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, c->stream), "tables upload");
    RW_CUDA(c, cudaMemcpyAsync(c->grad.p, grad_echo, ((size_t)p->n_echoes + 1) * 8, cudaMemcpyHostToDevice, c->stream),
            "grad upload");
    RW_CUDA(c, cudaMemsetAsync(c->status.p, 0, sizeof(unsigned), c->stream), "status reset");
    AdjointLaunch L{};
    L.n_echoes = p->n_echoes;
    L.steps_per_echo = p->steps_per_echo;
    L.t = c->tfp.p;
    L.tstride = (int)stride;
    L.grad = c->grad.p;
    L.partial = c->partial.p;
    L.status = c->status.p;
    RW_CUDA(c, cudaEventRecord(c->ev0, c->stream), "event");
    if (c->n > 0)
    {
        RW_CUDA(c, launch_cpmg_adjoint(bc_key(p->bc, p->shift), slots, c->image(p->bc, p->shift), c->state(), L, grid,
                                       c->stream), "adjoint kernel");
        c->launches++;
    }
    RW_CUDA(c, cudaEventRecord(c->ev1, c->stream), "event");
    std::vector<double> part((size_t)grid.x * slots, 0.0);
    if (c->n > 0)
        RW_CUDA(c, cudaMemcpyAsync(part.data(), c->partial.p, part.size() * 8, cudaMemcpyDeviceToHost, c->stream),
                "partials readback");
    RW_TRY(c->check_status("cpmg adjoint"));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->last_ms = ms;
    for (int q = 0; q < c->n_phases; q++)
    {
        double s = 0.0;
        for (unsigned b = 0; b < grid.x; b++) s += part[(size_t)b * slots + q];
        grad_dfactor[q] = s;
    }
    // echo 0 does not depend on the decrease factors
    return RWNMR_OK;
}

// ---- collision mapping ------------------------------------------------------------------------
static rwnmr_status map_impl(rwnmr_ctx *c, int32_t bc, int32_t shift, int64_t steps, uint32_t *collisions,
                             bool from_initial);

constexpr int64_t kMapResortSteps = 2048; // steps per launch of a re-sorted mapping walk

// Re-sorts the stored walkers by their current positions -- the upload-time order by start position
// loses its locality as a long walk spreads them: every persistent per-walker array is permuted
// alike and the stored-to-upload permutation is composed, so all outputs still come back in upload
// order.
static rwnmr_status reorder_walkers(rwnmr_ctx *c, int shift)
{
    const int64_t n = c->n;
    if (n <= 1) return RWNMR_OK;
    const size_t n1 = (size_t)n;
    const int slots = phase_slots(c->n_phases);
    RW_CUDA(c, c->sperm.ensure(n1), "walker reorder");
    RW_CUDA(c, walker_order(c->x.p, c->y.p, c->z.p, n, shift, c->order_scratch.p, c->sperm.p, c->stream),
            "walker reorder");
    RW_CUDA(c, c->ti32.ensure(n1), "walker reorder");
    for (DevBuf<int32_t> *a : {&c->x0, &c->y0, &c->z0, &c->x, &c->y, &c->z, &c->perm})
    {
        RW_CUDA(c, permute_u32(c->sperm.p, n, (const uint32_t *)a->p, (uint32_t *)c->ti32.p, c->stream), "walker reorder");
        std::swap(*a, c->ti32);
        RW_CUDA(c, c->ti32.ensure(n1), "walker reorder");
    }
    RW_CUDA(c, c->tu64.ensure(n1), "walker reorder");
    for (DevBuf<uint64_t> *a : {&c->seed0, &c->seed})
    {
        RW_CUDA(c, permute_u64(c->sperm.p, n, a->p, c->tu64.p, c->stream), "walker reorder");
        std::swap(*a, c->tu64);
        RW_CUDA(c, c->tu64.ensure(n1), "walker reorder");
    }
    RW_CUDA(c, c->tu32.ensure(n1 * slots), "walker reorder");
    for (int q = 0; q < slots; q++)
        RW_CUDA(c, permute_u32(c->sperm.p, n, c->coll.p + q * n1, c->tu32.p + q * n1, c->stream), "walker reorder");
    std::swap(c->coll, c->tu32);
    if (c->has_wf)
    {
        RW_CUDA(c, c->tf64.ensure(n1), "walker reorder");
        RW_CUDA(c, permute_u64(c->sperm.p, n, (const uint64_t *)c->wf.p, (uint64_t *)c->tf64.p, c->stream),
                "walker reorder");
        std::swap(c->wf, c->tf64);
    }
    c->h_perm_valid = false;
    c->launches += 7 + 9 + slots + (c->has_wf ? 1 : 0); // the sort's 7 kernels, one per permuted array
    return RWNMR_OK;
}

rwnmr_status rwnmr_map_run(rwnmr_ctx *c, int32_t bc, int32_t shift, int64_t steps, uint32_t *collisions)
{
    return map_impl(c, bc, shift, steps, collisions, true);
}

rwnmr_status rwnmr_map_continue(rwnmr_ctx *c, int32_t bc, int32_t shift, int64_t steps, uint32_t *collisions)
{
    return map_impl(c, bc, shift, steps, collisions, false);
}

static rwnmr_status map_impl(rwnmr_ctx *c, int32_t bc, int32_t shift, int64_t steps, uint32_t *collisions,
                             bool from_initial)
{
    NvtxRange nvtx(from_initial ? "rwnmr_map_run" : "rwnmr_map_continue");
    RW_TRY(need_run_state(c));
    RW_TRY(check_geom(c, bc, shift));
    if (steps < 0 || steps > (1ll << 31) - 1) return c->fail(RWNMR_ERR_INVALID, "bad step count");
    cudaSetDevice(c->device);
    const int slots = phase_slots(c->n_phases);
    RW_CUDA(c, cudaMemsetAsync(c->status.p, 0, sizeof(unsigned), c->stream), "status reset");
    CpmgLaunch L{};
    L.record = 0;
    L.status = c->status.p;
    L.tstride = 1;
    const DevImage im = c->image(bc, shift);
    WalkState st = c->state();
    // long walks of many walkers: shorter launches with the walkers re-sorted by position between
    // them, so a warp's gathers keep sharing cache lines (the sorted start order fades as they spread)
    const bool resort = c->n >= (1 << 16) && steps > 2 * kMapResortSteps;
    const int64_t chunk = resort ? kMapResortSteps : (1 << 14);
    RW_CUDA(c, cudaEventRecord(c->ev0, c->stream), "event");
    if (c->n > 0)
    {
        if (steps == 0)
        {
            L.e_begin = 0;
            L.e_end = 0;
            L.from_initial = from_initial ? 1 : 0;
            L.steps_per_echo = 1;
            RW_CUDA(c, launch_cpmg_walk(bc_key(bc, shift), slots, im, st, L, walk_grid(c->n), c->stream), "map kernel");
            c->launches++;
        }
        for (int64_t s = 0; s < steps; s += chunk)
        {
            if (resort && s > 0)
            {
                RW_TRY(reorder_walkers(c, shift));
                st = c->state();
            }
            L.e_begin = 0;
            L.e_end = 1;
            L.steps_per_echo = (int)std::min<int64_t>(chunk, steps - s);
            L.from_initial = (s == 0 && from_initial) ? 1 : 0;
            RW_CUDA(c, launch_cpmg_walk(bc_key(bc, shift), slots, im, st, L, walk_grid(c->n), c->stream), "map kernel");
            c->launches++;
        }
    }
    RW_CUDA(c, cudaEventRecord(c->ev1, c->stream), "event");
    RW_TRY(c->check_status("map walk"));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->last_ms = ms;
    if (collisions && c->n > 0)
    {
        const int P = c->n_phases;
        std::vector<uint32_t> tmp((size_t)c->n * P);
        RW_CUDA(c, cudaMemcpyAsync(tmp.data(), c->coll.p, tmp.size() * 4, cudaMemcpyDeviceToHost, c->stream), "readback");
        RW_CUDA(c, cudaStreamSynchronize(c->stream), "readback");
        RW_TRY(host_perm(c));
        for (int64_t i = 0; i < c->n; i++)
        {
            uint32_t s = 0;
            for (int q = 0; q < P; q++) s += tmp[(size_t)q * c->n + i];
            collisions[c->h_perm[(size_t)i]] = s;
        }
    }
    return RWNMR_OK;
}

// ---- PFGSE ------------------------------------------------------------------------------------
static rwnmr_status pfgse_impl(rwnmr_ctx *c, const rwnmr_pfgse_params *p, double *M, double *esum, uint64_t *msd,
                               bool want_grad, double kscale, const double *dir, double *dMdg)
{
    NvtxRange nvtx(want_grad ? "rwnmr_pfgse_grad_g" : "rwnmr_pfgse_run");
    RW_TRY(need_run_state(c));
    if (!p) return c->fail(RWNMR_ERR_INVALID, "params is NULL");
    RW_TRY(check_geom(c, p->bc, p->shift));
    const bool per_walker = p->dfactor == nullptr;
    RW_TRY(per_walker ? check_walker_dfactor(c) : check_dfactor(c, p->dfactor));
    if (p->n_delta < 0 || p->n_g < 0 || (p->n_delta > 0 && !p->steps) || (p->n_g > 0 && !p->kvec))
        return c->fail(RWNMR_ERR_INVALID, "bad PFGSE sizes");
    for (int i = 0; i < p->n_delta; i++)
        if (p->steps[i] < 0 || (i && p->steps[i] < p->steps[i - 1]))
            return c->fail(RWNMR_ERR_INVALID, "PFGSE steps must be non-negative and non-decreasing");
    const int smax = p->n_delta ? p->steps[p->n_delta - 1] : 0;
    if (smax > (1 << 20)) return c->fail(RWNMR_ERR_UNSUPPORTED, "PFGSE walks are limited to 2^20 steps");
    cudaSetDevice(c->device);
    // gradient along a single axis -> displacement histogram path
    int axis = -1;
    {
        bool nz[3] = {false, false, false};
        for (int j = 0; j < p->n_g; j++)
            for (int a = 0; a < 3; a++) nz[a] |= p->kvec[3 * j + a] != 0.0;
        int cnt = nz[0] + nz[1] + nz[2];
        if (cnt == 0) axis = 2;
        else if (cnt == 1) axis = nz[0] ? 0 : (nz[1] ? 1 : 2);
        if (want_grad && dir)
        {
            int dn = (dir[0] != 0.0) + (dir[1] != 0.0) + (dir[2] != 0.0);
            if (dn != 1 || (axis >= 0 && dir[axis] == 0.0 && cnt)) axis = -1;
            else if (cnt == 0) axis = dir[0] != 0.0 ? 0 : (dir[1] != 0.0 ? 1 : 2);
        }
        if (p->n_g > kDirectMaxG && axis < 0)
            return c->fail(RWNMR_ERR_UNSUPPORTED, "general-direction PFGSE handles at most %d gradient points", kDirectMaxG);
        if (axis < 0)
            for (int k = 0; k < 3 * p->n_g; k++)
                if (!(std::fabs(p->kvec[k] * p->res) < 0x1p40))
                    return c->fail(RWNMR_ERR_UNSUPPORTED, "general-direction PFGSE needs |k res| < 2^40 (got %g)",
                                   p->kvec[k] * p->res);
    }
    const int slots = phase_slots(c->n_phases);
    std::vector<uint64_t> fx;
    std::vector<double> t;
    if (!per_walker) build_tables(p->dfactor, c->n_phases, slots, smax, axis < 0 ? &t : nullptr, &fx);
    const int nd = p->n_delta, ng = p->n_g;
    const int hh = smax;
    const size_t nbins = 2 * (size_t)hh + 1;
    if (!per_walker)
    {
        RW_CUDA(c, c->tfx.ensure(fx.size()), "tables");
        RW_CUDA(c, cudaMemcpyAsync(c->tfx.p, fx.data(), fx.size() * 8, cudaMemcpyHostToDevice, c->stream), "tables");
    }
    if (axis < 0)
    {
        if (!per_walker)
        {
            RW_CUDA(c, c->tfp.ensure(t.size()), "tables");
            RW_CUDA(c, cudaMemcpyAsync(c->tfp.p, t.data(), t.size() * 8, cudaMemcpyHostToDevice, c->stream), "tables");
        }
        RW_CUDA(c, c->disp.ensure((size_t)std::max(nd, 1) * std::max<int64_t>(c->n, 1) * 3), "displacements");
        RW_CUDA(c, c->energy.ensure((size_t)std::max(nd, 1) * std::max<int64_t>(c->n, 1)), "energies");
    }
    else
    {
        RW_CUDA(c, c->hist.ensure((size_t)std::max(nd, 1) * nbins * 2), "histograms");
        RW_CUDA(c, cudaMemsetAsync(c->hist.p, 0, (size_t)nd * nbins * 16, c->stream), "histogram reset");
    }
    RW_CUDA(c, c->acc.ensure((size_t)std::max(nd, 1) * 6), "accumulators");
    RW_CUDA(c, cudaMemsetAsync(c->acc.p, 0, (size_t)nd * 6 * 8, c->stream), "accumulator reset");
    RW_CUDA(c, c->ibuf.ensure((size_t)std::max(nd, 1)), "steps");
    if (nd) RW_CUDA(c, cudaMemcpyAsync(c->ibuf.p, p->steps, (size_t)nd * 4, cudaMemcpyHostToDevice, c->stream), "steps");
    RW_CUDA(c, cudaMemsetAsync(c->status.p, 0, sizeof(unsigned), c->stream), "status reset");

    PfgseLaunch L{};
    L.n_delta = nd;
    L.steps = c->ibuf.p;
    L.tfx = c->tfx.p;
    L.t = c->tfp.p;
    L.tstride = smax + 1;
    L.acc = c->acc.p;
    L.axis = axis;
    L.hist_half = hh;
    L.hist = c->hist.p;
    L.disp = c->disp.p;
    L.energy = c->energy.p;
    L.wf = per_walker ? c->wf.p : nullptr;
    L.status = c->status.p;
    RW_CUDA(c, cudaEventRecord(c->ev0, c->stream), "event");
    if (c->n > 0 && nd > 0)
    {
        RW_CUDA(c, launch_pfgse_walk(bc_key(p->bc, p->shift), slots, c->image(p->bc, p->shift), c->state(), L,
                                     walk_grid(c->n), c->stream), "pfgse kernel");
        c->launches++;
    }
    // phase sums (the timed region ends after them)
    bool timed = false;
    std::vector<double> Mh((size_t)nd * ng, 0.0), Gh((size_t)nd * ng, 0.0);
    if (nd > 0 && ng > 0)
    {
        RW_CUDA(c, c->Mbuf.ensure((size_t)nd * ng), "phase buffer");
        RW_CUDA(c, c->gbuf.ensure((size_t)nd * ng), "phase buffer");
        if (axis >= 0)
        {
            std::vector<double> ka(ng);
            for (int j = 0; j < ng; j++) ka[j] = p->kvec[3 * j + axis];
            RW_CUDA(c, c->kbuf.ensure((size_t)ng * 3), "k buffer");
            RW_CUDA(c, cudaMemcpyAsync(c->kbuf.p, ka.data(), (size_t)ng * 8, cudaMemcpyHostToDevice, c->stream), "k upload");
            PhaseLaunch PL{};
            PL.hist = c->hist.p;
            PL.hist_half = hh;
            PL.kaxis = c->kbuf.p;
            PL.res = p->res;
            PL.kscale_axis = want_grad ? kscale * (dir ? dir[axis] : 0.0) : 0.0;
            PL.M = c->Mbuf.p;
            PL.dMdg = want_grad ? c->gbuf.p : nullptr;
            RW_CUDA(c, launch_pfgse_phase(PL, nd, ng, c->stream), "phase kernel");
            c->launches++;
            RW_CUDA(c, cudaEventRecord(c->ev1, c->stream), "event");
            timed = true;
            RW_CUDA(c, cudaMemcpyAsync(Mh.data(), c->Mbuf.p, Mh.size() * 8, cudaMemcpyDeviceToHost, c->stream), "readback");
            if (want_grad)
                RW_CUDA(c, cudaMemcpyAsync(Gh.data(), c->gbuf.p, Gh.size() * 8, cudaMemcpyDeviceToHost, c->stream), "readback");
        }
        else if (c->n > 0)
        {
            const int blocks = (int)std::min<int64_t>(1184, (c->n + 255) / 256);
            // k_ja res / (2 pi) mod 1 in 2^-64 turns, from the exact product k res (two FP64 terms)
            std::vector<uint64_t> kappa((size_t)ng * 3);
            for (size_t k = 0; k < kappa.size(); k++)
            {
                const double hi = p->kvec[k] * p->res, lo = std::fma(p->kvec[k], p->res, -hi);
                kappa[k] = fxcos::turns_q64_host(hi) + fxcos::turns_q64_host(lo);
            }
            RW_CUDA(c, c->kappa.ensure(kappa.size()), "k buffer");
            RW_CUDA(c, cudaMemcpyAsync(c->kappa.p, kappa.data(), kappa.size() * 8, cudaMemcpyHostToDevice, c->stream),
                    "k upload");
            RW_CUDA(c, c->dpart.ensure((size_t)nd * ng * blocks * 3), "partials");
            RW_CUDA(c, c->partial_g.ensure((size_t)nd * ng * blocks), "partials");
            DirectLaunch DL{};
            DL.n = c->n;
            DL.n_g = ng;
            DL.disp = c->disp.p;
            DL.energy = c->energy.p;
            DL.kappa = c->kappa.p;
            DL.res = p->res;
            DL.grad_on = want_grad ? 1 : 0;
            DL.kscale = kscale;
            for (int a = 0; a < 3; a++) DL.dir[a] = dir ? dir[a] : 0.0;
            DL.partial = c->dpart.p;
            DL.partial_g = c->partial_g.p;
            RW_CUDA(c, launch_pfgse_direct(DL, nd, blocks, c->stream), "direct phase kernel");
            c->launches++;
            RW_CUDA(c, cudaEventRecord(c->ev1, c->stream), "event");
            timed = true;
            std::vector<unsigned long long> part((size_t)nd * ng * blocks * 3);
            std::vector<double> partg;
            RW_CUDA(c, cudaMemcpyAsync(part.data(), c->dpart.p, part.size() * 8, cudaMemcpyDeviceToHost, c->stream), "readback");
            if (want_grad)
            {
                partg.resize((size_t)nd * ng * blocks);
                RW_CUDA(c, cudaMemcpyAsync(partg.data(), c->partial_g.p, partg.size() * 8, cudaMemcpyDeviceToHost, c->stream), "readback");
            }
            RW_CUDA(c, cudaStreamSynchronize(c->stream), "readback");
            // every walker added E cos 2^61 + 2^61 for every (i, j): exact sums, offset removed
            const __int128 offset = (__int128)c->n << 61;
            for (size_t k = 0; k < (size_t)nd * ng; k++)
            {
                __int128 v = -offset;
                double g = 0.0;
                for (int b = 0; b < blocks; b++)
                {
                    const unsigned long long *l = &part[(k * blocks + b) * 3];
                    v += (__int128)l[0] + ((__int128)l[1] << 21) + ((__int128)l[2] << 42);
                    if (want_grad) g += partg[k * blocks + b];
                }
                Mh[k] = std::ldexp((double)v, -61);
                Gh[k] = g;
            }
        }
    }
    if (!timed) RW_CUDA(c, cudaEventRecord(c->ev1, c->stream), "event");
    std::vector<unsigned long long> acc((size_t)nd * 6);
    if (nd) RW_CUDA(c, cudaMemcpyAsync(acc.data(), c->acc.p, acc.size() * 8, cudaMemcpyDeviceToHost, c->stream), "readback");
    RW_TRY(c->check_status("pfgse walk"));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->last_ms = ms;
    if (M) std::copy(Mh.begin(), Mh.end(), M);
    if (dMdg) std::copy(Gh.begin(), Gh.end(), dMdg);
    for (int i = 0; i < nd; i++)
    {
        if (esum) esum[i] = limbs_to_double(&acc[(size_t)i * 6]);
        if (msd)
            for (int a = 0; a < 3; a++) msd[(size_t)i * 3 + a] = acc[(size_t)i * 6 + 3 + a];
    }
    return RWNMR_OK;
}

rwnmr_status rwnmr_pfgse_run(rwnmr_ctx *c, const rwnmr_pfgse_params *p, double *M, double *esum, uint64_t *msd)
{
    return pfgse_impl(c, p, M, esum, msd, false, 0.0, nullptr, nullptr);
}

rwnmr_status rwnmr_pfgse_grad_g(rwnmr_ctx *c, const rwnmr_pfgse_params *p, double kscale, const double *dir,
                                double *dMdg)
{
    if (!c) return RWNMR_ERR_INVALID;
    if (!dir || !dMdg) return c->fail(RWNMR_ERR_INVALID, "NULL argument");
    return pfgse_impl(c, p, nullptr, nullptr, nullptr, true, kscale, dir, dMdg);
}

} // extern "C"
