// Test-oracle driver around the reference's own CPU implementation (RandomWalk_NMR).
//
// This file is compiled together with the reference's unmodified sources (Walker/, BitBlock/,
// RNG/, NMR_Simulation/, ConfigFiles/, FileHandler/, Math/, Utils/) by oracle/Makefile into
// oracle/_ref/librwnmr_ref.so. It is test infrastructure only: tests/ and the fixture script
// under tests/golden/ load it to pin the CPU restatement (oracle/rwnmr_oracle.cpp) and the
// product's host code against what the reference itself computes.
//
// The reference reads its configuration from ./config/default/<name>.config relative to the
// working directory (ConfigFiles/configFiles_defs.h:4-11), so every entry point writes those
// files into a caller-given scratch directory and runs with that directory as CWD. The user
// config path passed to each config class is the default path itself, so each file is read
// exactly once (ConfigFiles/rwnmr_config.cpp:18-22) and the RHO append quirk does not apply.
// GPU_USAGE is always false: the reference's CUDA methods are stubbed out below.

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include <malloc.h>
#include <unistd.h>
#include <sys/stat.h>

#include "NMR_Simulation/NMR_Simulation.h"
#include "NMR_Simulation/NMR_cpmg.h"
#include "NMR_Simulation/NMR_pfgse.h"
#include "NMR_Simulation/InternalField.h"
#include "NMR_Simulation/NMR_multitau.h"
#include "Walker/walker.h"

// ---------------------------------------------------------------------------------------------
// The reference's CUDA host methods live in *_cuda.cpp files that are not compiled here.
// GPU_USAGE is forced off, so these are never reached; they exist to satisfy the linker.
static void ref_no_gpu(const char *what)
{
    std::fprintf(stderr, "rwnmr oracle: reference GPU path %s is not built into the oracle\n", what);
    std::abort();
}
void NMR_cpmg::image_simulation_cuda() { ref_no_gpu("NMR_cpmg::image_simulation_cuda"); }
void NMR_PFGSE::simulation_cuda() { ref_no_gpu("NMR_PFGSE::simulation_cuda"); }
double **NMR_PFGSE::computeSamplesMagnitudeWithGpu()
{
    ref_no_gpu("NMR_PFGSE::computeSamplesMagnitudeWithGpu");
    return nullptr;
}
void NMR_Simulation::mapSimulation_CUDA_2D_histograms(bool) { ref_no_gpu("mapSimulation_CUDA_2D_histograms"); }
void NMR_Simulation::mapSimulation_CUDA_3D_histograms(bool) { ref_no_gpu("mapSimulation_CUDA_3D_histograms"); }

// ---------------------------------------------------------------------------------------------
extern "C" {

// Parameters that end up in the reference's rwnmr.config / uct.config.
struct ref_sim_params
{
    int32_t walkers;
    uint64_t seed;
    const char *placement;  // "random" | "point" | "cubic"
    int32_t deviation;      // PLACEMENT_DEVIATION
    const char *rho_type;   // "uniform" | "sigmoid"
    const double *rho;      // RHO values
    int32_t n_rho;
    double d0;              // um^2/ms
    double bulk_time;       // ms
    int32_t steps_per_echo;
    const char *bc;         // "noflux" | "periodic" | "mirror"
    double resolution;      // um
    int32_t voxel_division; // shifts
    double gamma;           // GIROMAGNETIC_RATIO
    const char *gamma_unit; // "mhertz" | "rad"
    int32_t histograms;
    int32_t histogram_size;
    const char *histogram_scale; // "linear" | "log"
};

struct ref_handle
{
    std::string workdir;
    NMR_Simulation *sim = nullptr;
};
}

namespace
{
std::string fmt_double(double v)
{
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.17g", v);
    return buf;
}

void mkdirs(const std::string &path)
{
    std::string acc;
    std::stringstream ss(path);
    std::string part;
    if (!path.empty() && path[0] == '/') acc = "/";
    while (std::getline(ss, part, '/'))
    {
        if (part.empty()) continue;
        acc += part + "/";
        ::mkdir(acc.c_str(), 0755);
    }
}

void write_file(const std::string &path, const std::string &text)
{
    std::ofstream f(path);
    f << text;
}

std::string rwnmr_text(const ref_sim_params &p)
{
    std::ostringstream o;
    o << "NAME: ref_oracle\n";
    o << "D0: " << fmt_double(p.d0) << "\n";
    o << "BULK_TIME: " << fmt_double(p.bulk_time) << "\n";
    o << "RHO_TYPE: " << p.rho_type << "\n";
    o << "RHO: {";
    for (int i = 0; i < p.n_rho; i++) o << (i ? ", " : "") << fmt_double(p.rho[i]);
    o << "}\n";
    o << "WALKERS: " << p.walkers << "\n";
    o << "WALKER_SAMPLES: 1\n";
    o << "WALKERS_PLACEMENT: " << p.placement << "\n";
    o << "PLACEMENT_DEVIATION: " << p.deviation << "\n";
    o << "STEPS_PER_ECHO: " << p.steps_per_echo << "\n";
    o << "SEED: " << p.seed << "\n";
    o << "BC: " << p.bc << "\n";
    o << "GIROMAGNETIC_RATIO: " << fmt_double(p.gamma) << "\n";
    o << "GIROMAGNETIC_UNIT: " << p.gamma_unit << "\n";
    o << "SAVE_IMG_INFO: false\nSAVE_BINIMG: false\nSAVE_WALKERS: false\n";
    o << "HISTOGRAMS: " << p.histograms << "\n";
    o << "HISTOGRAM_SIZE: " << p.histogram_size << "\n";
    o << "HISTOGRAM_SCALE: " << p.histogram_scale << "\n";
    o << "OPENMP_USAGE: false\nOPENMP_THREADS: 1\n";
    o << "GPU_USAGE: false\nBLOCKS: 4096\nTHREADSPERBLOCK: 1024\nECHOESPERKERNEL: 16\n";
    o << "REDUCE_IN_GPU: true\nMAX_RWSTEPS: 65536\n";
    return o.str();
}

std::string uct_text(const ref_sim_params &p, int nz)
{
    std::ostringstream o;
    o << "DIR_PATH: ./\nFILENAME: none\nFIRST_IDX: 0\nDIGITS: 1\nEXTENSION: .png\n";
    o << "SLICES: " << nz << "\n";
    o << "RESOLUTION: " << fmt_double(p.resolution) << "\n";
    o << "VOXEL_DIVISION: " << p.voxel_division << "\n";
    return o.str();
}

// Every config file the reference may open, written so that ./config/default/* exists.
void write_configs(const std::string &dir, const ref_sim_params &p, int nz, const std::string &cpmg,
                   const std::string &pfgse)
{
    mkdirs(dir + "/config/default");
    mkdirs(dir + "/config/imgs");
    mkdirs(dir + "/db");
    write_file(dir + "/config/default/rwnmr.config", rwnmr_text(p));
    write_file(dir + "/config/default/uct.config", uct_text(p, nz));
    write_file(dir + "/config/default/cpmg.config", cpmg);
    write_file(dir + "/config/default/pfgse.config", pfgse);
}

const char *kDefaultCpmg = "METHOD: image-based\nOBS_TIME: 1.0\nAPPLY_BULK: false\nTIME_VERBOSE: false\n"
                           "RESIDUAL_FIELD: none\nSAVE_MODE: false\n";
const char *kDefaultPfgse = "APPLY_BULK: false\nPULSE_WIDTH: 1.0\nMAX_GRADIENT: {0.0, 0.0, 1.0}\n"
                            "GRADIENT_SAMPLES: 2\nTIME_SEQ: manual\nTIME_SAMPLES: 1\nTIME_VALUES: {1.0}\n"
                            "APPLY_SCALE_FACTOR: false\nINSPECTION_LENGTH: 1.0\nTHRESHOLD_TYPE: samples\n"
                            "THRESHOLD_VALUE: 2\nALLOW_WALKER_SAMPLING: false\nSAVE_MODE: false\n";

struct cwd_guard
{
    char old[4096];
    explicit cwd_guard(const std::string &dir)
    {
        if (!getcwd(old, sizeof(old))) old[0] = 0;
        if (chdir(dir.c_str()) != 0) std::fprintf(stderr, "rwnmr oracle: chdir(%s) failed\n", dir.c_str());
    }
    ~cwd_guard()
    {
        if (old[0] && chdir(old) != 0) std::fprintf(stderr, "rwnmr oracle: chdir back failed\n");
    }
};
} // namespace

extern "C" {

// Builds an NMR_Simulation over a voxel image (uint8 [nz][ny][nx], 0 = pore, else solid) the way
// NMR_Simulation::readImage does after loading (NMR_Simulation.cpp:300-322: createBinaryMap's
// "non-zero is solid" rule, createBitBlockMap, countPoresInBitBlock, countInterfacePoreMatrix),
// then places the walkers with NMR_Simulation::setWalkers (NMR_Simulation.cpp:324-363).
void *ref_sim_create(const char *workdir, const uint8_t *vox, int nx, int ny, int nz, const ref_sim_params *p)
{
    ref_handle *h = new ref_handle();
    h->workdir = workdir;
    write_configs(h->workdir, *p, nz, kDefaultCpmg, kDefaultPfgse);
    cwd_guard g(h->workdir);
    rwnmr_config rw(std::string(CONFIG_ROOT) + RWNMR_CONFIG_DEFAULT);
    uct_config uct(std::string(CONFIG_ROOT) + UCT_CONFIG_DEFAULT);
    h->sim = new NMR_Simulation(rw, uct, "./");
    NMR_Simulation &s = *h->sim;
    s.numberOfImages = nz;
    s.depth = nz;
    s.height = ny;
    s.width = nx;
    s.binaryMap.clear();
    for (int z = 0; z < nz; z++)
    {
        cv::Mat slice = cv::Mat::zeros(ny, nx, CV_8UC1);
        for (int y = 0; y < ny; y++)
        {
            uchar *row = slice.ptr<uchar>(y);
            const uint8_t *src = vox + ((size_t)z * ny + y) * nx;
            for (int x = 0; x < nx; x++) row[x] = src[x] ? 255 : 0;
        }
        s.binaryMap.push_back(slice);
    }
    s.createBitBlockMap();
    s.countPoresInBitBlock();
    s.countInterfacePoreMatrix();
    s.setWalkers();
    return h;
}

void ref_sim_destroy(void *hv)
{
    ref_handle *h = (ref_handle *)hv;
    if (!h) return;
    delete h->sim;
    delete h;
}

// i64 out[12]: numberOfPores, interfacePoreMatrix, blockColumns, blockRows, blockDepth,
//              numberOfBlocks, width, height, depth, numberOfWalkers, voxelDivision, stepsPerEcho
// f64 outd[5]: porosity, SVp, timeInterval, imageVoxelResolution, giromagneticRatio
void ref_sim_info(void *hv, int64_t *out, double *outd)
{
    NMR_Simulation &s = *((ref_handle *)hv)->sim;
    out[0] = s.numberOfPores;
    out[1] = s.interfacePoreMatrix;
    out[2] = s.bitBlock.blockColumns;
    out[3] = s.bitBlock.blockRows;
    out[4] = s.bitBlock.blockDepth;
    out[5] = s.bitBlock.numberOfBlocks;
    out[6] = s.bitBlock.imageColumns;
    out[7] = s.bitBlock.imageRows;
    out[8] = s.bitBlock.imageDepth;
    out[9] = (int64_t)s.walkers.size();
    out[10] = s.voxelDivision;
    out[11] = s.stepsPerEcho;
    outd[0] = s.porosity;
    outd[1] = s.SVp;
    outd[2] = s.timeInterval;
    outd[3] = s.imageVoxelResolution;
    outd[4] = s.giromagneticRatio;
}

void ref_sim_blocks(void *hv, uint64_t *out)
{
    NMR_Simulation &s = *((ref_handle *)hv)->sim;
    std::memcpy(out, s.bitBlock.blocks, sizeof(uint64_t) * (size_t)s.bitBlock.numberOfBlocks);
}

// Initial walker state as the reference's setup left it.
void ref_sim_walkers(void *hv, int32_t *x0, int32_t *y0, int32_t *z0, uint64_t *seed0, double *dfactor)
{
    NMR_Simulation &s = *((ref_handle *)hv)->sim;
    for (size_t i = 0; i < s.walkers.size(); i++)
    {
        const Walker &w = s.walkers[i];
        x0[i] = w.initialPosition.x;
        y0[i] = w.initialPosition.y;
        z0[i] = w.initialPosition.z;
        seed0[i] = w.initialSeed;
        dfactor[i] = w.decreaseFactor;
    }
}

// Overrides every walker's decrease factor (for walks at a chosen relaxivity).
void ref_sim_set_dfactor(void *hv, double dfactor)
{
    NMR_Simulation &s = *((ref_handle *)hv)->sim;
    for (auto &w : s.walkers) w.decreaseFactor = dfactor;
}

// Steps every walker from its initial state for n_echoes x steps_per_echo steps with the
// reference's own Walker::map (mode 0, counts collisions) or Walker::walk (mode 1, relaxes
// energy) -- Walker/walker.cpp:197-231 -- in the serial walker-major order of
// NMR_cpmg::image_simulation_omp (NMR_cpmg.cpp:205-228).
//   per_echo: mode 0 -> sum over walkers of collisions gained during echo e ([n_echoes], u64)
//             mode 1 -> serial FP64 energy sum after echo e ([n_echoes + 1], index 0 = start)
//   final state per walker: position, collisions, energy, current seed.
void ref_walk(void *hv, int mode, int n_echoes, int steps_per_echo, void *per_echo, int32_t *xf, int32_t *yf,
              int32_t *zf, uint32_t *coll, double *energy, uint64_t *seed)
{
    NMR_Simulation &s = *((ref_handle *)hv)->sim;
    size_t n = s.walkers.size();
    for (auto &w : s.walkers)
    {
        w.resetPosition();
        w.resetSeed();
        w.resetEnergy();
        w.resetCollisions();
    }
    uint64_t *pc = (uint64_t *)per_echo;
    double *pe = (double *)per_echo;
    if (mode == 1)
    {
        double sum = 0.0;
        for (size_t i = 0; i < n; i++) sum += s.walkers[i].energy;
        pe[0] = sum;
    }
    for (int e = 0; e < n_echoes; e++)
    {
        uint64_t before = 0, after = 0;
        if (mode == 0)
            for (size_t i = 0; i < n; i++) before += s.walkers[i].collisions;
        for (size_t i = 0; i < n; i++)
            for (int st = 0; st < steps_per_echo; st++)
            {
                if (mode == 0) s.walkers[i].map(s.bitBlock);
                else s.walkers[i].walk(s.bitBlock);
            }
        if (mode == 0)
        {
            for (size_t i = 0; i < n; i++) after += s.walkers[i].collisions;
            pc[e] = after - before;
        }
        else
        {
            double sum = 0.0;
            for (size_t i = 0; i < n; i++) sum += s.walkers[i].energy;
            pe[e + 1] = sum;
        }
    }
    for (size_t i = 0; i < n; i++)
    {
        const Walker &w = s.walkers[i];
        if (xf) xf[i] = w.position_x;
        if (yf) yf[i] = w.position_y;
        if (zf) zf[i] = w.position_z;
        if (coll) coll[i] = w.collisions;
        if (energy) energy[i] = w.energy;
        if (seed) seed[i] = w.currentSeed;
    }
}

// The reference's CPMG sequence on CPU: NMR_cpmg::set() (time framework, collision-mapping walk,
// relaxivity update; NMR_cpmg.cpp:112-146) then image_simulation_omp (NMR_cpmg.cpp:177-233).
// raw[]: the un-normalised echo sums; out[]: after applyBulk (if apply_bulk) and normalizeSignal
// (NMR_cpmg.cpp:346-384). Returns the number of values (n_echoes + 1), or -1 if cap is too small.
int ref_cpmg(void *hv, double obs_time, int apply_bulk, double *raw, double *out, double *times, int cap,
             uint32_t *map_collisions)
{
    ref_handle *h = (ref_handle *)hv;
    NMR_Simulation &s = *h->sim;
    std::ostringstream c;
    c << "METHOD: image-based\nOBS_TIME: " << fmt_double(obs_time) << "\nAPPLY_BULK: " << (apply_bulk ? "true" : "false")
      << "\nTIME_VERBOSE: false\nRESIDUAL_FIELD: none\nSAVE_MODE: false\n";
    write_file(h->workdir + "/config/default/cpmg.config", c.str());
    cwd_guard g(h->workdir);
    cpmg_config cfg(std::string(CONFIG_ROOT) + CPMG_CONFIG_DEFAULT);
    NMR_cpmg cpmg(s, cfg);
    cpmg.set();
    if (map_collisions)
        for (size_t i = 0; i < s.walkers.size(); i++) map_collisions[i] = s.walkers[i].collisions;
    cpmg.image_simulation_omp();
    int n = (int)cpmg.signal_amps.size();
    if (n > cap) return -1;
    for (int i = 0; i < n; i++) raw[i] = cpmg.signal_amps[i];
    if (cpmg.getApplyBulkRelaxation()) cpmg.applyBulk();
    cpmg.normalizeSignal();
    for (int i = 0; i < n; i++) out[i] = cpmg.signal_amps[i];
    for (int i = 0; i < n && i < (int)cpmg.signal_times.size(); i++) times[i] = cpmg.signal_times[i];
    return n;
}

// The reference's CPMG sequence with a chosen METHOD ("image-based" or "histogram"): NMR_cpmg::set()
// (collision-mapping walk with HISTOGRAMS windows, xi-rate histograms, relaxivity update;
// NMR_cpmg.cpp:112-146, NMR_Simulation.cpp:1456-1479, 1787-1841) and the body of
// NMR_cpmg::run_simulation (NMR_cpmg.cpp:149-175): the image-based walk, or createPenaltiesVector +
// histogram_simulation (NMR_cpmg.cpp:235-343); then applyBulk and normalizeSignal.
//   raw[], out[], times[]: as ref_cpmg. hist_bins/hist_amps [histogram size]: the global xi-rate
//   histogram (NMR_Simulation::histogram); list_bins/list_amps [n_list][histogram size]: the
//   per-window histograms (NMR_Simulation::histogramList). sizes[0] <- histogram size,
//   sizes[1] <- number of windows. Returns the number of echo values, or -1 if a cap is too small.
int ref_cpmg_method(void *hv, const char *method, double obs_time, int apply_bulk, double *raw, double *out,
                    double *times, int cap, double *hist_bins, double *hist_amps, double *list_bins, double *list_amps,
                    int hcap, int32_t *sizes)
{
    ref_handle *h = (ref_handle *)hv;
    NMR_Simulation &s = *h->sim;
    std::ostringstream c;
    c << "METHOD: " << method << "\nOBS_TIME: " << fmt_double(obs_time)
      << "\nAPPLY_BULK: " << (apply_bulk ? "true" : "false")
      << "\nTIME_VERBOSE: false\nRESIDUAL_FIELD: none\nSAVE_MODE: false\n";
    write_file(h->workdir + "/config/default/cpmg.config", c.str());
    cwd_guard g(h->workdir);
    cpmg_config cfg(std::string(CONFIG_ROOT) + CPMG_CONFIG_DEFAULT);
    NMR_cpmg cpmg(s, cfg);
    cpmg.set();
    if (cpmg.getMethod() == "histogram")
    {
        std::vector<double> rho = s.rwNMR_config.getRho();
        if (s.rwNMR_config.getRhoType() == "uniform") cpmg.createPenaltiesVector(rho[0]);
        else cpmg.createPenaltiesVector(rho);
        cpmg.histogram_simulation();
    }
    else
        cpmg.image_simulation_omp();
    const int n = (int)cpmg.signal_amps.size();
    const int hs = s.histogram.getSize();
    const int nl = (int)s.histogramList.size();
    sizes[0] = hs;
    sizes[1] = nl;
    if (n > cap || hs > hcap || (int)s.histogram.bins.size() != hs) return -1;
    for (int i = 0; i < n; i++) raw[i] = cpmg.signal_amps[i];
    if (cpmg.getApplyBulkRelaxation()) cpmg.applyBulk();
    cpmg.normalizeSignal();
    for (int i = 0; i < n; i++) out[i] = cpmg.signal_amps[i];
    for (int i = 0; i < n && i < (int)cpmg.signal_times.size(); i++) times[i] = cpmg.signal_times[i];
    for (int i = 0; i < hs; i++)
    {
        hist_bins[i] = s.histogram.bins[i];
        hist_amps[i] = s.histogram.amps[i];
    }
    for (int l = 0; l < nl && list_bins; l++)
        for (int i = 0; i < hs; i++)
        {
            list_bins[(size_t)l * hs + i] = s.histogramList[l].bins[i];
            list_amps[(size_t)l * hs + i] = s.histogramList[l].amps[i];
        }
    return n;
}

// The reference's multitau sequence on CPU (NMR_multitau::run, NMR_multitau.cpp:187-204): one
// CPMG per echo time (setTauSequence), each run's first normalised echo kept. cpmg_text and
// multitau_text become default/cpmg.config and default/multitau.config. Writes steps[k], times[k]
// and amps[k]; returns the number of echo times, or -1 if cap is too small.
int ref_multitau(void *hv, const char *cpmg_text, const char *multitau_text, int cap, uint32_t *steps, double *times,
                 double *amps)
{
    ref_handle *h = (ref_handle *)hv;
    NMR_Simulation &s = *h->sim;
    write_file(h->workdir + "/config/default/cpmg.config", cpmg_text);
    write_file(h->workdir + "/config/default/multitau.config", multitau_text);
    cwd_guard g(h->workdir);
    multitau_config mcfg(std::string(CONFIG_ROOT) + MULTITAU_CONFIG_DEFAULT);
    cpmg_config ccfg(std::string(CONFIG_ROOT) + CPMG_CONFIG_DEFAULT);
    const uint32_t spe = s.getStepsPerEcho();
    NMR_multitau mt(s, mcfg, ccfg);
    mt.run();
    s.setNumberOfStepsPerEcho(spe); // multitau leaves the last echo time's steps behind
    const int n = (int)mt.signalAmps.size();
    if (n > cap || mt.requiredSteps.size() != (size_t)n || mt.signalTimes.size() != (size_t)n) return -1;
    for (int k = 0; k < n; k++)
    {
        steps[k] = mt.requiredSteps[k];
        times[k] = mt.signalTimes[k];
        amps[k] = mt.signalAmps[k];
    }
    return n;
}

// The reference's PFGSE sequence on CPU (NMR_PFGSE::run, NMR_pfgse.cpp:98-131, without file
// output): initial mapping walk to the longest time, then per exposure time the CPU simulation
// (simulation_omp, NMR_pfgse.cpp:1658-1806), bulk, and the D(t) recoveries.
//   Mkt [n_delta * n_g]: normalised M(k, Delta) after bulk;  steps[n_delta]: RW steps per Delta;
//   dsat/dmsd [n_delta]; kvec [n_g * 3]; delta_out [n_delta]: exposure times used.
// Returns n_delta, or -1 if cap_delta is too small.
} // extern "C"

// Outputs of one PFGSE sequence run beyond the sequence's own vectors (walker-sampling statistics).
struct pfgse_extra
{
    double *Mstd, *lhs, *lhs_std, *dsat_err, *dsat_std, *dmsd_std;
};

static int run_pfgse_sequence(ref_handle *h, const std::string &cfg_text, int n_g, int cap_delta, int samples,
                              double *Mkt, int32_t *steps, double *dsat, double *dmsd, double *kvec, double *delta_out,
                              const pfgse_extra *x)
{
    NMR_Simulation &s = *h->sim;
    write_file(h->workdir + "/config/default/pfgse.config", cfg_text);
    cwd_guard g(h->workdir);
    const uint old_samples = s.walkerSamples;
    if (samples > 0) s.walkerSamples = (uint)samples;
    pfgse_config cfg(std::string(CONFIG_ROOT) + PFGSE_CONFIG_DEFAULT);
    NMR_PFGSE pf(s, cfg);
    int nd = (int)pf.exposureTimes.size();
    if (nd > cap_delta)
    {
        s.walkerSamples = old_samples;
        return -1;
    }
    for (int j = 0; j < n_g; j++)
    {
        kvec[3 * j + 0] = pf.vecK[j].getX();
        kvec[3 * j + 1] = pf.vecK[j].getY();
        kvec[3 * j + 2] = pf.vecK[j].getZ();
    }
    // NMR_PFGSE::simulation_omp sums into a malloc'd array that it never zeroes
    // (Utils/myAllocator.cpp:43-51, NMR_pfgse.cpp:1673-1680), so later exposure times would pick
    // up recycled heap contents. glibc's M_PERTURB makes malloc return zero-filled memory (the
    // complement of 0xff), which gives the evidently intended zero-initialised sums. glibc's
    // per-thread cache bypasses M_PERTURB, so the calling process must also run with
    // GLIBC_TUNABLES=glibc.malloc.tcache_count=0 (tests/golden/make_golden.py does).
    mallopt(M_PERTURB, 0xff);
    pf.resetCurrentTime();
    pf.correctExposureTimes();
    pf.runInitialMapSimulation();
    pf.resetNMR();
    for (int t = 0; t < nd; t++)
    {
        pf.setExposureTime(pf.getExposureTime(t));
        pf.set();
        pf.runSequence();
        pf.recoverDsat();
        pf.recoverDmsd();
        for (int j = 0; j < n_g; j++) Mkt[(size_t)t * n_g + j] = pf.Mkt[j];
        steps[t] = (int32_t)s.simulationSteps;
        dsat[t] = pf.getD_sat();
        dmsd[t] = pf.getD_msd();
        delta_out[t] = pf.getExposureTime();
        if (x)
        {
            for (int j = 0; j < n_g; j++)
            {
                x->Mstd[(size_t)t * n_g + j] = pf.Mkt_stdev[j];
                x->lhs[(size_t)t * n_g + j] = pf.LHS[j];
                x->lhs_std[(size_t)t * n_g + j] = pf.LHS_stdev[j];
            }
            x->dsat_err[t] = pf.getD_sat_error();
            x->dsat_std[t] = pf.getD_sat_stdev();
            x->dmsd_std[t] = pf.getD_msd_stdev();
        }
        pf.incrementCurrentTime();
    }
    mallopt(M_PERTURB, 0);
    s.walkerSamples = old_samples;
    return nd;
}

static std::string pfgse_text(double pulse_width, double gx, double gy, double gz, int n_g, const char *time_seq, int n_t,
                              double t_min, double t_max, const double *t_values, int apply_bulk,
                              const char *threshold_type, double threshold_value, int threshold_window,
                              bool allow_sampling)
{
    std::ostringstream c;
    c << "APPLY_BULK: " << (apply_bulk ? "true" : "false") << "\n";
    c << "PULSE_WIDTH: " << fmt_double(pulse_width) << "\n";
    c << "MAX_GRADIENT: {" << fmt_double(gx) << ", " << fmt_double(gy) << ", " << fmt_double(gz) << "}\n";
    c << "GRADIENT_SAMPLES: " << n_g << "\n";
    c << "TIME_SEQ: " << time_seq << "\n";
    c << "TIME_SAMPLES: " << n_t << "\n";
    if (std::string(time_seq) == "manual")
    {
        c << "TIME_VALUES: {";
        for (int i = 0; i < n_t; i++) c << (i ? ", " : "") << fmt_double(t_values[i]);
        c << "}\n";
    }
    c << "TIME_MIN: " << fmt_double(t_min) << "\nTIME_MAX: " << fmt_double(t_max) << "\n";
    c << "APPLY_SCALE_FACTOR: false\nINSPECTION_LENGTH: 1.0\n";
    c << "THRESHOLD_TYPE: " << threshold_type << "\nTHRESHOLD_VALUE: " << fmt_double(threshold_value) << "\n";
    c << "THRESHOLD_WINDOW: " << threshold_window << "\n";
    c << "ALLOW_WALKER_SAMPLING: " << (allow_sampling ? "true" : "false") << "\nAPPLY_ABSORPTION: false\nSAVE_MODE: false\n";
    return c.str();
}

extern "C" {

int ref_pfgse(void *hv, double pulse_width, double gx, double gy, double gz, int n_g, const char *time_seq, int n_t,
              double t_min, double t_max, const double *t_values, int apply_bulk, const char *threshold_type,
              double threshold_value, int threshold_window, int cap_delta, double *Mkt, int32_t *steps, double *dsat,
              double *dmsd, double *kvec, double *delta_out)
{
    return run_pfgse_sequence((ref_handle *)hv,
                              pfgse_text(pulse_width, gx, gy, gz, n_g, time_seq, n_t, t_min, t_max, t_values, apply_bulk,
                                         threshold_type, threshold_value, threshold_window, false),
                              n_g, cap_delta, 0, Mkt, steps, dsat, dmsd, kvec, delta_out, nullptr);
}

// The same sequence with ALLOW_WALKER_SAMPLING: true and WALKER_SAMPLES = samples
// (recoverDsatWithSampling / recoverDmsdWithSampling, NMR_pfgse.cpp:876-1097, 1173-1290). Extra
// outputs per exposure time: Mstd, lhs, lhs_std [n_delta * n_g]; dsat_err, dsat_std, dmsd_std [n_delta].
int ref_pfgse_sampling(void *hv, int samples, double pulse_width, double gx, double gy, double gz, int n_g,
                       const char *time_seq, int n_t, const double *t_values, int apply_bulk, const char *threshold_type,
                       double threshold_value, int cap_delta, double *Mkt, int32_t *steps, double *dsat, double *dmsd,
                       double *kvec, double *delta_out, double *Mstd, double *lhs, double *lhs_std, double *dsat_err,
                       double *dsat_std, double *dmsd_std)
{
    pfgse_extra x{Mstd, lhs, lhs_std, dsat_err, dsat_std, dmsd_std};
    return run_pfgse_sequence((ref_handle *)hv,
                              pfgse_text(pulse_width, gx, gy, gz, n_g, time_seq, n_t, 0.0, 1.0, t_values, apply_bulk,
                                         threshold_type, threshold_value, 1, true),
                              n_g, cap_delta, samples, Mkt, steps, dsat, dmsd, kvec, delta_out, &x);
}

} // extern "C"

// Voxels [nz][ny][nx] (non-zero = solid) as the reference's image slices.
static std::vector<cv::Mat> voxel_slices(const uint8_t *vox, int nx, int ny, int nz)
{
    std::vector<cv::Mat> slices;
    for (int z = 0; z < nz; z++)
    {
        cv::Mat slice = cv::Mat::zeros(ny, nx, CV_8UC1);
        for (int y = 0; y < ny; y++)
        {
            uchar *row = slice.ptr<uchar>(y);
            const uint8_t *src = vox + ((size_t)z * ny + y) * nx;
            for (int x = 0; x < nx; x++) row[x] = src[x] ? 255 : 0;
        }
        slices.push_back(slice);
    }
    return slices;
}

extern "C" {

// The reference's bit-block packer on its own (BitBlock/bitBlock.cpp:138-221).
// dims[3] <- blockColumns, blockRows, blockDepth; blocks sized by a first call with blocks == NULL.
int ref_bitblock(const uint8_t *vox, int nx, int ny, int nz, uint64_t *blocks, int32_t *dims)
{
    std::vector<cv::Mat> slices = voxel_slices(vox, nx, ny, nz);
    BitBlock bb;
    bb.createBlockMap(slices);
    dims[0] = bb.blockColumns;
    dims[1] = bb.blockRows;
    dims[2] = bb.blockDepth;
    if (blocks) std::memcpy(blocks, bb.blocks, sizeof(uint64_t) * (size_t)bb.numberOfBlocks);
    return bb.numberOfBlocks;
}

// The reference's uniform internal field (NMR_Simulation/InternalField.cpp: the
// InternalField(BitBlock&, resolution, gradient, direction) constructor). out [nz][ny][nx].
int ref_uniform_field(const uint8_t *vox, int nx, int ny, int nz, double resolution, double gradient, int direction,
                      double *out)
{
    std::vector<cv::Mat> slices = voxel_slices(vox, nx, ny, nz);
    BitBlock bb;
    bb.createBlockMap(slices);
    InternalField field(bb, resolution, gradient, direction);
    if (field.getDimX() != nx || field.getDimY() != ny || field.getDimZ() != nz) return -1;
    std::memcpy(out, field.getData(), sizeof(double) * (size_t)nx * ny * nz);
    return 0;
}

} // extern "C"
