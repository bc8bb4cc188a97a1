// Host-side simulation and sequences: the reference's NMR_Simulation / NMR_cpmg / NMR_PFGSE
// orchestration (config -> image -> walkers -> walk -> outputs), with every walk on the GPU engine.
#pragma once
#include <cstdint>
#include <random>
#include <string>
#include <vector>

#include "config.h"
#include "rwnmr_gb300.h"

namespace rwnmr_host
{

struct Image
{
    int nx = 0, ny = 0, nz = 0, n_phases = 1;
    std::vector<uint8_t> labels; // [nz][ny][nx], 0 = pore, p = solid phase p
    std::vector<uint64_t> blocks;
    std::string source;
};

// Loads the image slices named by a uct config (PNG; any non-zero colour channel is solid, as in
// NMR_Simulation::createBinaryMap, NMR_Simulation.cpp:577-617).
bool load_uct_image(const UctConfig &uct, Image &img, std::string &err);
// Decodes one 8-bit PNG into a solid/pore mask (1 = solid). Non-interlaced PNGs, any colour type.
bool png_solid_mask(const std::string &path, int &width, int &height, std::vector<uint8_t> &mask, std::string &err);

// xi-rate collision histogram (NMR_Simulation/CollisionHistogram.cpp:59-249).
struct Histogram
{
    int size = 0;
    double gap = 0.0;
    std::string scale = "linear";
    int first_echo = 0, last_echo = 0;
    std::vector<double> bins, amps;
    void create(int size, const std::string &scale);
    void fill(const std::vector<uint32_t> &collisions, uint32_t steps);
};

class Simulation
{
  public:
    RwnmrConfig rw;
    UctConfig uct;
    std::string db_path, sim_dir;
    std::mt19937 rng;
    uint64_t initial_seed = 0;
    Image img;
    double resolution = 1.0, voxel_res = 1.0, dt = 0.0, gamma = 0.0;
    int shift = 0;
    bool voxel_division_applied = false;
    uint32_t pores = 0, interface_count = 0, clamped = 0;
    double porosity = 0.0, svp = 0.0, occupancy = 0.0;
    std::vector<int32_t> x0, y0, z0;
    std::vector<uint64_t> seed0;
    std::vector<double> rho_phase; // relaxivity per solid phase
    uint32_t steps = 0, echoes = 0;
    std::vector<uint32_t> collisions;
    std::vector<double> xi_rate;
    std::vector<double> walker_dfactors; // RHO_TYPE sigmoid: the factors last uploaded
    Histogram histogram;
    std::vector<Histogram> hist_list;
    rwnmr_ctx *ctx = nullptr;
    int device = 0;
    bool quiet = false;

    ~Simulation();
    // NMR_Simulation constructor (NMR_Simulation.cpp:44-108)
    bool init(const RwnmrConfig &rw, const UctConfig &uct, const std::string &project_root, int device,
              std::string &err);
    // readImage's bookkeeping after loading (pores, S/Vp) and the upload to the GPU
    bool set_image(Image &&image, std::string &err);
    // setWalkers (NMR_Simulation.cpp:324-409) and the upload to the GPU
    bool set_walkers(std::string &err);
    void set_time_framework_time(double time_ms); // NMR_Simulation.cpp:285-298
    void set_time_framework_steps(uint32_t steps);
    // collision-mapping walk with histogram windows (mapSimulation, NMR_Simulation.cpp:1787-1841)
    bool map_simulation(std::string &err);
    double decrease_factor(double rho) const; // Walker::computeDecreaseFactor
    double sigmoid_rho(double xi) const;      // Walker::setSurfaceRelaxivity(vector) at collision rate xi
    // per-walker decrease factors from the sigmoid of each walker's collision rate over `steps`
    // steps of the last mapping walk (NMR_Simulation::updateWalkersRelaxativity)
    bool upload_sigmoid_dfactors(uint32_t steps, std::string &err);
    std::vector<double> phase_dfactors() const;
    int bc_code() const;
    void save_info() const;
    void log(const std::string &msg) const;
};

class CpmgSequence
{
  public:
    Simulation &sim;
    CpmgConfig cfg;
    std::string parent, suffix; // NMR_cpmg::setName(parent, sufix): directory nesting, e.g. under a multitau run
    bool map = true;            // NMR_cpmg::setNMRTimeFramework(_map)
    std::string name, dir;
    std::vector<double> times, amps, raw, noise;
    std::vector<double> t2_bins, t2_amps;  // T2 distribution (apply_laplace)
    double t2_lambda = 0.0;
    std::vector<uint64_t> echo_collisions; // [echoes][phases]
    double kernel_ms = 0.0;
    CpmgSequence(Simulation &s, const CpmgConfig &c) : sim(s), cfg(c) {}
    bool run(std::string &err); // set + run_simulation + save (NMR_cpmg::run, NMR_cpmg.cpp:87-93)
    bool set(std::string &err);
    bool run_simulation(std::string &err);
    bool apply_laplace(std::string &err); // NMR_cpmg::applyLaplace (NMR_cpmg.cpp:387-453)
    void save() const;
};

class PfgseSequence
{
  public:
    Simulation &sim;
    PfgseConfig cfg;
    std::string dir;
    std::vector<double> exposure_times;
    std::vector<double> gradient;        // |g_j|
    std::vector<double> gvec, kvec;      // [n_g][3]
    int n_g = 0;
    // per exposure time
    std::vector<double> Mkt;             // [n_delta][n_g] un-normalised (sum E cos), after bulk and noise
    std::vector<double> esum, dsat, dsat_err, dmsd;
    std::vector<double> dsat_std, dmsd_std;      // walker-sampling deviations (0 without sampling)
    std::vector<double> m_std, lhs_std;          // [n_delta][n_g]
    std::vector<double> msd_vec_std, dmsd_vec_std; // [n_delta][3]
    std::vector<int> dsat_points;
    std::vector<double> msd_vec, dmsd_vec; // [n_delta][3]
    std::vector<double> lhs, rhs, raw_noise; // [n_delta][n_g]
    std::vector<uint32_t> steps;
    double kernel_ms = 0.0;
    PfgseSequence(Simulation &s, const PfgseConfig &c) : sim(s), cfg(c) {}
    bool run(std::string &err); // NMR_PFGSE::run (NMR_pfgse.cpp:98-131)
};

// Multi-echo-time CPMG (NMR_multitau.cpp:22-204): one CPMG per echo time te, keeping the first echo
// of each (or each full decay with COMPLETE_DECAY), written to multitau_decay.csv.
class MultitauSequence
{
  public:
    Simulation &sim;
    MultitauConfig cfg;
    CpmgConfig cpmg_cfg;
    std::string name, dir;
    std::vector<uint32_t> required_steps; // steps per echo of each run
    std::vector<double> signal_times, signal_amps;
    double kernel_ms = 0.0;
    MultitauSequence(Simulation &s, const MultitauConfig &c, const CpmgConfig &cc) : sim(s), cfg(c), cpmg_cfg(cc) {}
    void set_tau_sequence(); // NMR_multitau::setTauSequence
    bool run(std::string &err);
};

// The RWNMR command line (Utils/ArgsParser.cpp:10-152, App/rwnmrApp.cpp:106-231).
int cli_main(int argc, const char *const *argv);

} // namespace rwnmr_host
