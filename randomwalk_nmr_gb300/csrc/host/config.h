// Config files of the walker path: rwnmr / uct / cpmg / pfgse (the reference's ConfigFiles/).
#pragma once
#include <string>
#include <vector>

namespace rwnmr_host
{

// rwnmr.config (ConfigFiles/rwnmr_config.cpp:79-144)
struct RwnmrConfig
{
    std::string name = "NMR_simulation";
    double d0 = 2.5;
    double bulk_time = 2800.0;
    std::string rho_type = "uniform";
    std::vector<double> rho;
    int walkers = 50000;
    int walker_samples = 1;
    std::string placement = "random";
    int deviation = 0;
    int steps_per_echo = 1;
    unsigned long long seed = 0;
    std::string bc = "noflux";
    double gamma = 42.576;
    std::string gamma_unit = "mhertz";
    bool save_img_info = true, save_binimg = false, save_walkers = false;
    int histograms = 1;
    int histogram_size = 1024;
    std::string histogram_scale = "linear";
    bool openmp_usage = true;
    int openmp_threads = 4;
    bool gpu_usage = true;
    int blocks = 4096, threads_per_block = 1024, echoes_per_kernel = 16, max_rwsteps = 65536;
    bool reduce_in_gpu = true;
};

// uct.config (ConfigFiles/uct_config.cpp:65-79)
struct UctConfig
{
    std::string dir_path = "./";
    std::string filename = "image";
    int first_idx = 0;
    int digits = 1;
    std::string extension = ".png";
    int slices = 1;
    double resolution = 1.0;
    int voxel_division = 0;
    std::string img_files_list;
};

// cpmg.config (ConfigFiles/cpmg_config.cpp:79-108)
struct CpmgConfig
{
    double d0 = 2.5;
    double obs_time = 3000.0;
    std::string method = "image-based";
    bool apply_bulk = true;
    bool time_verbose = false;
    std::string residual_field = "none";
    double gradient_value = 0.0;
    int gradient_direction = 2;
    std::string path_to_field;
    double min_t2 = 0.1, max_t2 = 10000.0;
    bool use_t2_logspace = true;
    int num_t2_bins = 128;
    double min_lambda = -4, max_lambda = 2;
    int num_lambdas = 512, prune_num = 512;
    double noise_amp = 0.0;
    bool save_mode = true, save_t2 = true, save_walkers = false, save_decay = true, save_histogram = true,
         save_histogram_list = false;
};

// pfgse.config (ConfigFiles/pfgse_config.cpp:87-115, 191-240)
struct PfgseConfig
{
    double pulse_width = 0.1;
    double max_gradient[3] = {3000.0, 0.0, 0.0};
    int gradient_samples = 10;
    bool apply_bulk = true;
    std::string time_seq = "log";
    int time_samples = 3;
    std::vector<double> time_values;
    double time_min = -2.0, time_max = 0.3;
    bool apply_scale_factor = true;
    double inspection_length = 100.0;
    double noise_amp = 0.0;
    double target_snr = -1.0;
    std::string threshold_type = "samples";
    double threshold_value = 8;
    int threshold_window = 1;
    bool allow_walker_sampling = true;
    bool apply_absorption = false;
    bool save_mode = true, save_pfgse = true, save_walkers = false, save_histogram = true, save_histogram_list = false;
};

// multitau.config (ConfigFiles/multitau_config.cpp:65-178). The reference leaves every field without
// a default (its constructor reads the cpmg default file by mistake, so only the SAVE_* keys of
// cpmg.config reach it); these defaults stand in for the unset values.
struct MultitauConfig
{
    double tau_min = 0.0, tau_max = 0.0;
    int tau_points = 0;
    std::vector<double> tau_values;
    std::string tau_scale = "linear";
    bool complete_decay = false;
    bool save_mode = false, save_decay = false, save_walkers = false, save_histogram = false,
         save_histogram_list = false;
};

// Reads the default file (config_root + "default/<kind>.config") and then the user file, like
// the reference: rwnmr/uct/cpmg skip the user file when it is the default file itself; pfgse reads
// both regardless. A missing default file falls back to the values the reference ships.
// Vector keys (RHO) append across the two files, as in the reference (RHO in the default file
// comes first and RHO[0] is what a uniform walk uses); replace_vectors = true makes the user
// file's RHO replace the default's instead. Returns false and sets err if the user file is missing.
bool load_rwnmr(const std::string &config_root, const std::string &user, RwnmrConfig &c, std::string &err,
                bool replace_vectors = false);
bool load_uct(const std::string &config_root, const std::string &user, UctConfig &c, std::string &err);
bool load_cpmg(const std::string &config_root, const std::string &user, CpmgConfig &c, std::string &err);
bool load_pfgse(const std::string &config_root, const std::string &user, PfgseConfig &c, std::string &err);
// multitau: the reference reads config_root + "default/cpmg.config" first (multitau_config.cpp:16-22),
// then the user file (config_root + "default/multitau.config" when "default").
bool load_multitau(const std::string &config_root, const std::string &user, MultitauConfig &c, std::string &err);

// PFGSE exposure times (pfgse_config.cpp:191-240): log = 10^linspace, linear, manual (sorted).
std::vector<double> pfgse_time_samples(const PfgseConfig &c);

std::string to_json(const RwnmrConfig &c);
std::string to_json(const UctConfig &c);
std::string to_json(const CpmgConfig &c);
std::string to_json(const PfgseConfig &c);
std::string to_json(const MultitauConfig &c);

} // namespace rwnmr_host
