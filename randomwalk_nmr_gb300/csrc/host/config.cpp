// Config-file parsing with the reference's semantics (ConfigFiles/*.cpp): each line is scanned for
// "KEY: value" pairs separated by ": " (a line may hold several; text after the last separator is
// the value), unknown keys are ignored, booleans are the literal "true", and the default file is
// read before the user file.
#include "config.h"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <functional>
#include <sstream>

namespace rwnmr_host
{
namespace
{
using Handler = std::function<void(const std::string &key, const std::string &value)>;

// Returns false if the file cannot be opened.
bool scan_file(const std::string &path, const Handler &h)
{
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    while (std::getline(f, line))
    {
        std::string s = line;
        const std::string delim = ": ";
        size_t pos;
        while ((pos = s.find(delim)) != std::string::npos)
        {
            std::string key = s.substr(0, pos);
            std::string value = s.substr(pos + delim.size());
            s.erase(0, pos + delim.size());
            h(key, value);
        }
    }
    return true;
}

void scan_text(const std::string &text, const Handler &h)
{
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line))
    {
        size_t pos = line.find(": ");
        if (pos != std::string::npos) h(line.substr(0, pos), line.substr(pos + 2));
    }
}

// std::stod / std::stoi semantics (leading number, trailing text ignored); a value that is not a
// number leaves the field unchanged instead of aborting as the reference's uncaught exception does.
bool to_d(const std::string &s, double &out)
{
    try
    {
        out = std::stod(s);
        return true;
    }
    catch (...)
    {
        return false;
    }
}
bool to_i(const std::string &s, int &out)
{
    try
    {
        out = std::stoi(s);
        return true;
    }
    catch (...)
    {
        return false;
    }
}
bool is_true(const std::string &s) { return s == "true"; }

// "{a, b, c}" -> values; anything else -> one value (rwnmr_config.cpp:178-202).
std::vector<double> parse_list(const std::string &s, bool braces_required)
{
    std::vector<double> out;
    if (s.size() >= 2 && s.front() == '{' && s.back() == '}')
    {
        std::string body = s.substr(1, s.size() - 2);
        size_t pos;
        while ((pos = body.find(',')) != std::string::npos)
        {
            double v;
            if (to_d(body.substr(0, pos), v)) out.push_back(v);
            body.erase(0, pos + 1);
        }
        double v;
        if (to_d(body, v)) out.push_back(v);
    }
    else if (!braces_required)
    {
        double v;
        if (to_d(s, v)) out.push_back(v);
    }
    return out;
}

// The values the reference ships in config/default/, used when a default file is absent.
const char *kRwnmrDefaults = "NAME: NMR_simulation\nD0: 2.5\nBULK_TIME: 2800\nRHO_TYPE: uniform\nRHO: {0.0}\n"
                             "WALKERS: 50000\nWALKER_SAMPLES: 1\nWALKERS_PLACEMENT: random\nPLACEMENT_DEVIATION: 0\n"
                             "STEPS_PER_ECHO: 1\nSEED: 0\nBC: noflux\nSAVE_IMG_INFO: true\nSAVE_BINIMG: false\n"
                             "HISTOGRAMS: 1\nHISTOGRAM_SIZE: 1024\nOPENMP_USAGE: true\nOPENMP_THREADS: 4\n"
                             "GPU_USAGE: true\nBLOCKS: 4096\nTHREADSPERBLOCK: 1024\nECHOESPERKERNEL: 16\n"
                             "REDUCE_IN_GPU: true\nMAX_RWSTEPS: 65536\n";
const char *kUctDefaults = "DIR_PATH: path_to_folder_with_images\nFILENAME: imagefile_prefix\nFIRST_IDX: 0\nDIGITS: 1\n"
                           "EXTENSION: .png\nSLICES: 1\nRESOLUTION: 1.0\nVOXEL_DIVISION: 0\n";
const char *kCpmgDefaults = "METHOD: image-based\nOBS_TIME: 3000.0\nAPPLY_BULK: true\nMIN_T2: 0.1\nMAX_T2: 10000.0\n"
                            "USE_T2_LOGSPACE: true\nNUM_T2_BINS: 128\nMIN_LAMBDA: -4\nMAX_LAMBDA: 2\nNUM_LAMBDAS: 512\n"
                            "PRUNE_NUM: 512\nNOISE_AMP: 0.0\nSAVE_MODE: true\nSAVE_T2: true\n"
                            "SAVE_DECAY: true\nSAVE_HISTOGRAM: true\nSAVE_HISTOGRAM_LIST: false\n";
const char *kPfgseDefaults = "APPLY_BULK: true\nPULSE_WIDTH: 0.1\n"
                             "MAX_GRADIENT: {3000.0, 0.0, 0.0}\nGRADIENT_SAMPLES: 10\nTIME_SEQ: log\nTIME_SAMPLES: 3\n"
                             "TIME_MIN: -2.0\nTIME_MAX: 0.3\nAPPLY_SCALE_FACTOR: true\nINSPECTION_LENGTH: 100.0\n"
                             "THRESHOLD_TYPE: samples\nTHRESHOLD_VALUE: 8\n"
                             "ALLOW_WALKER_SAMPLING: true\nSAVE_MODE: true\nSAVE_PFGSE: true\nSAVE_HISTOGRAM: true\n"
                             "SAVE_HISTOGRAM_LIST: false\n";

bool load_two(const std::string &root, const char *name, const char *defaults, const std::string &user, bool always_user,
              const Handler &h, std::string &err)
{
    std::string dflt = root + "default/" + name + ".config";
    if (!scan_file(dflt, h)) scan_text(defaults, h);
    if (user.empty() || user == "default") return true;
    if (!always_user && user == dflt) return true;
    if (!scan_file(user, h))
    {
        err = std::string("could not open ") + name + " config file " + user;
        return false;
    }
    return true;
}

std::string q(const std::string &s)
{
    std::string o = "\"";
    for (char ch : s)
    {
        if (ch == '"' || ch == '\\') o += '\\';
        o += ch;
    }
    return o + "\"";
}
std::string num(double v)
{
    char b[64];
    snprintf(b, sizeof b, "%.17g", v);
    return b;
}
std::string arr(const std::vector<double> &v)
{
    std::string o = "[";
    for (size_t i = 0; i < v.size(); i++) o += (i ? "," : "") + num(v[i]);
    return o + "]";
}
const char *tf(bool b) { return b ? "true" : "false"; }
} // namespace

bool load_rwnmr(const std::string &root, const std::string &user, RwnmrConfig &c, std::string &err, bool replace_vectors)
{
    bool in_user = false;
    bool user_rho_seen = false;
    Handler h = [&](const std::string &k, const std::string &v) {
        int i;
        double d;
        if (k == "NAME") c.name = v;
        else if (k == "WALKERS") { if (to_i(v, i)) c.walkers = i; }
        else if (k == "WALKER_SAMPLES") { if (to_i(v, i)) c.walker_samples = i; }
        else if (k == "WALKERS_PLACEMENT") c.placement = v;
        else if (k == "PLACEMENT_DEVIATION") { if (to_i(v, i)) c.deviation = i; }
        else if (k == "RHO_TYPE") c.rho_type = (v == "uniform" || v == "sigmoid") ? v : "undefined";
        else if (k == "RHO")
        {
            if (replace_vectors && in_user && !user_rho_seen) c.rho.clear();
            if (in_user) user_rho_seen = true;
            for (double x : parse_list(v, false)) c.rho.push_back(x);
        }
        else if (k == "STEPS_PER_ECHO") { if (to_i(v, i)) c.steps_per_echo = i; }
        else if (k == "GIROMAGNETIC_RATIO") { if (to_d(v, d)) c.gamma = d; }
        else if (k == "GIROMAGNETIC_UNIT") c.gamma_unit = (v == "MHertz" || v == "mhertz") ? "mhertz" : "rad";
        else if (k == "D0") { if (to_d(v, d)) c.d0 = d; }
        else if (k == "BULK_TIME") { if (to_d(v, d)) c.bulk_time = d; }
        else if (k == "SEED")
        {
            try { c.seed = (unsigned long long)std::stoll(v); } catch (...) {}
        }
        else if (k == "BC")
            c.bc = v == "periodic" ? "periodic" : (v == "mirror" ? "mirror" : ((v == "debug" || v == "test") ? "test" : "noflux"));
        else if (k == "SAVE_IMG_INFO") c.save_img_info = is_true(v);
        else if (k == "SAVE_BINIMG") c.save_binimg = is_true(v);
        else if (k == "SAVE_WALKERS") c.save_walkers = is_true(v);
        else if (k == "HISTOGRAMS") { if (to_i(v, i)) c.histograms = i; }
        else if (k == "HISTOGRAM_SIZE") { if (to_i(v, i)) c.histogram_size = i; }
        else if (k == "HISTOGRAM_SCALE") c.histogram_scale = v == "log" ? "log" : "linear";
        else if (k == "OPENMP_USAGE") c.openmp_usage = is_true(v);
        else if (k == "OPENMP_THREADS") { if (to_i(v, i)) c.openmp_threads = i; }
        else if (k == "GPU_USAGE") c.gpu_usage = is_true(v);
        else if (k == "BLOCKS") { if (to_i(v, i)) c.blocks = i; }
        else if (k == "THREADSPERBLOCK") { if (to_i(v, i)) c.threads_per_block = i; }
        else if (k == "ECHOESPERKERNEL") { if (to_i(v, i)) c.echoes_per_kernel = i; }
        else if (k == "REDUCE_IN_GPU") c.reduce_in_gpu = is_true(v);
        else if (k == "MAX_RWSTEPS") { if (to_i(v, i)) c.max_rwsteps = i; }
    };
    std::string dflt = root + "default/rwnmr.config";
    if (!scan_file(dflt, h)) scan_text(kRwnmrDefaults, h);
    if (user.empty() || user == "default" || user == dflt) return true;
    in_user = true;
    if (!scan_file(user, h))
    {
        err = "could not open rwnmr config file " + user;
        return false;
    }
    return true;
}

bool load_uct(const std::string &root, const std::string &user, UctConfig &c, std::string &err)
{
    Handler h = [&](const std::string &k, const std::string &v) {
        int i;
        double d;
        if (k == "DIR_PATH") c.dir_path = v;
        else if (k == "FILENAME") c.filename = v;
        else if (k == "FIRST_IDX") { if (to_i(v, i)) c.first_idx = i; }
        else if (k == "DIGITS") { if (to_i(v, i)) c.digits = i; }
        else if (k == "EXTENSION") c.extension = v;
        else if (k == "SLICES") { if (to_i(v, i)) c.slices = i; }
        else if (k == "RESOLUTION") { if (to_d(v, d)) c.resolution = d; }
        else if (k == "VOXEL_DIVISION") { if (to_i(v, i)) c.voxel_division = i; }
        else if (k == "IMG_FILES_LIST") c.img_files_list = v;
    };
    return load_two(root, "uct", kUctDefaults, user, false, h, err);
}

bool load_cpmg(const std::string &root, const std::string &user, CpmgConfig &c, std::string &err)
{
    Handler h = [&](const std::string &k, const std::string &v) {
        int i;
        double d;
        if (k == "D0") { if (to_d(v, d)) c.d0 = d; }
        else if (k == "APPLY_BULK") c.apply_bulk = is_true(v);
        else if (k == "OBS_TIME") { if (to_d(v, d)) c.obs_time = d; }
        else if (k == "METHOD") c.method = v;
        else if (k == "TIME_VERBOSE") c.time_verbose = is_true(v);
        else if (k == "RESIDUAL_FIELD") c.residual_field = (v == "uniform" || v == "import") ? v : "none";
        else if (k == "GRADIENT_VALUE") { if (to_d(v, d)) c.gradient_value = d; }
        else if (k == "GRADIENT_DIRECTION") c.gradient_direction = (v == "0" || v == "x") ? 0 : ((v == "1" || v == "y") ? 1 : 2);
        else if (k == "PATH_TO_FIELD") c.path_to_field = v;
        else if (k == "MIN_T2") { if (to_d(v, d)) c.min_t2 = d; }
        else if (k == "MAX_T2") { if (to_d(v, d)) c.max_t2 = d; }
        else if (k == "USE_T2_LOGSPACE") c.use_t2_logspace = is_true(v);
        else if (k == "NUM_T2_BINS") { if (to_i(v, i)) c.num_t2_bins = i; }
        else if (k == "MIN_LAMBDA") { if (to_d(v, d)) c.min_lambda = d; }
        else if (k == "MAX_LAMBDA") { if (to_d(v, d)) c.max_lambda = d; }
        else if (k == "NUM_LAMBDAS") { if (to_i(v, i)) c.num_lambdas = i; }
        else if (k == "PRUNE_NUM") { if (to_i(v, i)) c.prune_num = i; }
        else if (k == "NOISE_AMP") { if (to_d(v, d)) c.noise_amp = d; }
        else if (k == "SAVE_MODE") c.save_mode = is_true(v);
        else if (k == "SAVE_T2") c.save_t2 = is_true(v);
        else if (k == "SAVE_WALKERS") c.save_walkers = is_true(v);
        else if (k == "SAVE_DECAY") c.save_decay = is_true(v);
        else if (k == "SAVE_HISTOGRAM") c.save_histogram = is_true(v);
        else if (k == "SAVE_HISTOGRAM_LIST") c.save_histogram_list = is_true(v);
    };
    return load_two(root, "cpmg", kCpmgDefaults, user, false, h, err);
}

bool load_multitau(const std::string &root, const std::string &user, MultitauConfig &c, std::string &err)
{
    Handler h = [&](const std::string &k, const std::string &v) {
        int i;
        double d;
        if (k == "TAU_MIN") { if (to_d(v, d)) c.tau_min = d; }
        else if (k == "TAU_MAX") { if (to_d(v, d)) c.tau_max = d; }
        else if (k == "TAU_POINTS") { if (to_i(v, i)) c.tau_points = i; }
        else if (k == "TAU_VALUES")
        {
            c.tau_values = parse_list(v, true);
            std::sort(c.tau_values.begin(), c.tau_values.end());
        }
        else if (k == "TAU_SCALE") c.tau_scale = (v == "log" || v == "linear") ? v : "manual";
        else if (k == "COMPLETE_DECAY") c.complete_decay = v == "true" || v == "True" || v == "TRUE";
        else if (k == "SAVE_MODE") c.save_mode = is_true(v);
        else if (k == "SAVE_DECAY") c.save_decay = is_true(v);
        else if (k == "SAVE_WALKERS") c.save_walkers = is_true(v);
        else if (k == "SAVE_HISTOGRAM") c.save_histogram = is_true(v);
        else if (k == "SAVE_HISTOGRAM_LIST") c.save_histogram_list = is_true(v);
    };
    const std::string cpmg_default = root + "default/cpmg.config";
    if (!scan_file(cpmg_default, h)) scan_text(kCpmgDefaults, h);
    const std::string path = (user.empty() || user == "default") ? root + "default/multitau.config" : user;
    if (path == cpmg_default) return true;
    if (!scan_file(path, h))
    {
        err = "could not open multitau config file " + path;
        return false;
    }
    return true;
}

bool load_pfgse(const std::string &root, const std::string &user, PfgseConfig &c, std::string &err)
{
    Handler h = [&](const std::string &k, const std::string &v) {
        int i;
        double d;
        if (k == "PULSE_WIDTH") { if (to_d(v, d)) c.pulse_width = d; }
        else if (k == "MAX_GRADIENT")
        {
            std::vector<double> g = parse_list(v, true);
            if (g.size() >= 3) for (int a = 0; a < 3; a++) c.max_gradient[a] = g[a];
        }
        else if (k == "GRADIENT_SAMPLES") { if (to_i(v, i)) c.gradient_samples = i; }
        else if (k == "APPLY_BULK") c.apply_bulk = is_true(v);
        else if (k == "TIME_SEQ") c.time_seq = v;
        else if (k == "TIME_SAMPLES") { if (to_i(v, i)) c.time_samples = i; }
        else if (k == "TIME_VALUES")
        {
            // only read while TIME_SEQ is "manual"; replaces earlier values (pfgse_config.cpp:166-190)
            c.time_values.clear();
            if (c.time_seq == "manual") c.time_values = parse_list(v, true);
        }
        else if (k == "TIME_MIN") { if (to_d(v, d)) c.time_min = d; }
        else if (k == "TIME_MAX") { if (to_d(v, d)) c.time_max = d; }
        else if (k == "APPLY_SCALE_FACTOR") c.apply_scale_factor = is_true(v);
        else if (k == "NOISE_AMP") { if (to_d(v, d) && d > 0.0) c.noise_amp = d; }
        else if (k == "TARGET_SNR") { if (to_d(v, d) && d > 0.0) c.target_snr = d; }
        else if (k == "INSPECTION_LENGTH") { if (to_d(v, d)) c.inspection_length = d; }
        else if (k == "THRESHOLD_TYPE") c.threshold_type = v;
        else if (k == "THRESHOLD_VALUE") { if (to_d(v, d)) c.threshold_value = d; }
        else if (k == "THRESHOLD_WINDOW") { if (to_i(v, i)) c.threshold_window = i; }
        else if (k == "ALLOW_WALKER_SAMPLING") c.allow_walker_sampling = is_true(v);
        else if (k == "APPLY_ABSORPTION") c.apply_absorption = is_true(v);
        else if (k == "SAVE_MODE") c.save_mode = is_true(v);
        else if (k == "SAVE_PFGSE") c.save_pfgse = is_true(v);
        else if (k == "SAVE_WALKERS") c.save_walkers = is_true(v);
        else if (k == "SAVE_HISTOGRAM") c.save_histogram = is_true(v);
        else if (k == "SAVE_HISTOGRAM_LIST") c.save_histogram_list = is_true(v);
    };
    return load_two(root, "pfgse", kPfgseDefaults, user, true, h, err);
}

std::vector<double> pfgse_time_samples(const PfgseConfig &c)
{
    std::vector<double> v;
    if (c.time_seq == "log" || c.time_seq == "linear")
    {
        const double step = (c.time_max - c.time_min) / ((double)c.time_samples - 1.0);
        for (int i = 0; i < c.time_samples; i++)
        {
            const double x = c.time_min + step * i;
            v.push_back(c.time_seq == "log" ? std::pow(10.0, x) : x);
        }
    }
    else if (c.time_seq == "manual")
    {
        v = c.time_values;
        std::sort(v.begin(), v.end());
    }
    return v;
}

std::string to_json(const RwnmrConfig &c)
{
    std::ostringstream o;
    o << "{\"NAME\":" << q(c.name) << ",\"D0\":" << num(c.d0) << ",\"BULK_TIME\":" << num(c.bulk_time)
      << ",\"RHO_TYPE\":" << q(c.rho_type) << ",\"RHO\":" << arr(c.rho) << ",\"WALKERS\":" << c.walkers
      << ",\"WALKER_SAMPLES\":" << c.walker_samples << ",\"WALKERS_PLACEMENT\":" << q(c.placement)
      << ",\"PLACEMENT_DEVIATION\":" << c.deviation << ",\"STEPS_PER_ECHO\":" << c.steps_per_echo
      << ",\"SEED\":" << c.seed << ",\"BC\":" << q(c.bc) << ",\"GIROMAGNETIC_RATIO\":" << num(c.gamma)
      << ",\"GIROMAGNETIC_UNIT\":" << q(c.gamma_unit) << ",\"HISTOGRAMS\":" << c.histograms
      << ",\"HISTOGRAM_SIZE\":" << c.histogram_size << ",\"HISTOGRAM_SCALE\":" << q(c.histogram_scale)
      << ",\"SAVE_IMG_INFO\":" << tf(c.save_img_info) << ",\"SAVE_BINIMG\":" << tf(c.save_binimg)
      << ",\"SAVE_WALKERS\":" << tf(c.save_walkers) << ",\"GPU_USAGE\":" << tf(c.gpu_usage)
      << ",\"MAX_RWSTEPS\":" << c.max_rwsteps << "}";
    return o.str();
}
std::string to_json(const UctConfig &c)
{
    std::ostringstream o;
    o << "{\"DIR_PATH\":" << q(c.dir_path) << ",\"FILENAME\":" << q(c.filename) << ",\"FIRST_IDX\":" << c.first_idx
      << ",\"DIGITS\":" << c.digits << ",\"EXTENSION\":" << q(c.extension) << ",\"SLICES\":" << c.slices
      << ",\"RESOLUTION\":" << num(c.resolution) << ",\"VOXEL_DIVISION\":" << c.voxel_division
      << ",\"IMG_FILES_LIST\":" << q(c.img_files_list) << "}";
    return o.str();
}
std::string to_json(const CpmgConfig &c)
{
    std::ostringstream o;
    o << "{\"OBS_TIME\":" << num(c.obs_time) << ",\"METHOD\":" << q(c.method) << ",\"APPLY_BULK\":" << tf(c.apply_bulk)
      << ",\"RESIDUAL_FIELD\":" << q(c.residual_field) << ",\"GRADIENT_VALUE\":" << num(c.gradient_value)
      << ",\"GRADIENT_DIRECTION\":" << c.gradient_direction << ",\"NOISE_AMP\":" << num(c.noise_amp)
      << ",\"SAVE_MODE\":" << tf(c.save_mode) << ",\"SAVE_DECAY\":" << tf(c.save_decay)
      << ",\"SAVE_WALKERS\":" << tf(c.save_walkers) << ",\"SAVE_HISTOGRAM\":" << tf(c.save_histogram) << "}";
    return o.str();
}
std::string to_json(const PfgseConfig &c)
{
    std::ostringstream o;
    o << "{\"PULSE_WIDTH\":" << num(c.pulse_width) << ",\"MAX_GRADIENT\":"
      << arr({c.max_gradient[0], c.max_gradient[1], c.max_gradient[2]}) << ",\"GRADIENT_SAMPLES\":" << c.gradient_samples
      << ",\"APPLY_BULK\":" << tf(c.apply_bulk) << ",\"TIME_SEQ\":" << q(c.time_seq)
      << ",\"TIME_SAMPLES\":" << c.time_samples << ",\"TIME_VALUES\":" << arr(pfgse_time_samples(c))
      << ",\"APPLY_SCALE_FACTOR\":" << tf(c.apply_scale_factor) << ",\"INSPECTION_LENGTH\":" << num(c.inspection_length)
      << ",\"NOISE_AMP\":" << num(c.noise_amp) << ",\"TARGET_SNR\":" << num(c.target_snr)
      << ",\"THRESHOLD_TYPE\":" << q(c.threshold_type) << ",\"THRESHOLD_VALUE\":" << num(c.threshold_value)
      << ",\"THRESHOLD_WINDOW\":" << c.threshold_window << ",\"ALLOW_WALKER_SAMPLING\":" << tf(c.allow_walker_sampling)
      << ",\"APPLY_ABSORPTION\":" << tf(c.apply_absorption) << ",\"SAVE_PFGSE\":" << tf(c.save_pfgse) << "}";
    return o.str();
}

std::string to_json(const MultitauConfig &c)
{
    std::ostringstream o;
    o << "{\"TAU_MIN\":" << num(c.tau_min) << ",\"TAU_MAX\":" << num(c.tau_max) << ",\"TAU_POINTS\":" << c.tau_points
      << ",\"TAU_VALUES\":" << arr(c.tau_values) << ",\"TAU_SCALE\":" << q(c.tau_scale)
      << ",\"COMPLETE_DECAY\":" << tf(c.complete_decay) << ",\"SAVE_MODE\":" << tf(c.save_mode)
      << ",\"SAVE_DECAY\":" << tf(c.save_decay) << ",\"SAVE_WALKERS\":" << tf(c.save_walkers)
      << ",\"SAVE_HISTOGRAM\":" << tf(c.save_histogram) << ",\"SAVE_HISTOGRAM_LIST\":" << tf(c.save_histogram_list)
      << "}";
    return o.str();
}

} // namespace rwnmr_host
