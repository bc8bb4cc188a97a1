// Host orchestration of the walker path (see sequences.h). Every walk runs on the GPU engine;
// this file does the reference's bookkeeping around it: time framework, relaxivity, bulk
// relaxation, normalisation, PFGSE wave vectors and D(t) fits, and the output files.
#include "sequences.h"

#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <random>
#include <sstream>

#include "host_internal.h"
#include "laplace.h"
#include "rwnmr_host.h"

namespace rwnmr_host
{
namespace
{
const double kTwoPi = 6.2831853071795864769252867665590057683943; // NMR_defs.h

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

// std::to_string(double) ("%f") cut two digits after the point, as NMR_cpmg::setName does.
std::string trimmed_time(double t)
{
    std::string s = std::to_string(t);
    size_t dot = s.find('.');
    return dot == std::string::npos ? s : s.substr(0, dot + 3);
}

std::ofstream open_out(const std::string &path, std::ios::openmode mode = std::ios::out)
{
    std::ofstream f(path, mode);
    f << std::setprecision(std::numeric_limits<double>::max_digits10);
    return f;
}

// Least squares through the origin over the first n points (Math/LeastSquareAdjust.cpp:77-170).
void lsq_no_intercept(const std::vector<double> &x, const std::vector<double> &y, int n, double &b, double &mse)
{
    double num = 0.0, den = 0.0;
    for (int i = 0; i < n; i++) num += x[i] * y[i];
    for (int i = 0; i < n; i++) den += x[i] * x[i];
    b = num / den;
    double r = 0.0;
    for (int i = 0; i < n; i++) r += std::pow(y[i] - b * x[i], 2.0);
    mse = r / (double)n;
}
} // namespace

// ---------------------------------------------------------------------------------------------
void Histogram::create(int sz, const std::string &sc)
{
    scale = sc;
    gap = 1.0 / (double)sz;
    size = scale == "log" ? sz + 1 : sz;
    bins.clear();
    amps.clear();
}

void Histogram::fill(const std::vector<uint32_t> &coll, uint32_t steps_)
{
    const double steps = (double)steps_;
    bins.clear();
    amps.assign(size, 0.0);
    const double n = (double)coll.size();
    if (scale == "log")
    {
        size_t first = 0;
        while (first < coll.size() && coll[first] == 0) first++;
        if (first < coll.size())
        {
            double min_rate = coll[first] / steps;
            for (size_t i = first; i < coll.size(); i++)
                if (coll[i] != 0) min_rate = std::min(min_rate, coll[i] / steps);
            const double lmin = std::round(std::log10(min_rate));
            bins.push_back(lmin - 1.0);
            const int pts = size - 1;
            const double stp = (0.0 - lmin) / ((double)pts - 1.0);
            for (int k = 0; k < pts; k++) bins.push_back(std::pow(10.0, lmin + stp * k));
        }
        else
            bins.assign(size, 0.0);
        const double lgap = std::log10(bins[2]) - std::log10(bins[1]);
        const double minv = std::log10(bins[1]);
        for (uint32_t c : coll)
        {
            if (c == 0) amps[0] += 1.0;
            else
            {
                int idx = (int)std::floor(std::round((std::log10(c / steps) - minv) / lgap)) + 1;
                if (idx > 0 && idx < size) amps[idx] += 1.0;
                else amps[1] += 1.0;
            }
        }
    }
    else
    {
        const double mean_bin = 0.5 * gap;
        for (int k = 0; k < size; k++) bins.push_back(k * gap + mean_bin);
        for (uint32_t c : coll)
        {
            int idx = (int)std::floor((c / steps) / gap);
            if (idx >= size) idx--;
            amps[idx] += 1.0;
        }
    }
    for (double &a : amps) a /= n;
}

// ---------------------------------------------------------------------------------------------
Simulation::~Simulation()
{
    if (ctx) rwnmr_ctx_destroy(ctx);
}

void Simulation::log(const std::string &msg) const
{
    if (!quiet) std::cout << msg << std::endl;
}

bool Simulation::init(const RwnmrConfig &r, const UctConfig &u, const std::string &root, int dev, std::string &err)
{
    rw = r;
    uct = u;
    device = dev;
    db_path = root + "./db/";
    sim_dir = db_path + rw.name;
    mkdirs(sim_dir);
    gamma = rw.gamma_unit == "mhertz" ? rw.gamma * kTwoPi : rw.gamma;
    seed_rng(rng, rw.seed);
    initial_seed = rw.seed;
    resolution = uct.resolution;
    voxel_res = resolution;
    shift = 0;
    voxel_division_applied = uct.voxel_division > 0;
    dt = voxel_res * voxel_res / (6.0 * rw.d0);
    if (rw.bc == "test")
    {
        err = "BC 'test' runs the reference's printf kernel; it has no walk to run";
        return false;
    }
    if (rw.rho.empty()) rw.rho.push_back(0.0);
    rwnmr_status st = rwnmr_ctx_create(&ctx, device);
    if (st != RWNMR_OK)
    {
        err = "no usable CUDA device (the walker engine has no CPU fallback)";
        return false;
    }
    return true;
}

bool Simulation::set_image(Image &&image, std::string &err)
{
    img = std::move(image);
    if (img.blocks.empty())
    {
        int32_t bd[3];
        int64_t nb = rwnmr_pack_blocks(img.labels.data(), img.nx, img.ny, img.nz, nullptr, bd);
        img.blocks.assign(nb, 0);
        rwnmr_pack_blocks(img.labels.data(), img.nx, img.ny, img.nz, img.blocks.data(), bd);
    }
    // countPoresInBitBlock + countInterfacePoreMatrix (periodic neighbours; NMR_Simulation.cpp:675-917)
    const int nx = img.nx, ny = img.ny, nz = img.nz;
    auto solid = [&](int x, int y, int z) { return img.labels[((size_t)z * ny + y) * nx + x] != 0; };
    pores = 0;
    interface_count = 0;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++)
            {
                const bool s = solid(x, y, z);
                if (!s) pores++;
                if (s != solid((x + 1) % nx, y, z)) interface_count++;
                if (s != solid(x, (y + 1) % ny, z)) interface_count++;
                if (nz > 1 && s != solid(x, y, (z + 1) % nz)) interface_count++;
            }
    porosity = (double)pores / ((double)nx * ny * nz);
    const double area = voxel_res * voxel_res;
    svp = ((double)interface_count * area) / ((double)pores * area * voxel_res);
    rwnmr_status st = rwnmr_image_upload_labels(ctx, img.labels.data(), nx, ny, nz, img.n_phases);
    if (st != RWNMR_OK)
    {
        err = std::string("image upload: ") + rwnmr_last_error(ctx);
        return false;
    }
    // relaxivity per solid phase: RHO[0] for every phase (the reference's uniform relaxivity), or
    // RHO values phase by phase where the image has as many phases as the user file's RHO list
    rho_phase.assign(img.n_phases, rw.rho[0]);
    if (img.n_phases > 1 && (int)rw.rho.size() >= img.n_phases + 1)
        for (int q = 0; q < img.n_phases; q++) rho_phase[q] = rw.rho[rw.rho.size() - img.n_phases + q];
    log("- image " + img.source + ": " + std::to_string(nx) + "x" + std::to_string(ny) + "x" + std::to_string(nz) +
        ", porosity " + std::to_string(porosity) + ", S/Vp " + std::to_string(svp));
    return true;
}

bool Simulation::set_walkers(std::string &err)
{
    PlacementRequest req;
    req.mode = rw.placement;
    req.deviation = rw.deviation;
    req.shift = voxel_division_applied ? uct.voxel_division : 0;
    req.n = rw.walkers;
    PlacementInfo info;
    if (place_walkers(rng, img.blocks.data(), img.nx, img.ny, img.nz, req, x0, y0, z0, seed0, info, err) != 0)
        return false;
    clamped = info.clamped;
    occupancy = info.occupancy;
    if (req.shift > 0)
    {
        // applyVoxelDivision (NMR_Simulation.cpp:192-268): finer walk grid and time step
        shift = req.shift;
        voxel_res = resolution / (double)(1 << shift);
        dt = voxel_res * voxel_res / (6.0 * rw.d0);
    }
    rwnmr_status st = rwnmr_walkers_upload(ctx, (int64_t)x0.size(), x0.data(), y0.data(), z0.data(), seed0.data());
    if (st != RWNMR_OK)
    {
        err = std::string("walker upload: ") + rwnmr_last_error(ctx);
        return false;
    }
    log("- " + std::to_string(x0.size()) + " walkers placed (" + rw.placement + ")" +
        (clamped ? ", " + std::to_string(clamped) + " one-past-the-end pore draws clamped" : ""));
    return true;
}

void Simulation::set_time_framework_time(double t)
{
    // setNumberOfStepsFromTime + setTimeFramework(double)
    steps = (uint32_t)std::round(t * (6.0 * rw.d0 / (voxel_res * voxel_res)));
    if (steps < (uint32_t)rw.steps_per_echo) steps = rw.steps_per_echo;
    echoes = (uint32_t)std::ceil((double)steps / (double)rw.steps_per_echo);
    steps = echoes * rw.steps_per_echo;
}

void Simulation::set_time_framework_steps(uint32_t s)
{
    if (s < (uint32_t)rw.steps_per_echo) s = rw.steps_per_echo;
    echoes = (uint32_t)std::ceil(s / (double)rw.steps_per_echo);
    steps = echoes * rw.steps_per_echo;
}

double Simulation::decrease_factor(double rho) const
{
    return 1.0 - (2.0 / 3.0) * ((rho * voxel_res) / (rw.d0 * 1e03));
}

double Simulation::sigmoid_rho(double xi) const
{
    // two sigmoids K + (A - K) / (1 + exp(-B (xi - eps))) (Walker/walker.h:174-196)
    const std::vector<double> &p = rw.rho;
    const double s1 = p[1] + ((p[0] - p[1]) / (1 + std::exp((-1) * p[3] * (xi - p[2]))));
    const double s2 = p[5] + ((p[4] - p[5]) / (1 + std::exp((-1) * p[7] * (xi - p[6]))));
    return s1 + s2;
}

bool Simulation::upload_sigmoid_dfactors(uint32_t map_steps, std::string &err)
{
    if (rw.rho.size() < 8)
    {
        err = "RHO_TYPE sigmoid needs 8 RHO values {K1, A1, eps1, B1, K2, A2, eps2, B2}";
        return false;
    }
    if (img.n_phases != 1)
    {
        err = "RHO_TYPE sigmoid needs a single-phase image";
        return false;
    }
    std::vector<double> f(collisions.size());
    for (size_t i = 0; i < f.size(); i++)
    {
        // updateXIrate (walker.h:162-172, LOG_XIRATE false) -> setSurfaceRelaxivity -> computeDecreaseFactor
        const double xi = (double)collisions[i] / (double)map_steps;
        f[i] = decrease_factor(sigmoid_rho(xi));
    }
    if (rwnmr_walkers_set_dfactor(ctx, f.data()) != RWNMR_OK)
    {
        err = std::string("per-walker decrease factors: ") + rwnmr_last_error(ctx);
        return false;
    }
    walker_dfactors = f;
    return true;
}

std::vector<double> Simulation::phase_dfactors() const
{
    std::vector<double> f(rho_phase.size());
    for (size_t q = 0; q < f.size(); q++) f[q] = decrease_factor(rho_phase[q]);
    return f;
}

int Simulation::bc_code() const
{
    return rw.bc == "periodic" ? RWNMR_BC_PERIODIC : (rw.bc == "mirror" ? RWNMR_BC_MIRROR : RWNMR_BC_NOFLUX);
}

bool Simulation::map_simulation(std::string &err)
{
    // initHistogramList (NMR_Simulation.cpp:1456-1479)
    int nh = rw.histograms;
    if ((int)echoes < nh) nh = 1;
    if (nh < 1) nh = 1;
    const int per = echoes / nh;
    hist_list.assign(nh, Histogram());
    for (int h = 0; h < nh; h++)
    {
        hist_list[h].first_echo = h * per;
        hist_list[h].last_echo = hist_list[h].first_echo + per;
    }
    hist_list.back().last_echo += echoes - nh * per;
    const size_t n = x0.size();
    std::vector<uint32_t> total(n, 0), prev(n, 0), window(n);
    for (int h = 0; h < nh; h++)
    {
        const uint32_t wsteps = rw.steps_per_echo * (hist_list[h].last_echo - hist_list[h].first_echo);
        rwnmr_status st = h == 0 ? rwnmr_map_run(ctx, bc_code(), shift, wsteps, total.data())
                                 : rwnmr_map_continue(ctx, bc_code(), shift, wsteps, total.data());
        if (st != RWNMR_OK)
        {
            err = std::string("collision mapping: ") + rwnmr_last_error(ctx);
            return false;
        }
        for (size_t i = 0; i < n; i++) window[i] = total[i] - prev[i];
        prev = total;
        hist_list[h].create(rw.histogram_size, rw.histogram_scale);
        hist_list[h].fill(window, wsteps);
    }
    collisions = total;
    histogram.create(rw.histogram_size, rw.histogram_scale);
    histogram.fill(collisions, hist_list.back().last_echo * rw.steps_per_echo);
    // updateXIrate (Walker/walker.h:162-172)
    xi_rate.resize(n);
    for (size_t i = 0; i < n; i++) xi_rate[i] = (double)collisions[i] / (double)steps;
    return true;
}

void Simulation::save_info() const
{
    std::ofstream f(sim_dir + "/SimInfo.txt");
    f << "------------------------------------------------------\n";
    f << ">>> NMR SIMULATION 3D PARAMETERS: " << rw.name << "\n";
    f << "------------------------------------------------------\n";
    f << "Data path: " << db_path + rw.name << "\n";
    f << "Image path: " << img.source << "\n";
    f << "Image resolution (um/voxel): " << voxel_res << "\n";
    f << "Diffusion coefficient (um^2/ms): " << rw.d0 << "\n";
    f << "Number of images: " << img.nz << "\n";
    f << "Walkers pore occupancy in simulation: " << occupancy * 100.0 << "%\n";
    f << "Initial seed: " << initial_seed << "\n";
    f << "GPU usage: ON (rwnmr_gb300, sm_103a)\n";
    // saveImageInfo (NMR_Simulation.cpp:1644-1672)
    if (rw.save_img_info)
    {
        std::ofstream g(sim_dir + "/ImageInfo.txt");
        g << "image path: " << img.source << "\n";
        g << "width(x): " << img.nx << "\nheight(y): " << img.ny << "\ndepth(z): " << img.nz << "\n";
        g << "resolution: " << resolution << "\nvoxel shift: " << (1 << shift) << "\nstep length: " << voxel_res << "\n";
        g << "porosity: " << porosity << "\nSVp: " << svp << "\n";
    }
    // saveBitBlock -> fileHandler::writeBitBlockObject3D (FileHandler/fileHandler.cpp:192-235)
    if (rw.save_binimg)
    {
        const int bc = (img.nx + 3) / 4, br = (img.ny + 3) / 4, bd = (img.nz + 3) / 4;
        std::ofstream b(sim_dir + "/NMR_binImage.txt");
        b << "blocks, bRows, bColumns, bDepth, imgRows, imgColumns, imgDepth, \n";
        b << img.blocks.size() << ", " << br << ", " << bc << ", " << bd << ", " << img.ny << ", " << img.nx << ", "
          << img.nz << "\n\nblockID, blockData\n";
        for (size_t k = 0; k < img.blocks.size(); k++) b << k << ", " << img.blocks[k] << "\n";
    }
    // saveWalkers (NMR_Simulation.cpp:1674-1712): the walkers as created, before any walk
    if (rw.save_walkers)
    {
        std::ofstream w(sim_dir + "/walkers.csv");
        w << std::setprecision(6);
        w << "PositionXi,PositionYi,PositionZi,PositionXf,PositionYf,PositionZf,Collisions,XIRate,Energy,RNGSeed\n";
        for (size_t i = 0; i < x0.size(); i++)
            w << x0[i] << "," << y0[i] << "," << z0[i] << "," << x0[i] << "," << y0[i] << "," << z0[i] << ",0,0,1,"
              << seed0[i] << "\n";
    }
}

// ---------------------------------------------------------------------------------------------
bool CpmgSequence::set(std::string &err)
{
    name = parent + "/NMR_cpmg_t=" + trimmed_time(cfg.obs_time) + "ms" + suffix;
    mkdirs(sim.db_path + sim.rw.name + "/" + name);
    dir = sim.db_path + sim.rw.name + "/" + name;
    sim.set_time_framework_time(cfg.obs_time);
    // signal times (NMR_cpmg.cpp:121-130): accumulated echo spacing
    times.clear();
    double t = 0.0;
    const double delta_t = sim.rw.steps_per_echo * sim.dt;
    times.push_back(t);
    for (uint32_t e = 0; e < sim.echoes; e++)
    {
        t += delta_t;
        times.push_back(t);
    }
    // The reference always runs the collision-mapping walk here (NMR_cpmg.cpp:134). With uniform
    // relaxivity nothing but the histogram / walker outputs depends on it, so it runs only when one
    // of those is requested.
    if (!map) return true;
    const bool need_map = sim.rw.rho_type == "sigmoid" || cfg.method == "histogram" ||
                          (cfg.save_mode && (cfg.save_histogram || cfg.save_histogram_list || cfg.save_walkers));
    if (need_map && !sim.map_simulation(err)) return false;
    // updateWalkersRelaxativity(sigmoid) (NMR_cpmg.cpp:137-146): a decrease factor per walker
    if (sim.rw.rho_type == "sigmoid" && cfg.method != "histogram" && !sim.upload_sigmoid_dfactors(sim.steps, err))
        return false;
    return true;
}

bool CpmgSequence::run_simulation(std::string &err)
{
    const uint32_t E = sim.echoes;
    if (cfg.method == "histogram")
    {
        // createPenaltiesVector + histogram_simulation (NMR_cpmg.cpp:235-343)
        const int hs = sim.histogram.size;
        std::vector<double> pen(hs);
        for (int k = 0; k < hs; k++)
        {
            const double xi = sim.histogram.bins[k];
            double rho = sim.rho_phase[0];
            if (sim.rw.rho_type == "sigmoid" && sim.rw.rho.size() >= 8) rho = sim.sigmoid_rho(xi);
            pen[k] = std::pow(sim.decrease_factor(rho), xi * (double)sim.rw.steps_per_echo);
        }
        amps.assign(1, 1.0);
        std::vector<double> dist(hs);
        for (const Histogram &h : sim.hist_list)
        {
            for (int k = 0; k < hs; k++) dist[k] = amps.back() * h.amps[k];
            for (int e = h.first_echo; e < h.last_echo; e++)
            {
                for (int k = 0; k < hs; k++) dist[k] *= pen[k];
                double lvl = 0.0;
                for (int k = 0; k < hs; k++) lvl += dist[k];
                amps.push_back(lvl);
            }
        }
        raw = amps;
    }
    else if (cfg.residual_field != "none")
    {
        // RESIDUAL_FIELD (NMR_cpmg.cpp:48-64): the reference applies the field in its GPU walk
        // (CPMG_walk_*_field, NMR_cpmg_cuda.cpp:1008-1012, 1184-1258); its OpenMP walk ignores it.
        rwnmr_status st;
        if (cfg.residual_field == "uniform")
            st = rwnmr_field_set_uniform(sim.ctx, cfg.gradient_value, cfg.gradient_direction, sim.resolution);
        else
        {
            // InternalField::readDataFromFile: raw doubles, x fastest, exactly one per voxel
            const int64_t vol = (int64_t)sim.img.nx * sim.img.ny * sim.img.nz;
            std::ifstream in(cfg.path_to_field, std::ios::binary | std::ios::ate);
            if (!in)
            {
                err = "cannot open internal field file " + cfg.path_to_field;
                return false;
            }
            const int64_t bytes = (int64_t)in.tellg();
            if (bytes / (int64_t)sizeof(double) != vol)
            {
                err = "internal field dims don't match the image: " + std::to_string(bytes / (int64_t)sizeof(double)) +
                      " vs. " + std::to_string(vol);
                return false;
            }
            std::vector<double> field((size_t)vol);
            in.seekg(0);
            in.read(reinterpret_cast<char *>(field.data()), vol * (int64_t)sizeof(double));
            if (!in)
            {
                err = "error reading internal field file " + cfg.path_to_field;
                return false;
            }
            st = rwnmr_field_upload(sim.ctx, field.data(), vol);
        }
        std::vector<double> f = sim.phase_dfactors();
        rwnmr_field_cpmg_params p{};
        p.bc = sim.bc_code();
        p.shift = sim.shift;
        p.steps_per_echo = sim.rw.steps_per_echo;
        p.n_echoes = (int32_t)E;
        p.dfactor = sim.rw.rho_type == "sigmoid" ? nullptr : f.data(); // NULL: per-walker factors
        p.gamma = 1.0e+06 * sim.gamma;   // image_simulation_cuda: gamma = 1e6 * giromagneticRatio
        p.time_interval = 1.0e-3 * sim.dt; // timeInterval = 1e-3 * NMR.getTimeInterval()
        raw.assign(E + 1, 0.0);
        echo_collisions.assign((size_t)E * sim.img.n_phases, 0); // the field walk records no collisions per echo
        if (st == RWNMR_OK) st = rwnmr_cpmg_field_run(sim.ctx, &p, raw.data(), nullptr, nullptr);
        if (st != RWNMR_OK)
        {
            err = std::string("CPMG field walk: ") + rwnmr_last_error(sim.ctx);
            return false;
        }
        kernel_ms = rwnmr_ctx_last_kernel_ms(sim.ctx);
        amps = raw;
    }
    else
    {
        std::vector<double> f = sim.phase_dfactors();
        rwnmr_cpmg_params p{};
        p.bc = sim.bc_code();
        p.shift = sim.shift;
        p.steps_per_echo = sim.rw.steps_per_echo;
        p.n_echoes = (int32_t)E;
        p.dfactor = sim.rw.rho_type == "sigmoid" ? nullptr : f.data(); // NULL: per-walker factors
        raw.assign(E + 1, 0.0);
        echo_collisions.assign((size_t)E * sim.img.n_phases, 0);
        rwnmr_status st = rwnmr_cpmg_run(sim.ctx, &p, raw.data(), nullptr, echo_collisions.data());
        if (st != RWNMR_OK)
        {
            err = std::string("CPMG walk: ") + rwnmr_last_error(sim.ctx);
            return false;
        }
        kernel_ms = rwnmr_ctx_last_kernel_ms(sim.ctx);
        amps = raw;
    }
    if (cfg.apply_bulk)
    {
        // applyBulk (NMR_cpmg.cpp:346-359)
        const double bulk = -1.0 / sim.rw.bulk_time;
        if (amps.size() == times.size())
            for (size_t e = 0; e < amps.size(); e++) amps[e] = std::exp(bulk * times[e]) * amps[e];
    }
    // normalizeSignal (NMR_cpmg.cpp:369-384)
    if (!amps.empty())
    {
        const double norm = 1.0 / amps[0];
        for (double &a : amps) a = norm * a;
    }
    noise.assign(amps.size(), 0.0);
    t2_bins.clear();
    t2_amps.clear();
    return true;
}

bool CpmgSequence::apply_laplace(std::string &err)
{
    // Tikhonov-ILT of the normalised decay without its t = 0 point; with NOISE_AMP the inverted
    // decay carries Gaussian noise, which becomes the decay file's noise column.
    t2_bins.clear();
    t2_amps.clear();
    if (amps.size() < 3 || times.size() != amps.size())
    {
        sim.log("- T2 inversion skipped: the decay has fewer than 3 points");
        return true;
    }
    T2InversionConfig c;
    c.min_t2 = cfg.min_t2;
    c.max_t2 = cfg.max_t2;
    c.use_logspace = cfg.use_t2_logspace;
    c.num_t2_bins = cfg.num_t2_bins;
    c.min_lambda = cfg.min_lambda;
    c.max_lambda = cfg.max_lambda;
    c.num_lambdas = cfg.num_lambdas;
    c.prune_num = cfg.prune_num;
    c.noise_amp = cfg.noise_amp;
    c.noise_seed = sim.rw.seed;
    if (c.noise_amp != 0.0 && c.noise_seed == 0)
    {
        std::random_device dev;
        c.noise_seed = ((uint64_t)dev() << 32) | dev();
    }
    T2Inversion r;
    if (!invert_t2(times, amps, c, r, err)) return false;
    t2_bins = r.bins;
    t2_amps = r.amps;
    t2_lambda = r.lambda;
    noise.assign(amps.size(), 0.0);
    if (r.noise.size() + 1 == amps.size())
        for (size_t i = 1; i < amps.size(); i++) noise[i] = r.noise[i - 1];
    std::ostringstream m;
    m << "- T2 inversion: " << t2_bins.size() << " bins, filtering lambda " << t2_lambda << ", "
      << r.nnls_solves << " NNLS solves";
    sim.log(m.str());
    return true;
}

void CpmgSequence::save() const
{
    if (!cfg.save_mode) return;
    if (cfg.save_decay)
    {
        std::ofstream f = open_out(dir + "/cpmg_decay.csv");
        f << "time,signal,noise,noiseless\n";
        for (size_t i = 0; i < amps.size(); i++)
            f << times[i] << "," << amps[i] + noise[i] << "," << noise[i] << "," << amps[i] << "\n";
        // writeT2dist (NMR_cpmg.cpp:514-535)
        std::ofstream t = open_out(dir + "/cpmg_T2.csv");
        t << "NMRT2_bins,NMRT2_amps\n";
        for (size_t i = 0; i < t2_bins.size() && i < t2_amps.size(); i++) t << t2_bins[i] << "," << t2_amps[i] << "\n";
        if (!echo_collisions.empty())
        {
            // per-echo collision counts per phase (an output the reference does not have)
            std::ofstream c = open_out(dir + "/cpmg_echo_collisions.csv");
            const int P = sim.img.n_phases;
            c << "echo";
            for (int q = 0; q < P; q++) c << ",collisions_phase" << q + 1;
            c << "\n";
            for (size_t e = 0; e < echo_collisions.size() / P; e++)
            {
                c << e + 1;
                for (int q = 0; q < P; q++) c << "," << echo_collisions[e * P + q];
                c << "\n";
            }
        }
    }
    if (cfg.save_walkers && !sim.collisions.empty())
    {
        std::ofstream f(dir + "/cpmg_walkers.csv");
        f << std::setprecision(6);
        std::vector<int32_t> x(sim.x0.size()), y(x.size()), z(x.size());
        rwnmr_walkers_download(sim.ctx, x.data(), y.data(), z.data(), nullptr, nullptr);
        f << "PositionXi,PositionYi,PositionZi,PositionXf,PositionYf,PositionZf,Collisions,XIRate,Energy,RNGSeed\n";
        const double fd = sim.decrease_factor(sim.rho_phase[0]);
        const bool per_walker = sim.walker_dfactors.size() == x.size();
        for (size_t i = 0; i < x.size(); i++)
            f << sim.x0[i] << "," << sim.y0[i] << "," << sim.z0[i] << "," << x[i] << "," << y[i] << "," << z[i] << ","
              << sim.collisions[i] << "," << sim.xi_rate[i] << ","
              << std::pow(per_walker ? sim.walker_dfactors[i] : fd, (double)sim.collisions[i]) << "," << sim.seed0[i]
              << "\n";
    }
    if (cfg.save_histogram && !sim.histogram.bins.empty())
    {
        std::ofstream f = open_out(dir + "/cpmg_histogram.csv");
        f << "Bins,Amps\n";
        for (int i = 0; i < sim.histogram.size; i++) f << sim.histogram.bins[i] << "," << sim.histogram.amps[i] << "\n";
    }
    if (cfg.save_histogram_list && !sim.hist_list.empty())
    {
        std::ofstream f = open_out(dir + "/cpmg_histList.csv");
        for (size_t h = 0; h < sim.hist_list.size(); h++) f << "Bins" << h << ",Amps" << h << ",";
        f << "\n";
        for (int i = 0; i < sim.histogram.size; i++)
        {
            for (const Histogram &h : sim.hist_list) f << h.bins[i] << "," << h.amps[i] << ",";
            f << "\n";
        }
    }
}

bool CpmgSequence::run(std::string &err)
{
    if (!set(err) || !run_simulation(err) || !apply_laplace(err)) return false;
    save();
    sim.log("- CPMG: " + std::to_string(sim.echoes) + " echoes x " + std::to_string(sim.rw.steps_per_echo) +
            " steps, walk " + std::to_string(kernel_ms) + " ms on the GPU");
    return true;
}

// ---------------------------------------------------------------------------------------------
namespace
{
// std::to_string(v) cut `digits` places after the point of std::to_string(ref), the way
// NMR_multitau::setName / setCPMG trim (the point is looked up in a second string).
std::string trimmed_like(double v, double ref, int digits)
{
    const std::string s = std::to_string(v);
    const size_t dot = std::to_string(ref).find('.');
    return s.substr(0, dot == std::string::npos ? std::string::npos : dot + digits + 1);
}
} // namespace

void MultitauSequence::set_tau_sequence()
{
    std::vector<double> t;
    if (cfg.tau_scale == "manual") t = cfg.tau_values;
    else
    {
        // linspace / logspace (NMR_multitau.cpp:51-78)
        const int n = std::max(cfg.tau_points, 0);
        const bool lg = cfg.tau_scale == "log";
        const double a = lg ? std::log10(cfg.tau_min) : cfg.tau_min;
        const double b = lg ? std::log10(cfg.tau_max) : cfg.tau_max;
        const double step = (b - a) / ((double)n - 1.0);
        for (int i = 0; i < n; i++)
        {
            const double x = a + step * i;
            t.push_back(lg ? std::pow(10.0, x) : x);
        }
    }
    required_steps.clear();
    signal_times.clear();
    uint32_t min_steps = 0;
    for (double tau : t)
    {
        // ceil to whole steps, even, strictly increasing by at least two
        int steps = (int)std::ceil(tau / sim.dt);
        if (steps % 2 != 0) steps++;
        if ((uint32_t)steps <= min_steps) steps = (int)min_steps + 2;
        required_steps.push_back((uint32_t)steps);
        min_steps = (uint32_t)steps;
        signal_times.push_back(steps * sim.dt);
    }
}

bool MultitauSequence::run(std::string &err)
{
    // setName (NMR_multitau.cpp:45-66)
    std::string lo, hi, pts;
    if (cfg.tau_scale == "manual")
    {
        if (cfg.tau_values.empty())
        {
            err = "TAU_SCALE manual needs TAU_VALUES";
            return false;
        }
        lo = std::to_string(cfg.tau_values.front());
        hi = std::to_string(cfg.tau_values.back());
        pts = std::to_string(cfg.tau_values.size());
    }
    else
    {
        lo = std::to_string(cfg.tau_min);
        hi = std::to_string(cfg.tau_max);
        pts = std::to_string(cfg.tau_points);
    }
    {
        const size_t dmin = std::to_string(cfg.tau_min).find('.'), dmax = std::to_string(cfg.tau_max).find('.');
        lo = lo.substr(0, dmin == std::string::npos ? std::string::npos : dmin + 3);
        hi = hi.substr(0, dmax == std::string::npos ? std::string::npos : dmax + 3);
    }
    name = "/NMR_multitau_min=" + lo + "ms_max=" + hi + "ms_pts=" + pts + "_scale=" + cfg.tau_scale;
    mkdirs(sim.db_path + sim.rw.name + "/" + name);
    dir = sim.db_path + sim.rw.name + "/" + name;
    set_tau_sequence();
    // a sigmoid relaxivity keeps each walker's current factor (none mapped yet: collision rate 0)
    if (sim.rw.rho_type == "sigmoid" && sim.walker_dfactors.size() != sim.x0.size())
    {
        sim.collisions.assign(sim.x0.size(), 0);
        if (!sim.upload_sigmoid_dfactors(1, err)) return false;
    }
    signal_amps.clear();
    for (size_t k = 0; k < required_steps.size(); k++)
    {
        // setCPMG (NMR_multitau.cpp:119-131): te = required steps, one echo unless COMPLETE_DECAY
        sim.rw.steps_per_echo = (int)required_steps[k];
        CpmgSequence seq(sim, cpmg_cfg);
        if (!cfg.complete_decay) seq.cfg.obs_time = signal_times[k];
        seq.map = false;
        seq.parent = name;
        const double te = required_steps[k] * sim.dt;
        seq.suffix = "_te=" + trimmed_like(te, te, 3);
        if (!seq.set(err) || !seq.run_simulation(err)) return false;
        kernel_ms += seq.kernel_ms;
        if (seq.amps.size() > 1) signal_amps.push_back(seq.amps[1]);
        if (cfg.complete_decay)
        {
            // runCPMG inverts complete decays (NMR_multitau.cpp:146-149)
            if (!seq.apply_laplace(err)) return false;
            // saveCPMG (NMR_multitau.cpp:154-185): the multitau SAVE_* flags pick the files
            seq.cfg.save_mode = true;
            seq.cfg.save_walkers = cfg.save_walkers;
            seq.cfg.save_histogram = cfg.save_histogram;
            seq.cfg.save_histogram_list = cfg.save_histogram_list;
            seq.cfg.save_decay = cfg.save_decay;
            seq.save();
        }
    }
    if (cfg.save_decay)
    {
        // writeDecay (NMR_multitau.cpp:221-248)
        std::ofstream f = open_out(dir + "/multitau_decay.csv");
        f << "echo_time,signal\n";
        if (signal_times.size() == signal_amps.size())
            for (size_t k = 0; k < signal_amps.size(); k++) f << signal_times[k] << "," << signal_amps[k] << "\n";
    }
    sim.log("- multitau: " + std::to_string(required_steps.size()) + " echo times, walks " + std::to_string(kernel_ms) +
            " ms on the GPU");
    return true;
}

// ---------------------------------------------------------------------------------------------
bool PfgseSequence::run(std::string &err)
{
    Simulation &S = sim;
    n_g = cfg.gradient_samples;
    if (n_g < 2)
    {
        err = "GRADIENT_SAMPLES must be at least 2";
        return false;
    }
    // gradient ramp and wave vectors (NMR_pfgse.cpp:272-313, 483-486): accumulated steps
    gvec.assign((size_t)n_g * 3, 0.0);
    kvec.assign((size_t)n_g * 3, 0.0);
    gradient.assign(n_g, 0.0);
    double gap[3], gv[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < 3; a++) gap[a] = cfg.max_gradient[a] / ((double)(n_g - 1));
    for (int j = 0; j < n_g; j++)
    {
        for (int a = 0; a < 3; a++)
        {
            gvec[3 * j + a] = gv[a];
            kvec[3 * j + a] = (cfg.pulse_width * 1.0e-03) * (S.gamma * 1.0e+06) * (gv[a] * 1.0e-08);
        }
        gradient[j] = std::sqrt(gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]);
        for (int a = 0; a < 3; a++) gv[a] += gap[a];
    }
    exposure_times = pfgse_time_samples(cfg);
    if (cfg.apply_scale_factor)
    {
        const double sf = (cfg.inspection_length * cfg.inspection_length) / S.rw.d0;
        for (double &t : exposure_times) t *= sf;
    }
    const int nd = (int)exposure_times.size();
    dir = S.db_path + S.rw.name + "//NMR_pfgse";
    mkdirs(dir + "/timesamples");
    if (cfg.save_mode && cfg.save_pfgse)
    {
        std::ofstream r = open_out(dir + "/PFGSE_results.csv");
        r << "Time,D_sat,D_sat(error),D_sat(std),D_sat(pts),D_msd,D_msd(std),D_msdX,D_msdX(std),D_msdY,D_msdY(std),"
             "D_msdZ,D_msdZ(std)\n";
        std::ofstream p = open_out(dir + "/PFGSE_parameters.txt");
        const double gx = gvec[3 * (n_g - 1)], gy = gvec[3 * (n_g - 1) + 1], gz = gvec[3 * (n_g - 1) + 2];
        const double gn = std::sqrt(gx * gx + gy * gy + gz * gz);
        p << "RWNMR-PFGSE Parameters\nD_0: " << S.rw.d0 << "\nPulse width: " << cfg.pulse_width
          << "\nGiromagnetic Ratio: " << S.gamma << "\nGradient direction: {" << gx / gn << ", " << gy / gn << ", "
          << gz / gn << "}\nGradients: " << n_g << "\nTimes: [";
        for (int i = 0; i < nd; i++) p << (i ? ", " : "") << exposure_times[i];
        p << "]\n";
        std::ofstream g = open_out(dir + "/PFGSE_gradient.csv");
        g << "Id,Gx,Gy,Gz,Kx,Ky,Kz\n";
        for (int j = 0; j < n_g; j++)
            g << j << "," << gvec[3 * j] << "," << gvec[3 * j + 1] << "," << gvec[3 * j + 2] << "," << kvec[3 * j] << ","
              << kvec[3 * j + 1] << "," << kvec[3 * j + 2] << "\n";
    }
    if (nd == 0) return true;
    // walk steps per exposure time (setTimeFramework(double) per Delta)
    steps.assign(nd, 0);
    for (int i = 0; i < nd; i++)
    {
        S.set_time_framework_time(exposure_times[i]);
        steps[i] = S.steps;
    }
    if (S.rw.rho_type == "sigmoid")
    {
        // runInitialMapSimulation (NMR_pfgse.cpp:322-346): a mapping walk as long as the longest
        // exposure time sets each walker's collision rate, hence its relaxivity
        const uint32_t map_steps = steps[nd - 1];
        S.collisions.assign(S.x0.size(), 0);
        if (rwnmr_map_run(S.ctx, S.bc_code(), S.shift, map_steps, S.collisions.data()) != RWNMR_OK)
        {
            err = std::string("collision mapping: ") + rwnmr_last_error(S.ctx);
            return false;
        }
        if (!S.upload_sigmoid_dfactors(map_steps, err)) return false;
    }
    // one GPU call walks all exposure times cumulatively (the reference GPU path's stepsTaken)
    std::vector<double> f = S.phase_dfactors();
    std::vector<int32_t> st32(steps.begin(), steps.end());
    rwnmr_pfgse_params p{};
    p.bc = S.bc_code();
    p.shift = S.shift;
    p.n_delta = nd;
    p.steps = st32.data();
    p.n_g = n_g;
    p.kvec = kvec.data();
    p.res = S.voxel_res;
    p.dfactor = S.rw.rho_type == "sigmoid" ? nullptr : f.data(); // NULL: per-walker factors
    Mkt.assign((size_t)nd * n_g, 0.0);
    esum.assign(nd, 0.0);
    std::vector<uint64_t> msd((size_t)nd * 3);
    rwnmr_status rs = rwnmr_pfgse_run(S.ctx, &p, Mkt.data(), esum.data(), msd.data());
    if (rs != RWNMR_OK)
    {
        err = std::string("PFGSE walk: ") + rwnmr_last_error(S.ctx);
        return false;
    }
    kernel_ms = rwnmr_ctx_last_kernel_ms(S.ctx);
    // Walker sampling (ALLOW_WALKER_SAMPLING with WALKER_SAMPLES > 1; NMR_pfgse.cpp:605-640, 876-1097,
    // 1173-1290): the walkers split into WALKER_SAMPLES contiguous groups of N / WALKER_SAMPLES (the
    // rest are left out), each group's M(k) and mean squared displacement computed on its own. The
    // groups are walked as separate populations; every walker's trajectory is the same as in the
    // full walk.
    const int n_samples = S.rw.walker_samples;
    const bool sampling = cfg.allow_walker_sampling && n_samples > 1;
    const int64_t per = sampling ? (int64_t)S.x0.size() / n_samples : 0;
    std::vector<double> Ms, es;      // [sample][n_delta][n_g], [sample][n_delta]
    std::vector<uint64_t> msds;      // [sample][n_delta][3]
    if (sampling)
    {
        Ms.assign((size_t)n_samples * nd * n_g, 0.0);
        es.assign((size_t)n_samples * nd, 0.0);
        msds.assign((size_t)n_samples * nd * 3, 0);
        for (int smp = 0; smp < n_samples && rs == RWNMR_OK; smp++)
        {
            const size_t o = (size_t)smp * per;
            rs = rwnmr_walkers_upload(S.ctx, per, S.x0.data() + o, S.y0.data() + o, S.z0.data() + o, S.seed0.data() + o);
            if (rs == RWNMR_OK && p.dfactor == nullptr) rs = rwnmr_walkers_set_dfactor(S.ctx, S.walker_dfactors.data() + o);
            if (rs == RWNMR_OK)
                rs = rwnmr_pfgse_run(S.ctx, &p, &Ms[(size_t)smp * nd * n_g], &es[(size_t)smp * nd], &msds[(size_t)smp * nd * 3]);
            kernel_ms += rwnmr_ctx_last_kernel_ms(S.ctx);
        }
        // the full population back in the engine for what runs next
        if (rs == RWNMR_OK)
            rs = rwnmr_walkers_upload(S.ctx, (int64_t)S.x0.size(), S.x0.data(), S.y0.data(), S.z0.data(), S.seed0.data());
        if (rs == RWNMR_OK && p.dfactor == nullptr) rs = rwnmr_walkers_set_dfactor(S.ctx, S.walker_dfactors.data());
        if (rs != RWNMR_OK)
        {
            err = std::string("PFGSE walker samples: ") + rwnmr_last_error(S.ctx);
            return false;
        }
    }
    auto mean_of = [](const std::vector<double> &v) {
        double sum = 0.0;
        for (double x : v) sum += x;
        return sum / (double)v.size();
    };
    auto std_of = [](const std::vector<double> &v, double m) { // population deviation (NMR_pfgse.cpp:1863-1891)
        double sum = 0.0;
        for (double x : v) sum += (x - m) * (x - m);
        return std::sqrt(sum / (double)v.size());
    };
    dsat_std.assign(nd, 0.0);
    dmsd_std.assign(nd, 0.0);
    dmsd_vec_std.assign((size_t)nd * 3, 0.0);
    msd_vec_std.assign((size_t)nd * 3, 0.0);
    m_std.assign((size_t)nd * n_g, 0.0);
    lhs_std.assign((size_t)nd * n_g, 0.0);
    lhs.assign((size_t)nd * n_g, 0.0);
    rhs.assign((size_t)nd * n_g, 0.0);
    raw_noise.assign((size_t)nd * n_g, 0.0);
    dsat.assign(nd, 0.0);
    dsat_err.assign(nd, 0.0);
    dmsd.assign(nd, 0.0);
    dsat_points.assign(nd, n_g);
    msd_vec.assign((size_t)nd * 3, 0.0);
    dmsd_vec.assign((size_t)nd * 3, 0.0);
    double noise_amp = cfg.noise_amp;
    const double N = (double)S.x0.size();
    for (int i = 0; i < nd; i++)
    {
        const double delta = exposure_times[i];
        double *M = &Mkt[(size_t)i * n_g];
        if (cfg.apply_bulk)
        {
            const double bm = std::exp((-1.0 / S.rw.bulk_time) * delta);
            for (int j = 0; j < n_g; j++) M[j] *= bm;
        }
        // createNoiseVector / applyNoiseToSignal (NMR_pfgse.cpp:527-591): the draws always happen
        double basis = N;
        if (cfg.target_snr > 0.0)
        {
            double sss = 0.0, uss = 0.0;
            for (int j = 0; j < n_g; j++)
            {
                sss += M[j] * M[j];
                uss += M[j];
            }
            sss /= (double)n_g;
            uss /= (double)n_g;
            noise_amp = std::sqrt((sss - uss * uss) / cfg.target_snr);
            basis = 1.0;
        }
        {
            std::normal_distribution<double> nd_(0.0, basis * noise_amp);
            for (int j = 0; j < n_g; j++) raw_noise[(size_t)i * n_g + j] = nd_(S.rng);
        }
        if (noise_amp > 0.0)
            for (int j = 0; j < n_g; j++) M[j] += raw_noise[(size_t)i * n_g + j];
        // recoverDsatWithoutSampling (NMR_pfgse.cpp:641-692)
        double *L = &lhs[(size_t)i * n_g];
        double *R = &rhs[(size_t)i * n_g];
        auto lhs_of = [&](const double *m, double *out) {
            std::vector<double> norm(n_g);
            for (int j = 0; j < n_g; j++) norm[j] = m[j] / m[0];
            for (int j = 0; j < n_g; j++)
            {
                const double ratio = norm[j] / norm[0];
                out[j] = ratio > 1.0e-06 ? std::log(ratio) : std::log(1.0e-06);
            }
        };
        lhs_of(M, L);
        for (int j = 0; j < n_g; j++)
        {
            const double k = std::sqrt(kvec[3 * j] * kvec[3 * j] + kvec[3 * j + 1] * kvec[3 * j + 1] +
                                       kvec[3 * j + 2] * kvec[3 * j + 2]);
            R[j] = (-1.0) * k * k * (delta - (cfg.pulse_width / 3.0));
        }
        // recoverDsatWithSampling (NMR_pfgse.cpp:876-1097): per-sample magnitudes (bulk, then noise of
        // amplitude (N / samples) * NOISE_AMP drawn per sample when NOISE_AMP > 0), normalised per
        // sample; the mean and population deviation over samples replace M and the LHS
        std::vector<double> LS; // [sample][n_g]
        if (sampling)
        {
            const double bm = cfg.apply_bulk ? std::exp((-1.0 / S.rw.bulk_time) * delta) : 1.0;
            std::vector<double> Msmp((size_t)n_samples * n_g), Nsmp((size_t)n_samples * n_g, 0.0);
            LS.assign((size_t)n_samples * n_g, 0.0);
            for (int smp = 0; smp < n_samples; smp++)
                for (int j = 0; j < n_g; j++)
                    Msmp[(size_t)smp * n_g + j] = Ms[((size_t)smp * nd + i) * n_g + j] * bm;
            if (noise_amp > 0.0)
            {
                const double m0 = N / (double)n_samples;
                for (int smp = 0; smp < n_samples; smp++)
                {
                    std::normal_distribution<double> nd_(0.0, m0 * noise_amp);
                    for (int j = 0; j < n_g; j++) Nsmp[(size_t)smp * n_g + j] = nd_(S.rng);
                }
                for (size_t k = 0; k < Msmp.size(); k++) Msmp[k] += Nsmp[k];
            }
            for (int smp = 0; smp < n_samples; smp++) lhs_of(&Msmp[(size_t)smp * n_g], &LS[(size_t)smp * n_g]);
            for (int j = 0; j < n_g; j++)
            {
                std::vector<double> mv(n_samples), nv(n_samples), lv(n_samples);
                for (int smp = 0; smp < n_samples; smp++)
                {
                    mv[smp] = Msmp[(size_t)smp * n_g + j];
                    nv[smp] = Nsmp[(size_t)smp * n_g + j];
                    lv[smp] = LS[(size_t)smp * n_g + j];
                }
                M[j] = mean_of(mv);
                m_std[(size_t)i * n_g + j] = std_of(mv, M[j]);
                raw_noise[(size_t)i * n_g + j] = mean_of(nv);
                L[j] = mean_of(lv);
                lhs_std[(size_t)i * n_g + j] = std_of(lv, L[j]);
            }
        }
        int pts = n_g;
        int window = std::min(cfg.threshold_window, n_g);
        if (cfg.threshold_type == "lhs")
        {
            const double v = cfg.threshold_value;
            if (n_g >= window && v > 0.0 && v < 1.0)
            {
                const double lv = std::log(v);
                int idx;
                if (noise_amp == 0.0)
                {
                    idx = window - 1;
                    bool greater = true;
                    while (idx < n_g && greater)
                    {
                        if (L[idx] < lv) greater = false;
                        else idx++;
                    }
                    if (greater) idx--;
                }
                else
                {
                    std::vector<double> wv(L, L + window);
                    auto mean = [&]() {
                        double s = 0.0;
                        for (double x : wv) s += x;
                        return s / (double)wv.size();
                    };
                    idx = window;
                    bool greater = mean() >= lv;
                    while (idx < n_g && greater)
                    {
                        wv[idx % window] = L[idx];
                        if (mean() < lv) greater = false;
                        else idx++;
                    }
                    if (greater) idx--;
                }
                pts = idx;
            }
        }
        else if (cfg.threshold_type == "samples")
        {
            const int s = (int)cfg.threshold_value;
            if (s <= n_g && s > 1) pts = s;
        }
        dsat_points[i] = pts;
        std::vector<double> xs(R, R + pts);
        if (!sampling)
        {
            std::vector<double> ys(L, L + pts);
            double b, mse;
            lsq_no_intercept(xs, ys, pts, b, mse);
            dsat[i] = b;
            dsat_err[i] = std::sqrt(mse * (((double)pts) / ((double)pts - 1.0)));
        }
        else
        {
            std::vector<double> bs(n_samples), errs(n_samples);
            for (int smp = 0; smp < n_samples; smp++)
            {
                std::vector<double> ys(&LS[(size_t)smp * n_g], &LS[(size_t)smp * n_g] + pts);
                double b, mse;
                lsq_no_intercept(xs, ys, pts, b, mse);
                bs[smp] = b;
                errs[smp] = std::sqrt(mse * (((double)pts) / ((double)pts - 1.0)));
            }
            dsat[i] = mean_of(bs);
            dsat_err[i] = mean_of(errs);
            dsat_std[i] = std_of(bs, dsat[i]);
        }
        // recoverDmsdWithoutSampling (NMR_pfgse.cpp:1098-1171): exact integer sums of dR^2; with
        // sampling the per-sample values' means and population deviations (NMR_pfgse.cpp:1173-1290)
        const double r2 = S.voxel_res * S.voxel_res;
        if (!sampling)
        {
            double tot = 0.0;
            for (int a = 0; a < 3; a++)
            {
                msd_vec[(size_t)i * 3 + a] = r2 * (double)msd[(size_t)i * 3 + a] / N;
                dmsd_vec[(size_t)i * 3 + a] = msd_vec[(size_t)i * 3 + a] / (2.0 * delta);
                tot += msd_vec[(size_t)i * 3 + a];
            }
            dmsd[i] = tot / (6.0 * delta);
        }
        else
        {
            std::vector<double> dm(n_samples), mv[3], dv[3];
            for (int a = 0; a < 3; a++)
            {
                mv[a].resize(n_samples);
                dv[a].resize(n_samples);
            }
            for (int smp = 0; smp < n_samples; smp++)
            {
                double tot = 0.0;
                for (int a = 0; a < 3; a++)
                {
                    mv[a][smp] = r2 * (double)msds[((size_t)smp * nd + i) * 3 + a] / (double)per;
                    dv[a][smp] = mv[a][smp] / (2.0 * delta);
                    tot += mv[a][smp];
                }
                dm[smp] = tot / (6.0 * delta);
            }
            dmsd[i] = mean_of(dm);
            dmsd_std[i] = std_of(dm, dmsd[i]);
            for (int a = 0; a < 3; a++)
            {
                msd_vec[(size_t)i * 3 + a] = mean_of(mv[a]);
                msd_vec_std[(size_t)i * 3 + a] = std_of(mv[a], msd_vec[(size_t)i * 3 + a]);
                dmsd_vec[(size_t)i * 3 + a] = mean_of(dv[a]);
                dmsd_vec_std[(size_t)i * 3 + a] = std_of(dv[a], dmsd_vec[(size_t)i * 3 + a]);
            }
        }
        if (cfg.save_mode && cfg.save_pfgse)
        {
            std::ofstream r = open_out(dir + "/PFGSE_results.csv", std::ios::app);
            r << delta << "," << dsat[i] << "," << dsat_err[i] << "," << dsat_std[i] << "," << pts << "," << dmsd[i] << ","
              << dmsd_std[i];
            for (int a = 0; a < 3; a++) r << "," << dmsd_vec[(size_t)i * 3 + a] << "," << dmsd_vec_std[(size_t)i * 3 + a];
            r << "\n";
            std::ofstream e = open_out(dir + "/timesamples/echoes_" + std::to_string(i) + ".csv");
            e << "Idx,Gradient,NMR_signal(mean),NMR_signal(noise),NMR_signal(std),SAT_lhs(mean),SAT_lhs(std),SAT_rhs\n";
            for (int j = 0; j < n_g; j++)
                e << j << "," << gradient[j] << "," << M[j] << "," << raw_noise[(size_t)i * n_g + j] << ","
                  << m_std[(size_t)i * n_g + j] << "," << L[j] << "," << lhs_std[(size_t)i * n_g + j] << "," << R[j] << "\n";
            std::ofstream m = open_out(dir + "/timesamples/msd_" + std::to_string(i) + ".csv");
            m << "msdX(mean),msdX(std),msdY(mean),msdY(std),msdZ(mean),msdZ(std),DmsdX(mean),DmsdX(std),"
                 "DmsdY(mean),DmsdY(std),DmsdZ(mean),DmsdZ(std)\n";
            for (int a = 0; a < 3; a++) m << msd_vec[(size_t)i * 3 + a] << "," << msd_vec_std[(size_t)i * 3 + a] << ",";
            for (int a = 0; a < 3; a++)
                m << dmsd_vec[(size_t)i * 3 + a] << "," << dmsd_vec_std[(size_t)i * 3 + a] << (a < 2 ? "," : "");
        }
        S.log("- D(" + std::to_string(delta) + " ms) {s&t} = " + std::to_string(dsat[i]) + ", {msd} = " +
              std::to_string(dmsd[i]));
    }
    return true;
}

} // namespace rwnmr_host
