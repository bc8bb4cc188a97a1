// Command-line application: the reference's RWNMR driver (src/backend/main.cpp, App/rwnmrApp.cpp,
// Utils/ArgsParser.cpp) over the GPU engine.
//
//   rwnmr_gb300 [-rwconfig FILE] [-uctconfig FILE] cpmg [-config FILE] pfgse [-config FILE]
//               multitau [-config MT CPMG | -mtconfig MT | -cpmgconfig CPMG] ...
//
// Commands run in the order given, on one simulation (image + walkers), exactly as the reference's
// rwnmrApp::exec does. Options beyond the reference's:
//   --config-root DIR      where default/<kind>.config live (reference: ./config/)
//   --synthetic NX,NY,NZ,RMIN,RMAX,POROSITY,PHASES,SEED   sphere-pack image instead of the uct slices
//   --labels FILE --shape NZ,NY,NX                         raw uint8 label volume instead of the slices
//   --device N             CUDA device
//   --quiet
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "rwnmr_host.h"
#include "sequences.h"

namespace rwnmr_host
{
namespace
{
std::vector<double> csv_numbers(const std::string &s)
{
    std::vector<double> v;
    std::stringstream ss(s);
    std::string tok;
    while (std::getline(ss, tok, ','))
        if (!tok.empty()) v.push_back(std::stod(tok));
    return v;
}

int usage()
{
    std::cerr << "usage: rwnmr_gb300 [-rwconfig FILE] [-uctconfig FILE] [cpmg [-config FILE]] [pfgse [-config FILE]]\n"
                 "       [multitau [-config MTFILE CPMGFILE | -mtconfig MTFILE | -cpmgconfig CPMGFILE]]\n"
                 "       [--config-root DIR] [--synthetic NX,NY,NZ,RMIN,RMAX,POROSITY,PHASES,SEED]\n"
                 "       [--labels FILE --shape NZ,NY,NX] [--device N] [--quiet]\n";
    return 2;
}
} // namespace

int cli_main(int argc, const char *const *argv)
{
    std::string rw_path = "default", uct_path = "default", root = "./config/", labels_path;
    struct Command
    {
        std::string name, path = "default", path2 = "default"; // path2: multitau's cpmg config
    };
    std::vector<Command> commands;
    std::vector<double> synth, shape;
    int device = 0;
    bool quiet = false;
    for (int i = 1; i < argc; i++)
    {
        std::string a = argv[i];
        auto next = [&](std::string &out) {
            if (i + 1 < argc) out = argv[++i];
        };
        if (a == "-rwconfig") next(rw_path);
        else if (a == "-uctconfig") next(uct_path);
        else if (a == "cpmg" || a == "pfgse" || a == "ga")
        {
            Command c{a};
            if (i + 2 < argc && std::string(argv[i + 1]) == "-config")
            {
                c.path = argv[i + 2];
                i += 2;
            }
            commands.push_back(c);
        }
        else if (a == "multitau")
        {
            // multitau [-config MT CPMG | -mtconfig MT | -cpmgconfig CPMG] (Utils/ArgsParser.cpp:104-145)
            Command c{a};
            const std::string flag = i + 1 < argc ? argv[i + 1] : "";
            if (flag == "-config" && i + 3 < argc)
            {
                c.path = argv[i + 2];
                c.path2 = argv[i + 3];
                i += 3;
            }
            else if (flag == "-mtconfig" && i + 2 < argc)
            {
                c.path = argv[i + 2];
                i += 2;
            }
            else if (flag == "-cpmgconfig" && i + 2 < argc)
            {
                c.path2 = argv[i + 2];
                i += 2;
            }
            commands.push_back(c);
        }
        else if (a == "--config-root")
        {
            next(root);
            if (!root.empty() && root.back() != '/') root += "/";
        }
        else if (a == "--synthetic")
        {
            std::string s;
            next(s);
            synth = csv_numbers(s);
        }
        else if (a == "--labels") next(labels_path);
        else if (a == "--shape")
        {
            std::string s;
            next(s);
            shape = csv_numbers(s);
        }
        else if (a == "--device")
        {
            std::string s;
            next(s);
            device = std::stoi(s);
        }
        else if (a == "--quiet") quiet = true;
        else if (a == "-h" || a == "--help") return usage();
    }
    std::string err;
    RwnmrConfig rw;
    UctConfig uct;
    if (!load_rwnmr(root, rw_path == "default" ? root + "default/rwnmr.config" : rw_path, rw, err) ||
        !load_uct(root, uct_path == "default" ? root + "default/uct.config" : uct_path, uct, err))
    {
        std::cerr << err << std::endl;
        return 1;
    }
    Simulation sim;
    sim.quiet = quiet;
    if (!sim.init(rw, uct, "", device, err))
    {
        std::cerr << err << std::endl;
        return 1;
    }
    Image img;
    if (synth.size() == 8)
    {
        img.nx = (int)synth[0];
        img.ny = (int)synth[1];
        img.nz = (int)synth[2];
        img.n_phases = (int)synth[6];
        img.labels.assign((size_t)img.nx * img.ny * img.nz, 0);
        double por = 0.0;
        if (rwnmr_synth_spheres(img.labels.data(), img.nx, img.ny, img.nz, synth[3], synth[4], synth[5], img.n_phases,
                                (uint64_t)synth[7], &por) < 0)
        {
            std::cerr << "invalid --synthetic parameters" << std::endl;
            return 1;
        }
        img.source = "synthetic sphere pack";
    }
    else if (!labels_path.empty())
    {
        if (shape.size() != 3) return usage();
        img.nz = (int)shape[0];
        img.ny = (int)shape[1];
        img.nx = (int)shape[2];
        img.labels.assign((size_t)img.nx * img.ny * img.nz, 0);
        std::ifstream f(labels_path, std::ios::binary);
        if (!f.read((char *)img.labels.data(), (std::streamsize)img.labels.size()))
        {
            std::cerr << "could not read " << img.labels.size() << " bytes from " << labels_path << std::endl;
            return 1;
        }
        uint8_t mx = 0;
        for (uint8_t v : img.labels) mx = std::max(mx, v);
        img.n_phases = std::max<int>(1, mx);
        img.source = labels_path;
    }
    else if (!load_uct_image(uct, img, err))
    {
        std::cerr << err << std::endl;
        return 1;
    }
    if (!sim.set_image(std::move(img), err) || !sim.set_walkers(err))
    {
        std::cerr << err << std::endl;
        return 1;
    }
    sim.save_info(); // NMR_Simulation::save (rwnmrApp.cpp:68): SimInfo + the SAVE_IMG_INFO / SAVE_BINIMG / SAVE_WALKERS files
    for (auto &cmd : commands)
    {
        if (cmd.name == "cpmg")
        {
            CpmgConfig c;
            if (!load_cpmg(root, cmd.path == "default" ? root + "default/cpmg.config" : cmd.path, c, err))
            {
                std::cerr << err << std::endl;
                return 1;
            }
            CpmgSequence seq(sim, c);
            if (!seq.run(err))
            {
                std::cerr << err << std::endl;
                return 1;
            }
        }
        else if (cmd.name == "pfgse")
        {
            PfgseConfig c;
            if (!load_pfgse(root, cmd.path == "default" ? root + "default/pfgse.config" : cmd.path, c, err))
            {
                std::cerr << err << std::endl;
                return 1;
            }
            PfgseSequence seq(sim, c);
            if (!seq.run(err))
            {
                std::cerr << err << std::endl;
                return 1;
            }
        }
        else if (cmd.name == "ga")
            std::cout << "-- GA is under construction." << std::endl; // as the reference (App/rwnmrApp.cpp:204-207)
        else
        {
            // rwnmrApp::MultiTau (App/rwnmrApp.cpp:129-150)
            MultitauConfig mc;
            CpmgConfig cc;
            if (!load_multitau(root, cmd.path, mc, err) ||
                !load_cpmg(root, cmd.path2 == "default" ? root + "default/cpmg.config" : cmd.path2, cc, err))
            {
                std::cerr << err << std::endl;
                return 1;
            }
            MultitauSequence seq(sim, mc, cc);
            if (!seq.run(err))
            {
                std::cerr << err << std::endl;
                return 1;
            }
        }
    }
    return 0;
}

} // namespace rwnmr_host

extern "C" {

int rwnmr_cli_main(int argc, const char *const *argv) { return rwnmr_host::cli_main(argc, argv); }

int rwnmr_config_json(const char *kind, const char *config_root, const char *user_path, char *out, int cap)
{
    using namespace rwnmr_host;
    std::string root = config_root ? config_root : "./config/";
    if (!root.empty() && root.back() != '/') root += "/";
    std::string user = user_path ? user_path : "default";
    std::string err, js;
    std::string k = kind ? kind : "";
    bool ok = false;
    if (k == "rwnmr")
    {
        RwnmrConfig c;
        ok = load_rwnmr(root, user, c, err);
        js = to_json(c);
    }
    else if (k == "uct")
    {
        UctConfig c;
        ok = load_uct(root, user, c, err);
        js = to_json(c);
    }
    else if (k == "cpmg")
    {
        CpmgConfig c;
        ok = load_cpmg(root, user, c, err);
        js = to_json(c);
    }
    else if (k == "pfgse")
    {
        PfgseConfig c;
        ok = load_pfgse(root, user, c, err);
        js = to_json(c);
    }
    else if (k == "multitau")
    {
        MultitauConfig c;
        ok = load_multitau(root, user, c, err);
        js = to_json(c);
    }
    else
        err = "unknown config kind";
    const std::string &res = ok ? js : err;
    if (out && cap > 0)
    {
        std::strncpy(out, res.c_str(), (size_t)cap - 1);
        out[cap - 1] = 0;
    }
    return ok ? (int)res.size() : -1;
}

} // extern "C"
