// T2 distribution from a CPMG decay: Tikhonov-regularised non-negative inverse Laplace transform,
// the reference's NMRInverter path (Laplace/src/nmrinv_core.cpp, TikhonovSolver.cpp, NNLS.hpp)
// as used by NMR_cpmg::applyLaplace (NMR_Simulation/NMR_cpmg.cpp:387-453). Self-contained dense
// linear algebra (the reference uses Eigen): a QR-preconditioned one-sided Jacobi SVD for the
// L-curve and a Lawson-Hanson active-set NNLS on incrementally updated Householder QR.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace rwnmr_host
{

struct T2InversionConfig
{
    double min_t2 = 0.1, max_t2 = 10000.0; // T2 bin range (ms)
    bool use_logspace = true;
    int num_t2_bins = 128;
    double min_lambda = -4.0, max_lambda = 2.0; // log10 range of the Tikhonov parameter
    int num_lambdas = 512;
    int prune_num = 512;   // 0: no prune-averaging
    double noise_amp = 0.0; // standard deviation of added Gaussian noise (0: none)
    uint64_t noise_seed = 0;
};

struct T2Inversion
{
    std::vector<double> bins, amps;             // the T2 distribution
    std::vector<double> used_times, used_amps;  // decay after noise and pruning
    std::vector<double> noise;                  // noise added to each decay point (empty: none)
    std::vector<double> lambdas, curvature, singular_values;
    double lambda = 0.0;
    int lambda_index = -1;
    int nnls_solves = 0;
};

// Log-spaced T2 bins (get_t2_bins, nmrinv_core.cpp:129-142).
std::vector<double> t2_bins(const T2InversionConfig &cfg);

// Prune-averaging of a decay (nmrinv_core.cpp:145-239). Returns false (nothing written) when the
// decay has no more points than num_pruning, or the log grid leaves no slice to average.
bool prune_decay(const std::vector<double> &times, const std::vector<double> &amps, int num_pruning,
                 std::vector<double> &out_times, std::vector<double> &out_amps);

// L-curve over lambdas = logspace(min_lambda, max_lambda, n) for kernel A (m x n, column-major) and
// data b; returns the index of the first curvature maximum (TikhonovSolver.cpp:14-116).
int lcurve(const std::vector<double> &A, int m, int n, const std::vector<double> &b, double min_lambda,
           double max_lambda, int num_lambdas, std::vector<double> &lambdas, std::vector<double> &curvature,
           std::vector<double> &singular_values);

// Non-negative least squares min ||A x - b||, x >= 0 (A m x n column-major). Returns the number of
// least-squares solves, or -1 if max_solves is reached.
int nnls(const std::vector<double> &A, int m, int n, const std::vector<double> &b, std::vector<double> &x,
         double eps = 1e-10, int max_solves = 0);

// The whole inversion of a decay whose first point is t = 0 (dropped, as applyLaplace does).
bool invert_t2(const std::vector<double> &times, const std::vector<double> &amps, const T2InversionConfig &cfg,
               T2Inversion &out, std::string &err);

} // namespace rwnmr_host
