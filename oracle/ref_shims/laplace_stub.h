// Force-included when compiling the reference's CPU sources as a test oracle.
// The reference's Laplace inversion needs Eigen, which this image lacks. Defining the
// header guards of its two Laplace headers first turns their #include into no-ops, and
// the no-op NMRInverter below satisfies NMR_cpmg::applyLaplace(). The oracle never calls
// applyLaplace(): the walk path under test ends at the echo train.
#ifndef RWNMR_ORACLE_LAPLACE_STUB_H
#define RWNMR_ORACLE_LAPLACE_STUB_H

#define NMRINV_CORE_H
#define TIKHONOV_H

#ifdef __cplusplus
#include <vector>
#include <string>

struct NMRInverterConfig
{
    NMRInverterConfig(double = 0.1, double = 1e4, bool = true, int = 256, double = -4, double = 2, int = 512,
                      int = 512, double = 0.0) {}
};

class NMRInverter
{
public:
    std::vector<double> used_t2_bins;
    std::vector<double> used_t2_amps;
    void set_config(NMRInverterConfig, std::vector<double> &) {}
    void find_best_lambda(int, double *) {}
    void invert(int, double *) {}
    std::vector<double> get_raw_noise() { return std::vector<double>(); }
    double get_inversion_lambda() { return 0.0; }
};
#endif

#endif
