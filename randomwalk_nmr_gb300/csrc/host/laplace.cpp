// T2 inversion of CPMG decays (see laplace.h). Host code: the inversion of one decay is a few
// dense factorisations of a ~640 x 128 matrix (tens of milliseconds on one core), after a walk
// of seconds on the GPU, so it stays on the host like the reference's.
#include "laplace.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>

#include "../../../include/rwnmr_host.h"

namespace rwnmr_host
{
namespace
{

// linspace with the final point, accumulated step by step (vector_funcs.cpp:85-100); the
// accumulation, not start + i * step, fixes the bin values.
std::vector<double> linspace_acc(double a, double b, int n)
{
    std::vector<double> v;
    v.reserve(n > 0 ? n : 0);
    const double step = (b - a) / (n - 1);
    double x = a;
    for (int i = 0; i < n; i++)
    {
        v.push_back(x);
        x += step;
    }
    return v;
}

// 10^linspace (vector_funcs.cpp:102-107).
std::vector<double> logspace_acc(double a, double b, int n)
{
    std::vector<double> v = linspace_acc(a, b, n);
    for (double &x : v) x = std::pow(10.0, x);
    return v;
}

// Householder reflector H = I - tau [1; v][1; v]^T with H x = [beta; 0]: x[0] becomes beta and
// x[1..len) becomes v. tau = 0 when x[1..) is zero (no reflection).
void make_reflector(double *x, int len, double &tau)
{
    double ss = 0.0;
    for (int i = 1; i < len; i++) ss += x[i] * x[i];
    if (ss == 0.0)
    {
        tau = 0.0;
        return;
    }
    const double alpha = x[0];
    const double beta = -std::copysign(std::sqrt(alpha * alpha + ss), alpha);
    tau = (beta - alpha) / beta;
    const double inv = 1.0 / (alpha - beta);
    for (int i = 1; i < len; i++) x[i] *= inv;
    x[0] = beta;
}

// y[0..len) <- H y for the reflector stored in v[1..len) (v[0] is the implicit 1).
void apply_reflector(const double *v, int len, double tau, double *y)
{
    if (tau == 0.0) return;
    double s = y[0];
    for (int i = 1; i < len; i++) s += v[i] * y[i];
    s *= tau;
    y[0] -= s;
    for (int i = 1; i < len; i++) y[i] -= s * v[i];
}

// In-place Householder QR of a column-major rows x cols matrix (rows >= cols), applying every
// reflector to rhs as well; on return the upper triangle holds R.
void householder_qr(std::vector<double> &M, int rows, int cols, std::vector<double> &rhs)
{
    std::vector<double> tau(cols, 0.0);
    for (int j = 0; j < cols; j++)
    {
        double *cj = &M[(size_t)j * rows];
        make_reflector(cj + j, rows - j, tau[j]);
        for (int k = j + 1; k < cols; k++) apply_reflector(cj + j, rows - j, tau[j], &M[(size_t)k * rows] + j);
        apply_reflector(cj + j, rows - j, tau[j], rhs.data() + j);
    }
}

// Lawson-Hanson active-set NNLS (the algorithm of Laplace/include/NNLS.hpp:289-406): the passive
// set P grows by the free index of largest gradient w = A^T (b - A x) until none exceeds eps; each
// least-squares solve on P uses a Householder QR of P's columns kept up to date as columns join
// (appended) or leave (the last passive column takes the leaving one's slot and the columns from
// there on are re-reduced); an infeasible solve moves x to the boundary and drops the one passive
// index that reaches zero first.
class Nnls
{
  public:
    Nnls(const std::vector<double> &A, int m, int n) : A_(A), m_(m), n_(n), qr_((size_t)m * n), tau_(n)
    {
        ata_.assign((size_t)n * n, 0.0);
        for (int i = 0; i < n; i++)
            for (int j = i; j < n; j++)
            {
                double s = 0.0;
                const double *ci = &A[(size_t)i * m], *cj = &A[(size_t)j * m];
                for (int r = 0; r < m; r++) s += ci[r] * cj[r];
                ata_[(size_t)i * n + j] = ata_[(size_t)j * n + i] = s;
            }
    }

    int solve(const std::vector<double> &b, std::vector<double> &x, double eps, int max_solves)
    {
        const int n = n_, m = m_;
        std::vector<double> atb(n), w(n), y(n), tmp(m);
        for (int j = 0; j < n; j++)
        {
            double s = 0.0;
            const double *cj = &A_[(size_t)j * m];
            for (int r = 0; r < m; r++) s += cj[r] * b[r];
            atb[j] = s;
        }
        x.assign(n, 0.0);
        perm_.resize(n);
        std::iota(perm_.begin(), perm_.end(), 0);
        int np = 0, solves = 0;
        for (;;)
        {
            for (int j = 0; j < n; j++)
            {
                double s = atb[j];
                const double *row = &ata_[(size_t)j * n];
                for (int k = 0; k < n; k++) s -= row[k] * x[k];
                w[j] = s;
            }
            if (np == n) return solves;
            int zi = np;
            for (int i = np + 1; i < n; i++)
                if (w[perm_[zi]] < w[perm_[i]]) zi = i;
            if (w[perm_[zi]] - eps < 0.0) return solves;
            if (np >= m) return solves; // no more independent columns (underdetermined kernel)
            std::swap(perm_[zi], perm_[np]);
            reduce_column(np, perm_[np]);
            np++;
            for (;;)
            {
                if (solves >= max_solves) return -1;
                // least squares on P: Q^T b, then back substitution with R
                std::copy(b.begin(), b.end(), tmp.begin());
                for (int i = 0; i < np; i++) apply_reflector(&qr_[(size_t)i * m] + i, m - i, tau_[i], tmp.data() + i);
                for (int i = np - 1; i >= 0; i--)
                {
                    double s = tmp[i];
                    for (int k = i + 1; k < np; k++) s -= qr_[(size_t)k * m + i] * tmp[k];
                    tmp[i] = s / qr_[(size_t)i * m + i];
                }
                std::fill(y.begin(), y.end(), 0.0);
                for (int i = 0; i < np; i++) y[perm_[i]] = tmp[i];
                solves++;
                double alpha = std::numeric_limits<double>::max();
                int rem = -1;
                for (int i = 0; i < np; i++)
                {
                    const int j = perm_[i];
                    if (y[j] <= 0.0)
                    {
                        const double t = -x[j] / (y[j] - x[j]);
                        if (alpha > t)
                        {
                            alpha = t;
                            rem = i;
                        }
                    }
                }
                if (rem < 0)
                {
                    x = y;
                    break;
                }
                for (int i = 0; i < np; i++)
                {
                    const int j = perm_[i];
                    x[j] += alpha * (y[j] - x[j]);
                }
                std::swap(perm_[rem], perm_[np - 1]);
                np--;
                for (int i = rem; i < np; i++) reduce_column(i, perm_[i]);
            }
        }
    }

  private:
    // QR column k <- A column col with reflectors 0..k-1 applied, then reflector k formed.
    void reduce_column(int k, int col)
    {
        double *c = &qr_[(size_t)k * m_];
        std::memcpy(c, &A_[(size_t)col * m_], sizeof(double) * m_);
        for (int i = 0; i < k; i++) apply_reflector(&qr_[(size_t)i * m_] + i, m_ - i, tau_[i], c + i);
        make_reflector(c + k, m_ - k, tau_[k]);
    }

    const std::vector<double> &A_;
    int m_, n_;
    std::vector<double> ata_, qr_, tau_;
    std::vector<int> perm_;
};

} // namespace

std::vector<double> t2_bins(const T2InversionConfig &cfg)
{
    if (cfg.use_logspace) return logspace_acc(std::log10(cfg.min_t2), std::log10(cfg.max_t2), cfg.num_t2_bins);
    return linspace_acc(cfg.min_t2, cfg.max_t2, cfg.num_t2_bins);
}

bool prune_decay(const std::vector<double> &times, const std::vector<double> &amps, int P,
                 std::vector<double> &out_times, std::vector<double> &out_amps)
{
    // get_nmr_pruning_slices (nmrinv_core.cpp:145-179): a log grid of P points from the first to
    // the last time; points before the first grid point that lies beyond the echo times stay as
    // they are, later grid intervals average the echoes whose log-time falls inside them.
    const int n = (int)times.size();
    if (P < 3 || n <= P || (int)amps.size() != n) return false;
    std::vector<double> lg(n), nl(P);
    for (int i = 0; i < n; i++) lg[i] = std::log10(times[i]);
    const double d = (lg[n - 1] - lg[0]) / (P - 1);
    for (int i = 0; i < P; i++) nl[i] = lg[0] + d * i;
    int ps = 1;
    while (ps < P - 1 && std::pow(10.0, nl[ps]) - times[ps] <= 0.0) ps++;
    ps -= 1;
    int ib = 0;
    while (ib < n && lg[ib] - nl[ps] <= 0.0) ib++;
    if (ib >= n) return false;
    struct Slice
    {
        int p, b0, b1;
    };
    std::vector<Slice> sl;
    for (int pi = ps; pi < P - 1; pi++)
    {
        const int b0 = ib;
        const double lo = nl[pi], hi = nl[pi + 1];
        while (ib < n && lg[ib] >= lo && lg[ib] < hi) ib++;
        sl.push_back({pi, b0, ib});
    }
    // prune_nmr_data_from_slices (nmrinv_core.cpp:182-239): geometric means of the times,
    // arithmetic means of the amplitudes, the last point kept.
    out_times.assign(P, 0.0);
    out_amps.assign(P, 0.0);
    std::copy(times.begin(), times.begin() + ps, out_times.begin());
    std::copy(amps.begin(), amps.begin() + ps, out_amps.begin());
    for (const Slice &s : sl)
    {
        double lt = 0.0, sa = 0.0;
        for (int i = s.b0; i < s.b1; i++)
        {
            lt += std::log10(times[i]);
            sa += amps[i];
        }
        const double cnt = (double)(s.b1 - s.b0); // an empty slice gives NaN, as in the reference
        out_times[s.p] = std::pow(10.0, lt / cnt);
        out_amps[s.p] = sa / cnt;
    }
    out_times[P - 1] = times[n - 1];
    out_amps[P - 1] = amps[n - 1];
    return true;
}

int lcurve(const std::vector<double> &A, int m, int n, const std::vector<double> &b, double min_lambda,
           double max_lambda, int num_lambdas, std::vector<double> &lambdas, std::vector<double> &curvature,
           std::vector<double> &singular_values)
{
    // Thin SVD A = U S V^T through a square k x k factor C with the same singular values and a
    // vector c with U^T b = U_C^T c: m >= n: A = Q R, C = R, c = (Q^T b)[0:n]; m < n: A^T = Q R,
    // C = R^T, c = b. Then one-sided Jacobi (Hestenes) rotations orthogonalise the columns of C;
    // the column norms are the singular values and the normalised columns U_C.
    const int k = std::min(m, n);
    std::vector<double> C((size_t)k * k, 0.0), c(k);
    if (m >= n)
    {
        std::vector<double> Q(A), rhs(b);
        householder_qr(Q, m, n, rhs);
        for (int j = 0; j < n; j++)
            for (int i = 0; i <= j; i++) C[(size_t)j * k + i] = Q[(size_t)j * m + i];
        std::copy(rhs.begin(), rhs.begin() + n, c.begin());
    }
    else
    {
        std::vector<double> At((size_t)n * m), dummy(n, 0.0);
        for (int i = 0; i < m; i++)
            for (int j = 0; j < n; j++) At[(size_t)i * n + j] = A[(size_t)j * m + i];
        householder_qr(At, n, m, dummy);
        for (int j = 0; j < m; j++)
            for (int i = 0; i <= j; i++) C[(size_t)i * k + j] = At[(size_t)j * n + i];
        std::copy(b.begin(), b.begin() + m, c.begin());
    }
    const double tol = 1e-15;
    for (int sweep = 0; sweep < 100; sweep++)
    {
        bool rotated = false;
        for (int p = 0; p < k - 1; p++)
        {
            double *cp = &C[(size_t)p * k];
            for (int q = p + 1; q < k; q++)
            {
                double *cq = &C[(size_t)q * k];
                double al = 0.0, be = 0.0, ga = 0.0;
                for (int i = 0; i < k; i++)
                {
                    al += cp[i] * cp[i];
                    be += cq[i] * cq[i];
                    ga += cp[i] * cq[i];
                }
                if (ga == 0.0 || std::fabs(ga) <= tol * std::sqrt(al * be)) continue;
                const double zeta = (be - al) / (2.0 * ga);
                const double t = std::copysign(1.0, zeta) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                const double cs = 1.0 / std::sqrt(1.0 + t * t), sn = cs * t;
                for (int i = 0; i < k; i++)
                {
                    const double a = cp[i], bb = cq[i];
                    cp[i] = cs * a - sn * bb;
                    cq[i] = sn * a + cs * bb;
                }
                rotated = true;
            }
        }
        if (!rotated) break;
    }
    std::vector<double> sv(k), uatb(k);
    for (int j = 0; j < k; j++)
    {
        const double *cj = &C[(size_t)j * k];
        double ss = 0.0, dot = 0.0;
        for (int i = 0; i < k; i++)
        {
            ss += cj[i] * cj[i];
            dot += cj[i] * c[i];
        }
        sv[j] = std::sqrt(ss);
        uatb[j] = sv[j] > 0.0 ? dot / sv[j] : 0.0;
    }
    std::vector<int> order(k);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b2) { return sv[a] > sv[b2]; });
    // singular values up to the first zero (TikhonovSolver.cpp:22-30)
    singular_values.clear();
    std::vector<double> u;
    for (int j : order)
    {
        if (sv[j] == 0.0) break;
        singular_values.push_back(sv[j]);
        u.push_back(uatb[j]);
    }
    const size_t ns = singular_values.size();
    std::vector<double> d(ns), d2(ns);
    for (size_t j = 0; j < ns; j++)
    {
        d[j] = u[j] / singular_values[j];
        d2[j] = d[j] * d[j];
    }
    // L-curve values per lambda (TikhonovSolver.cpp:82-116): eta = ||x||^2, rho = ||r||^2 of the
    // Tikhonov solution from the filter factors s^2 / (s^2 + lambda^2), and the curvature of
    // (log rho, log eta) in Hansen's closed form.
    lambdas = logspace_acc(min_lambda, max_lambda, num_lambdas);
    curvature.assign(num_lambdas, 0.0);
    for (int il = 0; il < num_lambdas; il++)
    {
        const double lam = lambdas[il], sql = lam * lam;
        double eta = 0.0, rho = 0.0, deta = 0.0;
        for (size_t j = 0; j < ns; j++)
        {
            const double s2 = singular_values[j] * singular_values[j];
            const double ft = s2 / (s2 + sql), om = 1.0 - ft;
            const double xe = ft * d[j], re = om * u[j];
            eta += xe * xe;
            rho += re * re;
            deta += om * ft * ft * d2[j];
        }
        deta *= -4.0 / lam;
        const double mult = -2.0 * eta * rho / deta;
        const double num = sql * deta * rho + 2.0 * lam * eta * rho + sql * sql * eta * deta;
        const double den = std::pow(sql * eta * eta + rho * rho, 1.5);
        curvature[il] = mult * num / den;
    }
    if (num_lambdas <= 0) return -1;
    return (int)(std::max_element(curvature.begin(), curvature.end()) - curvature.begin());
}

int nnls(const std::vector<double> &A, int m, int n, const std::vector<double> &b, std::vector<double> &x, double eps,
         int max_solves)
{
    // The reference iterates without a limit; 50 (n + 1) least-squares solves is far above what
    // the active-set method needs on these kernels and turns a cycling case into an error.
    if (max_solves <= 0) max_solves = 50 * (n + 1);
    Nnls s(A, m, n);
    return s.solve(b, x, eps, max_solves);
}

bool invert_t2(const std::vector<double> &times, const std::vector<double> &amps, const T2InversionConfig &cfg,
               T2Inversion &out, std::string &err)
{
    if (times.size() != amps.size() || times.size() < 3)
    {
        err = "T2 inversion needs a decay of at least 3 points with matching times";
        return false;
    }
    if (cfg.num_t2_bins < 1 || cfg.num_lambdas < 1 || !(cfg.max_t2 > cfg.min_t2) ||
        (cfg.use_logspace && !(cfg.min_t2 > 0.0)))
    {
        err = "T2 inversion: bad bin or lambda settings (NUM_T2_BINS, NUM_LAMBDAS >= 1, 0 < MIN_T2 < MAX_T2)";
        return false;
    }
    // applyLaplace drops the t = 0 point (NMR_cpmg.cpp:404-408)
    std::vector<double> t(times.begin() + 1, times.end()), a(amps.begin() + 1, amps.end());
    for (double v : t)
        if (!(v > 0.0))
        {
            err = "T2 inversion: echo times must be positive";
            return false;
        }
    out.noise.clear();
    if (cfg.noise_amp != 0.0)
    {
        // generate_noise / add_noise_to_decays (nmrinv_core.cpp:76-97, 303-315): N(0, NOISE_AMP)
        // per echo; the reference seeds from std::random_device, here the seed is explicit.
        std::mt19937_64 gen(cfg.noise_seed);
        std::normal_distribution<double> nd(0.0, cfg.noise_amp);
        out.noise.resize(a.size());
        for (size_t i = 0; i < a.size(); i++)
        {
            out.noise[i] = nd(gen);
            a[i] += out.noise[i];
        }
    }
    out.bins = t2_bins(cfg);
    const int nb = (int)out.bins.size();
    if (!(cfg.prune_num > 0 && prune_decay(t, a, cfg.prune_num, out.used_times, out.used_amps)))
    {
        out.used_times = t;
        out.used_amps = a;
    }
    const int m = (int)out.used_times.size();
    std::vector<double> K((size_t)m * nb);
    for (int j = 0; j < nb; j++)
        for (int i = 0; i < m; i++) K[(size_t)j * m + i] = std::exp(-out.used_times[i] / out.bins[j]);
    out.lambda_index = lcurve(K, m, nb, out.used_amps, cfg.min_lambda, cfg.max_lambda, cfg.num_lambdas, out.lambdas,
                              out.curvature, out.singular_values);
    out.lambda = out.lambdas[out.lambda_index];
    // [K; lambda I] x = [b; 0] (create_nmr_inversion_matrix / set_inversion_lambda, nmrinv_core.cpp:99-126, 317-336)
    std::vector<double> Ka, ba(out.used_amps);
    int ma = m;
    if (out.lambda != 0.0)
    {
        ma = m + nb;
        Ka.assign((size_t)ma * nb, 0.0);
        for (int j = 0; j < nb; j++)
        {
            std::copy(&K[(size_t)j * m], &K[(size_t)j * m] + m, &Ka[(size_t)j * ma]);
            Ka[(size_t)j * ma + m + j] = out.lambda;
        }
        ba.resize(ma, 0.0);
    }
    else
    {
        Ka.swap(K);
    }
    out.nnls_solves = nnls(Ka, ma, nb, ba, out.amps);
    if (out.nnls_solves < 0)
    {
        err = "T2 inversion: NNLS did not converge";
        return false;
    }
    return true;
}

} // namespace rwnmr_host

using namespace rwnmr_host;

extern "C" int32_t rwnmr_t2_invert(const double *times, const double *amps, int32_t n, const rwnmr_t2_config *c,
                                   double *t2_bins_out, double *t2_amps_out, double *lambda, double *noise, char *err,
                                   int32_t errlen)
{
    auto fail = [&](const std::string &m) {
        if (err && errlen > 0)
        {
            std::strncpy(err, m.c_str(), (size_t)errlen - 1);
            err[errlen - 1] = 0;
        }
        return -1;
    };
    if (!times || !amps || !c || n < 3) return fail("rwnmr_t2_invert: null argument or fewer than 3 points");
    T2InversionConfig cfg;
    cfg.min_t2 = c->min_t2;
    cfg.max_t2 = c->max_t2;
    cfg.use_logspace = c->use_logspace != 0;
    cfg.num_t2_bins = c->num_t2_bins;
    cfg.min_lambda = c->min_lambda;
    cfg.max_lambda = c->max_lambda;
    cfg.num_lambdas = c->num_lambdas;
    cfg.prune_num = c->prune_num;
    cfg.noise_amp = c->noise_amp;
    cfg.noise_seed = c->noise_seed;
    T2Inversion r;
    std::string e;
    if (!invert_t2(std::vector<double>(times, times + n), std::vector<double>(amps, amps + n), cfg, r, e))
        return fail(e);
    if (t2_bins_out) std::copy(r.bins.begin(), r.bins.end(), t2_bins_out);
    if (t2_amps_out) std::copy(r.amps.begin(), r.amps.end(), t2_amps_out);
    if (lambda) *lambda = r.lambda;
    if (noise)
    {
        noise[0] = 0.0;
        for (int32_t i = 1; i < n; i++) noise[i] = r.noise.empty() ? 0.0 : r.noise[i - 1];
    }
    return (int32_t)r.bins.size();
}

extern "C" int32_t rwnmr_t2_prune(const double *times, const double *amps, int32_t n, int32_t prune_num,
                                  double *out_times, double *out_amps)
{
    if (!times || !amps || n < 1) return -1;
    std::vector<double> t, a;
    if (!prune_decay(std::vector<double>(times, times + n), std::vector<double>(amps, amps + n), prune_num, t, a))
        return 0;
    if (out_times) std::copy(t.begin(), t.end(), out_times);
    if (out_amps) std::copy(a.begin(), a.end(), out_amps);
    return (int32_t)t.size();
}

extern "C" int32_t rwnmr_t2_lcurve(const double *a, int32_t m, int32_t n, const double *b, double min_lambda,
                                   double max_lambda, int32_t num_lambdas, double *curvature, double *singular_values,
                                   int32_t *n_singular)
{
    if (!a || !b || m < 1 || n < 1 || num_lambdas < 1) return -1;
    std::vector<double> lam, curv, sv;
    const int best = lcurve(std::vector<double>(a, a + (size_t)m * n), m, n, std::vector<double>(b, b + m), min_lambda,
                            max_lambda, num_lambdas, lam, curv, sv);
    if (curvature) std::copy(curv.begin(), curv.end(), curvature);
    if (singular_values) std::copy(sv.begin(), sv.end(), singular_values);
    if (n_singular) *n_singular = (int32_t)sv.size();
    return best;
}

extern "C" int32_t rwnmr_nnls(const double *a, int32_t m, int32_t n, const double *b, double *x, int32_t max_solves)
{
    if (!a || !b || !x || m < 1 || n < 1) return -1;
    std::vector<double> xv;
    const int r = nnls(std::vector<double>(a, a + (size_t)m * n), m, n, std::vector<double>(b, b + m), xv, 1e-10,
                       max_solves);
    if (r >= 0) std::copy(xv.begin(), xv.end(), x);
    return r;
}
