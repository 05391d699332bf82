// Host check of the integer-pipe exponential and logarithm (cantera_gb300/csrc/fastexp.h)
// against the C library: prints the largest errors over sweeps.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../cantera_gb300/csrc/fastexp.h"

using namespace gbchem;

static double ulp_err(double a, double b) {
    if (a == b) return 0.0;
    double u = std::nextafter(std::fabs(b), INFINITY) - std::fabs(b);
    return std::fabs(a - b) / u;
}

int main(int argc, char** argv) {
    long n = argc > 1 ? atol(argv[1]) : 2000000;
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> wide(-699.0, 699.0), narrow(-3.0, 3.0), tiny(-1e-6, 1e-6);
    double worst = 0.0, worstx = 0.0;
    double worstpm = 0.0;
    for (long i = 0; i < n; i++) {
        double x = (i % 3 == 0) ? wide(rng) : (i % 3 == 1) ? narrow(rng) : tiny(rng);
        double e = ulp_err(gbx_exp(x, gbx_t63), std::exp(x));
        if (e > worst) { worst = e; worstx = x; }
        XVal a, b;
        gbx_exp_pm(x, a, b, gbx_t63);
        double em = gbx_todouble(b);
        double e2 = ulp_err(em, std::exp(-x));
        if (e2 > worstpm) worstpm = e2;
    }
    // products of exponentials (equilibrium constants) against exp of the sum
    double worstprod = 0.0;
    for (long i = 0; i < n / 10; i++) {
        double g1 = wide(rng) / 4, g2 = wide(rng) / 4, g3 = wide(rng) / 4;
        XVal a1, b1, a2, b2, a3, b3;
        gbx_exp_pm(g1, a1, b1, gbx_t63);
        gbx_exp_pm(g2, a2, b2, gbx_t63);
        gbx_exp_pm(g3, a3, b3, gbx_t63);
        XVal v = gbx_mul(gbx_mul(a1, a2), b3);
        double got = gbx_todouble(v);
        long double want = expl((long double)g1 + (long double)g2 - (long double)g3);
        double rel = std::fabs((double)((got - want) / want));
        if (rel > worstprod) worstprod = rel;
    }
    // logarithm: ulp error where |ln x| > 1/256, absolute error near x = 1 (against long double)
    uint64_t tab[kGbxTableWords];
    gbx_host_table(tab);
    std::uniform_real_distribution<double> lexp(-690.0, 709.0), temp(200.0, 4000.0), near1(-0.004, 0.004);
    double worstlog = 0.0, worstlog1 = 0.0;
    for (long i = 0; i < n; i++) {
        const int mode = (int)(i % 3);
        const double x = mode == 0 ? std::exp(lexp(rng)) : (mode == 1 ? temp(rng) : 1.0 + near1(rng));
        const double a = gbx_log(x, tab), b = std::log(x);
        if (std::fabs(b) > 1.0 / 256) {
            const double e = ulp_err(a, b);
            if (e > worstlog) worstlog = e;
        } else {
            const double ab = std::fabs((double)((long double)a - logl((long double)x)));
            if (ab > worstlog1) worstlog1 = ab;
        }
    }
    std::printf("max_ulp %.3f at %.17g max_ulp_neg %.3f max_rel_product %.3e max_ulp_log %.3f max_abs_log_near1 %.3e\n",
                worst, worstx, worstpm, worstprod, worstlog, worstlog1);
    return 0;
}
