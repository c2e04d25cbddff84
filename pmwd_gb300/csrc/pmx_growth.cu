// Growth-function ODEs of the background cosmology, integrated on the host.
//
// pmwd integrates its growth ODEs (boltzmann.py:163-229, right-hand side
// boltzmann.py:196-203) with JAX's odeint, a Dormand-Prince 5(4) method with
// adaptive steps.  This is the same method in plain C++: a handful of
// doubles per parameter set, so a native loop takes microseconds where an
// interpreted right-hand side costs tens of milliseconds.  Host only: no
// device memory, callable without a GPU.
//
// State per parameter set (Omega_m, Omega_k, w_0, w_a), as functions of
// ln a:  y = (G1, dG1/dlna, G2, dG2/dlna), with G_m = D_m / a^m.

#include <cmath>
#include <cstdint>
#include <utility>
#include <vector>

#include "pmx_internal.cuh"

namespace pmx {
namespace {

struct Bg {
    double Om, Ok, w0, wa;
};

// dy/dlna (boltzmann.py:196-203)
void rhs(double lna, const double y[4], const Bg &c, double dy[4]) {
    const double a = std::exp(lna);
    const double Ode = 1.0 - (c.Om + c.Ok);
    const double p = -3.0 * (1.0 + c.w0 + c.wa);
    const double q = -3.0 * c.wa;
    const double de = std::pow(a, p) * std::exp(q * (1.0 - a));
    const double a3 = a * a * a, a2 = a * a;
    const double E2 = c.Om / a3 + c.Ok / a2 + Ode * de;
    const double dlnH = 0.5 * (-3.0 * c.Om / a3 - 2.0 * c.Ok / a2 + Ode * de * (p - q * a)) / E2;
    const double Of = 1.5 * c.Om / (a3 * E2);
    dy[0] = y[1];
    dy[1] = -(3.0 + dlnH - Of) * y[0] - (4.0 + dlnH) * y[1];
    dy[2] = y[3];
    dy[3] = Of * y[0] * y[0] - (8.0 + 2.0 * dlnH - Of) * y[2] - (6.0 + dlnH) * y[3];
}

// Dormand-Prince 5(4) tableau (Dormand & Prince 1980, the coefficients every
// RK45 implementation publishes); b5 is the propagated 5th-order solution.
constexpr double C2 = 1.0 / 5, C3 = 3.0 / 10, C4 = 4.0 / 5, C5 = 8.0 / 9;
constexpr double A21 = 1.0 / 5;
constexpr double A31 = 3.0 / 40, A32 = 9.0 / 40;
constexpr double A41 = 44.0 / 45, A42 = -56.0 / 15, A43 = 32.0 / 9;
constexpr double A51 = 19372.0 / 6561, A52 = -25360.0 / 2187, A53 = 64448.0 / 6561,
                 A54 = -212.0 / 729;
constexpr double A61 = 9017.0 / 3168, A62 = -355.0 / 33, A63 = 46732.0 / 5247, A64 = 49.0 / 176,
                 A65 = -5103.0 / 18656;
constexpr double B1 = 35.0 / 384, B3 = 500.0 / 1113, B4 = 125.0 / 192, B5 = -2187.0 / 6784,
                 B6 = 11.0 / 84;
// error coefficients b5 - b4
constexpr double E1 = 35.0 / 384 - 5179.0 / 57600, E3 = 500.0 / 1113 - 7571.0 / 16695,
                 E4 = 125.0 / 192 - 393.0 / 640, E5 = -2187.0 / 6784 + 92097.0 / 339200,
                 E6 = 11.0 / 84 - 187.0 / 2100, E7 = -1.0 / 40;

// All parameter sets at once, on one shared step sequence (so that the
// central differences of neighbouring sets see the same discretisation):
// y at every output point t[0..n) (t increasing), written (n, P, 4), with
// y(t[0]) = (1, 0, 3/7, 0) for every set.  Steps are adaptive (RMS error
// norm over all components) and end exactly on each output point.
struct Work {
    std::vector<double> y, yt, y5, k1, k2, k3, k4, k5, k6, k7;
    explicit Work(size_t m)
        : y(m), yt(m), y5(m), k1(m), k2(m), k3(m), k4(m), k5(m), k6(m), k7(m) {}
};

void rhs_all(double lna, const double *y, const std::vector<Bg> &c, double *dy) {
    for (size_t p = 0; p < c.size(); ++p) rhs(lna, y + 4 * p, c[p], dy + 4 * p);
}

int integrate(const std::vector<Bg> &c, const double *t, int64_t n, double rtol, double atol,
              double *yout, double *dyout) {
    const size_t P = c.size(), m = 4 * P;
    Work w(m);
    double *y = w.y.data(), *yt = w.yt.data(), *y5 = w.y5.data(), *k1 = w.k1.data(),
           *k2 = w.k2.data(), *k3 = w.k3.data(), *k4 = w.k4.data(), *k5 = w.k5.data(),
           *k6 = w.k6.data(), *k7 = w.k7.data();
    for (size_t p = 0; p < P; ++p) {
        y[4 * p] = 1.0;
        y[4 * p + 1] = 0.0;
        y[4 * p + 2] = 3.0 / 7.0;
        y[4 * p + 3] = 0.0;
    }
    double x = t[0];
    rhs_all(x, y, c, k1);
    for (size_t i = 0; i < m; ++i) {
        yout[i] = y[i];
        dyout[i] = k1[i];
    }
    double h = 1e-3;
    int64_t steps = 0;
    for (int64_t s = 1; s < n; ++s) {
        const double tend = t[s];
        while (x < tend) {
            if (++steps > 10000000) return -1;
            bool last = false;
            double hs = h;
            if (x + hs >= tend) {
                hs = tend - x;
                last = true;
            }
            for (size_t i = 0; i < m; ++i) yt[i] = y[i] + hs * A21 * k1[i];
            rhs_all(x + C2 * hs, yt, c, k2);
            for (size_t i = 0; i < m; ++i) yt[i] = y[i] + hs * (A31 * k1[i] + A32 * k2[i]);
            rhs_all(x + C3 * hs, yt, c, k3);
            for (size_t i = 0; i < m; ++i)
                yt[i] = y[i] + hs * (A41 * k1[i] + A42 * k2[i] + A43 * k3[i]);
            rhs_all(x + C4 * hs, yt, c, k4);
            for (size_t i = 0; i < m; ++i)
                yt[i] = y[i] + hs * (A51 * k1[i] + A52 * k2[i] + A53 * k3[i] + A54 * k4[i]);
            rhs_all(x + C5 * hs, yt, c, k5);
            for (size_t i = 0; i < m; ++i)
                yt[i] = y[i] + hs * (A61 * k1[i] + A62 * k2[i] + A63 * k3[i] + A64 * k4[i] +
                                     A65 * k5[i]);
            rhs_all(x + hs, yt, c, k6);
            for (size_t i = 0; i < m; ++i)
                y5[i] = y[i] + hs * (B1 * k1[i] + B3 * k3[i] + B4 * k4[i] + B5 * k5[i] + B6 * k6[i]);
            const double xn = last ? tend : x + hs;
            rhs_all(xn, y5, c, k7);
            double err = 0.0;
            for (size_t i = 0; i < m; ++i) {
                const double e = hs * (E1 * k1[i] + E3 * k3[i] + E4 * k4[i] + E5 * k5[i] +
                                       E6 * k6[i] + E7 * k7[i]);
                const double sc = atol + rtol * std::fmax(std::fabs(y[i]), std::fabs(y5[i]));
                err += (e / sc) * (e / sc);
            }
            err = std::sqrt(err / (double)m);
            if (err <= 1.0) {  // accept (first same as last: k7 is the next k1)
                x = xn;
                std::swap(w.y, w.y5);
                std::swap(w.k1, w.k7);
                y = w.y.data();
                y5 = w.y5.data();
                k1 = w.k1.data();
                k7 = w.k7.data();
            }
            const double fac = err > 0.0 ? 0.9 * std::pow(err, -0.2) : 5.0;
            const double hn = hs * std::fmin(5.0, std::fmax(0.2, fac));
            // an accepted step cut short at an output point does not shrink h
            h = (last && err <= 1.0) ? std::fmax(h, hn) : hn;
            if (!(h > 0.0) || !std::isfinite(h)) return -1;
        }
        for (size_t i = 0; i < m; ++i) {
            yout[s * m + i] = y[i];
            dyout[s * m + i] = k1[i];
        }
    }
    return 0;
}

}  // namespace
}  // namespace pmx

using namespace pmx;

extern "C" int pmx_growth_ode(const double *params, int64_t nparam, const double *lna,
                              int64_t num, double rtol, double atol, double *y, double *dy) {
    clear_error();
    if (!params || !lna || !y || !dy) return fail(PMX_ERR_ARG, "null argument");
    if (nparam < 1 || num < 1 || !(rtol > 0.0) || !(atol > 0.0))
        return fail(PMX_ERR_ARG, "need nparam >= 1, num >= 1 and positive tolerances");
    for (int64_t i = 1; i < num; ++i)
        if (!(lna[i] > lna[i - 1])) return fail(PMX_ERR_ARG, "lna must increase");
    std::vector<Bg> c((size_t)nparam);
    for (int64_t p = 0; p < nparam; ++p)
        c[(size_t)p] = Bg{params[4 * p], params[4 * p + 1], params[4 * p + 2], params[4 * p + 3]};
    if (integrate(c, lna, num, rtol, atol, y, dy) != 0)
        return fail(PMX_ERR_ARG, "growth ODE: step size underflow or too many steps");
    return PMX_OK;
}
