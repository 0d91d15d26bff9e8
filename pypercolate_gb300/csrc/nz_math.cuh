// nz_math.cuh -- FP64 special functions for the confidence intervals.
//
// The reference calls scipy.stats.t.interval (percolate/hpc.py:818-823,
// percolate/percolate.py:621-633, 691-703) and scipy.stats.beta.ppf
// (percolate/percolate.py:564-566).  These are computed here on the device
// from the mathematics:
//   * the regularized incomplete beta function I_x(a, b) by its continued
//     fraction (DLMF 8.17.22), evaluated by the forward recurrence of its
//     convergents (division-free after an equivalence transformation), and
//     the symmetry I_x(a, b) = 1 - I_{1-x}(b, a) outside its fast region;
//   * Student-t CDF F(t; v) = 1 - I_{v/(v+t^2)}(v/2, 1/2) / 2 for t >= 0;
//   * quantiles by Newton's method on the CDF inside a maintained bracket,
//     falling back to bisection whenever a Newton step leaves the bracket.
//     The t start value is the Cornish-Fisher expansion (Abramowitz & Stegun
//     26.7.5) about the normal quantile; v = 1, 2 use their closed forms.
//     The Beta start value is the normal approximation with its skewness
//     term; Beta(1, b) and Beta(a, 1) use their closed forms.
// lgamma, log1p, exp, normcdfinv are CUDA's own functions.
#pragma once

#include <cmath>
#include <cstdint>

namespace nz {

#ifdef __CUDA_ARCH__
#define NZ_HD __host__ __device__
#else
#define NZ_HD __host__ __device__
#endif

// Continued fraction of I_x(a, b) (without the prefactor), x < (a+1)/(a+b+2):
//   f = 1 / (1 + d_1 / (1 + d_2 / (1 + ...))),  d_j = p_j / q_j,
//   d_1 = -(a + b) x / (a + 1),
//   d_2m = m (b - m) x / ((a + 2m - 1)(a + 2m)),
//   d_2m+1 = -(a + m)(a + b + m) x / ((a + 2m)(a + 2m + 1)).
// Evaluated by the forward recurrence of its convergents A_j / B_j after the
// equivalence transformation that clears the q_j (partial numerators
// q_{j-1} p_j, partial denominators q_j), so that no term needs a division
// -- FP64 division is a long dependent sequence on this chip -- with A and B
// rescaled by 1 / B every 8 terms (keeping them in range and A / B = A),
// until two rescaled values agree to 1e-15.
NZ_HD inline double incbeta_cf(double a, double b, double x) {
    double Ap = 0.0, Ac = 1.0, Bp = 1.0, Bc = 1.0, ql = 1.0;
    auto term = [&](double p, double q) {
        const double An = q * Ac + ql * p * Ap, Bn = q * Bc + ql * p * Bp;
        Ap = Ac; Ac = An; Bp = Bc; Bc = Bn; ql = q;
    };
    term(-(a + b) * x, a + 1.0);
    double f = 1.0;
    for (int m = 1; m <= 2000; m += 4) {
        for (int i = 0; i < 4; ++i) {
            const double mm = m + i, m2 = 2.0 * mm;
            term(mm * (b - mm) * x, (a + m2 - 1.0) * (a + m2));
            term(-(a + mm) * (a + b + mm) * x, (a + m2) * (a + m2 + 1.0));
        }
        if (!(Bc != 0.0) || !isfinite(Bc)) break;  // (not in the convergent region)
        const double r = 1.0 / Bc;
        Ap *= r; Ac *= r; Bp *= r; Bc = 1.0;
        const bool done = fabs(Ac - f) <= 1e-15 * fabs(Ac);
        f = Ac;
        if (done) break;
    }
    return f;
}

// I_x(a, b) with y = 1 - x supplied separately (no cancellation near 1);
// lbeta = ln B(a, b) = lgamma(a) + lgamma(b) - lgamma(a + b).
NZ_HD inline double incbeta_lb(double a, double b, double x, double y, double lbeta) {
    if (x <= 0.0) return 0.0;
    if (y <= 0.0) return 1.0;
    const double bt = exp(a * log(x) + b * log(y) - lbeta);
    if (x < (a + 1.0) / (a + b + 2.0)) return bt * incbeta_cf(a, b, x) / a;
    return 1.0 - bt * incbeta_cf(b, a, y) / b;
}

// Upper tail 1 - I_x(a, b) with the same arguments, accurate when small.
NZ_HD inline double incbeta_upper_lb(double a, double b, double x, double y, double lbeta) {
    if (x <= 0.0) return 1.0;
    if (y <= 0.0) return 0.0;
    const double bt = exp(a * log(x) + b * log(y) - lbeta);
    if (x < (a + 1.0) / (a + b + 2.0)) return 1.0 - bt * incbeta_cf(a, b, x) / a;
    return bt * incbeta_cf(b, a, y) / b;
}

NZ_HD inline double log_beta(double a, double b) { return lgamma(a) + lgamma(b) - lgamma(a + b); }

NZ_HD inline double incbeta(double a, double b, double x, double y) {
    return incbeta_lb(a, b, x, y, log_beta(a, b));
}

// Probability that a Student-t variable with v dof exceeds t >= 0.
NZ_HD inline double t_upper_tail(double t, double v) {
    const double t2 = t * t;
    const double x = v / (v + t2), y = t2 / (v + t2);
    return 0.5 * incbeta(0.5 * v, 0.5, x, y);
}

NZ_HD inline double t_log_pdf(double t, double v) {
    return lgamma(0.5 * (v + 1.0)) - lgamma(0.5 * v) - 0.5 * log(v * M_PI) -
           0.5 * (v + 1.0) * log1p(t * t / v);
}

#ifdef __CUDA_ARCH__
__device__ inline double nz_normal_quantile(double q) { return normcdfinv(q); }
#else
inline double nz_normal_quantile(double q) {
    // host fallback is only used by host-side unit checks; bisection on erfc
    double lo = -40.0, hi = 40.0;
    for (int i = 0; i < 200; ++i) {
        double mid = 0.5 * (lo + hi);
        double c = 0.5 * erfc(-mid / M_SQRT2);
        if (c < q) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}
#endif

// Quantile t_q(v): P(T <= t) = q.  NaN for v <= 0 or q outside (0, 1),
// +-inf at q = 1 / 0 (scipy's conventions).
NZ_HD inline double student_t_quantile(double q, double v) {
    if (!(v > 0.0) || !(q >= 0.0 && q <= 1.0)) return NAN;
    if (q == 0.0) return -INFINITY;
    if (q == 1.0) return INFINITY;
    if (q == 0.5) return 0.0;
    const double sgn = q > 0.5 ? 1.0 : -1.0;
    const double tail = q > 0.5 ? 1.0 - q : q;  // upper-tail probability of |t|
    if (v == 1.0) return sgn * tan(M_PI * (0.5 - tail));
    if (v == 2.0) { const double p2 = 2.0 * tail; return sgn * sqrt(2.0 / (p2 * (2.0 - p2)) - 2.0); }
    // Cornish-Fisher expansion about the normal quantile (Abramowitz & Stegun
    // 26.7.5).  With four terms it is the quantile to double precision for
    // v >= 1e4 (<= 1e-15 relative against scipy for tails 1e-8 .. 0.5), and
    // the Newton iteration below, whose incomplete-beta continued fraction
    // needs hundreds of terms at large v, is skipped; below it is the start.
    const double z = -nz_normal_quantile(tail);
    const double z2 = z * z;
    double t = z + (z2 + 1.0) * z / (4.0 * v) + ((5.0 * z2 + 16.0) * z2 + 3.0) * z / (96.0 * v * v) +
               (((3.0 * z2 + 19.0) * z2 + 17.0) * z2 - 15.0) * z / (384.0 * v * v * v);
    if (v >= 1e4 && isfinite(z)) {
        t += ((((79.0 * z2 + 776.0) * z2 + 1482.0) * z2 - 1920.0) * z2 - 945.0) * z / (92160.0 * v * v * v * v);
        return sgn * t;
    }
    if (!(t > 0.0) || !isfinite(t)) t = z > 0.0 ? z : 1.0;
    // bracket [lo, hi] with tail(lo) >= target >= tail(hi)
    double lo = 0.0, hi = t;
    for (int i = 0; i < 200 && t_upper_tail(hi, v) > tail; ++i) { lo = hi; hi *= 2.0; }
    t = hi;
    for (int it = 0; it < 100; ++it) {
        const double g = t_upper_tail(t, v) - tail;  // decreasing in t
        if (g > 0.0) lo = t; else hi = t;
        const double dens = exp(t_log_pdf(t, v));
        double tn = t + g / dens;
        if (!(tn > lo && tn < hi) || !isfinite(tn)) tn = 0.5 * (lo + hi);
        if (fabs(tn - t) <= 1e-15 * fabs(t) || hi - lo <= 1e-15 * hi) { t = tn; break; }
        t = tn;
    }
    return sgn * t;
}

// Beta(a, b) quantile: I_x(a, b) = q.  NaN outside the domain.
NZ_HD inline double beta_quantile(double q, double a, double b) {
    if (!(a > 0.0) || !(b > 0.0) || !(q >= 0.0 && q <= 1.0)) return NAN;
    if (q == 0.0) return 0.0;
    if (q == 1.0) return 1.0;
    // the one-parameter families in closed form -- I_x(1, b) = 1 - (1 - x)^b
    // and I_x(a, 1) = x^a -- which are the Bayesian spanning bounds of every
    // n where no run or every run spans (most n of an ensemble)
    if (a == 1.0) return -expm1(log1p(-q) / b);
    if (b == 1.0) return exp(log(q) / a);
    const double lbeta = log_beta(a, b);
    // start: the normal approximation with its first skewness correction
    // (Cornish-Fisher, Abramowitz & Stegun 26.2.49 with the Beta's skewness),
    // clamped into (0, 1)
    const double s = a + b;
    const double mu = a / s;
    const double sd = sqrt(a * b / (s * s * (s + 1.0)));
    const double skew = 2.0 * (b - a) * sqrt(s + 1.0) / ((s + 2.0) * sqrt(a * b));
    const double z = nz_normal_quantile(q);
    double x = mu + sd * (z + skew * (z * z - 1.0) / 6.0);
    double lo = 0.0, hi = 1.0;
    if (!(x > 0.0 && x < 1.0)) x = mu;
    for (int it = 0; it < 200; ++it) {
        const double y = 1.0 - x;
        // work on whichever tail is smaller for accuracy
        double g;
        if (q < 0.5) g = incbeta_lb(a, b, x, y, lbeta) - q;
        else g = (1.0 - q) - incbeta_upper_lb(a, b, x, y, lbeta);  // I - q written via the upper tail
        if (g < 0.0) lo = x; else hi = x;
        const double ldens = (a - 1.0) * log(x) + (b - 1.0) * log1p(-x) - lbeta;
        double xn = x - g / exp(ldens);
        const bool newton = xn > lo && xn < hi && isfinite(xn);
        if (!newton) xn = 0.5 * (lo + hi);
        // a Newton step of relative size d leaves an error of order d^2:
        // below 1e-10 the new iterate is converged to double precision
        if ((newton && fabs(xn - x) <= 1e-10 * fmax(x, 1e-300)) || hi - lo <= 1e-16 * hi) { x = xn; break; }
        x = xn;
    }
    return x;
}

}  // namespace nz
