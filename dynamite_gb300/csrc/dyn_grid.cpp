// Grid/table generator (the reference's `RG-Evo grid`, poly method):
// theta grid (theta_grid.cpp:12-125), phi grids (phi_grid.cpp:17-34),
// int.dat quadrature weights (integration.cpp:14-195), local barycentric
// stencils for A1/A2/B2 (interpolation_weights.cpp:12-147, grid_cli.cpp:78-215).
//
// Published methods restated here: the knot-span search and the Cox-de Boor
// basis recurrence of Piegl & Tiller, "The NURBS Book" (algorithms A2.1 and
// A2.2) for the spline quadrature; barycentric Lagrange interpolation
// (Berrut & Trefethen, SIAM Review 46, 2004) for the polynomial stencils;
// Floater & Hormann's rational interpolant (Numer. Math. 107, 2007) for the
// rational ones; Halley's iteration for the Lambert W_{-1} branch.  The steps
// follow the reference generator's, so that the tables are bit-identical.
//
// Arithmetic is long double like the reference built without Boost
// (mp_type.hpp), with its transcendental calls in double (see dexp below):
// on x86-64 long double is the same 80-bit format, so the tables match the
// reference generator's bit for bit; on aarch64 long double is 128-bit and
// the tables agree to the last few bits of a double.
// Values that the reference writes as text are passed through the same
// 17-digit text round trip, so they equal what the solver reads back.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dyn.h"

namespace {

using ld = long double;

const ld PI_L = 3.141592653589793238462643383279502884L;

// The reference calls exp/log/atan/sqrt unqualified on long double values;
// with libstdc++ those resolve to the double-precision C functions, so the
// transcendental parts of its "long double" grid are evaluated in double.
// These wrappers make that explicit.
ld dexp(ld x) { return (ld)::exp((double)x); }
ld dlog(ld x) { return (ld)::log((double)x); }
ld datan(ld x) { return (ld)::atan((double)x); }
ld dsqrt(ld x) { return (ld)::sqrt((double)x); }

// W_{-1}(x) for x in [-1/e, 0): Halley iteration from the asymptotic
// (x near 0) or branch-point (x near -1/e) starting value.
ld lambert_wm1(ld x) {
    if (!(x <= 0)) throw std::domain_error("lambert_wm1: x must be <= 0");
    const ld minus_inv_e = -ld(1) / dexp(ld(1));
    if (x < minus_inv_e) throw std::domain_error("lambert_wm1: x must be >= -1/e");
    if (x == 0) return -std::numeric_limits<double>::infinity();
    ld w;
    if (x > ld(-0.1)) {
        const ld l1 = dlog(-x), l2 = dlog(-l1);
        w = l1 - l2 + (l2 / l1);
    } else {
        ld u = x * dexp(ld(1)) + ld(1);
        if (u > 0) u = 0;
        if (u < -1) u = -1;
        const ld sq = dsqrt(-ld(2) * u);
        w = -ld(1) - sq + (sq * sq) / ld(3);
    }
    for (int it = 0; it < 80; ++it) {
        const ld ew = dexp(w);
        const ld f = w * ew - x;
        const ld wp1 = w + ld(1);
        const ld den = ew * wp1 - (wp1 + ld(1)) * f / (ld(2) * wp1);
        ld dw = f / den;
        ld wn = w - dw;
        if (!std::isfinite(static_cast<double>(wn))) {
            dw = f / (ew * (w + ld(1)));
            wn = w - dw;
        }
        w = wn;
        // The reference's unqualified abs() on this long double picks the int
        // overload, so its loop stops as soon as |dw| < 1 (after one Halley
        // step from these starting values); kept so the grids coincide.
        if (std::abs((int)dw) <= std::numeric_limits<double>::epsilon()) break;
    }
    return w;
}

// Optional smooth index remap (alpha, delta): theta_grid.cpp:12-33
ld remap_index(ld x1, size_t len, double alpha, double delta) {
    if (alpha == 0.0) return x1;
    const ld N = (ld)len;
    const ld c = (N - 1.0L) / 2.0L;
    const ld t = 2.0L * x1 - N - 1.0L;
    ld s = t / (N - 1.0L);
    if (s > 1.0L) s = 1.0L;
    if (s < -1.0L) s = -1.0L;
    const ld a = std::fabs(s), d = (ld)delta;
    const ld inner = std::pow(a * a * a + d * d * d, 1.0L / 3.0L) - d;
    const ld S = s < 0 ? -1.0L : (s > 0 ? 1.0L : 0.0L);
    const ld g1 = std::pow(1.0L + d * d * d, 1.0L / 3.0L) - d;
    ld mapped = c * ((S * inner / g1) + 1.0L) + 1.0L;
    ld out = (ld)alpha * mapped + (1.0L - (ld)alpha) * x1;
    if (out < 1.0L) out = 1.0L;
    if (out > N) out = N;
    return out;
}

// theta(i) = [T(1) - T(i)] / [T(L/2+) - T(L/2-)] with T(x) = (2/pi) atan(exp(-(x - L/2 - 1/2) eta)),
// eta = -(2/L) W_{-1}(-1/(10 Tmax))   (theta_grid.cpp:37-125)
// theta at 0-based fractional indices (theta_of_vec, theta_grid.cpp:72-110)
std::vector<ld> theta_at(const std::vector<double>& indices, size_t len, double Tmax, double alpha, double delta) {
    const ld Lm = (ld)len;
    const ld Wm1 = lambert_wm1(-ld(1) / (ld(10) * (ld)Tmax));
    const ld eta = -(ld(2) / Lm) * Wm1;
    const ld tref = (ld(1) - (Lm / ld(2)) - ld(1) / ld(2)) * eta;
    const ld term_ref = (ld(2) / PI_L) * datan(ld(1) / dexp(tref));
    const ld thalf = ((Lm / ld(2)) - ld(1) / ld(2)) * eta;
    const ld den = (ld(2) / PI_L) * datan(dexp(thalf)) - (ld(2) / PI_L) * datan(dexp(-thalf));
    std::vector<ld> th(indices.size());
    for (size_t k = 0; k < indices.size(); ++k) {
        const ld x1 = remap_index((ld)indices[k] + 1.0L, len, alpha, delta);
        const ld idx = (ld)(double)x1;
        const ld t1 = (idx - (Lm / ld(2)) - ld(1) / ld(2)) * eta;
        const ld term1 = (ld(2) / PI_L) * datan(ld(1) / dexp(t1));
        const ld num = (ld(1) - term1) - (ld(1) - term_ref);
        ld v = (ld)(num / den);
        if (v < 0.0) v = 0.0;
        if (v > 1.0) v = 1.0;
        th[k] = v;
    }
    return th;
}

std::vector<ld> theta_grid(size_t len, double Tmax, double alpha, double delta) {
    std::vector<double> idx(len);
    for (size_t k = 0; k < len; ++k) idx[k] = (double)k;
    std::vector<ld> th = theta_at(idx, len, Tmax, alpha, delta);
    for (size_t k = 1; k < len; ++k)
        if (th[k] < th[k - 1]) th[k] = th[k - 1];
    return th;
}

// ---- position grids (pos_grid.cpp:111-205): the inverse map theta -> 1-based
// fractional index, as a local barycentric interpolant of m = 12 nodes through
// theta sampled at 20 len points, evaluated at phi1, phi2 and theta_i / phi2 ----
struct InverseTheta {
    std::vector<ld> x, y;  // theta samples (strictly increasing), 1-based positions
    std::vector<int> left;  // first node of the window of interval i
    std::vector<ld> w;      // barycentric weights of every window start
    int m = 12;

    void build(size_t len, double Tmax, double alpha, double delta, size_t oversample, int m_req) {
        const size_t M = len * oversample;
        std::vector<double> idx(M);
        y.resize(M);
        for (size_t k = 0; k < M; ++k) {
            y[k] = 1.0L + ((ld)len - 1.0L) * ((ld)k / (ld)(M - 1));
            idx[k] = (double)(y[k] - 1.0L);
        }
        x = theta_at(idx, len, Tmax, alpha, delta);
        for (size_t k = 1; k < M; ++k)
            if (x[k] <= x[k - 1]) x[k] = std::nextafter(x[k - 1], std::numeric_limits<ld>::infinity());
        m = std::max(4, std::min(16, m_req));
        if (m > (int)M) m = (int)M;
        const int Nm = (int)M - m, nleft = std::max(0, Nm) + 1;
        left.resize(M - 1);
        for (size_t i = 0; i + 1 < M; ++i) left[i] = std::min(std::max((int)i - m / 2 + 1, 0), std::max(0, Nm));
        w.assign((size_t)nleft * m, 0.0L);
        for (int L0 = 0; L0 < nleft; ++L0)
            for (int j = 0; j < m; ++j) {
                ld prod = 1.0L;
                for (int k = 0; k < m; ++k)
                    if (k != j) prod *= x[(size_t)(L0 + j)] - x[(size_t)(L0 + k)];
                w[(size_t)L0 * m + j] = 1.0L / prod;
            }
    }

    ld operator()(ld v) const {
        if (v <= x.front()) return y.front();
        if (v >= x.back()) return y.back();
        const size_t i = std::max<size_t>(1, (size_t)(std::upper_bound(x.begin(), x.end(), v) - x.begin())) - 1;
        const int nleft = std::max(0, (int)x.size() - m) + 1;
        const int L0 = std::min(std::max(left[i], 0), nleft - 1);
        const ld* wp = &w[(size_t)L0 * m];
        for (int j = 0; j < m; ++j)
            if (v == x[(size_t)(L0 + j)]) return y[(size_t)(L0 + j)];
        ld num = 0.0L, den = 0.0L;
        for (int j = 0; j < m; ++j) {
            const ld q = wp[j] / (v - x[(size_t)(L0 + j)]);
            den += q;
            num += q * y[(size_t)(L0 + j)];
        }
        return num / den;
    }
};

// the reference reads these two tuning variables (clamped the same way)
size_t env_size(const char* name, size_t def, long lo) {
    if (const char* e = std::getenv(name)) {
        const long v = std::strtol(e, nullptr, 10);
        if (v > lo) return (size_t)v;
    }
    return def;
}

// ---- integration weights: spline-consistent quadrature (integration.cpp) ----
std::vector<ld> open_knots(const std::vector<ld>& x, int p) {
    const int N = (int)x.size(), K = N + p + 1;
    std::vector<ld> t(K);
    for (int i = 0; i <= p; ++i) t[i] = x.front();
    for (int i = 0; i <= p; ++i) t[K - 1 - i] = x.back();
    for (int j = p + 1; j <= N - 1; ++j) {
        ld sum = 0.0L;
        for (int i = j - p; i <= j - 1; ++i) sum += x[i];
        t[j] = sum / (ld)p;
    }
    return t;
}

int find_span(int nb, int p, ld u, const std::vector<ld>& t) {
    const int n = nb - 1;
    if (u >= t[n + 1]) return n;
    if (u <= t[p]) return p;
    int lo = p, hi = n + 1, mid = (lo + hi) / 2;
    while (!(u >= t[mid] && u < t[mid + 1])) {
        if (u < t[mid]) hi = mid; else lo = mid;
        mid = (lo + hi) / 2;
    }
    return mid;
}

void basis(int span, ld u, int p, const std::vector<ld>& t, std::vector<ld>& Nv) {
    Nv.assign(p + 1, 0.0L);
    std::vector<ld> left(p + 1), right(p + 1);
    Nv[0] = 1.0L;
    for (int j = 1; j <= p; ++j) {
        left[j] = u - t[span + 1 - j];
        right[j] = t[span + j] - u;
        ld saved = 0.0L;
        for (int r = 0; r < j; ++r) {
            const ld den = right[r + 1] + left[j - r];
            const ld tmp = den != 0.0L ? Nv[r] / den : 0.0L;
            Nv[r] = saved + right[r + 1] * tmp;
            saved = left[j - r] * tmp;
        }
        Nv[j] = saved;
    }
}

std::vector<ld> integration_weights(const std::vector<ld>& th, int order) {
    const int N = (int)th.size();
    int p = order;
    if (p < 1) p = 1;
    if (p > N - 1) p = std::max(1, N - 1);
    const std::vector<ld> kn = open_knots(th, p);
    // banded collocation matrix, stored dense row-major like the reference
    std::vector<ld> A((size_t)N * N, 0.0L), Nv(p + 1);
    for (int i = 0; i < N; ++i) {
        const int span = find_span(N, p, th[i], kn);
        basis(span, th[i], p, kn, Nv);
        for (int j = 0; j <= p; ++j) {
            const int col = span - p + j;
            if (col >= 0 && col < N) A[(size_t)i * N + col] = Nv[j];
        }
    }
    // LU without pivoting, band p
    for (int k = 0; k < N; ++k) {
        const ld akk = A[(size_t)k * N + k];
        for (int i = k + 1; i <= std::min(N - 1, k + p); ++i) {
            const ld lik = A[(size_t)i * N + k] /= akk;
            for (int j = k + 1; j <= std::min(N - 1, k + p); ++j) A[(size_t)i * N + j] -= lik * A[(size_t)k * N + j];
        }
    }
    // basis integrals M_j = (t_{j+p+1} - t_j)/(p+1); solve A^T w = M
    std::vector<ld> w(N);
    for (int j = 0; j < N; ++j) w[j] = (kn[j + p + 1] - kn[j]) / (ld)(p + 1);
    for (int i = 0; i < N; ++i) {
        for (int j = std::max(0, i - p); j < i; ++j) w[i] -= A[(size_t)j * N + i] * w[j];
        w[i] /= A[(size_t)i * N + i];
    }
    for (int i = N - 1; i >= 0; --i)
        for (int j = i + 1; j <= std::min(N - 1, i + p); ++j) w[i] -= A[(size_t)j * N + i] * w[j];
    return w;
}

// ---- local barycentric stencils (interpolation_weights.cpp:12-147) ----
// start of the m-point window around xq whose farther end is nearest
// (pick_stencil_start with m = n + 1, pick_window_start for any m)
int window_start(const std::vector<ld>& x, int m, ld xq) {
    const int N = (int)x.size();
    const int hi = (int)(std::lower_bound(x.begin(), x.end(), xq) - x.begin());
    int start = hi - m / 2;
    if (start < 0) start = 0;
    if (start > N - m) start = N - m;
    auto spread = [&](int s) {
        const ld l = std::fabs(xq - x[s]), r = std::fabs(xq - x[s + m - 1]);
        return l < r ? r : l;
    };
    ld best = spread(start);
    for (int s = std::max(0, start - 2); s <= std::min(N - m, start + 2); ++s) {
        const ld v = spread(s);
        if (v < best) { best = v; start = s; }
    }
    return start;
}

void stencils(const std::vector<ld>& x, const std::vector<ld>& xq, int n, int64_t* inds, double* w) {
    const int m = n + 1;
    const long long Q = (long long)xq.size();
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < Q; ++k) {
        const ld q = xq[k];
        const int start = window_start(x, m, q);
        ld xn[64], wl[64], tmp[64];
        for (int j = 0; j < m; ++j) xn[j] = x[start + j];
        int exact = -1;
        for (int j = 0; j < m; ++j) if (q == xn[j]) { exact = j; break; }
        double* out = w + (size_t)k * m;
        inds[k] = start;
        if (exact >= 0) {
            for (int j = 0; j < m; ++j) out[j] = 0.0;
            out[exact] = 1.0;
            continue;
        }
        for (int j = 0; j < m; ++j) {
            ld den = 1.0L;
            for (int l = 0; l < m; ++l) if (l != j) den *= (xn[j] - xn[l]);
            wl[j] = 1.0L / den;
        }
        ld sum = 0.0L;
        for (int j = 0; j < m; ++j) { tmp[j] = wl[j] / (q - xn[j]); sum += tmp[j]; }
        const ld inv = 1.0L / sum;
        for (int j = 0; j < m; ++j) out[j] = (double)(tmp[j] * inv);
    }
}

// ---- Floater-Hormann rational stencils (interpolation_weights.cpp:72-290) ----
// Barycentric weights of the order-d Floater-Hormann interpolant on the m
// nodes xn: w_j = sum over the (d+1)-node subsets i..i+d holding j of
// (-1)^i / prod_{k != j} (x_j - x_k).
void fh_node_weights(const ld* xn, int m, int d, ld* w) {
    for (int j = 0; j < m; ++j) {
        const int r0 = std::max(0, j - (m - d - 1)), r1 = std::min(d, j);
        ld sum = 0.0L;
        for (int r = r0; r <= r1; ++r) {
            const int i = j - r;
            ld prod = 1.0L;
            bool dup = false;
            for (int k = 0; k <= d; ++k) {
                if (k == r) continue;
                const ld diff = xn[j] - xn[i + k];
                if (diff == 0.0L) { dup = true; break; }
                prod *= diff;
            }
            if (dup || prod == 0.0L) continue;
            sum += (((j - r) & 1) ? -1.0L : 1.0L) / prod;
        }
        w[j] = sum;
    }
}

// Neumaier-compensated barycentric evaluation at qn: alpha_j = (w_j / (qn - y_j)) / sum.
// Returns the denominator (NaN/inf if ill-defined), the sum of |terms| and the
// Lebesgue sum of the double weights (inf if the denominator is not finite).
ld bary_eval(const ld* w, const ld* y, int m, ld qn, double* alpha, ld* sumabs, ld* lebesgue) {
    ld tmp[256];
    ld den = 0.0L, comp = 0.0L, sa = 0.0L;
    for (int j = 0; j < m; ++j) {
        const ld v = w[j] / (qn - y[j]);
        tmp[j] = v;
        sa += std::fabs(v);
        const ld t = den + v;
        if (std::fabs(den) >= std::fabs(v)) comp += (den - t) + v;
        else comp += (v - t) + den;
        den = t;
    }
    den += comp;
    *sumabs = sa;
    *lebesgue = std::numeric_limits<ld>::infinity();
    if (den == den && std::isfinite(den)) {
        const ld inv = 1.0L / den;
        ld leb = 0.0L;
        for (int j = 0; j < m; ++j) {
            const double a = (double)(tmp[j] * inv);
            alpha[j] = a;
            leb += std::fabs(a);
        }
        *lebesgue = leb;
    }
    return den;
}

// Order-d Floater-Hormann stencils on m-point windows; the polynomial stencil
// of the same window where FH cancels (|den| <= 1e-10 sum |terms|) or has a
// Lebesgue sum more than twice the polynomial's.
void stencils_fh(const std::vector<ld>& x, const std::vector<ld>& xq, int d, int m, int64_t* inds, double* w) {
    const long long Q = (long long)xq.size();
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < Q; ++k) {
        const ld q = xq[k];
        const int start = window_start(x, m, q);
        ld xn[256], yn[256], wl[256];
        for (int j = 0; j < m; ++j) xn[j] = x[start + j];
        double* out = w + (size_t)k * m;
        inds[k] = start;
        const ld span = xn[m - 1] - xn[0];
        const ld tol = 64 * std::numeric_limits<ld>::epsilon() * (span > 0.0L ? span : 1.0L);
        int hit = -1;
        for (int j = 0; j < m; ++j) if (std::fabs(q - xn[j]) <= tol) { hit = j; break; }
        if (hit >= 0) {
            for (int j = 0; j < m; ++j) out[j] = 0.0;
            out[hit] = 1.0;
            continue;
        }
        const ld a = xn[0], b = xn[m - 1], c = 0.5L * (a + b);
        ld sc = b - a;
        if (sc <= 0.0L) sc = 1.0L;
        for (int j = 0; j < m; ++j) yn[j] = (xn[j] - c) / sc;
        const ld qn = (q - c) / sc;
        double afh[256], apl[256];
        for (int j = 0; j < m; ++j) afh[j] = apl[j] = 0.0;
        ld sa_fh, leb_fh, sa_pl, leb_pl;
        fh_node_weights(yn, m, d, wl);
        const ld den_fh = bary_eval(wl, yn, m, qn, afh, &sa_fh, &leb_fh);
        for (int j = 0; j < m; ++j) {
            ld den = 1.0L;
            for (int l = 0; l < m; ++l) if (l != j) den *= (yn[j] - yn[l]);
            wl[j] = 1.0L / den;
        }
        bary_eval(wl, yn, m, qn, apl, &sa_pl, &leb_pl);
        const ld inf = std::numeric_limits<ld>::infinity();
        bool poly = !(den_fh == den_fh) || !std::isfinite(den_fh) || (sa_fh > 0.0L && std::fabs(den_fh) <= 1e-10L * sa_fh);
        if (!poly && leb_pl < inf && leb_fh < inf && leb_fh > 2.0L * leb_pl) poly = true;
        for (int j = 0; j < m; ++j) out[j] = poly ? apl[j] : afh[j];
    }
}

// grid_io.cpp writes long-double grids at 17 digits after the point;
// io_input.cpp reads them back as double.
double text_trip(ld v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.17Le", v);
    return std::strtod(buf, nullptr);
}

}  // namespace

// The generator behind both entry points: rational = false is -m poly
// (depth interp_order + 1), true is -m rational (depth fh_depth(...)).
static dyn_status generate(size_t len, double Tmax, int spline_order, int interp_order, bool rational, int fh_window,
                           double alpha, double delta, double* theta, double* phi1, double* phi2, double* integ,
                           int64_t* indsA1, double* wA1, int64_t* indsA2, double* wA2, int64_t* indsB2, double* wB2) {
    const int n = std::max(1, interp_order);
    if (len < (size_t)(n + 1) || len > 8192 || !(Tmax > 0)) return DYN_ERR_INVALID;
    if (!theta || !phi2 || !integ || !indsA1 || !wA1 || !indsA2 || !wA2 || !indsB2 || !wB2) return DYN_ERR_INVALID;
    const int mfh = (int)std::min<size_t>(len, (size_t)std::max(n + 1, fh_window > 0 ? fh_window : n + 1));
    if (rational && mfh > 256) return DYN_ERR_INVALID;
    auto tables = [&](const std::vector<ld>& th, const std::vector<ld>& q, int64_t* inds, double* w) {
        if (rational) stencils_fh(th, q, n, mfh, inds, w);
        else stencils(th, q, n, inds, w);
    };
    try {
        const std::vector<ld> th = theta_grid(len, Tmax, alpha, delta);
        const size_t N = len, N2 = N * N;
        std::vector<ld> p1(N2), p2(N2), xb(N2);
        for (size_t i = 0; i < N; ++i) {
            const ld ti = th[i], omt = 1.0L - ti;
            for (size_t j = 0; j < N; ++j) {
                p1[i * N + j] = ti * th[j];
                p2[i * N + j] = ti + omt * th[j];
            }
        }
        const double tiny = 1e-200;
        for (size_t i = 0; i < N; ++i) {
            const ld ti = th[i];
            for (size_t j = 0; j < N; ++j) {
                const ld den = p2[i * N + j] - tiny;
                xb[i * N + j] = std::fabs(den) < 1e-300L ? (ti > 0 ? th.back() : th.front()) : ti / den;
            }
        }
        const std::vector<ld> wint = integration_weights(th, spline_order);
        for (size_t i = 0; i < N; ++i) {
            theta[i] = (double)th[i];
            integ[i] = (double)wint[i];
        }
        for (size_t k = 0; k < N2; ++k) {
            if (phi1) phi1[k] = text_trip(p1[k]);
            phi2[k] = text_trip(p2[k]);
        }
        tables(th, p1, indsA1, wA1);
        tables(th, p2, indsA2, wA2);
        tables(th, xb, indsB2, wB2);
    } catch (...) {
        return DYN_ERR_INVALID;
    }
    return DYN_OK;
}

extern "C" dyn_status dyn_grid_generate(size_t len, double Tmax, int spline_order, int interp_order, double alpha,
                                        double delta, double* theta, double* phi1, double* phi2, double* integ,
                                        int64_t* indsA1, double* wA1, int64_t* indsA2, double* wA2, int64_t* indsB2,
                                        double* wB2) {
    return generate(len, Tmax, spline_order, interp_order, false, 0, alpha, delta, theta, phi1, phi2, integ, indsA1,
                    wA1, indsA2, wA2, indsB2, wB2);
}

extern "C" dyn_status dyn_grid_positions(size_t len, double Tmax, double alpha, double delta, double* posA1y,
                                         double* posA2y, double* posB2y) {
    if (len < 4 || len > 8192 || !(Tmax > 0) || !posA1y || !posA2y || !posB2y) return DYN_ERR_INVALID;
    try {
        const std::vector<ld> th = theta_grid(len, Tmax, alpha, delta);
        InverseTheta inv;
        int m_req = 12;
        if (const char* e = std::getenv("DMFE_POS_BARY_M")) m_req = std::max(2, std::min(32, (int)std::strtol(e, nullptr, 10)));
        inv.build(len, Tmax, alpha, delta, env_size("DMFE_POS_OVERSAMPLE", 20, 1), m_req);
        const ld tmin = inv.x.front(), tmax = inv.x.back(), tiny = 1e-200L;
        const size_t N = len;
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)N; ++i) {
            const ld ti = th[(size_t)i], omt = 1.0L - ti;
            for (size_t j = 0; j < N; ++j) {
                const size_t k = (size_t)i * N + j;
                const ld v1 = ti * th[j], v2 = ti + omt * th[j];
                posA1y[k] = (double)inv(v1);
                posA2y[k] = (double)inv(v2);
                const ld den = v2 - tiny;
                const ld arg = std::fabs(den) < 1e-300L ? (ti > 0 ? tmax : tmin) : ti / den;
                posB2y[k] = (double)inv(arg);
            }
        }
    } catch (...) {
        return DYN_ERR_INVALID;
    }
    return DYN_OK;
}

extern "C" int dyn_grid_rational_depth(size_t len, int interp_order, int fh_window) {
    const int n = std::max(1, interp_order);
    return (int)std::min<size_t>(len, (size_t)std::max(n + 1, fh_window > 0 ? fh_window : n + 1));
}

extern "C" dyn_status dyn_grid_generate_rational(size_t len, double Tmax, int spline_order, int interp_order,
                                                 int fh_window, double alpha, double delta, double* theta,
                                                 double* phi1, double* phi2, double* integ, int64_t* indsA1,
                                                 double* wA1, int64_t* indsA2, double* wA2, int64_t* indsB2,
                                                 double* wB2) {
    return generate(len, Tmax, spline_order, interp_order, true, fh_window, alpha, delta, theta, phi1, phi2, integ,
                    indsA1, wA1, indsA2, wA2, indsB2, wB2);
}
