// Test infrastructure only: a C-ABI harness around the reference DYNAMITE CPU
// implementation, compiled by oracle/Makefile from the reference's own sources
// into oracle/_ref/libdynref.so.  The harness owns the three globals the
// reference expects (`config`, `sim`, `rk`, defined in the reference at
// main.cpp:32-37) and forwards to the reference functions unchanged.  Nothing
// in the product links this file; tests and the golden-vector generator load
// it with ctypes to pin the C restatement (oracle/dyn_oracle.c) and the CUDA
// path against the real reference.
//
// The few pieces of driver logic that live in files not compiled here
// (t=0 state, controller, CPU energy) are restated with citations.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <omp.h>

#include "core/config.hpp"
#include "simulation/simulation_data.hpp"
#include "EOMs/rk_data.hpp"
#include "interpolation/interpolation_core.hpp"
#include "EOMs/time_steps.hpp"
#include "EOMs/runge_kutta.hpp"
#include "sparsify/sparsify_utils.hpp"
#include "simulation/tail_fit.hpp"
#include "convolution/convolution.hpp"
#include "math/math_sigma.hpp"
#include "math/math_ops.hpp"
#include "search/search_utils.hpp"
#include "grid/theta_grid.hpp"
#include "grid/phi_grid.hpp"
#include "grid/pos_grid.hpp"
#include "grid/integration.hpp"
#include "grid/interpolation_weights.hpp"

SimulationConfig config;
int last_rollback_loop = -1000;  // simulation_runner.cpp:53 (read by the tail fit)
SimulationData* sim = nullptr;
RKData* rk = nullptr;

namespace {

std::vector<double> copy_in(const double* p, size_t n) { return std::vector<double>(p, p + n); }

// Grid files are text: theta/int are written as doubles, phi1/phi2 as long
// doubles at 17 digits after the point (grid_io.cpp:26-76,138-154) and read
// back with `ifstream >> double` (io_input.cpp:60-88).  Reproduce that trip.
double text_round_trip(long double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.17Le", v);
    return std::strtod(buf, nullptr);
}

}  // namespace

extern "C" {

// The -R option (config.cpp:164-166): QR gathered in log space by
// indexVecLN3 / indexVecN / indexMatAll.  dynref_setup resets it to off.
void dynref_set_log_response(int on) { config.log_response_interp = on != 0; }

// --tail-fit (config.hpp:55): dynref_run applies tailFitBlendCPU after each
// update; dynref_tail_fit applies it once to the current state.  The fit keeps
// its window / smoothing state in function statics (tail_fit.cpp:81-85), so a
// process sees one fit history: drive it from a fresh process.
void dynref_set_tail_fit(int on) { config.tail_fit_enabled = on != 0; }
void dynref_tail_fit(void) { tailFitBlendCPU(); }
void dynref_set_rollback_loop(int loop) { last_rollback_loop = loop; }

// Model / controller parameters (config.hpp:18-56).
int dynref_setup(int p, int p2, double lambda, double T0, double Gamma, size_t len,
                 double delta_t_min, double delta_max, int nthreads) {
    config = SimulationConfig();
    config.p = p;
    config.p2 = p2;
    config.lambda = lambda;
    config.T0 = T0;
    config.Gamma = Gamma;
    config.len = len;
    config.delta_t_min = delta_t_min;
    config.delta_max = delta_max;
    config.gpu = false;
    config.debug = false;
    config.log_response_interp = false;
    config.tail_fit_enabled = false;
    delete sim;
    delete rk;
    sim = new SimulationData();
    rk = new RKData();
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return 0;
}

// Table import: the same vectors io_input.cpp:90-110 fills from Grid_data/<L>.
int dynref_set_tables(const double* theta, const double* phi1, const double* phi2,
                      const double* integ, const int64_t* indsA1, const int64_t* indsA2,
                      const int64_t* indsB2, const double* wA1, const double* wA2,
                      const double* wB2, size_t depth) {
    const size_t L = config.len, L2 = L * L;
    sim->h_theta = copy_in(theta, L);
    sim->h_phi1 = copy_in(phi1, L2);
    sim->h_phi2 = copy_in(phi2, L2);
    sim->h_integ = copy_in(integ, L);
    sim->h_indsA1y.assign(indsA1, indsA1 + L2);
    sim->h_indsA2y.assign(indsA2, indsA2 + L2);
    sim->h_indsB2y.assign(indsB2, indsB2 + L2);
    sim->h_weightsA1y = copy_in(wA1, L2 * depth);
    sim->h_weightsA2y = copy_in(wA2, L2 * depth);
    sim->h_weightsB2y = copy_in(wB2, L2 * depth);
    config.ord = static_cast<int>(depth) - 2;
    return 0;
}

static void size_scratch() {
    // initialization.cpp:234-256
    const size_t L = config.len, L2 = L * L;
    for (auto* v : {&sim->h_SigmaKA1int, &sim->h_SigmaRA1int, &sim->h_SigmaKB1int, &sim->h_SigmaRB1int,
                    &sim->h_SigmaKA2int, &sim->h_SigmaRA2int, &sim->h_SigmaKB2int, &sim->h_SigmaRB2int,
                    &sim->h_QKA1int, &sim->h_QRA1int, &sim->h_QKB1int, &sim->h_QRB1int,
                    &sim->h_QKA2int, &sim->h_QRA2int, &sim->h_QKB2int, &sim->h_QRB2int})
        v->assign(L2, 0.0);
    sim->h_rInt.assign(L, 0.0);
    sim->h_drInt.assign(L, 0.0);
}

// t=0 state, initialization.cpp:204-222 and 234-256, CPU branch :276-283.
void dynref_init_state(double delta_t) {
    const size_t L = config.len;
    sim->h_t1grid.assign(1, 0.0);
    sim->h_delta_t_ratio.assign(1, 0.0);
    config.specRad = 4 * std::sqrt(DDflambda(1));
    config.delta_t = delta_t > 0 ? delta_t : config.delta_t_min;
    config.loop = 0;
    config.delta = 1;
    config.delta_old = 0;
    sim->h_QKv.assign(L, 1.0);
    sim->h_QRv.assign(L, 1.0);
    sim->h_dQKv.assign(L, 0.0);
    sim->h_dQRv.assign(L, 0.0);
    sim->h_rvec.assign(1, config.Gamma + Dflambda(1) / config.T0);
    sim->h_drvec.assign(1, rstep());
    sim->h_posB1xOld.assign(L, 1.0);
    sim->h_posB2xOld.assign(L * L, 0.0);
    size_scratch();
    rk->init = (config.delta_t < config.rmax[0] / config.specRad) ? 1 : 2;
    interpolate();
}

void dynref_set_state(size_t n, const double* t1grid, const double* dtr, const double* QK,
                      const double* QR, const double* dQK, const double* dQR, const double* rvec,
                      const double* drvec, const double* posB1xOld, const double* posB2xOld) {
    const size_t L = config.len;
    sim->h_t1grid = copy_in(t1grid, n);
    sim->h_delta_t_ratio = copy_in(dtr, n);
    sim->h_QKv = copy_in(QK, n * L);
    sim->h_QRv = copy_in(QR, n * L);
    sim->h_dQKv = copy_in(dQK, n * L);
    sim->h_dQRv = copy_in(dQR, n * L);
    sim->h_rvec = copy_in(rvec, n);
    sim->h_drvec = copy_in(drvec, n);
    if (posB1xOld) sim->h_posB1xOld = copy_in(posB1xOld, L); else sim->h_posB1xOld.assign(L, 1.0);
    if (posB2xOld) sim->h_posB2xOld = copy_in(posB2xOld, L * L); else sim->h_posB2xOld.assign(L * L, 0.0);
    size_scratch();
    config.specRad = 4 * std::sqrt(DDflambda(1));
}

size_t dynref_get_n(void) { return sim->h_t1grid.size(); }

void dynref_get_state(double* t1grid, double* dtr, double* QK, double* QR, double* dQK,
                      double* dQR, double* rvec, double* drvec, double* posB1xOld,
                      double* posB2xOld) {
    auto out = [](const std::vector<double>& v, double* dst) {
        if (dst) std::memcpy(dst, v.data(), v.size() * sizeof(double));
    };
    out(sim->h_t1grid, t1grid);
    out(sim->h_delta_t_ratio, dtr);
    out(sim->h_QKv, QK);
    out(sim->h_QRv, QR);
    out(sim->h_dQKv, dQK);
    out(sim->h_dQRv, dQR);
    out(sim->h_rvec, rvec);
    out(sim->h_drvec, drvec);
    out(sim->h_posB1xOld, posB1xOld);
    out(sim->h_posB2xOld, posB2xOld);
}

// interpolation_core.cpp:19 — empty position vectors select the binary search.
void dynref_interpolate(const double* posB1xIn, const double* posB2xIn, int same) {
    const size_t L = config.len;
    std::vector<double> b1 = posB1xIn ? copy_in(posB1xIn, L) : std::vector<double>{};
    std::vector<double> b2 = posB2xIn ? copy_in(posB2xIn, L * L) : std::vector<double>{};
    interpolate(b1, b2, same != 0);
}

// which: 0..7 = QK/QR for A1, A2, B1, B2; 8..15 = SigmaK/SigmaR for A1, A2, B1, B2; 16 = rInt
void dynref_get_interp(int which, double* out) {
    const std::vector<double>* tab[17] = {
        &sim->h_QKA1int, &sim->h_QRA1int, &sim->h_QKA2int, &sim->h_QRA2int,
        &sim->h_QKB1int, &sim->h_QRB1int, &sim->h_QKB2int, &sim->h_QRB2int,
        &sim->h_SigmaKA1int, &sim->h_SigmaRA1int, &sim->h_SigmaKA2int, &sim->h_SigmaRA2int,
        &sim->h_SigmaKB1int, &sim->h_SigmaRB1int, &sim->h_SigmaKB2int, &sim->h_SigmaRB2int,
        &sim->h_rInt};
    if (which < 0 || which > 16) return;
    std::memcpy(out, tab[which]->data(), tab[which]->size() * sizeof(double));
}

void dynref_qkstep(double* out) {
    std::vector<double> v = QKstep();
    std::memcpy(out, v.data(), v.size() * sizeof(double));
}

void dynref_qrstep(double* out) {
    std::vector<double> v = QRstep();
    std::memcpy(out, v.data(), v.size() * sizeof(double));
}

double dynref_rstep(void) { return rstep(); }

double dynref_drstep2(const double* qK, const double* qR, const double* dqK, const double* dqR,
                      double t) {
    const size_t L = config.len;
    return drstep2(copy_in(qK, L), copy_in(qR, L), copy_in(dqK, L), copy_in(dqR, L), t);
}

// CPU energy, simulation_runner.cpp:334-336, evaluated at time t.
double dynref_energy(double t) {
    const size_t L = config.len;
    std::vector<double> q = getLastLenEntries(sim->h_QKv, L);
    std::vector<double> r = getLastLenEntries(sim->h_QRv, L);
    std::vector<double> sk(L, 0.0);
    SigmaK(q, sk);
    return -(ConvA(sk, r, t)[0] + Dflambda(q[0]) / config.T0);
}

std::vector<double> conv_out;

// ConvA/ConvR (convolution.cpp:5-50) on caller arrays; depth = size(f)/L.
void dynref_conv(int kind, const double* f, const double* g, size_t n, double t, double* out) {
    std::vector<double> vf = copy_in(f, n), vg = copy_in(g, n);
    std::vector<double> v = kind == 0 ? ConvA(vf, vg, t) : ConvR(vf, vg, t);
    std::memcpy(out, v.data(), v.size() * sizeof(double));
}

void dynref_bsearch(const double* list, size_t nlist, const double* elem, size_t nelem,
                    double* out) {
    std::vector<double> v = bsearchPosSorted(copy_in(list, nlist), copy_in(elem, nelem));
    std::memcpy(out, v.data(), nelem * sizeof(double));
}

// isearchPosSortedInit scales elem by list.back() itself (search_utils.cpp:77).
void dynref_isearch(const double* list, size_t nlist, const double* elem, size_t nelem,
                    const double* inits, double* out) {
    std::vector<double> v = isearchPosSortedInit(copy_in(list, nlist), copy_in(elem, nelem),
                                                 copy_in(inits, nelem));
    std::memcpy(out, v.data(), nelem * sizeof(double));
}

// One RK step through update() (runge_kutta.cpp:254-261): init 1 = RK54, else SSPRK104.
double dynref_update(int init, double delta_t) {
    rk->init = init;
    config.delta_t = delta_t;
    return update();
}

void dynref_sparsify(double threshold) { sparsifyNscale(threshold); }

// The CPU branch of the driver loop, simulation_runner.cpp:125-278 (no
// rollback on CPU, :280 is GPU-only), run for exactly `nsteps` controller
// iterations.  With `schedule` non-null the step sizes and methods are
// replayed instead of adapted (frozen schedule).  Per step it records the
// step size used, the method, the error estimate and the energy
// (simulation_runner.cpp:334-336) at the loop's own t (:128).
// With sparsify_every > 0 the periodic block of :148-237 (CPU branch: one
// sparsifyNscale pass at delta_max, interpolate(), then the halving with
// rk->init = 2 when delta < delta_max/2; no rollback on the CPU, so the last
// rollback loop stays at its initial -1000, :53).
// With dynref_set_tail_fit(1), tailFitBlendCPU after every update, as the CUDA
// build's loop does when --tail-fit is on (:135-141; the CPU-only build's loop
// has no tail fit).
int dynref_run(int nsteps, const double* schedule_dt, const int* schedule_method,
               double* out_dt, int* out_method, double* out_delta, double* out_t,
               double* out_energy, long long sparsify_every) {
    const size_t L = config.len;
    for (int k = 0; k < nsteps; ++k) {
        if (schedule_dt) {
            config.delta_t = schedule_dt[k];
            rk->init = schedule_method[k];
        }
        const double t = sim->h_t1grid.back() + config.delta_t;
        if (out_dt) out_dt[k] = config.delta_t;
        if (out_method) out_method[k] = rk->init;
        config.delta_old = config.delta;
        config.delta = update();
        if (config.tail_fit_enabled) tailFitBlendCPU();
        config.loop++;
        if (sparsify_every > 0 && config.loop % sparsify_every == 0) {
            sparsifyNscale(config.delta_max);
            interpolate();
            if (!schedule_dt && config.delta < config.delta_max / 2 && config.loop - last_rollback_loop > 1000) {
                config.delta_t *= 0.5;
                rk->init = 2;
            }
        }
        if (!schedule_dt) {
            if (config.delta < config.delta_max && config.loop > 5 &&
                (config.delta < 1.1 * config.delta_old || config.delta_old < config.delta_max / 1000) &&
                config.rmax[rk->init - 1] / config.specRad > config.delta_t &&
                sim->h_delta_t_ratio.back() == 1.0) {
                config.delta_t *= 1.01;
            } else if (config.delta > 2 * config.delta_max && config.delta_t > config.delta_t_min) {
                config.delta_t *= 0.9;
            }
            if (rk->init == 2 && config.delta > config.delta_max &&
                config.rmax[0] / config.specRad > config.delta_t) {
                rk->init = 1;
                config.delta_t *= 0.5;
            }
        }
        if (out_delta) out_delta[k] = config.delta;
        if (out_t) out_t[k] = t;
        if (out_energy) {
            const size_t n = sim->h_t1grid.size();
            double qk0 = sim->h_QKv[(n - 1) * L];
            std::vector<double> sk(L, 0.0);
            SigmaK(getLastLenEntries(sim->h_QKv, L), sk);
            out_energy[k] = -(ConvA(sk, getLastLenEntries(sim->h_QRv, L), t)[0] + Dflambda(qk0) / config.T0);
        }
    }
    return 0;
}

double dynref_get_delta_t(void) { return config.delta_t; }
int dynref_get_method(void) { return rk->init; }
double dynref_spec_rad(void) { return config.specRad; }

// SERK coefficient solver (runge_kutta.cu:228-272 is GPU-build only; the
// host version is in the same .cu file, so it is not available here).

// Grid generation: the same calls and post-processing as grid_cli.cpp:78-215
// (poly method), returning the values the solver reads back from the files.
// grid_cli.cpp:84-215 for -m poly (fh_window < 0) or -m rational (window size
// min(len, max(n + 1, fh_window)), fh_window 0: n + 1); weights hold that depth
int dynref_grid_method(size_t len, double Tmax, int spline_order, int interp_order, int fh_window, double alpha,
                       double delta, double* theta, double* phi1, double* phi2, double* integ,
                       int64_t* indsA1, double* wA1, int64_t* indsA2, double* wA2, int64_t* indsB2,
                       double* wB2);

// generate_pos_grids (pos_grid.cpp:111-205) on the generator's theta and phi grids
int dynref_grid_positions(size_t len, double Tmax, double alpha, double delta, double* posA1y, double* posA2y,
                          double* posB2y) {
    std::vector<long double> th, p1, p2;
    generate_theta_grid(len, Tmax, th, alpha, delta);
    generate_phi_grids(th, p1, p2);
    std::vector<double> a1, a2, b2;
    generate_pos_grids(len, Tmax, th, p1, p2, a1, a2, b2, alpha, delta);
    std::copy(a1.begin(), a1.end(), posA1y);
    std::copy(a2.begin(), a2.end(), posA2y);
    std::copy(b2.begin(), b2.end(), posB2y);
    return 0;
}

int dynref_grid(size_t len, double Tmax, int spline_order, int interp_order, double alpha,
                double delta, double* theta, double* phi1, double* phi2, double* integ,
                int64_t* indsA1, double* wA1, int64_t* indsA2, double* wA2, int64_t* indsB2,
                double* wB2) {
    return dynref_grid_method(len, Tmax, spline_order, interp_order, -1, alpha, delta, theta, phi1, phi2, integ,
                              indsA1, wA1, indsA2, wA2, indsB2, wB2);
}

int dynref_grid_method(size_t len, double Tmax, int spline_order, int interp_order, int fh_window, double alpha,
                       double delta, double* theta, double* phi1, double* phi2, double* integ,
                       int64_t* indsA1, double* wA1, int64_t* indsA2, double* wA2, int64_t* indsB2,
                       double* wB2) {
    std::vector<long double> th;
    generate_theta_grid(len, Tmax, th, alpha, delta);
    std::vector<long double> p1, p2;
    generate_phi_grids(th, p1, p2);
    std::vector<long double> wint;
    compute_integration_weights(th, spline_order, wint);
    const size_t N = len;
    const int n = interp_order < 1 ? 1 : interp_order;
    const bool rational = fh_window >= 0;
    const int mfh = (int)std::min<size_t>(N, (size_t)std::max(n + 1, fh_window > 0 ? fh_window : n + 1));
    const int m = rational ? mfh : n + 1;
    auto weights = [&](const std::vector<long double>& q) {
        return rational ? dmfe::grid::compute_barycentric_rational_weights(th, q, n, mfh)
                        : dmfe::grid::compute_barycentric_weights(th, q, n);
    };
    for (size_t i = 0; i < N; ++i) theta[i] = static_cast<double>(th[i]);
    for (size_t i = 0; i < N; ++i) integ[i] = static_cast<double>(wint[i]);
    for (size_t k = 0; k < N * N; ++k) {
        phi1[k] = text_round_trip(p1[k]);
        phi2[k] = text_round_trip(p2[k]);
    }
    auto st1 = weights(p1);
    auto st2 = weights(p2);
    const double tiny = 1e-200;
    std::vector<long double> xqB2;
    xqB2.reserve(N * N);
    for (size_t i = 0; i < N; ++i) {
        const long double ti = th[i];
        for (size_t j = 0; j < N; ++j) {
            const long double denom = p2[i * N + j] - tiny;
            long double arg;
            if (std::fabs(denom) < 1e-300L) arg = (ti > 0) ? th.back() : th.front();
            else arg = ti / denom;
            xqB2.push_back(arg);
        }
    }
    auto st3 = weights(xqB2);
    for (size_t k = 0; k < N * N; ++k) {
        indsA1[k] = st1[k].start;
        indsA2[k] = st2[k].start;
        indsB2[k] = st3[k].start;
        for (int j = 0; j < m; ++j) {
            wA1[k * m + j] = st1[k].alpha[j];
            wA2[k * m + j] = st2[k].alpha[j];
            wB2[k * m + j] = st3[k].alpha[j];
        }
    }
    return 0;
}

}  // extern "C"
