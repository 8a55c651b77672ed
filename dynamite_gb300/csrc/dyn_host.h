// Host-side constants and helpers shared by the single-quench context
// (dyn_api.cu) and the batched quenches (dyn_batch.cu): the RK tableaux,
// the step-size limits and the model's f', f'' in the reference's host
// expression order.
#pragma once
#include <nvtx3/nvToolsExt.h>
#include <cstdlib>
#include <string>
#include <vector>
#include "../../include/dyn.h"

namespace dyn {

// A named NVTX range over one host call or one step, for Nsight timelines and
// `ncu --nvtx` filters.  Off unless the environment sets DYN_NVTX=1 (read once).
inline bool trace_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("DYN_NVTX");
        return e && e[0] == '1';
    }();
    return on;
}
struct TraceRange {
    const bool on;
    explicit TraceRange(const char* name) : on(trace_enabled()) {
        if (on) nvtxRangePushA(name);
    }
    ~TraceRange() {
        if (on) nvtxRangePop();
    }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

// rmax (config.hpp:33): stability radius of method m is RMAX[m-1] / specRad
inline constexpr double RMAX[11] = {3, 13, 20, 80, 180, 320, 500, 720, 980, 1280, 1620};

// Dormand-Prince tableau (runge_kutta.cpp:149-159)
inline constexpr double RK54_A[7][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {1.0 / 5, 0, 0, 0, 0, 0, 0},
    {3.0 / 40, 9.0 / 40, 0, 0, 0, 0, 0},
    {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0, 0, 0},
    {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0, 0, 0},
    {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656, 0, 0},
    {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84, 0}};
inline constexpr double RK54_B[7] = {35.0 / 384, 0.0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84, 0.0};
inline constexpr double RK54_B2[7] = {5179.0 / 57600, 0.0, 7571.0 / 16695, 393.0 / 640, -92097.0 / 339200, 187.0 / 2100, 1.0 / 40};

// SSPRK(10,4) tableau (runge_kutta.cpp:22-35)
inline double ssp_a(int r, int c) {
    if (c >= r) return 0.0;
    return (r <= 4 || c >= 5) ? 1.0 / 6 : 1.0 / 15;
}
inline constexpr double SSP_B[10] = {1.0 / 10, 1.0 / 10, 1.0 / 10, 1.0 / 10, 1.0 / 10,
                                     1.0 / 10, 1.0 / 10, 1.0 / 10, 1.0 / 10, 1.0 / 10};
inline constexpr double SSP_B2[10] = {0., 2.0 / 9, 0, 0, 5.0 / 18, 1.0 / 3, 0., 0., 0., 1.0 / 6};

// SERK2(q) combination coefficients b[0..2q] (runge_kutta.cu:202-272), long double solve
std::vector<double> serk_coeffs(int q);

// Sparsify passes of one periodic block (simulation_runner.cpp:163-183, 187):
// requested < 0 is the reference's "auto" (2 when more than half of the
// device's memory is in use, else 1), 0 none, otherwise at most 10
int sparsify_block_sweeps(int requested);

// pow_int (math_ops.cpp:7-21) on the host
inline double pow_int_h(double b, int e) {
    if (e == 0) return 1.0;
    if (e == 1) return b;
    if (e == 2) return b * b;
    if (e == 3) return b * b * b;
    if (e == 4) { double sq = b * b; return sq * sq; }
    double r = 1.0, c = b;
    while (e > 0) { if (e & 1) r *= c; c *= c; e >>= 1; }
    return r;
}

// Dflambda / DDflambda (math_ops.cpp:27-37)
inline double Df_host(double lambda, int p, int p2, double q) {
    return lambda * p * pow_int_h(q, p - 1) + (1 - lambda) * p2 * pow_int_h(q, p2 - 1);
}
inline double DDf_host(double lambda, int p, int p2, double q) {
    return lambda * p * (p - 1) * pow_int_h(q, p - 2) + (1 - lambda) * p2 * (p2 - 1) * pow_int_h(q, p2 - 2);
}

void set_last_error(const std::string& msg);

// Validates a table set and returns the stencil starts as int32 (dyn_api.cu)
bool check_tables(size_t L, size_t m, const dyn_tables* tb, std::vector<int> i32[3], std::string& why);
bool check_model(int p, int p2, double lambda, double T0, double Gamma, std::string& why);

// Keep list, derivative rows with their time factors, and the new t1grid /
// delta_t_ratio of one sparsify pass from its node flags (dyn_api.cu); false
// when variant 0 erases nothing
bool sparsify_indices(const unsigned char* fl, size_t n, int variant, const std::vector<double>& t1,
                      const std::vector<double>& dtr, std::vector<int>& inds, std::vector<int>& indsD,
                      std::vector<double>& tfac, std::vector<double>& t1n, std::vector<double>& dtrn);

}  // namespace dyn
