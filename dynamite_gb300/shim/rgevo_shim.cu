// RG-Evo's hot-path symbols on top of libdynamite_gb300 (include/dyn.h).
//
// Drop-in layer for the reference driver: built inside an RG-Evo tree (it
// includes the reference's own headers for SimulationData, RKData,
// SimulationConfig and StreamPool) in place of the hot-path CUDA sources
// src/{interpolation,convolution,EOMs,search,sparsify}/*.cu and
// src/math/{math_ops,math_sigma}.cu (CMakeLists.txt:184-202).  It defines
// exactly the symbols the rest of RG-Evo calls from those files:
//
//   interpolateGPU     interpolation_core.hpp:20-23   (simulation_runner.cpp:212,477,
//                                                       initialization.cpp:274,
//                                                       simulation_control.cpp:54)
//   updateGPU, RK54GPU, SSPRK104GPU, SERK2GPU, init_RK54GPU, init_SSPRK104GPU,
//   init_SERK2         runge_kutta.hpp:23-37           (simulation_runner.cpp:134, 222-229, ...)
//   energyGPU          time_steps.hpp:176-182          (simulation_runner.cpp:330, io/*)
//   sparsifyNscaleGPU, sparsifyNscale
//                      sparsify_utils.hpp:17-24        (simulation_runner.cpp:195)
//   DflambdaGPU        math_ops.hpp:46 (device)        (io_output.cu:61-122)
//
// State: one library context holds the two-time history, the tables and the
// scratch; RG-Evo's thrust vectors in `sim` stay the record the rest of the
// driver reads (printing, saves, rollback, the energy log).  Every call first
// brings the context in line with `sim` (a full upload when the history's
// length or last time changed behind its back -- rollbackState, a loaded
// checkpoint, the CPU path -- and the newest row again in any case, since the
// tail fit edits it in place), runs, and writes what changed back into `sim`
// (the new row, the compacted history, the interpolation arrays).  After a
// step the B1 pair sim->d_QKB1int / d_QRB1int is refreshed, as the
// reference's closing interpolation leaves it for the compressed saves; the
// other fourteen interpolation arrays are filled by interpolateGPU only (no
// part of RG-Evo outside the hot path reads them).
//
// Arithmetic: the plain FP64 form of the library with the reference CUDA
// path's lower-bound position search (search_utils.cu:71-112).  Errors
// abort with the library's message, as RG-Evo's own CUDA error checks do.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>
#include <thrust/device_vector.h>

#include "core/config.hpp"
#include "core/device_constants.hpp"
#include "core/globals.hpp"
#include "core/stream_pool.hpp"
#include "EOMs/rk_data.hpp"
#include "EOMs/runge_kutta.hpp"
#include "EOMs/time_steps.hpp"
#include "interpolation/interpolation_core.hpp"
#include "math/math_ops.hpp"
#include "simulation/simulation_data.hpp"
#include "sparsify/sparsify_utils.hpp"

#include "dyn.h"

extern SimulationConfig config;

namespace {

void* g_ctx = nullptr;
size_t g_n = 0;      // rows of sim's history the context last agreed with
double g_t = -1.0;   // and the time of the newest of them

void check(int status, const char* what) {
    if (status == DYN_OK) return;
    std::fprintf(stderr, "dynamite_gb300 drop-in: %s failed (status %d): %s\n", what, status, dyn_last_error());
    std::abort();
}

double* raw(thrust::device_vector<double>& v) { return thrust::raw_pointer_cast(v.data()); }

dyn_state_dev sim_state() {
    dyn_state_dev s;
    s.n = sim->d_t1grid.size();
    s.t1grid = raw(sim->d_t1grid);
    s.delta_t_ratio = raw(sim->d_delta_t_ratio);
    s.QK = raw(sim->d_QKv);
    s.QR = raw(sim->d_QRv);
    s.dQK = raw(sim->d_dQKv);
    s.dQR = raw(sim->d_dQRv);
    s.rvec = raw(sim->d_rvec);
    s.drvec = raw(sim->d_drvec);
    return s;
}

// The context, created on first use from the run's configuration and the
// tables import() left in sim's host vectors (io_input.cpp:90-110)
void* ctx() {
    if (g_ctx) return g_ctx;
    const size_t L = config.len, L2 = L * L;
    dyn_config cfg{};
    cfg.p = config.p;
    cfg.p2 = config.p2;
    cfg.lambda = config.lambda;
    cfg.T0 = config.T0;
    cfg.Gamma = config.Gamma;
    cfg.len = L;
    cfg.depth = sim->h_weightsA1y.size() / L2;
    cfg.delta_t_min = config.delta_t_min;
    cfg.delta_max = config.delta_max;
    cfg.precision = DYN_FP64;
    cfg.search = DYN_SEARCH_LOWER_BOUND;
    cfg.device = 0;
    cudaGetDevice(&cfg.device);
    cfg.use_graph = 1;
    cfg.log_response = config.log_response_interp ? 1 : 0;
    std::vector<int64_t> i1(sim->h_indsA1y.begin(), sim->h_indsA1y.end());
    std::vector<int64_t> i2(sim->h_indsA2y.begin(), sim->h_indsA2y.end());
    std::vector<int64_t> i3(sim->h_indsB2y.begin(), sim->h_indsB2y.end());
    dyn_tables tb{sim->h_theta.data(), sim->h_phi2.data(), sim->h_integ.data(), i1.data(), i2.data(), i3.data(),
                  sim->h_weightsA1y.data(), sim->h_weightsA2y.data(), sim->h_weightsB2y.data()};
    check(dyn_ctx_create(&cfg, &tb, &g_ctx), "dyn_ctx_create");
    g_n = 0;
    g_t = -1.0;
    return g_ctx;
}

// Bring the context in line with sim's device history
void sync_from_sim() {
    void* c = ctx();
    dyn_state_dev st = sim_state();
    const double t = st.n ? static_cast<double>(sim->d_t1grid.back()) : -1.0;
    if (st.n != g_n || t != g_t) {
        check(dyn_state_upload_dev(c, &st), "dyn_state_upload_dev");
        g_n = st.n;
        g_t = t;
    } else {
        check(dyn_state_rows_load_dev(c, st.n - 1, 1, &st), "dyn_state_rows_load_dev");
    }
}

void resize_history(size_t n) {
    const size_t L = config.len;
    for (auto* v : {&sim->d_QKv, &sim->d_QRv, &sim->d_dQKv, &sim->d_dQRv}) v->resize(n * L);
    for (auto* v : {&sim->d_t1grid, &sim->d_delta_t_ratio, &sim->d_rvec, &sim->d_drvec}) v->resize(n);
}

void refresh_b1() {
    const size_t L2 = config.len * config.len;
    sim->d_QKB1int.resize(L2);
    sim->d_QRB1int.resize(L2);
    check(dyn_interp_b1_dev(ctx(), raw(sim->d_QKB1int), raw(sim->d_QRB1int)), "dyn_interp_b1_dev");
}

// One RK step of `method` (rk->init numbering) with config.delta_t; the new
// row is appended to sim's history (appendAllGPU_ptr, time_steps.cu:766-919)
double step(int method) {
    sync_from_sim();
    dyn_step_result r{};
    check(dyn_update(ctx(), method, config.delta_t, &r), "dyn_update");
    const size_t n = g_n + 1;
    resize_history(n);
    dyn_state_dev st = sim_state();
    check(dyn_state_rows_store_dev(ctx(), n - 1, 1, &st), "dyn_state_rows_store_dev");
    refresh_b1();
    g_n = n;
    g_t = r.t;
    return r.delta;
}

// fast integer power for DflambdaGPU: q^e by squaring, 1 for e <= 0
__device__ __forceinline__ double ipow(double q, int e) {
    double r = 1.0;
    while (e > 0) {
        if (e & 1) r *= q;
        q *= q;
        e >>= 1;
    }
    return r;
}

}  // namespace

// ------------------------------------------------ runge_kutta.hpp:23-37
double RK54GPU(StreamPool*) { return step(DYN_RK54); }
double SSPRK104GPU(StreamPool*) { return step(DYN_SSPRK104); }
double SERK2GPU(int q, StreamPool*) { return step(2 + q / 2); }
double updateGPU(StreamPool*) { return step(rk->init >= 1 ? rk->init : DYN_RK54); }

// The method switches of the driver loop: the library keeps its own tableaux
// and scratch, so only the selection is recorded (runge_kutta.cu:71-297)
void init_RK54GPU() {
    rk->init = DYN_RK54;
    rk->stages = 7;
}
void init_SSPRK104GPU() {
    rk->init = DYN_SSPRK104;
    rk->stages = 10;
    rk->posCount = 3;
}
void init_SERK2(int q) {
    rk->init = 2 + q / 2;
    rk->stages = 2 * q;
}

// ------------------------------------------- interpolation_core.hpp:20-23
// The reference's GPU form searches the positions itself whatever posB1xIn,
// posB2xIn and same say (interpolation_core.cu:63-81); so does this one.
void interpolateGPU(const double*, const double*, const bool, StreamPool*) {
    sync_from_sim();
    void* c = ctx();
    check(dyn_interpolate(c, nullptr, nullptr), "dyn_interpolate");
    const size_t L = config.len, L2 = L * L;
    thrust::device_vector<double>* arrays[16] = {
        &sim->d_QKA1int, &sim->d_QRA1int, &sim->d_QKA2int, &sim->d_QRA2int,
        &sim->d_QKB1int, &sim->d_QRB1int, &sim->d_QKB2int, &sim->d_QRB2int,
        &sim->d_SigmaKA1int, &sim->d_SigmaRA1int, &sim->d_SigmaKA2int, &sim->d_SigmaRA2int,
        &sim->d_SigmaKB1int, &sim->d_SigmaRB1int, &sim->d_SigmaKB2int, &sim->d_SigmaRB2int};
    for (int w = 0; w < 16; ++w) {
        arrays[w]->resize(L2);
        check(dyn_get_interp_dev(c, w, raw(*arrays[w])), "dyn_get_interp_dev");
    }
    sim->d_rInt.resize(L);
    sim->d_posB1xOld.resize(L);
    sim->d_posB2xOld.resize(L2);
    check(dyn_get_interp_dev(c, DYN_RINT, raw(sim->d_rInt)), "dyn_get_interp_dev");
    check(dyn_get_interp_dev(c, DYN_POSB1X, raw(sim->d_posB1xOld)), "dyn_get_interp_dev");
    check(dyn_get_interp_dev(c, DYN_POSB2X, raw(sim->d_posB2xOld)), "dyn_get_interp_dev");
}

// ------------------------------------------------ time_steps.hpp:176-182
// E of sim's newest row; the arguments are sim's own vectors at every call
// site of RG-Evo (simulation_runner.cpp:330, io_output.cpp, io_save_params.cpp)
double energyGPU(const thrust::device_vector<double>& QKv, const thrust::device_vector<double>&,
                 const thrust::device_vector<double>&, const thrust::device_vector<double>&,
                 const thrust::device_vector<double>&, double T0) {
    if (&QKv != &sim->d_QKv || T0 != config.T0) {
        std::fprintf(stderr, "dynamite_gb300 drop-in: energyGPU takes the run's own history and T0\n");
        std::abort();
    }
    sync_from_sim();
    double e = 0.0;
    check(dyn_energy(ctx(), &e), "dyn_energy");
    return e;
}

// --------------------------------------------- sparsify_utils.hpp:17-24
// The GPU path's sparsify (sparsify_utils.cu:154-290: even-index flags, tfac
// rescaling), sim's history compacted in place
void sparsifyNscaleGPU(double threshold, cudaStream_t) {
    sync_from_sim();
    size_t k = 0;
    check(dyn_sparsify(ctx(), threshold, DYN_SPARSIFY_GPU, &k), "dyn_sparsify");
    resize_history(k);
    dyn_state_dev st = sim_state();
    check(dyn_state_rows_store_dev(ctx(), 0, k, &st), "dyn_state_rows_store_dev");
    g_n = k;
    g_t = sim->d_t1grid.back();
}

// The CUDA build's host-side sparsify of the CPU path (sparsify_utils.cu:38-113,
// used when RG-Evo runs with -g false): sim's host history through the library
// and back
void sparsifyNscale(double threshold) {
    void* c = ctx();
    const size_t L = config.len, n = sim->h_t1grid.size();
    dyn_state st{n, sim->h_t1grid.data(), sim->h_delta_t_ratio.data(), sim->h_QKv.data(), sim->h_QRv.data(),
                 sim->h_dQKv.data(), sim->h_dQRv.data(), sim->h_rvec.data(), sim->h_drvec.data()};
    check(dyn_state_upload(c, &st), "dyn_state_upload");
    size_t k = 0;
    check(dyn_sparsify(c, threshold, DYN_SPARSIFY_CUDA_HOST, &k), "dyn_sparsify");
    for (auto* v : {&sim->h_QKv, &sim->h_QRv, &sim->h_dQKv, &sim->h_dQRv}) v->resize(k * L);
    for (auto* v : {&sim->h_t1grid, &sim->h_delta_t_ratio, &sim->h_rvec, &sim->h_drvec}) v->resize(k);
    dyn_state out{k, sim->h_t1grid.data(), sim->h_delta_t_ratio.data(), sim->h_QKv.data(), sim->h_QRv.data(),
                  sim->h_dQKv.data(), sim->h_dQRv.data(), sim->h_rvec.data(), sim->h_drvec.data()};
    check(dyn_state_download(c, &out), "dyn_state_download");
    g_n = 0;  // the device history is sim's again from here on
    g_t = -1.0;
}

// ---------------------------------------------------- math_ops.hpp:46
// f'(q) = lambda p q^(p-1) + (1 - lambda) p2 q^(p2-1) with the run's model in
// constant memory (device_constants.cu:4-6); the save-time energy history
// kernel (io_output.cu:61-122) calls it
__device__ double DflambdaGPU(double q) {
    return d_lambda * d_p * ipow(q, d_p - 1) + (1 - d_lambda) * d_p2 * ipow(q, d_p2 - 1);
}
