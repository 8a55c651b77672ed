// Test infrastructure: drives the host-side sparsifyNscale of the reference's
// CUDA build (sparsify_utils.cu:38-113, the "cuda_host" variant), compiled from
// the reference's own source file, on a caller-given history.  Only host code
// runs; no GPU is needed.
#include <cstddef>
#include <cstring>
#include <vector>

#include "core/config.hpp"
#include "simulation/simulation_data.hpp"
#include "sparsify/sparsify_utils.hpp"

SimulationConfig config;
SimulationData* sim = nullptr;

extern "C" {

// history in (n rows of len); compacted history out (the caller's arrays hold n rows)
int dynref_sparsify_cudahost(size_t n, size_t len, const double* t1grid, const double* dtr, const double* QK,
                             const double* QR, const double* dQK, const double* dQR, const double* rvec,
                             const double* drvec, double threshold, size_t* n_out, double* t1o, double* dtro,
                             double* QKo, double* QRo, double* dQKo, double* dQRo, double* ro, double* dro) {
    if (!sim) sim = new SimulationData();  // empty device vectors: nothing touches the GPU
    config.len = len;
    sim->h_t1grid.assign(t1grid, t1grid + n);
    sim->h_delta_t_ratio.assign(dtr, dtr + n);
    sim->h_QKv.assign(QK, QK + n * len);
    sim->h_QRv.assign(QR, QR + n * len);
    sim->h_dQKv.assign(dQK, dQK + n * len);
    sim->h_dQRv.assign(dQR, dQR + n * len);
    sim->h_rvec.assign(rvec, rvec + n);
    sim->h_drvec.assign(drvec, drvec + n);
    sparsifyNscale(threshold);
    const size_t k = sim->h_t1grid.size();
    *n_out = k;
    std::memcpy(t1o, sim->h_t1grid.data(), k * sizeof(double));
    std::memcpy(dtro, sim->h_delta_t_ratio.data(), k * sizeof(double));
    std::memcpy(QKo, sim->h_QKv.data(), k * len * sizeof(double));
    std::memcpy(QRo, sim->h_QRv.data(), k * len * sizeof(double));
    std::memcpy(dQKo, sim->h_dQKv.data(), k * len * sizeof(double));
    std::memcpy(dQRo, sim->h_dQRv.data(), k * len * sizeof(double));
    std::memcpy(ro, sim->h_rvec.data(), k * sizeof(double));
    std::memcpy(dro, sim->h_drvec.data(), k * sizeof(double));
    return 0;
}

}  // extern "C"
