// Test infrastructure: exposes SERKcoeffs (runge_kutta.cu:228-272) of the
// reference's CUDA build, compiled from the reference's own source file, so the
// oracle's SERK2(q) weights can be compared with it.  Only that host function
// runs; no GPU is needed.  runge_kutta.cu also references the driver's globals
// and, from its GPU steppers, a few kernels (by address, for their launches): they
// are defined here so the library loads.  The host functions those steppers call
// (interpolateGPU, QKRstepGPU, ...) stay unresolved: the library is loaded with
// lazy binding and none of them is ever called.
#include <cstddef>
#include <vector>

#include "core/compute_utils.hpp"
#include "core/config.hpp"
#include "core/globals.hpp"
#include "EOMs/runge_kutta.hpp"

SimulationConfig config;
SimulationData* sim = nullptr;
RKData* rk = nullptr;

__global__ void computeScale(double*, double, size_t) {}
__global__ void computeMA(double*, const double*, double, size_t) {}
__global__ void computeMAD(double*, const double*, const double*, double, size_t) {}
__global__ void computeWeightedSum(const double* __restrict__, const double* __restrict__, const double* __restrict__,
                                   double* __restrict__, double, int, size_t) {}

extern "C" int dynref_serk_coeffs(int q, double* out) {
    const std::vector<double> b = SERKcoeffs(q);
    for (size_t i = 0; i < b.size(); ++i) out[i] = b[i];
    return (int)b.size();
}
