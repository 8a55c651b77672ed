// dyn_rhs_noalloc: the fused right-hand side without any device allocation.
//
// Who needs this: callers that must not call cudaMalloc after start-up —
// a host driver that runs inside a memory-capped or pre-partitioned device
// pool it does not own, code that records work while another library owns
// the allocator, or a process that has already handed all free device memory
// to its history buffers.  Such a caller passes its own device buffers for
// the tables, the history and the output; the scratch the two stage kernels
// need (row partial sums, epilogue partials, row values, positions, 1/ratio
// table, the stage descriptor, the reduction ticket) lives in one
// file-scope __device__ array of fixed size, allocated when the library is
// loaded and held by every GPU that loads it until the process exits.
//
// Limits: 4 <= len <= DYN_NOALLOC_MAX_LEN (1024), 2 <= history rows <=
// DYN_NOALLOC_MAX_ROWS (16384), 2 <= stencil depth <= len; the array is
// DYN_NOALLOC_SCRATCH_BYTES (448 KiB).  The device tables are not read on
// the host, so their stencil starts are the caller's to keep within
// [0, len - depth] (dyn_check_tables checks host copies).
//
// Set-up: the first call on a device looks up the device address of the
// array (cudaGetSymbolAddress, with that device current) and caches it for
// that device for the rest of the process (a cudaDeviceReset of that device
// would leave the cached address stale); make that first call before any
// stream capture.  All calls share the one array and it keeps the last
// call's contents; the parts that must start at zero are cleared by every
// call.  Two calls whose kernels
// overlap on the GPU (different streams, or different host threads on the
// same device) race on the array: serialize them.
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/dyn.h"
#include "dyn_kernels.cuh"

using namespace dyn;

namespace dyn {
void set_last_error(const std::string& msg);  // dyn_api.cu: the text dyn_last_error() returns
}

namespace {

constexpr int MAX_LEN = DYN_NOALLOC_MAX_LEN;
constexpr int MAX_ROWS = DYN_NOALLOC_MAX_ROWS;
constexpr int TPB = 64;
constexpr int MAX_NCH = 4;  // chunks per row for the tile shapes chosen below (<= 4 for len <= 1024)
constexpr int MAX_G = (MAX_LEN + EPI_ROWS - 1) / EPI_ROWS;

// scratch layout, in doubles
constexpr size_t OFF_PART = 0;
constexpr size_t N_PART = (size_t)MAX_LEN * MAX_NCH * 8;
constexpr size_t OFF_EPART = OFF_PART + N_PART;
constexpr size_t N_EPART = (size_t)MAX_G * EP_N;
constexpr size_t OFF_ROWVAL = OFF_EPART + N_EPART;        // double2[MAX_LEN]
constexpr size_t OFF_H = OFF_ROWVAL + 2 * (size_t)MAX_LEN; // double2[MAX_LEN]
constexpr size_t OFF_POS = OFF_H + 2 * (size_t)MAX_LEN;    // double[MAX_LEN]
constexpr size_t OFF_INV = OFF_POS + MAX_LEN;              // double[MAX_ROWS]
constexpr size_t OFF_SLOTS = OFF_INV + MAX_ROWS;           // Slots, rounded up
constexpr size_t N_SLOTS = (sizeof(Slots) + 7) / 8 + 8;
constexpr size_t OFF_STAGE = OFF_SLOTS + N_SLOTS;          // StageDev
constexpr size_t N_STAGE = (sizeof(StageDev) + 7) / 8 + 8;
constexpr size_t N_TOTAL = OFF_STAGE + N_STAGE;
constexpr size_t N_ARRAY = DYN_NOALLOC_SCRATCH_BYTES / sizeof(double);
static_assert(N_TOTAL <= N_ARRAY, "the scratch layout outgrows DYN_NOALLOC_SCRATCH_BYTES");
static_assert(N_ARRAY * sizeof(double) == DYN_NOALLOC_SCRATCH_BYTES, "whole doubles");

__device__ __align__(256) double g_noalloc_scratch[N_ARRAY];

std::mutex g_mu;
double* g_addr[64] = {nullptr};

dyn_status err(dyn_status s, const char* what, cudaError_t e = cudaSuccess) {
    std::string m(what);
    if (e != cudaSuccess) m += std::string(": ") + cudaGetErrorString(e);
    dyn::set_last_error(m);
    return s;
}

__global__ void k_noalloc_prep(double* inv, const double* dtr, const double* t1grid, int n, StageDev* sp,
                               Slots* slots) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        inv[k] = dtr[k] != 0.0 ? 1.0 / dtr[k] : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        StageDev z;
        memset(&z, 0, sizeof z);
        z.kind = KIND_RHS;
        z.nrows = n;
        z.n0 = n;
        z.T = t1grid[n - 1];
        z.maxceil = n - 1 < 1 ? 1 : n - 1;  // as Ctx::set_clamps
        z.maxX = n - 1;
        z.b2_save = z.b2_reuse = z.pos_save = z.pos_reuse = z.nb2_save = z.nb2_reuse = -1;
        *sp = z;
        slots->counter = 0;
    }
}

}  // namespace

extern "C" dyn_status dyn_rhs_noalloc(const dyn_noalloc_rhs* a, void* stream) {
    if (!a) return err(DYN_ERR_INVALID, "dyn_rhs_noalloc: null argument");
    if (a->len < 4 || a->len > (size_t)MAX_LEN)
        return err(DYN_ERR_INVALID, "dyn_rhs_noalloc: len must be in [4, DYN_NOALLOC_MAX_LEN=1024]");
    // at least two rows: the B1/B2 clamps of a one-row history point at row 1
    if (a->rows < 2 || a->rows > (size_t)MAX_ROWS)
        return err(DYN_ERR_INVALID, "dyn_rhs_noalloc: rows must be in [2, DYN_NOALLOC_MAX_ROWS=16384]");
    if (a->depth < 2 || a->depth > a->len) return err(DYN_ERR_INVALID, "dyn_rhs_noalloc: bad stencil depth");
    if (a->search != DYN_SEARCH_BINARY && a->search != DYN_SEARCH_LOWER_BOUND)
        return err(DYN_ERR_INVALID, "dyn_rhs_noalloc: search must be DYN_SEARCH_BINARY or DYN_SEARCH_LOWER_BOUND");
    if (!a->theta || !a->phi2 || !a->integ || !a->indsA1y || !a->indsA2y || !a->indsB2y || !a->weightsA1y ||
        !a->weightsA2y || !a->weightsB2y || !a->KR || !a->dKR || !a->t1grid || !a->delta_t_ratio || !a->rvec ||
        !a->drvec || !a->out)
        return err(DYN_ERR_INVALID, "dyn_rhs_noalloc: null device pointer");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return err(DYN_ERR_CUDA, "cudaGetDevice", e);
    if (dev < 0 || dev >= 64) return err(DYN_ERR_INVALID, "dyn_rhs_noalloc: device ordinal above 63");
    double* base;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return err(DYN_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch)", e);
            g_addr[dev] = static_cast<double*>(p);
        }
        base = g_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    DevCtx c;
    std::memset(&c, 0, sizeof c);
    const int L = (int)a->len;
    c.L = L;
    c.m = (int)a->depth;
    c.search = a->search;
    c.tpb = TPB;
    c.kpt = L >= 512 ? 4 : (L >= 256 ? 2 : 1);
    c.nch = (L + c.tpb * c.kpt - 1) / (c.tpb * c.kpt);
    DModel& M = c.M;
    M.p = a->p;
    M.p2 = a->p2;
    M.cA = a->lambda * a->p;
    M.cB = (1 - a->lambda) * a->p2;
    M.cC = a->lambda * a->p * (a->p - 1);
    M.cD = (1 - a->lambda) * a->p2 * (a->p2 - 1);
    M.cE = a->lambda * a->p * (a->p - 1) * (a->p - 2);
    M.cF = (1 - a->lambda) * a->p2 * (a->p2 - 1) * (a->p2 - 2);
    M.T0 = a->T0;
    M.Gamma = a->Gamma;
    c.theta = a->theta;
    c.phi2 = a->phi2;
    c.integ = a->integ;
    c.iA1 = a->indsA1y;
    c.iA2 = a->indsA2y;
    c.iB2 = a->indsB2y;
    c.wA1 = a->weightsA1y;
    c.wA2 = a->weightsA2y;
    c.wB2 = a->weightsB2y;
    c.KR = reinterpret_cast<double2*>(const_cast<double*>(a->KR));
    c.dKR = reinterpret_cast<double2*>(const_cast<double*>(a->dKR));
    c.t1grid = const_cast<double*>(a->t1grid);
    c.dtr = const_cast<double*>(a->delta_t_ratio);
    c.rvec = const_cast<double*>(a->rvec);
    c.drvec = const_cast<double*>(a->drvec);
    c.part = base + OFF_PART;
    c.epart = base + OFF_EPART;
    c.rowval = reinterpret_cast<double2*>(base + OFF_ROWVAL);
    c.h = reinterpret_cast<double2*>(base + OFF_H);
    c.posB1x = base + OFF_POS;
    c.inv_dtr = base + OFF_INV;
    c.slots = reinterpret_cast<Slots*>(base + OFF_SLOTS);
    c.stages = reinterpret_cast<StageDev*>(base + OFF_STAGE);
    c.rhs_out = reinterpret_cast<double2*>(a->out);

    const int n = (int)a->rows;
    if (c.nch > MAX_NCH) return err(DYN_ERR_INVALID, "dyn_rhs_noalloc: tile shape exceeds the scratch layout");
    k_noalloc_prep<<<(n + 255) / 256, 256, 0, st>>>(c.inv_dtr, c.dtr, c.t1grid, n, c.stages, c.slots);
    if ((e = cudaGetLastError()) != cudaSuccess) return err(DYN_ERR_CUDA, "k_noalloc_prep", e);
    if ((e = launch_pos_init(c, n, st)) != cudaSuccess) return err(DYN_ERR_CUDA, "positions", e);
    if ((e = launch_stage(c, 0, st)) != cudaSuccess) return err(DYN_ERR_CUDA, "stage kernels", e);
    return DYN_OK;
}
