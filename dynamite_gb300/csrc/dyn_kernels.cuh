// Kernel-side structures shared by dyn_kernels.cu and dyn_api.cu.
#pragma once
#include <atomic>
#include <cstddef>
#include <cuda_runtime.h>
#include "dyn_common.cuh"

namespace dyn {

constexpr int SMAX = 32;      // most stages of one step (SERK2 with q <= 16)
constexpr int NSAVE = 3;      // SSPRK(10,4) keeps positions of stages 2..4
constexpr int EPI_T = 32;     // threads per epilogue CTA (one warp)
constexpr int EPI_ROWS = 32;  // rows per epilogue CTA (one row per lane; spreading rows over
                              // more SMs did not shorten its FP64 dependency chain)
constexpr int EP_N = 16;      // per-CTA epilogue partials

enum StageKind { KIND_TABLEAU = 0, KIND_SERK = 1, KIND_RHS = 2 };

// One RK stage as the device sees it; the host fills an array of these per
// step (pinned buffer -> one H2D copy), so a captured graph replays any step.
struct StageDev {
    int s, kind, last, nrows, n0, nrows_next;
    int b2_save, b2_reuse;   // main(s): posB2x save/reuse slot, -1 none
    int pos_save, pos_reuse; // epilogue(s): next stage's posB1x save/reuse slot
    int nb2_reuse, nb2_save; // next stage's posB2x flags (for the B2 clamp)
    int ncoef, serk_mode;    // serk_mode: 0 first stage, 1 even, 2 odd
    int maxceil, maxX;       // B1 Floor clamp and B2 row clamp of this stage (from nrows)
    int fresh;               // 1: the gather searches the B1 positions itself (after a rollback)
    int pad_;
    double T;        // t1grid.back() while this stage's RHS is evaluated
    double T_next;   // time of the row this stage writes
    double tdiff;    // T_next - t1grid[n0-1]
    double dtr_new;  // delta_t_ratio of the written row
    double serk_c, serk_c2, serk_b0, serk_bnext;
    double coef[SMAX];    // tableau: g = g0 + sum_j h_j coef[j]
    double coef_e[SMAX];  // embedded solution coefficients (last stage)
};

struct Slots {
    double q0;            // C(t, theta=0) of the current last row
    double dr;            // drstep2 of the current step
    int maxceil;          // B1 Floor clamp of the current stage
    int maxX;             // B2 clamp of the current stage
    int saved_maxX[NSAVE];
    unsigned int counter; // last-block election in the epilogue
    int pad;
    // step result, written by the last epilogue block of the last stage
    double res_err, res_energy, res_r, res_qk0, res_dr;
};

// Per-target gathered values of one stage, recorded by k_main when
// DevCtx::rec is set (the adjoint's recompute) and read back by k_adj_targets
// instead of gathering again.
struct GatherRec {
    double2 a1, a2, b1, b2;  // (QK, QR) at the A1, A2, B1, B2 points
    double x;                // B2 position fraction
    int X;                   // B2 row (clamped)
    int pad;
};

struct DevCtx {
    int L, m, nch, search, kpt, tpb;
    int mixed;             // 1: FP32 gathers/convolutions (dyn_mixed.cu); 2: with (hi, lo) inputs
    int logr;              // 1: QR gathers in log space (FP64 form only)
    DModel M;
    const double* theta;
    const double* phi2;
    const double* integ;
    const int* iA1;
    const int* iA2;
    const int* iB2;
    const double* wA1;
    const double* wA2;
    const double* wB2;
    double2* KR;
    double2* dKR;
    double* t1grid;
    double* dtr;
    double* inv_dtr;
    double* rvec;
    double* drvec;
    double* posB1x;        // [L]
    double* posB1x_next;   // [L] next stage's positions, written by the gather kernel
    double* posB1x_saved;  // [NSAVE][L]
    double* posB2x;        // [L*L]
    double* posB2x_saved;  // [NSAVE][L*L]
    double2* h;            // [SMAX][L]
    double2* gS;           // SERK running stage value [L]
    double2* geS;          // SERK previous odd value [L]
    double2* gfS;          // SERK combination [L]
    double* part;          // [L][nch][8]
    double2* rowval;       // [L] (QK^{B1}[i,0], rInt_i)
    double* epart;         // [G][EP_N]
    Slots* slots;
    StageDev* stages;      // [SMAX]
    double2* rhs_out;      // [L]
    // mixed form: FP32 copies of the weights, tap-major ([ceil(m/2)][L*L] tap
    // pairs), and FP32 mirror of the history
    const float2* wA1f;
    const float2* wA2f;
    const float2* wB2f;
    float2* KRf;
    float2* dKRf;
    float2* KRl;           // mixed 2: low parts of (QK, QR), KR - (double)KRf
    const float2* wA1l;    // mixed 2: low parts of the FP32 weights (same layout as wA1f)
    const float2* wA2l;
    const float2* wB2l;
    const float* integ_f;  // [L]   int.dat in FP32
    const float* integ_l;  // [L]   its low parts, int.dat - (double)integ_f (mixed forms)
    float* inv_dtr_f;      // [cap] 1/delta_t_ratio in FP32
    float* inv_len_f;      // [cap] 1/(t1grid[k+1]-t1grid[k]) in FP32
    // materialized interpolation (dyn_interpolate)
    double* ip;            // [16][L*L]
    double* rint;          // [L]
    GatherRec* rec;        // [L*L] gathered values of this stage, or null
};

// Adjoint state of the FP64 path (dyn_adjoint.cu): cotangents of the
// history and per-step stage snapshots from the recompute.
struct AdjDev {
    double2* HKR;      // [cap][L] cotangents of (QK, QR)
    double2* HdKR;     // [cap][L] cotangents of (dQK, dQR)
    double* Hr;        // [cap]
    double* Hdr;       // [cap]
    double2* Gsave;    // [SMAX][L] row n0 (QK, QR) after stage s
    double2* Dsave;    // [SMAX][L] row n0 (dQK, dQR) after stage s
    double* rsave;     // [SMAX] r of row n0 after stage s
    double* drsave;    // [SMAX]
    double* Psave;     // [SMAX][L] B1 positions stage s read
    double2* hbar;     // [SMAX][L] cotangents of the stage right-hand sides
    double2* g0bar;    // [L] cotangent of the step's base row
    double2* Gbar;     // [L] cotangent of row n0's (QK, QR) after the current stage
    double2* Dbar;     // [L]
    double* abar;      // [L][8] cotangents of the eight memory-integral rows
    double2* lbar_part;  // [L][L] per-target-row last-row stencil cotangents
    double2* abarA;      // [L*L][2] cotangents of each target's A1 and A2 gathers
    double* sc;        // scalars: rho, delta, DR, Gamma, lambda
    // B2 cotangents of one stage, one packet per target, stored in the static
    // (iB2, phi2) order: the targets that share a B2 stencil row (X, iB2) in a
    // stage then sit next to each other (X is monotonic in phi2).
    struct B2Packet {
        int ij, X;
        double x, gK, gR;
    };
    B2Packet* b2pk;      // [L*L]
    int* b2rank;         // [L*L] packet slot of target ij
    GatherRec* rec;      // [SMAX][L*L] gathered values of each stage of the recomputed step
    // A1 and A2 gathers of each target row as one column-sorted sparse
    // matrix onto the last row (static): entry p of row i adds
    // lrW[p] * (cotangent 2j+t of the row) to column k for lrC[k] <= p < lrC[k+1]
    double* lrW;         // [L][2*L*m]
    int* lrS;            // [L][2*L*m] source 2j+t
    int* lrC;            // [L][L+1] column starts
};
struct AdjModel {
    int p, p2;
    double lam, T0, Gamma;
};

// Model coefficients in the reference's host evaluation order
// (math_ops.cpp:27-37: (lambda*p)*(p-1)... with p as the integer exponent)
inline DModel make_model(int p, int p2, double lambda, double T0, double Gamma) {
    DModel M;
    M.p = p;
    M.p2 = p2;
    M.cA = lambda * p;
    M.cB = (1 - lambda) * p2;
    M.cC = lambda * p * (p - 1);
    M.cD = (1 - lambda) * p2 * (p2 - 1);
    M.cE = lambda * p * (p - 1) * (p - 2);
    M.cF = (1 - lambda) * p2 * (p2 - 1) * (p2 - 2);
    M.T0 = T0;
    M.Gamma = Gamma;
    return M;
}

// Launch with programmatic stream serialization (overlaps the launch with the
// previous kernel's tail; the kernel itself calls wait_prior_grid first).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

// Dynamic shared memory above the 48 KB default needs the kernel's
// MaxDynamicSharedMemorySize attribute, which is per device: raise it to
// `limit` once per (kernel, device); `devs` is the caller's per-kernel record.
template <typename Kern>
inline cudaError_t raise_smem_limit(Kern kern, size_t bytes, int limit, std::atomic<unsigned long long>& devs) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (devs.load() & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
    if (e == cudaSuccess) devs.fetch_or(bit);
    return e;
}

// Window / smoothing state of the tail fit across calls (the reference keeps it
// in function statics, tail_fit.cpp:81-85); dyn_tail.cu
struct TailState {
    long long prev_off;   // offset of the last chosen window (-1: none yet)
    long long prev_n;     // history rows at the last call
    double alpha;         // smoothed alpha
    int last_rb;          // rollback loop seen last (-1000 initially)
    int applied;          // last call: 1 if QK was blended
    double alpha_raw;     // last call: the chosen window's mean
    int j0;               // last call: first blended column
    int pad;
};
cudaError_t launch_tail_fit(const DevCtx& c, int nrows, int rollback_loop, double delta_max, TailState* ts,
                            cudaStream_t st);

// launch wrappers (dyn_kernels.cu)
cudaError_t launch_stage(const DevCtx& c, int s, cudaStream_t st);
cudaError_t launch_main_only(const DevCtx& c, int s, cudaStream_t st);
cudaError_t launch_epi_only(const DevCtx& c, int s, cudaStream_t st);
cudaError_t launch_pos_init(const DevCtx& c, int nrows, cudaStream_t st);
cudaError_t launch_interp_exact(const DevCtx& c, int nrows, const double* pos1_given,
                                const double* pos2_given, cudaStream_t st);
cudaError_t launch_qkr_exact(const DevCtx& c, int nrows, double2* out, cudaStream_t st);
// posB1x of the state's last time and the reference-order B1 pair of every target
cudaError_t launch_b1_exact(const DevCtx& c, int nrows, double* qk, double* qr, cudaStream_t st);
cudaError_t launch_rstep_exact(const DevCtx& c, int nrows, double* out, cudaStream_t st);
cudaError_t launch_drstep2_exact(const DevCtx& c, const double* qK, const double* qR,
                                 const double* dqK, const double* dqR, double t, double* out,
                                 cudaStream_t st);
cudaError_t launch_energy_exact(const DevCtx& c, int nrows, double* out, cudaStream_t st);
cudaError_t launch_energy_history(const DevCtx& c, int nrows, double* out, cudaStream_t st);
cudaError_t launch_conv_exact(const DevCtx& c, int kind, const double* f, const double* g,
                              size_t n, double t, double* out, cudaStream_t st);
cudaError_t launch_search(const DevCtx& c, const double* list, size_t nlist, const double* elem,
                          size_t nelem, double* out, cudaStream_t st);
cudaError_t launch_sparsify_flags(const DevCtx& c, int nrows, int variant, double threshold,
                                  unsigned char* flags, cudaStream_t st);
cudaError_t launch_compact(const DevCtx& c, const int* inds, const int* indsD, const double* tfac,
                           int k, double2* KRn, double2* dKRn, double* rn, double* drn,
                           cudaStream_t st);
cudaError_t launch_pack_rows(const double* QK, const double* QR, double2* out, size_t count,
                             cudaStream_t st);
cudaError_t launch_main_mixed(const DevCtx& c, int s, cudaStream_t st);
cudaError_t launch_mirror_rows(const double2* in, float2* out, size_t count, cudaStream_t st);
cudaError_t launch_mirror_lo(const double2* in, float2* out, size_t count, cudaStream_t st);
// Rows past a history meet the zero taps of the mixed gathers' segment loads
// (the element after a stencil window that ends a row is the next row's first),
// so they must hold finite values: zero the FP32 mirror rows [r0, r1) that a
// shortened or replaced history leaves behind (they may hold a failed step's NaN).
cudaError_t clear_mirror_rows(const DevCtx& c, size_t r0, size_t r1, cudaStream_t st);
cudaError_t launch_weights_tapmajor_lo(const double* in, float2* out, size_t targets, int m, cudaStream_t st);
// [L*L][m] FP64 stencil rows to the tap-major FP32 pair planes of the mixed form
cudaError_t launch_weights_tapmajor(const double* in, float2* out, size_t targets, int m, cudaStream_t st);
cudaError_t launch_time_f32(const double* t1, const double* dtr, int n, float* inv_len, float* inv_dtr,
                            cudaStream_t st);
cudaError_t launch_fp64_probe(double* out, int blocks, int threads, int iters, cudaStream_t st);
cudaError_t launch_unpack_rows(const double2* in, double* QK, double* QR, size_t count,
                               cudaStream_t st);

cudaError_t launch_adj_seed(const DevCtx& c, const AdjDev& a, const AdjModel& am, int nl, double wE, double wR,
                            double wDr, const double* cK, const double* cR, const double* cdK, const double* cdR,
                            cudaStream_t st);
cudaError_t launch_adj_step(const DevCtx& c, const AdjDev& a, const AdjModel& am, int S, int n0, cudaStream_t st);
cudaError_t launch_adj_initial(const AdjDev& a, const AdjModel& am, cudaStream_t st);
cudaError_t launch_adj_verify(const DevCtx& c, const AdjDev& a, const double2* snapKR, const double2* snapdKR,
                              const double* snapr, const double* snapdr, int n0, cudaStream_t st);
cudaError_t adj_targets_smem_attr(int L, int m);

}  // namespace dyn
