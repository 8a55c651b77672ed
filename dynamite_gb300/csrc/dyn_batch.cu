// Batched quenches: many independent DYNAMITE quenches (own model, grid
// length, history, step controller, stopping rule) advance together on one
// GPU.
//
// One "tick" moves every running quench by one RK stage with two kernels:
//
//   k_batch_gather (persistent, nSM x k CTAs): CTAs pull (quench, target
//     row) items from an atomic counter, heaviest grids first, and run the
//     mixed-precision row set-up and chunk functions of the single-quench
//     kernel (dyn_mixed.cuh) on that quench's current stage; the last CTA to
//     leave resets the counter, so the kernel is idempotent per stage.
//   k_batch_epi (one one-warp CTA per 32 history rows of every quench): the
//     epilogue functions of the single-quench kernel (dyn_epi.cuh); the last
//     CTA of each quench folds its partials and then plans that quench's next
//     stage: at the end of a step it applies the step-size controller of
//     dyn_run (simulation_runner.cpp:252-304, rollback included), checks the
//     stopping rule and writes the next step's stage descriptors with the
//     same operation order as the host planner (so times are bit-identical).
//
// The host replays a CUDA graph of `ticks_per_launch` ticks and reads the
// quench plans back between replays; nothing else crosses PCIe.  A quench's
// one-warp epilogue latency overlaps the other quenches' gathers, which is
// what a single quench cannot do.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dyn.h"
#include "dyn_epi.cuh"
#include "dyn_host.h"
#include "dyn_mixed.cuh"

namespace dyn {
namespace {

constexpr int QMAX = SMAX / 2;  // largest SERK2 q (2q stages)

// RK tableaux and limits in device memory (copied from dyn_host.h)
struct TabDev {
    double rk_A[7][7], rk_B[7], rk_B2[7];
    double ssp_A[11][10], ssp_B[10], ssp_B2[10];
    double serk_b[QMAX + 1][SMAX + 1];
    double serk_alpha[QMAX + 1];
    double rmax[11];
};

// Step state and controller of one quench (the device owns it while ticks run)
struct Plan {
    int status, method, S, s, sidx, loop, fresh, n;
    long long steps;
    double dt, delta, delta_old, err_t;
    double T_last, T_prev;  // t1grid[n-1], t1grid[n-2]
    double energy, r, qk0;
    double dtr_last;        // delta_t_ratio of the newest row (the controller's ratio == 1 test)
    int spars_loop;         // loop of the last periodic sparsify (-1: none)
    int last_rb;            // loop of the last rollback (simulation_runner.cpp:53: -1000)
};

struct Quench {
    DevCtx c;
    StageDev* stg;  // [2][SMAX]: the current step's stages and the next step's
    int cap, rollback;
    long long max_steps;
    double t_stop, dmin, dmax, specRad;
    long long spars_every;  // periodic sparsify every this many loops (0: never)
};

struct Work {
    unsigned next, done;
};

// ------------------------------------------------------------------ planner
// Stage descriptors of the next step (Ctx::build_step in dyn_api.cu, itself
// runge_kutta.cpp:182-252 / runge_kutta.cu:397-487 time arithmetic) with the
// host's operation order: every product and sum rounded as written.
__device__ void begin_step(const Quench& q, Plan& pl, const TabDev& tb) {
    if (pl.status == DYN_QUENCH_FAILED) return;  // only a new state (dyn_batch_upload) restarts it
    if (q.t_stop > 0.0 && pl.T_last >= q.t_stop) { pl.status = DYN_QUENCH_DONE; return; }
    if (q.max_steps > 0 && pl.steps >= q.max_steps) { pl.status = DYN_QUENCH_MAXSTEPS; return; }
    if (pl.n + 1 > q.cap) { pl.status = DYN_QUENCH_FULL; return; }
    pl.status = DYN_QUENCH_RUNNING;
    const int method = pl.method, n0 = pl.n;
    const double dt = pl.dt, T0 = pl.T_last;
    const double prev = n0 >= 2 ? __dsub_rn(T0, pl.T_prev) : 0.0;
    const int nb = pl.sidx ^ 1;
    StageDev* st = q.stg + nb * SMAX;
    double Tn[SMAX];
    int S;
    if (method == DYN_RK54 || method == DYN_SSPRK104) {
        const bool ssp = method == DYN_SSPRK104;
        S = ssp ? 10 : 7;
        const double* B = ssp ? tb.ssp_B : tb.rk_B;
        const double* B2 = ssp ? tb.ssp_B2 : tb.rk_B2;
        for (int s = 0; s < S; ++s) {
            StageDev& sp = st[s];
            sp.kind = KIND_TABLEAU;
            sp.ncoef = s + 1;
            double gt = T0;
            if (s == S - 1) {
                for (int j = 0; j < S; ++j) {
                    const double cf = __dmul_rn(dt, B[j]);
                    gt = __dadd_rn(gt, cf);
                    sp.coef[j] = cf;
                }
                for (int j = 0; j < S; ++j) sp.coef_e[j] = __dmul_rn(dt, B2[j]);
            } else {
                for (int j = 0; j <= s; ++j) {
                    const double cf = __dmul_rn(dt, ssp ? tb.ssp_A[s + 1][j] : tb.rk_A[s + 1][j]);
                    gt = __dadd_rn(gt, cf);
                    sp.coef[j] = cf;
                }
            }
            Tn[s] = gt;
            // SSPRK(10,4) reuses the positions of stages 2..4 at stages 5..7
            sp.b2_save = (ssp && s >= 2 && s <= 4) ? s - 2 : -1;
            sp.b2_reuse = (ssp && s >= 5 && s <= 7) ? s - 5 : -1;
            const int nx = s + 1;
            sp.pos_save = (ssp && nx >= 2 && nx <= 4) ? nx - 2 : -1;
            sp.pos_reuse = (ssp && nx >= 5 && nx <= 7) ? nx - 5 : -1;
            sp.nb2_save = sp.pos_save;
            sp.nb2_reuse = sp.pos_reuse;
            sp.serk_mode = 0;
            sp.serk_c = sp.serk_c2 = sp.serk_b0 = sp.serk_bnext = 0.0;
        }
        double gte = T0;
        for (int j = 0; j < S; ++j) gte = __dadd_rn(gte, __dmul_rn(dt, B2[j]));
        pl.err_t = fabs(__dsub_rn(Tn[S - 1], gte));
    } else {
        const int qq = 2 * (method - 2);
        S = 2 * qq;
        const double alpha = tb.serk_alpha[qq];
        const double ca = __dmul_rn(dt, alpha), c2 = __dmul_rn(__dmul_rn(2.0, dt), alpha);
        double gt = T0, gte = T0;
        for (int s = 0; s < S; ++s) {
            StageDev& sp = st[s];
            sp.kind = KIND_SERK;
            sp.ncoef = 0;
            sp.serk_c = ca;
            sp.serk_c2 = c2;
            sp.serk_b0 = tb.serk_b[qq][0];
            sp.serk_bnext = tb.serk_b[qq][s + 1];
            sp.b2_save = sp.b2_reuse = sp.pos_save = sp.pos_reuse = sp.nb2_save = sp.nb2_reuse = -1;
            if (s == 0) {
                sp.serk_mode = 0;
                gt = __dadd_rn(T0, ca);
            } else if (s % 2 == 0) {
                sp.serk_mode = 1;
                gt = __dadd_rn(gt, ca);
            } else {
                sp.serk_mode = 2;
                gt = __dadd_rn(__dsub_rn(__dmul_rn(2.0, gt), gte), c2);
                gte = gt;
            }
            Tn[s] = gt;
        }
        pl.err_t = fabs(__dsub_rn(__dadd_rn(T0, dt), gt));
    }
    for (int s = 0; s < S; ++s) {
        StageDev& sp = st[s];
        sp.s = s;
        sp.last = s == S - 1;
        sp.n0 = n0;
        sp.nrows = s == 0 ? n0 : n0 + 1;
        sp.maxceil = sp.nrows - 1 < 1 ? 1 : sp.nrows - 1;
        sp.maxX = sp.nrows - 1;
        sp.fresh = s == 0 ? pl.fresh : 0;
        sp.nrows_next = n0 + 1;
        sp.T = s == 0 ? T0 : Tn[s - 1];
        sp.T_next = Tn[s];
        sp.tdiff = __dsub_rn(Tn[s], T0);
        sp.dtr_new = n0 >= 2 ? __ddiv_rn(sp.tdiff, prev) : 0.0;
    }
    pl.fresh = 0;
    pl.S = S;
    pl.s = 0;
    pl.sidx = nb;
}

// End of a step: the step result and the controller of dyn_run without a
// schedule (simulation_runner.cpp:252-304), same operation order.
// The step's bookkeeping: error estimate, loop count, the new row's time
__device__ void finish_step(const Quench& q, Plan& pl, const StageDev& last) {
    const Slots* sl = q.c.slots;
    const double delta = __dadd_rn(sl->res_err, pl.err_t);
    pl.delta_old = pl.delta;
    pl.delta = delta;
    pl.loop += 1;
    pl.steps += 1;
    pl.n += 1;
    pl.T_prev = pl.T_last;
    pl.T_last = last.T_next;
    pl.dtr_last = last.dtr_new;
    pl.energy = sl->res_energy;
    pl.r = sl->res_r;
    pl.qk0 = sl->res_qk0;
}

// The periodic sparsify falls due at the end of this loop (simulation_runner.cpp:148)
__device__ __forceinline__ bool sparsify_due(const Quench& q, const Plan& pl) {
    return q.spars_every > 0 && pl.loop > 0 && pl.loop % q.spars_every == 0 && pl.loop != pl.spars_loop;
}

// The step-size controller of dyn_run (simulation_runner.cpp:252-304)
__device__ void adapt_step(const Quench& q, Plan& pl, const TabDev& tb) {
    const double delta = pl.delta;
    const double dmax = q.dmax, dmin = q.dmin, sr = q.specRad;
    double dt = pl.dt;
    int method = pl.method;
    if (delta < dmax && pl.loop > 5 && (delta < __dmul_rn(1.1, pl.delta_old) || pl.delta_old < __ddiv_rn(dmax, 1000.0)) &&
        __ddiv_rn(tb.rmax[method - 1], sr) > dt && pl.dtr_last == 1.0) {
        dt = __dmul_rn(dt, 1.01);
    } else if (delta > __dmul_rn(2.0, dmax) && dt > dmin) {
        dt = __dmul_rn(dt, 0.9);
    }
    if (method == DYN_SSPRK104 && delta > dmax && __ddiv_rn(tb.rmax[0], sr) > dt) {
        method = DYN_RK54;
        dt = __dmul_rn(dt, 0.5);
    }
    if (q.rollback && delta > __dmul_rn(2.0, dmax)) {
        // rollbackState(nr) (simulation_control.cpp:14-123) of the CUDA build
        const int nr = min(10, max(0, pl.n - 2));
        if (nr > 0) {
            const int target = pl.n - nr;
            pl.n = target;
            pl.T_last = q.c.t1grid[target - 1];
            pl.T_prev = q.c.t1grid[target - 2];
            dt = __dsub_rn(pl.T_last, pl.T_prev);
            pl.loop -= nr;
            pl.last_rb = pl.loop;
            pl.fresh = 1;
        }
        dt = __dmul_rn(0.5, fmin(fmax(dt, dmin), __ddiv_rn(tb.rmax[method - 1], sr)));
        method = method > 3 ? 2 + (2 * (method - 3)) / 2 : DYN_SSPRK104;
    }
    pl.dt = dt;
    pl.method = method;
}

// ------------------------------------------------------------------ kernels
// TPB threads per CTA; the register cap keeps DYN_BATCH_TPSM (K = 1) or 512
// (K = 2) threads resident per SM: the gathers are latency-bound.
#ifndef DYN_BATCH_TPSM
#define DYN_BATCH_TPSM 1280
#endif
#ifndef DYN_BATCH_SHIFT
#define DYN_BATCH_SHIFT 0
#endif
#ifndef DYN_BATCH_DF_TPSM
#define DYN_BATCH_DF_TPSM 1024
#endif
// DF: the (hi, lo) form (mdf::chunk_dd): twice the staged row and a double-float
// tail; a cap of 64 registers (DYN_BATCH_DF_TPSM = 1024 threads per SM) spills a
// little but measures best for 64 quenches at L=512: 1.55 ms against 1.62 (56
// registers), 1.61 (72) and 1.74 (80).
template <int M, int K, int P, int P2, int TPB, bool DF = false>
__global__ void __launch_bounds__(TPB, DF ? DYN_BATCH_DF_TPSM / TPB : (K == 1 ? DYN_BATCH_TPSM : 512) / TPB)
    k_batch_gather(const Quench* __restrict__ Q, const Plan* __restrict__ PL, const unsigned* __restrict__ items,
                   const unsigned nitems, Work* work) {
    wait_prior_grid();
    extern __shared__ float2 s_lastf[];
    __shared__ mixed::RowShared sh;
    __shared__ float s_clo[4];
    __shared__ unsigned s_item[2];  // the item being worked on and the next one
    constexpr int GMAX = mixed::RED_CAP / (8 * (TPB / 32));  // chunks per fold
    int p = 0;
    if (threadIdx.x == 0) s_item[0] = atomicAdd(&work->next, 1u);
    __syncthreads();
    for (;;) {
        const unsigned it = s_item[p];
        if (it >= nitems) break;
        const unsigned e = __ldg(items + it);
        const Quench& q = Q[e >> 16];
        const Plan& pl = PL[e >> 16];
        if (pl.status == DYN_QUENCH_RUNNING) {
            const int i = (int)(e & 0xffffu);
            const StageDev& sp = q.stg[pl.sidx * SMAX + pl.s];
            float2* s_lo = s_lastf + (q.c.L + 2);
            if constexpr (DF) {
                mixed::row_setup(q.c, sp, i, true, s_lastf, sh, s_clo);
                mdf::stage_lo(q.c, sp, s_lo);
            } else {
                mixed::row_setup(q.c, sp, i, true, s_lastf, sh);
            }
            __syncthreads();
            const int nch = q.c.nch;
            for (int ch0 = 0; ch0 < nch; ch0 += GMAX) {
                const int ng = min(GMAX, nch - ch0);
                for (int g = 0; g < ng; ++g) {
                    if constexpr (DF) mdf::chunk_dd<M, K, P, P2>(q.c, sp, ch0 + g, g, s_lastf, s_lo, s_clo, sh, i);
                    else mixed::chunk_sums<M, K, P, P2, DYN_BATCH_SHIFT>(q.c, sp, ch0 + g, g, s_lastf, sh, i);
                }
                __syncthreads();
                mixed::fold_chunks(q.c, i, nch, ch0, ng, sh);
                if (ch0 + GMAX < nch) __syncthreads();
            }
        }
        // the next item goes to the other slot: threads still reading s_item[p] are unaffected
        if (threadIdx.x == 0) s_item[p ^ 1] = atomicAdd(&work->next, 1u);
        __syncthreads();
        p ^= 1;
    }
    if (threadIdx.x == 0 && atomicAdd(&work->done, 1u) == gridDim.x - 1) {
        // every CTA has made its last fetch: reset for the next launch
        work->next = 0;
        work->done = 0;
    }
}

template <int P, int P2>
__global__ void __launch_bounds__(EPI_T) k_batch_epi(const Quench* __restrict__ Q, Plan* __restrict__ PL,
                                                     const unsigned* __restrict__ eitems, const TabDev* __restrict__ tb) {
    wait_prior_grid();
    const unsigned e = eitems[blockIdx.x];
    const Quench& q = Q[e >> 16];
    Plan& pl = PL[e >> 16];
    if (pl.status != DYN_QUENCH_RUNNING) return;
    const unsigned blk = e & 0xffffu;
    const int s = pl.s;
    const StageDev& sp = q.stg[pl.sidx * SMAX + s];
    const DevCtx& c = q.c;
    const unsigned G = (unsigned)((c.L + EPI_ROWS - 1) / EPI_ROWS);
    double ep[EP_N];
    epi::rows<P, P2, true>(c, sp, s, (int)blk, ep);
    if (!epi::elect_last(c, ep, blk, G)) return;
    epi::fold<P, P2, true>(c, sp, s, G);
    if (threadIdx.x != 0) return;
    c.slots->counter = 0;
    if (!sp.last) {
        pl.s = s + 1;
        return;
    }
    finish_step(q, pl, sp);
    if (!isfinite(pl.delta)) {
        // non-finite values in the state (dyn_run's DYN_ERR_NONFINITE): stop this quench
        pl.status = DYN_QUENCH_FAILED;
        return;
    }
    if (sparsify_due(q, pl)) {
        // the host compacts the history, then k_batch_resume adapts and plans
        pl.status = DYN_QUENCH_SPARSIFY;
        return;
    }
    adapt_step(q, pl, *tb);
    begin_step(q, pl, *tb);
}

// (Re)start quench b's planning from its plan (after creation, upload or new limits)
__global__ void k_batch_begin(const Quench* Q, Plan* PL, const TabDev* tb, int b) {
    if (threadIdx.x == 0 && blockIdx.x == 0) begin_step(Q[b], PL[b], *tb);
}

// Continue quench b after its periodic sparsify: the controller of the loop
// that ended, then the next step's plan
__global__ void k_batch_resume(const Quench* Q, Plan* PL, const TabDev* tb, int b) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        adapt_step(Q[b], PL[b], *tb);
        begin_step(Q[b], PL[b], *tb);
    }
}

// ------------------------------------------------------------------ host side
#define BCK(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return bfail(DYN_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

dyn_status bfail(dyn_status s, const std::string& msg) {
    set_last_error(msg);
    return s;
}

struct GridDev {
    size_t L = 0, m = 0;
    double* theta = nullptr;
    double* phi2 = nullptr;
    double* integ = nullptr;
    float* integ_f = nullptr;
    int* iA[3] = {nullptr, nullptr, nullptr};
    float2* wf[3] = {nullptr, nullptr, nullptr};  // tap-major FP32 pair planes
    float2* wl[3] = {nullptr, nullptr, nullptr};  // their low parts (DYN_MIXED_DF)
};

struct Batch {
    dyn_batch_config cfg{};
    cudaStream_t st = nullptr;
    bool own_stream = false;
    int nsm = 0;
    std::vector<GridDev> grids;
    std::vector<dyn_batch_quench> spec;
    std::vector<Quench> qh;  // host copy: pointers and constants (pl is the device's)
    std::vector<Plan> plan_h;
    Plan* plan_pin = nullptr;
    double2* row_pin = nullptr;
    size_t row_pin_len = 0;
    Quench* qd = nullptr;
    Plan* pd = nullptr;
    TabDev* tabd = nullptr;
    unsigned* items = nullptr;
    unsigned nitems = 0;
    unsigned* eitems = nullptr;
    unsigned neitems = 0;
    Work* work = nullptr;
    int tpb = 128, kpt = 1, ctas = 0;
    int M = 10, pp = 0;  // template selectors: stencil depth, (p, p2) kind
    bool df = false;     // DYN_MIXED_DF: (hi, lo) inputs (mdf::chunk)
    size_t smem = 0, Lmax = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_ticks = 0;
    std::vector<void*> allocs;

    ~Batch() {
        if (graph) cudaGraphExecDestroy(graph);
        for (void* p : allocs) cudaFree(p);
        if (plan_pin) cudaFreeHost(plan_pin);
        if (row_pin) cudaFreeHost(row_pin);
        if (own_stream && st) cudaStreamDestroy(st);
    }

    template <typename T>
    dyn_status alloc(T** p, size_t count) {
        *p = nullptr;
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
        if (e != cudaSuccess) return bfail(DYN_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs.push_back((void*)*p);
        return DYN_OK;
    }

    template <int M_, int K_, int P_, int P2_, int TPB_>
    cudaError_t gather_t() {
        if (df)  // the (hi, lo) form runs one target per thread
            return launch_pdl(k_batch_gather<M_, 1, P_, P2_, TPB_, true>, dim3(nsm * ctas), dim3(TPB_), smem, st,
                              (const Quench*)qd, (const Plan*)pd, (const unsigned*)items, nitems, work);
        return launch_pdl(k_batch_gather<M_, K_, P_, P2_, TPB_>, dim3(nsm * ctas), dim3(TPB_), smem, st,
                          (const Quench*)qd, (const Plan*)pd, (const unsigned*)items, nitems, work);
    }
    template <int M_, int K_, int P_, int P2_>
    cudaError_t gather_b() { return tpb == 256 ? gather_t<M_, K_, P_, P2_, 256>() : gather_t<M_, K_, P_, P2_, 128>(); }
    template <int M_, int P_, int P2_>
    cudaError_t gather_k() { return kpt == 2 ? gather_b<M_, 2, P_, P2_>() : gather_b<M_, 1, P_, P2_>(); }
    template <int P_, int P2_>
    cudaError_t gather_m() { return M == 10 ? gather_k<10, P_, P2_>() : gather_k<0, P_, P2_>(); }
    cudaError_t launch_gather() {
        if (pp == 1) return gather_m<3, 4>();
        if (pp == 2) return gather_m<3, 0>();
        return gather_m<-1, -1>();
    }
    cudaError_t launch_epi() {
        const Quench* q = qd;
        const unsigned* ei = eitems;
        const TabDev* tb = tabd;
        if (pp == 1) return launch_pdl(k_batch_epi<3, 4>, dim3(neitems), dim3(EPI_T), 0, st, q, pd, ei, tb);
        if (pp == 2) return launch_pdl(k_batch_epi<3, 0>, dim3(neitems), dim3(EPI_T), 0, st, q, pd, ei, tb);
        return launch_pdl(k_batch_epi<-1, -1>, dim3(neitems), dim3(EPI_T), 0, st, q, pd, ei, tb);
    }

    int occupancy(int threads, int targets) {
        int nb = 0;
        const void* f;
#define OCC_T(M_, K_, P_, P2_)                                                                        \
    (df ? (threads == 256 ? (const void*)k_batch_gather<M_, 1, P_, P2_, 256, true>                        \
                          : (const void*)k_batch_gather<M_, 1, P_, P2_, 128, true>)                       \
        : (threads == 256 ? (const void*)k_batch_gather<M_, K_, P_, P2_, 256> : (const void*)k_batch_gather<M_, K_, P_, P2_, 128>))
#define OCC_SEL(P_, P2_) \
    f = M == 10 ? (targets == 2 ? OCC_T(10, 2, P_, P2_) : OCC_T(10, 1, P_, P2_)) \
                : (targets == 2 ? OCC_T(0, 2, P_, P2_) : OCC_T(0, 1, P_, P2_))
        if (pp == 1) { OCC_SEL(3, 4); } else if (pp == 2) { OCC_SEL(3, 0); } else { OCC_SEL(-1, -1); }
#undef OCC_SEL
#undef OCC_T
        // the (hi, lo) form stages 2 (Lmax + 2) float2: above 48 KB from Lmax = 3071 on; the
        // attribute is set here, before the tile's first launch and any graph capture
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, threads, smem) != cudaSuccess) return 1;
        nb = nb > 0 ? nb : 1;
        // ask for the smallest shared-memory carveout that still holds nb CTAs, so the rest
        // of the SM's unified 256 KB stays L1 for the gathers' history lines and spills.  The
        // hint belongs to the kernel, not to this batch: of two live batches with different
        // row lengths the later tile setting decides, and a batch whose CTAs then do not all
        // fit at once runs them in waves (no CTA of the gather waits on another).
        cudaFuncAttributes fa;
        int dev = 0, smem_sm = 0, reserved = 0;
        if (cudaFuncGetAttributes(&fa, f) == cudaSuccess && cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess &&
            smem_sm > 0) {
            const size_t need = (size_t)nb * (fa.sharedSizeBytes + smem + (size_t)reserved);
            const int pct = (int)std::min<size_t>(100, (need * 100 + smem_sm - 1) / smem_sm);
            cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
            int nb2 = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb2, f, threads, smem) == cudaSuccess && nb2 < nb)
                cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, -1);  // keep nb resident
        }
        cudaGetLastError();  // a refused hint is not an error of the batch
        return nb;
    }

    dyn_status set_tile(int threads, int targets, int ctas_per_sm) {
        if (threads != 128 && threads != 256) return bfail(DYN_ERR_INVALID, "threads must be 128 or 256");
        if (targets != 1 && targets != 2) return bfail(DYN_ERR_INVALID, "targets must be 1 or 2");
        if (df) targets = 1;
        tpb = threads;
        kpt = targets;
        const int occ = occupancy(threads, targets);
        ctas = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ;
        for (size_t b = 0; b < qh.size(); ++b) {
            const int L = qh[b].c.L;
            qh[b].c.tpb = tpb;
            qh[b].c.kpt = kpt;
            qh[b].c.nch = (L + tpb * kpt - 1) / (tpb * kpt);
            BCK(cudaMemcpyAsync(&qd[b].c, &qh[b].c, sizeof(DevCtx), cudaMemcpyHostToDevice, st));
        }
        BCK(cudaStreamSynchronize(st));
        if (graph) {
            cudaGraphExecDestroy(graph);
            graph = nullptr;
        }
        return DYN_OK;
    }

    dyn_status read_plans() {
        const size_t B = qh.size();
        BCK(cudaMemcpyAsync(plan_pin, pd, B * sizeof(Plan), cudaMemcpyDeviceToHost, st));
        BCK(cudaStreamSynchronize(st));
        plan_h.assign(plan_pin, plan_pin + B);
        return DYN_OK;
    }

    dyn_status begin(int b) {
        k_batch_begin<<<1, 32, 0, st>>>(qd, pd, tabd, b);
        BCK(cudaGetLastError());
        return DYN_OK;
    }

    int running() const {
        int k = 0;
        for (const Plan& p : plan_h) k += p.status == DYN_QUENCH_RUNNING || p.status == DYN_QUENCH_SPARSIFY;
        return k;
    }

    // One sparsify pass over quench b's history (the same flag and compaction
    // kernels and index logic as dyn_sparsify), in place: rows are compacted
    // into scratch and copied back, times, FP32 mirrors and the plan's row
    // count follow.  Call at a step boundary (status other than running).
    dyn_status sparsify_pass(int b, double thr, int variant, int* n_out) {
        Quench& q = qh[b];
        Plan& pl = plan_h[b];
        const size_t n = (size_t)pl.n, L = q.c.L;
        *n_out = pl.n;
        if (n < 3) return DYN_OK;
        unsigned char* fl_d = nullptr;
        BCK(cudaMalloc(&fl_d, n));
        std::vector<unsigned char> fl(n);
        std::vector<double> t1(n), dtr(n);
        cudaError_t e = launch_sparsify_flags(q.c, (int)n, variant, thr, fl_d, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fl.data(), fl_d, n, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(t1.data(), q.c.t1grid, n * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dtr.data(), q.c.dtr, n * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(fl_d);
        BCK(e);
        std::vector<int> inds, indsD;
        std::vector<double> tfac, t1n, dtrn;
        if (!sparsify_indices(fl.data(), n, variant, t1, dtr, inds, indsD, tfac, t1n, dtrn)) return DYN_OK;
        const size_t k = inds.size();
        double2 *KRn = nullptr, *dKRn = nullptr;
        double *rn = nullptr, *drn = nullptr, *tf = nullptr;
        int* id = nullptr;
        auto release = [&]() {
            cudaFree(KRn); cudaFree(dKRn); cudaFree(rn); cudaFree(drn); cudaFree(tf); cudaFree(id);
        };
        if ((e = cudaMalloc(&KRn, k * L * sizeof(double2))) != cudaSuccess ||
            (e = cudaMalloc(&dKRn, k * L * sizeof(double2))) != cudaSuccess ||
            (e = cudaMalloc(&rn, k * sizeof(double))) != cudaSuccess ||
            (e = cudaMalloc(&drn, k * sizeof(double))) != cudaSuccess ||
            (e = cudaMalloc(&tf, k * sizeof(double))) != cudaSuccess ||
            (e = cudaMalloc(&id, 2 * k * sizeof(int))) != cudaSuccess) {
            release();
            return bfail(DYN_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        std::vector<double> inv(k);
        for (size_t r = 0; r < k; ++r) inv[r] = dtrn[r] != 0.0 ? 1.0 / dtrn[r] : 0.0;
        const bool ok =
            cudaMemcpyAsync(id, inds.data(), k * sizeof(int), cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(id + k, indsD.data(), k * sizeof(int), cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(tf, tfac.data(), k * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess &&
            launch_compact(q.c, id, id + k, variant == 0 ? nullptr : tf, (int)k, KRn, dKRn, rn, drn, st) == cudaSuccess &&
            cudaMemcpyAsync(q.c.KR, KRn, k * L * sizeof(double2), cudaMemcpyDeviceToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(q.c.dKR, dKRn, k * L * sizeof(double2), cudaMemcpyDeviceToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(q.c.rvec, rn, k * sizeof(double), cudaMemcpyDeviceToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(q.c.drvec, drn, k * sizeof(double), cudaMemcpyDeviceToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(q.c.t1grid, t1n.data(), k * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(q.c.dtr, dtrn.data(), k * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(q.c.inv_dtr, inv.data(), k * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess &&
            launch_mirror_rows(q.c.KR, q.c.KRf, k * L, st) == cudaSuccess &&
            launch_mirror_rows(q.c.dKR, q.c.dKRf, k * L, st) == cudaSuccess &&
            (!q.c.KRl || launch_mirror_lo(q.c.KR, q.c.KRl, k * L, st) == cudaSuccess) &&
            launch_time_f32(q.c.t1grid, q.c.dtr, (int)k, q.c.inv_len_f, q.c.inv_dtr_f, st) == cudaSuccess &&
            clear_mirror_rows(q.c, k, std::min((size_t)pl.n + 1, (size_t)q.cap), st) == cudaSuccess;
        e = cudaStreamSynchronize(st);  // the host vectors above are sources of the copies
        release();
        if (!ok || e != cudaSuccess) return bfail(DYN_ERR_CUDA, "batch sparsify: " + std::string(cudaGetErrorString(cudaGetLastError())));
        pl.n = (int)k;
        pl.T_last = t1n[k - 1];
        pl.T_prev = k >= 2 ? t1n[k - 2] : 0.0;
        pl.dtr_last = dtrn[k - 1];
        pl.fresh = 1;
        *n_out = (int)k;
        return DYN_OK;
    }

    // Quenches paused for their periodic sparsify (simulation_runner.cpp:148-237):
    // passes while the history shrinks, then the step halving when delta <
    // delta_max/2 and the last rollback is more than 1000 loops back, then the
    // controller of the loop and the next step's plan on the device.
    dyn_status service_sparsify() {
        bool any = false;
        for (size_t b = 0; b < qh.size(); ++b) {
            if (plan_h[b].status != DYN_QUENCH_SPARSIFY) continue;
            any = true;
            Plan& pl = plan_h[b];
            const double dmax = qh[b].dmax;
            const int sweeps = sparsify_block_sweeps(cfg.sparsify_sweeps);
            int prev = pl.n;
            for (int sw = 0; sw < sweeps; ++sw) {
                int nn = prev;
                dyn_status s = sparsify_pass((int)b, dmax, cfg.sparsify_variant, &nn);
                if (s) return s;
                if (nn >= prev) break;
                prev = nn;
            }
            if (pl.delta < dmax / 2 && pl.loop - pl.last_rb > 1000) {
                pl.dt *= 0.5;
                if (pl.method == DYN_RK54) pl.method = DYN_SSPRK104;
                else if (cfg.use_serk2 && pl.method < 2 + QMAX / 2) pl.method++;  // as dyn_run
            }
            pl.spars_loop = pl.loop;
            pl.status = DYN_QUENCH_RUNNING;
            BCK(cudaMemcpyAsync(pd + b, &pl, sizeof(Plan), cudaMemcpyHostToDevice, st));
            k_batch_resume<<<1, 32, 0, st>>>(qd, pd, tabd, (int)b);
            BCK(cudaGetLastError());
            BCK(cudaStreamSynchronize(st));  // &pl is host memory the copy reads
        }
        return any ? read_plans() : DYN_OK;
    }

    dyn_status enqueue_ticks(int n) {
        for (int k = 0; k < n; ++k) {
            BCK(launch_gather());
            BCK(launch_epi());
        }
        return DYN_OK;
    }

    dyn_status ensure_graph() {
        if (graph) return DYN_OK;
        const int T = cfg.ticks_per_launch > 0 ? cfg.ticks_per_launch : 32;
        cudaGraph_t g;
        BCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        dyn_status es = enqueue_ticks(T);
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (es) return es;
        BCK(ce);
        cudaError_t ie = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        BCK(ie);
        graph_ticks = T;
        return DYN_OK;
    }

    // t = 0 state of quench b (dyn_state_init: initialization.cpp:204-222)
    dyn_status init_state(int b) {
        Quench& q = qh[b];
        const dyn_batch_quench& sq = spec[b];
        const int L = q.c.L;
        std::vector<double2> row(L, make_double2(1.0, 1.0)), zero(L, make_double2(0.0, 0.0));
        BCK(cudaMemcpyAsync(q.c.KR, row.data(), L * sizeof(double2), cudaMemcpyHostToDevice, st));
        BCK(cudaMemcpyAsync(q.c.dKR, zero.data(), L * sizeof(double2), cudaMemcpyHostToDevice, st));
        const double r0 = sq.Gamma + Df_host(sq.lambda, sq.p, sq.p2, 1) / sq.T0;
        const double z = 0.0;
        BCK(cudaMemcpyAsync(q.c.rvec, &r0, sizeof(double), cudaMemcpyHostToDevice, st));
        BCK(cudaMemcpyAsync(q.c.t1grid, &z, sizeof(double), cudaMemcpyHostToDevice, st));
        BCK(cudaMemcpyAsync(q.c.dtr, &z, sizeof(double), cudaMemcpyHostToDevice, st));
        BCK(cudaMemcpyAsync(q.c.inv_dtr, &z, sizeof(double), cudaMemcpyHostToDevice, st));
        BCK(launch_time_f32(q.c.t1grid, q.c.dtr, 1, q.c.inv_len_f, q.c.inv_dtr_f, st));
        BCK(launch_rstep_exact(q.c, 1, q.c.drvec, st));
        BCK(launch_mirror_rows(q.c.KR, q.c.KRf, L, st));
        BCK(launch_mirror_rows(q.c.dKR, q.c.dKRf, L, st));
        if (q.c.KRl) BCK(launch_mirror_lo(q.c.KR, q.c.KRl, L, st));
        Plan p{};
        p.status = DYN_QUENCH_RUNNING;
        p.n = 1;
        p.dt = sq.delta_t > 0 ? sq.delta_t : sq.delta_t_min;
        p.delta = 1;
        p.delta_old = 0;
        p.loop = 0;
        p.method = p.dt < RMAX[0] / q.specRad ? DYN_RK54 : DYN_SSPRK104;
        p.fresh = 1;
        p.T_last = 0.0;
        p.T_prev = 0.0;
        p.dtr_last = 0.0;
        p.spars_loop = -1;
        p.last_rb = -1000;
        BCK(cudaMemcpyAsync(pd + b, &p, sizeof(Plan), cudaMemcpyHostToDevice, st));
        BCK(cudaStreamSynchronize(st));  // the host vectors above are stack memory
        return begin(b);
    }
};

Batch* BT(void* p) { return static_cast<Batch*>(p); }

}  // namespace
}  // namespace dyn

using namespace dyn;

extern "C" {

dyn_status dyn_batch_create(const dyn_batch_config* cfg, const dyn_batch_grid* grids, int ngrids,
                            const dyn_batch_quench* quenches, int nquench, void** out) {
    if (!cfg || !grids || !quenches || !out) return bfail(DYN_ERR_INVALID, "null argument");
    *out = nullptr;
    if (ngrids < 1 || nquench < 1 || nquench > 65535) return bfail(DYN_ERR_INVALID, "need 1..65535 quenches and at least one grid");
    if (cfg->search != DYN_SEARCH_BINARY && cfg->search != DYN_SEARCH_LOWER_BOUND) return bfail(DYN_ERR_INVALID, "unknown search");
    if (cfg->sparsify_variant < 0 || cfg->sparsify_variant > 2) return bfail(DYN_ERR_INVALID, "unknown sparsify variant");
    for (int g = 0; g < ngrids; ++g) {
        const size_t L = grids[g].len, m = grids[g].depth;
        if (L < 4 || L > 4096 || m < 2 || m > L) return bfail(DYN_ERR_INVALID, "len must be in [4, 4096] and 2 <= depth <= len");
    }
    for (int b = 0; b < nquench; ++b) {
        const dyn_batch_quench& q = quenches[b];
        if (q.grid < 0 || q.grid >= ngrids) return bfail(DYN_ERR_INVALID, "quench grid index out of range");
        if (q.p < 2 || q.p2 < 0 || q.p2 == 1) return bfail(DYN_ERR_INVALID, "quench exponents: p >= 2, p2 = 0 or >= 2");
        if (!(q.T0 > 0) || !(q.delta_t_min > 0) || !(q.delta_max > 0)) return bfail(DYN_ERR_INVALID, "T0, delta_t_min and delta_max must be positive");
        if (q.capacity != 0 && q.capacity < 2) return bfail(DYN_ERR_INVALID, "capacity must be at least 2 rows");
        std::string why;
        if (!check_model(q.p, q.p2, q.lambda, q.T0, q.Gamma, why)) return bfail(DYN_ERR_INVALID, why);
    }
    // every table on the host before any CUDA call
    for (int g = 0; g < ngrids; ++g) {
        std::vector<int> i32[3];
        std::string why;
        if (!check_tables(grids[g].len, grids[g].depth, &grids[g].tables, i32, why))
            return bfail(DYN_ERR_INVALID, "grid " + std::to_string(g) + ": " + why);
    }
    if (cfg->precision != 0 && cfg->precision != DYN_MIXED && cfg->precision != DYN_MIXED_DF)
        return bfail(DYN_ERR_INVALID, "batch precision: DYN_MIXED_DF (or 0) or DYN_MIXED");
    Batch* bt = new Batch();
    bt->cfg = *cfg;
    bt->df = cfg->precision != DYN_MIXED;  // 0 (the default) and DYN_MIXED_DF: the (hi, lo) form
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) { delete bt; return bfail(DYN_ERR_CUDA, cudaGetErrorString(e)); }
    if (cfg->stream) {
        bt->st = (cudaStream_t)cfg->stream;
    } else {
        e = cudaStreamCreateWithFlags(&bt->st, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete bt; return bfail(DYN_ERR_CUDA, cudaGetErrorString(e)); }
        bt->own_stream = true;
    }
    cudaDeviceGetAttribute(&bt->nsm, cudaDevAttrMultiProcessorCount, cfg->device);
    dyn_status s;
    // ---- grids: FP64 theta/phi2/int.dat, int32 starts, FP32 weights and int.dat
    bt->grids.resize(ngrids);
    bool all10 = true;
    for (int g = 0; g < ngrids; ++g) {
        GridDev& gd = bt->grids[g];
        const size_t L = grids[g].len, m = grids[g].depth, L2 = L * L;
        gd.L = L;
        gd.m = m;
        all10 = all10 && m == 10 && L % 2 == 0;  // depth-10 kernels need an even L
        bt->Lmax = std::max(bt->Lmax, L);
        std::vector<int> i32[3];
        std::string why;
        if (!check_tables(L, m, &grids[g].tables, i32, why)) { delete bt; return bfail(DYN_ERR_INVALID, why); }
        const dyn_tables& tb = grids[g].tables;
        if ((s = bt->alloc(&gd.theta, L)) || (s = bt->alloc(&gd.phi2, L2)) || (s = bt->alloc(&gd.integ, L)) ||
            (s = bt->alloc(&gd.integ_f, 2 * L))) { delete bt; return s; }
        std::vector<float> f(2 * L);  // int.dat as FP32 (hi, lo) planes
        for (size_t k = 0; k < L; ++k) {
            f[k] = (float)tb.integ[k];
            f[L + k] = (float)(tb.integ[k] - (double)f[k]);
        }
#define BUP(dst, src, bytes)                                                                       \
    if ((e = cudaMemcpy((void*)(dst), (src), (bytes), cudaMemcpyHostToDevice)) != cudaSuccess) {  \
        delete bt;                                                                                 \
        return bfail(DYN_ERR_CUDA, cudaGetErrorString(e));                                         \
    }
        BUP(gd.theta, tb.theta, L * sizeof(double));
        BUP(gd.phi2, tb.phi2, L2 * sizeof(double));
        BUP(gd.integ, tb.integ, L * sizeof(double));
        BUP(gd.integ_f, f.data(), 2 * L * sizeof(float));
        const double* w[3] = {tb.weightsA1y, tb.weightsA2y, tb.weightsB2y};
        const size_t planes = (m + 1) / 2;
        std::vector<float2> wt(planes * L2);
        for (int k = 0; k < 3; ++k) {
            if ((s = bt->alloc(&gd.iA[k], L2)) || (s = bt->alloc(&gd.wf[k], planes * L2))) { delete bt; return s; }
            BUP(gd.iA[k], i32[k].data(), L2 * sizeof(int));
            // the layout of k_weights_tapmajor (dyn_mixed.cu)
            for (size_t tg = 0; tg < L2; ++tg)
                for (size_t d = 0; d < m; d += 2)
                    wt[(d >> 1) * L2 + tg] =
                        make_float2((float)w[k][tg * m + d], d + 1 < m ? (float)w[k][tg * m + d + 1] : 0.0f);
            BUP(gd.wf[k], wt.data(), planes * L2 * sizeof(float2));
            if (bt->df) {
                if ((s = bt->alloc(&gd.wl[k], planes * L2))) { delete bt; return s; }
                auto lo = [](double v) { return (float)(v - (double)(float)v); };
                for (size_t tg = 0; tg < L2; ++tg)
                    for (size_t d = 0; d < m; d += 2)
                        wt[(d >> 1) * L2 + tg] = make_float2(lo(w[k][tg * m + d]), d + 1 < m ? lo(w[k][tg * m + d + 1]) : 0.0f);
                BUP(gd.wl[k], wt.data(), planes * L2 * sizeof(float2));
            }
        }
    }
    bt->M = all10 ? 10 : 0;
    // (p, p2) kind shared by all quenches selects the compiled exponents
    int pp = -1;
    for (int b = 0; b < nquench; ++b) {
        const int k = (quenches[b].p == 3 && quenches[b].p2 == 4) ? 1 : (quenches[b].p == 3 && quenches[b].p2 == 0) ? 2 : 0;
        pp = pp < 0 ? k : (pp == k ? pp : 0);
    }
    bt->pp = pp;
    bt->smem = (bt->df ? 2 : 1) * (bt->Lmax + 2) * sizeof(float2);

    // ---- tableaux
    {
        TabDev th{};
        std::memcpy(th.rk_A, RK54_A, sizeof th.rk_A);
        std::memcpy(th.rk_B, RK54_B, sizeof th.rk_B);
        std::memcpy(th.rk_B2, RK54_B2, sizeof th.rk_B2);
        for (int r = 0; r < 11; ++r)
            for (int c = 0; c < 10; ++c) th.ssp_A[r][c] = ssp_a(r, c);
        std::memcpy(th.ssp_B, SSP_B, sizeof th.ssp_B);
        std::memcpy(th.ssp_B2, SSP_B2, sizeof th.ssp_B2);
        for (int q = 1; q <= QMAX; ++q) {
            const std::vector<double> b = serk_coeffs(q);
            for (int k = 0; k <= 2 * q && k <= SMAX; ++k) th.serk_b[q][k] = b[k];
            th.serk_alpha[q] = 1.0 / (4 * q);
        }
        std::memcpy(th.rmax, RMAX, sizeof th.rmax);
        if ((s = bt->alloc(&bt->tabd, 1))) { delete bt; return s; }
        BUP(bt->tabd, &th, sizeof th);
    }

    // ---- quenches
    bt->spec.assign(quenches, quenches + nquench);
    bt->qh.resize(nquench);
    const int nch_max_of = 64;  // smallest tile (threads x targets) the part buffers admit
    for (int b = 0; b < nquench; ++b) {
        const dyn_batch_quench& sq = quenches[b];
        const GridDev& gd = bt->grids[sq.grid];
        Quench& q = bt->qh[b];
        std::memset(&q, 0, sizeof q);
        DevCtx& d = q.c;
        const size_t L = gd.L, cap = sq.capacity ? sq.capacity : 4096;
        d.L = (int)L;
        d.m = (int)gd.m;
        d.search = cfg->search;
        d.mixed = bt->df ? 2 : 1;
        d.M = make_model(sq.p, sq.p2, sq.lambda, sq.T0, sq.Gamma);
        d.theta = gd.theta;
        d.phi2 = gd.phi2;
        d.integ = gd.integ;
        d.integ_f = gd.integ_f;
        d.integ_l = gd.integ_f + gd.L;
        d.iA1 = gd.iA[0];
        d.iA2 = gd.iA[1];
        d.iB2 = gd.iA[2];
        d.wA1f = gd.wf[0];
        d.wA2f = gd.wf[1];
        d.wB2f = gd.wf[2];
        d.wA1l = gd.wl[0];
        d.wA2l = gd.wl[1];
        d.wB2l = gd.wl[2];
        const size_t G = (L + EPI_ROWS - 1) / EPI_ROWS, nchm = (L + nch_max_of - 1) / nch_max_of;
        if ((s = bt->alloc(&d.KR, cap * L)) || (s = bt->alloc(&d.dKR, cap * L)) ||
            (s = bt->alloc(&d.KRf, cap * L + 16)) || (s = bt->alloc(&d.dKRf, cap * L + 16)) ||
            (s = bt->alloc(&d.t1grid, cap)) || (s = bt->alloc(&d.dtr, cap)) || (s = bt->alloc(&d.inv_dtr, cap)) ||
            (s = bt->alloc(&d.rvec, cap)) || (s = bt->alloc(&d.drvec, cap)) || (s = bt->alloc(&d.inv_len_f, cap)) ||
            (s = bt->alloc(&d.inv_dtr_f, cap)) || (s = bt->alloc(&d.posB1x, L)) || (s = bt->alloc(&d.posB1x_next, L)) ||
            (s = bt->alloc(&d.posB1x_saved, NSAVE * L)) || (s = bt->alloc(&d.h, (size_t)SMAX * L)) ||
            (s = bt->alloc(&d.gS, L)) || (s = bt->alloc(&d.geS, L)) || (s = bt->alloc(&d.gfS, L)) ||
            (s = bt->alloc(&d.part, L * nchm * 8)) || (s = bt->alloc(&d.rowval, L)) ||
            (s = bt->alloc(&d.epart, G * EP_N)) || (s = bt->alloc(&d.slots, 1)) || (s = bt->alloc(&d.rhs_out, L)) ||
            (s = bt->alloc(&q.stg, 2 * SMAX))) {
            delete bt;
            return s;
        }
        if (bt->df) {
            if ((s = bt->alloc(&d.KRl, cap * L + 16))) { delete bt; return s; }
            cudaMemset(d.KRl, 0, (cap * L + 16) * sizeof(float2));
        }
        // the 16-byte segment loads may touch one element past the last row
        cudaMemset(d.KRf, 0, (cap * L + 16) * sizeof(float2));
        cudaMemset(d.dKRf, 0, (cap * L + 16) * sizeof(float2));
        cudaMemset(d.slots, 0, sizeof(Slots));
        cudaMemset(q.stg, 0, 2 * SMAX * sizeof(StageDev));
        q.cap = (int)cap;
        q.rollback = cfg->gpu_rollback ? 1 : 0;
        q.spars_every = cfg->sparsify_every > 0 ? cfg->sparsify_every : 0;
        q.max_steps = sq.max_steps;
        q.t_stop = sq.t_stop;
        q.dmin = sq.delta_t_min;
        q.dmax = sq.delta_max;
        q.specRad = 4 * std::sqrt(DDf_host(sq.lambda, sq.p, sq.p2, 1));
    }
    if ((s = bt->alloc(&bt->qd, nquench)) || (s = bt->alloc(&bt->pd, nquench)) || (s = bt->alloc(&bt->work, 1))) {
        delete bt;
        return s;
    }
    BUP(bt->qd, bt->qh.data(), nquench * sizeof(Quench));
    if ((e = cudaMemset(bt->work, 0, sizeof(Work))) != cudaSuccess) { delete bt; return bfail(DYN_ERR_CUDA, cudaGetErrorString(e)); }
    if (cudaMallocHost((void**)&bt->plan_pin, nquench * sizeof(Plan)) != cudaSuccess) {
        delete bt;
        return bfail(DYN_ERR_NOMEM, "cudaMallocHost failed");
    }

    // ---- work items: (quench, row) gather items, largest grids first; epilogue items
    {
        std::vector<int> order(nquench);
        for (int b = 0; b < nquench; ++b) order[b] = b;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return bt->qh[a].c.L > bt->qh[b].c.L; });
        std::vector<unsigned> it, ei;
        for (int b : order)
            for (int i = 0; i < bt->qh[b].c.L; ++i) it.push_back(((unsigned)b << 16) | (unsigned)i);
        for (int b = 0; b < nquench; ++b)
            for (int g = 0; g < (bt->qh[b].c.L + EPI_ROWS - 1) / EPI_ROWS; ++g) ei.push_back(((unsigned)b << 16) | (unsigned)g);
        bt->nitems = (unsigned)it.size();
        bt->neitems = (unsigned)ei.size();
        if ((s = bt->alloc(&bt->items, it.size())) || (s = bt->alloc(&bt->eitems, ei.size()))) { delete bt; return s; }
        BUP(bt->items, it.data(), it.size() * sizeof(unsigned));
        BUP(bt->eitems, ei.data(), ei.size() * sizeof(unsigned));
    }
#undef BUP
    if ((s = bt->set_tile(cfg->threads ? cfg->threads : 128, cfg->targets ? cfg->targets : 1, cfg->ctas_per_sm))) {
        delete bt;
        return s;
    }
    for (int b = 0; b < nquench; ++b)
        if ((s = bt->init_state(b))) { delete bt; return s; }
    if ((s = bt->read_plans())) { delete bt; return s; }
    *out = bt;
    return DYN_OK;
}

dyn_status dyn_batch_destroy(void* p) {
    if (!p) return DYN_OK;
    Batch* bt = BT(p);
    cudaSetDevice(bt->cfg.device);
    cudaStreamSynchronize(bt->st);
    delete bt;
    return DYN_OK;
}

dyn_status dyn_batch_upload(void* p, int qi, const dyn_state* stt, const dyn_controller* ctl) {
    if (!p || !stt || !ctl) return bfail(DYN_ERR_INVALID, "null argument");
    Batch* bt = BT(p);
    if (qi < 0 || qi >= (int)bt->qh.size()) return bfail(DYN_ERR_INVALID, "quench index out of range");
    Quench& q = bt->qh[qi];
    const size_t n = stt->n, L = q.c.L;
    if (n < 1 || n + 1 > (size_t)q.cap) return bfail(DYN_ERR_INVALID, "state rows must be in [1, capacity-1]");
    if (!stt->t1grid || !stt->delta_t_ratio || !stt->QK || !stt->QR || !stt->dQK || !stt->dQR || !stt->rvec || !stt->drvec)
        return bfail(DYN_ERR_INVALID, "missing state array");
    for (size_t k = 0; k < n; ++k) {
        if (!(stt->t1grid[k] >= 0.0) || !std::isfinite(stt->t1grid[k]))
            return bfail(DYN_ERR_INVALID, "t1grid must be finite and non-negative");
        if (k && !(stt->t1grid[k] >= stt->t1grid[k - 1])) return bfail(DYN_ERR_INVALID, "t1grid must be non-decreasing");
        if (!std::isfinite(stt->delta_t_ratio[k]) || !std::isfinite(stt->rvec[k]) || !std::isfinite(stt->drvec[k]))
            return bfail(DYN_ERR_INVALID, "delta_t_ratio, rvec and drvec must be finite");
    }
    for (size_t e = 0; e < n * L; ++e)
        if (!std::isfinite(stt->QK[e]) || !std::isfinite(stt->QR[e]) || !std::isfinite(stt->dQK[e]) ||
            !std::isfinite(stt->dQR[e]))
            return bfail(DYN_ERR_INVALID, "QK, QR, dQK and dQR must be finite");
    if (ctl->method < 1 || ctl->method > 2 + QMAX / 2) return bfail(DYN_ERR_INVALID, "method out of range");
    if (!(ctl->delta_t > 0)) return bfail(DYN_ERR_INVALID, "delta_t must be positive");
    std::vector<double2> kr(n * L), dkr(n * L);
    for (size_t e = 0; e < n * L; ++e) {
        kr[e] = make_double2(stt->QK[e], stt->QR[e]);
        dkr[e] = make_double2(stt->dQK[e], stt->dQR[e]);
    }
    std::vector<double> inv(n);
    for (size_t k = 0; k < n; ++k) inv[k] = stt->delta_t_ratio[k] != 0.0 ? 1.0 / stt->delta_t_ratio[k] : 0.0;
    cudaStream_t st = bt->st;
    BCK(cudaMemcpyAsync(q.c.KR, kr.data(), n * L * sizeof(double2), cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(q.c.dKR, dkr.data(), n * L * sizeof(double2), cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(q.c.rvec, stt->rvec, n * sizeof(double), cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(q.c.drvec, stt->drvec, n * sizeof(double), cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(q.c.t1grid, stt->t1grid, n * sizeof(double), cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(q.c.dtr, stt->delta_t_ratio, n * sizeof(double), cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(q.c.inv_dtr, inv.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
    BCK(launch_mirror_rows(q.c.KR, q.c.KRf, n * L, st));
    BCK(launch_mirror_rows(q.c.dKR, q.c.dKRf, n * L, st));
    if (q.c.KRl) BCK(launch_mirror_lo(q.c.KR, q.c.KRl, n * L, st));
    BCK(clear_mirror_rows(q.c, n, (size_t)q.cap, st));  // whatever the previous history left
    BCK(launch_time_f32(q.c.t1grid, q.c.dtr, (int)n, q.c.inv_len_f, q.c.inv_dtr_f, st));
    Plan pl{};
    pl.status = DYN_QUENCH_RUNNING;
    pl.n = (int)n;
    pl.T_last = stt->t1grid[n - 1];
    pl.T_prev = n >= 2 ? stt->t1grid[n - 2] : 0.0;
    pl.dt = ctl->delta_t;
    pl.delta = ctl->delta;
    pl.delta_old = ctl->delta_old;
    pl.loop = ctl->loop;
    pl.method = ctl->method;
    pl.fresh = 1;
    pl.sidx = 0;
    pl.dtr_last = stt->delta_t_ratio[n - 1];
    pl.spars_loop = -1;
    pl.last_rb = -1000;
    BCK(cudaMemcpyAsync(bt->pd + qi, &pl, sizeof(Plan), cudaMemcpyHostToDevice, st));
    BCK(cudaStreamSynchronize(st));
    dyn_status s = bt->begin(qi);
    if (s) return s;
    return bt->read_plans();
}

dyn_status dyn_batch_download(void* p, int qi, dyn_state* stt) {
    if (!p || !stt) return bfail(DYN_ERR_INVALID, "null argument");
    Batch* bt = BT(p);
    if (qi < 0 || qi >= (int)bt->qh.size()) return bfail(DYN_ERR_INVALID, "quench index out of range");
    dyn_status s = bt->read_plans();
    if (s) return s;
    const Quench& q = bt->qh[qi];
    const size_t n = bt->plan_h[qi].n, L = q.c.L;
    if (stt->n < n) return bfail(DYN_ERR_INVALID, "state buffers hold fewer rows than the history");
    stt->n = n;
    std::vector<double2> kr(n * L), dkr(n * L);
    cudaStream_t st = bt->st;
    BCK(cudaMemcpyAsync(kr.data(), q.c.KR, n * L * sizeof(double2), cudaMemcpyDeviceToHost, st));
    BCK(cudaMemcpyAsync(dkr.data(), q.c.dKR, n * L * sizeof(double2), cudaMemcpyDeviceToHost, st));
    if (stt->rvec) BCK(cudaMemcpyAsync(stt->rvec, q.c.rvec, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (stt->drvec) BCK(cudaMemcpyAsync(stt->drvec, q.c.drvec, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (stt->t1grid) BCK(cudaMemcpyAsync(stt->t1grid, q.c.t1grid, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (stt->delta_t_ratio) BCK(cudaMemcpyAsync(stt->delta_t_ratio, q.c.dtr, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    BCK(cudaStreamSynchronize(st));
    for (size_t e = 0; e < n * L; ++e) {
        if (stt->QK) stt->QK[e] = kr[e].x;
        if (stt->QR) stt->QR[e] = kr[e].y;
        if (stt->dQK) stt->dQK[e] = dkr[e].x;
        if (stt->dQR) stt->dQR[e] = dkr[e].y;
    }
    return DYN_OK;
}

dyn_status dyn_batch_get_info(void* p, int qi, dyn_batch_info* info) {
    if (!p || !info) return bfail(DYN_ERR_INVALID, "null argument");
    Batch* bt = BT(p);
    if (qi < 0 || qi >= (int)bt->qh.size()) return bfail(DYN_ERR_INVALID, "quench index out of range");
    const Plan& pl = bt->plan_h[qi];
    std::memset(info, 0, sizeof *info);
    info->status = pl.status;
    info->method = pl.method;
    info->loop = pl.loop;
    info->steps = pl.steps;
    info->n = (size_t)pl.n;
    info->t = pl.T_last;
    info->delta_t = pl.dt;
    info->delta = pl.delta;
    info->delta_old = pl.delta_old;
    info->energy = pl.energy;
    info->r = pl.r;
    info->qk0 = pl.qk0;
    return DYN_OK;
}

dyn_status dyn_batch_set_limits(void* p, int qi, double t_stop, long long max_steps) {
    if (!p) return bfail(DYN_ERR_INVALID, "null argument");
    Batch* bt = BT(p);
    if (qi < 0 || qi >= (int)bt->qh.size()) return bfail(DYN_ERR_INVALID, "quench index out of range");
    Quench& q = bt->qh[qi];
    q.t_stop = t_stop;
    q.max_steps = max_steps;
    BCK(cudaMemcpyAsync(&bt->qd[qi].t_stop, &q.t_stop, sizeof(double), cudaMemcpyHostToDevice, bt->st));
    BCK(cudaMemcpyAsync(&bt->qd[qi].max_steps, &q.max_steps, sizeof(long long), cudaMemcpyHostToDevice, bt->st));
    dyn_status s = bt->read_plans();
    if (s) return s;
    const int stt = bt->plan_h[qi].status;
    if (stt == DYN_QUENCH_DONE || stt == DYN_QUENCH_MAXSTEPS) {
        if ((s = bt->begin(qi))) return s;
    }
    return bt->read_plans();
}

dyn_status dyn_batch_run(void* p, long long max_ticks, long long* ticks_out) {
    if (!p) return bfail(DYN_ERR_INVALID, "null argument");
    TraceRange tr("dyn_batch_run");
    Batch* bt = BT(p);
    long long done = 0;
    dyn_status s = bt->read_plans();
    if (s) return s;
    while (done < max_ticks && bt->running() > 0) {
        if ((s = bt->ensure_graph())) return s;
        if (max_ticks - done >= bt->graph_ticks) {
            BCK(cudaGraphLaunch(bt->graph, bt->st));
            done += bt->graph_ticks;
        } else {
            if ((s = bt->enqueue_ticks((int)(max_ticks - done)))) return s;
            done = max_ticks;
        }
        if ((s = bt->read_plans())) return s;
        if ((s = bt->service_sparsify())) return s;
    }
    if (ticks_out) *ticks_out = done;
    return DYN_OK;
}

dyn_status dyn_batch_enqueue(void* p, long long ticks) {
    if (!p || ticks < 0) return bfail(DYN_ERR_INVALID, "bad argument");
    TraceRange tr("dyn_batch_enqueue");
    Batch* bt = BT(p);
    dyn_status s = bt->ensure_graph();
    if (s) return s;
    long long done = 0;
    for (; done + bt->graph_ticks <= ticks; done += bt->graph_ticks) BCK(cudaGraphLaunch(bt->graph, bt->st));
    return bt->enqueue_ticks((int)(ticks - done));
}

dyn_status dyn_batch_sync(void* p) {
    if (!p) return bfail(DYN_ERR_INVALID, "null argument");
    dyn_status s = BT(p)->read_plans();
    return s ? s : BT(p)->service_sparsify();
}

dyn_status dyn_batch_last_row(void* p, int qi, double* qK, double* qR) {
    if (!p || !qK || !qR) return bfail(DYN_ERR_INVALID, "null argument");
    Batch* bt = BT(p);
    if (qi < 0 || qi >= (int)bt->qh.size()) return bfail(DYN_ERR_INVALID, "quench index out of range");
    const Quench& q = bt->qh[qi];
    const int L = q.c.L;
    const size_t n = (size_t)bt->plan_h[qi].n;
    if (bt->row_pin_len < (size_t)L) {
        if (bt->row_pin) cudaFreeHost(bt->row_pin);
        bt->row_pin = nullptr;
        bt->row_pin_len = 0;
        if (cudaMallocHost((void**)&bt->row_pin, L * sizeof(double2)) != cudaSuccess)
            return bfail(DYN_ERR_NOMEM, "cudaMallocHost failed");
        bt->row_pin_len = L;
    }
    BCK(cudaMemcpyAsync(bt->row_pin, q.c.KR + (n - 1) * L, L * sizeof(double2), cudaMemcpyDeviceToHost, bt->st));
    BCK(cudaStreamSynchronize(bt->st));
    for (int i = 0; i < L; ++i) {
        qK[i] = bt->row_pin[i].x;
        qR[i] = bt->row_pin[i].y;
    }
    return DYN_OK;
}

dyn_status dyn_batch_profile(void* p, int reps, float* ms) {
    if (!p || !ms || reps < 1) return bfail(DYN_ERR_INVALID, "bad argument");
    Batch* bt = BT(p);
    cudaEvent_t a, b;
    BCK(cudaEventCreate(&a));
    BCK(cudaEventCreate(&b));
    BCK(bt->launch_gather());  // warm
    BCK(cudaEventRecord(a, bt->st));
    for (int k = 0; k < reps; ++k) BCK(bt->launch_gather());
    BCK(cudaEventRecord(b, bt->st));
    BCK(cudaEventSynchronize(b));
    float t = 0;
    cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = t / reps;
    return DYN_OK;
}

dyn_status dyn_batch_tune(void* p, int reps, int* threads, int* targets, int* ctas_per_sm, float* ms_best) {
    if (!p || reps < 1) return bfail(DYN_ERR_INVALID, "bad argument");
    Batch* bt = BT(p);
    float best = 1e30f;
    int bt_t = bt->tpb, bt_k = bt->kpt, bt_c = bt->ctas;
    dyn_status s;
    for (int t : {128, 256}) {
        for (int k : {1, 2}) {
            if (bt->df && k == 2) continue;
            const int occ = bt->occupancy(t, k);
            std::vector<int> cands = {occ};
            if (occ >= 4) cands.push_back(occ / 2);
            for (int c : cands) {
                if ((s = bt->set_tile(t, k, c))) return s;
                float ms = 0;
                if ((s = dyn_batch_profile(p, reps, &ms))) return s;
                if (ms < best) { best = ms; bt_t = t; bt_k = k; bt_c = bt->ctas; }
            }
        }
    }
    if ((s = bt->set_tile(bt_t, bt_k, bt_c))) return s;
    if (threads) *threads = bt_t;
    if (targets) *targets = bt_k;
    if (ctas_per_sm) *ctas_per_sm = bt_c;
    if (ms_best) *ms_best = best;
    return DYN_OK;
}

}  // extern "C"
