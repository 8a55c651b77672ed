// Host side of the GB300-native DYNAMITE hot path: the C ABI of include/dyn.h.
//
// The host owns what is scalar and sequential — the time grid arithmetic
// (replicated operation by operation from the reference so that t1grid and
// delta_t_ratio come out bit-identical), the RK tableaux, the step-size
// controller — and keeps a mirror of t1grid/delta_t_ratio.  Everything of
// size L or L^2 lives on the device.  One RK step is one H2D copy of the
// stage descriptors, 2 kernels per stage, and one D2H copy of the step result,
// optionally replayed as a CUDA graph.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/dyn.h"
#include "dyn_host.h"
#include "dyn_kernels.cuh"

using namespace dyn;

namespace {

thread_local std::string g_err;

dyn_status fail(dyn_status s, const std::string& msg) {
    g_err = msg;
    return s;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(DYN_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
    } while (0)

template <typename T>
dyn_status dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) return fail(DYN_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return DYN_OK;
}

struct Ctx {
    dyn_config cfg{};
    int L = 0, m = 0;
    size_t L2 = 0;
    DevCtx d{};
    cudaStream_t st = nullptr;
    bool own_stream = false;
    // host mirrors of the time grid
    std::vector<double> t1, dtr;
    size_t n = 0, cap = 0;
    dyn_controller ctl{};
    int last_rollback_loop = -1000;  // loop of the last rollback (simulation_runner.cpp:53, :290)
    TailState* tail = nullptr;       // tail fit state across calls (device)
    double specRad = 0.0;
    // pinned staging
    StageDev* stages_h = nullptr;
    Slots* slots_h = nullptr;
    double2* rhs_h = nullptr;
    double* scratch_dev = nullptr;  // small device scratch for the exact kernels
    std::map<int, cudaGraphExec_t> graphs;
    std::map<int, int> warm;
    bool interp_alloc = false;
    unsigned long long gen = 0;  // bumped by every change of the history
    // discrete adjoint (FP64, fixed schedule): the recorded forward and its buffers
    AdjDev ad{};
    size_t ad_cap = 0;
    double* ad_ck = nullptr;        // [4][L] objective weights on the final row (K, R, dK, dR)
    double2* snap_KR = nullptr;     // history snapshot restored after the reverse sweep
    double2* snap_dKR = nullptr;
    double* snap_time = nullptr;    // [5][cap]: t1grid, dtr, inv_dtr, rvec, drvec
    bool adj_recorded = false;
    unsigned long long adj_gen = 0;
    size_t adj_n_start = 0;
    std::vector<double> adj_dt;
    std::vector<int> adj_method;
    double adj_ms_forward = 0.0;
    cudaEvent_t stages_copied = nullptr;  // the last async copy out of stages_h has run

    ~Ctx() { release(); }

    void drop_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }

    void release_adjoint() {
        void* ab[] = {ad.HKR, ad.HdKR, ad.Hr, ad.Hdr, ad.Gsave, ad.Dsave, ad.rsave, ad.drsave, ad.Psave, ad.hbar,
                      ad.g0bar, ad.Gbar, ad.Dbar, ad.abar, ad.lbar_part, ad.abarA, ad.sc, ad.b2pk, ad.b2rank, ad.rec, ad.lrW, ad.lrS, ad.lrC, ad_ck, snap_KR, snap_dKR, snap_time};
        for (void* b : ab) if (b) cudaFree(b);
        std::memset(&ad, 0, sizeof ad);
        ad_ck = nullptr;
        snap_KR = snap_dKR = nullptr;
        snap_time = nullptr;
        ad_cap = 0;
    }

    void release() {
        drop_graphs();
        release_adjoint();
        if (stages_copied) cudaEventDestroy(stages_copied);
        stages_copied = nullptr;
        void* bufs[] = {(void*)d.theta, (void*)d.phi2, (void*)d.integ, (void*)d.iA1, (void*)d.iA2, (void*)d.iB2,
                        (void*)d.wA1, (void*)d.wA2, (void*)d.wB2, d.KR, d.dKR, d.t1grid, d.dtr, d.inv_dtr,
                        d.rvec, d.drvec, d.posB1x, d.posB1x_next, d.posB1x_saved, d.posB2x, d.posB2x_saved, d.h, d.gS,
                        d.geS, d.gfS, d.part, d.rowval, d.epart, d.slots, d.stages, d.rhs_out, d.ip,
                        d.rint, scratch_dev, (void*)d.wA1f, (void*)d.wA2f, (void*)d.wB2f, d.KRf, d.dKRf,
                        (void*)d.integ_f, d.inv_len_f, d.inv_dtr_f, d.KRl, (void*)d.wA1l, (void*)d.wA2l,
                        (void*)d.wB2l, tail};
        for (void* b : bufs) if (b) cudaFree(b);
        std::memset(&d, 0, sizeof d);
        scratch_dev = nullptr;
        tail = nullptr;
        if (stages_h) cudaFreeHost(stages_h);
        if (slots_h) cudaFreeHost(slots_h);
        if (rhs_h) cudaFreeHost(rhs_h);
        stages_h = nullptr; slots_h = nullptr; rhs_h = nullptr;
        if (own_stream && st) cudaStreamDestroy(st);
        st = nullptr;
    }

    double Df_h(double q) const { return Df_host(cfg.lambda, cfg.p, cfg.p2, q); }
    double DDf_h(double q) const { return DDf_host(cfg.lambda, cfg.p, cfg.p2, q); }

    dyn_status ensure_rows(size_t rows) {
        if (rows <= cap) return DYN_OK;
        size_t ncap = cap ? cap : 1024;
        while (ncap < rows) ncap *= 2;
        double2 *KR, *dKR;
        double *t1g, *dt, *idt, *rv, *drv;
        dyn_status s;
        if ((s = dalloc(&KR, ncap * L)) || (s = dalloc(&dKR, ncap * L)) || (s = dalloc(&t1g, ncap)) ||
            (s = dalloc(&dt, ncap)) || (s = dalloc(&idt, ncap)) || (s = dalloc(&rv, ncap)) || (s = dalloc(&drv, ncap)))
            return s;
        float2 *KRf = nullptr, *dKRf = nullptr;
        float *ilen = nullptr, *idtf = nullptr;
        if (d.mixed && ((s = dalloc(&ilen, ncap)) || (s = dalloc(&idtf, ncap)))) return s;
        // +16 elements: the 16-byte segment loads of the mixed kernel may touch
        // one element past the end of the last row
        if (d.mixed && ((s = dalloc(&KRf, ncap * L + 16)) || (s = dalloc(&dKRf, ncap * L + 16)))) return s;
        float2* KRl = nullptr;
        if (d.mixed == 2 && (s = dalloc(&KRl, ncap * L + 16))) return s;
        // rows not written yet meet the zero taps of the gather segments: keep them finite
        if (d.mixed) {
            CK(cudaMemsetAsync(KRf, 0, (ncap * L + 16) * sizeof(float2), st));
            CK(cudaMemsetAsync(dKRf, 0, (ncap * L + 16) * sizeof(float2), st));
        }
        if (KRl) CK(cudaMemsetAsync(KRl, 0, (ncap * L + 16) * sizeof(float2), st));
        if (n && d.mixed) {
            CK(cudaMemcpyAsync(KRf, d.KRf, n * L * sizeof(float2), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(dKRf, d.dKRf, n * L * sizeof(float2), cudaMemcpyDeviceToDevice, st));
        }
        if (n && KRl) CK(cudaMemcpyAsync(KRl, d.KRl, n * L * sizeof(float2), cudaMemcpyDeviceToDevice, st));
        if (n) {
            CK(cudaMemcpyAsync(KR, d.KR, n * L * sizeof(double2), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(dKR, d.dKR, n * L * sizeof(double2), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(t1g, d.t1grid, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(dt, d.dtr, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(idt, d.inv_dtr, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(rv, d.rvec, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(drv, d.drvec, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            CK(cudaStreamSynchronize(st));
        }
        for (void* b : {(void*)d.KR, (void*)d.dKR, (void*)d.t1grid, (void*)d.dtr, (void*)d.inv_dtr, (void*)d.rvec,
                        (void*)d.drvec})
            if (b) cudaFree(b);
        d.KR = KR; d.dKR = dKR; d.t1grid = t1g; d.dtr = dt; d.inv_dtr = idt; d.rvec = rv; d.drvec = drv;
        if (d.mixed) {
            if (d.KRf) cudaFree(d.KRf);
            if (d.dKRf) cudaFree(d.dKRf);
            if (d.inv_len_f) cudaFree(d.inv_len_f);
            if (d.inv_dtr_f) cudaFree(d.inv_dtr_f);
            if (d.KRl) cudaFree(d.KRl);
            d.KRf = KRf;
            d.dKRf = dKRf;
            d.KRl = KRl;
            d.inv_len_f = ilen;
            d.inv_dtr_f = idtf;
            if (n) CK(launch_time_f32(d.t1grid, d.dtr, (int)n, d.inv_len_f, d.inv_dtr_f, st));
        }
        cap = ncap;
        drop_graphs();
        return DYN_OK;
    }

    dyn_status upload_times() {
        std::vector<double> inv(n);
        for (size_t k = 0; k < n; ++k) inv[k] = dtr[k] != 0.0 ? 1.0 / dtr[k] : 0.0;
        CK(cudaMemcpyAsync(d.t1grid, t1.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(d.dtr, dtr.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(d.inv_dtr, inv.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
        if (d.mixed) CK(launch_time_f32(d.t1grid, d.dtr, (int)n, d.inv_len_f, d.inv_dtr_f, st));
        CK(cudaStreamSynchronize(st));
        return DYN_OK;
    }

    // FP32 mirror of rows [0, n) from the FP64 master (mixed form)
    dyn_status mirror_all() {
        if (!d.mixed || n == 0) return DYN_OK;
        CK(launch_mirror_rows(d.KR, d.KRf, n * L, st));
        CK(launch_mirror_rows(d.dKR, d.dKRf, n * L, st));
        if (d.KRl) CK(launch_mirror_lo(d.KR, d.KRl, n * L, st));
        return DYN_OK;
    }

    dyn_status pos_init() {
        CK(launch_pos_init(d, (int)n, st));
        return DYN_OK;
    }

    // After the history shrank or was replaced (old length n_old): the FP32 mirror
    // rows [n, n_old + 1) leave the history and are zeroed (clear_mirror_rows)
    dyn_status clear_tail(size_t n_old) {
        if (!d.mixed) return DYN_OK;
        CK(clear_mirror_rows(d, n, std::min(std::max(n_old, n) + 1, cap), st));
        return DYN_OK;
    }

    // With theta[L-1] == phi2[L*L-1] == 1 (checked at creation) the largest
    // position of both searches is the last row exactly, so the reference's
    // clamps ceil(max posB1x) - 1 (interpolation_core.cpp:58-67) and
    // (size_t)(posB2x[L*L-1] - 0.5) (index_mat.cpp:189) are nrows - 1.
    static void set_clamps(StageDev& sp) {
        sp.maxceil = sp.nrows - 1 < 1 ? 1 : sp.nrows - 1;
        sp.maxX = sp.nrows - 1;
    }

    // Fill stages_h for one step; returns the host-side part of the error
    // estimate (|gt - gte|) and the final time through the out-params.
    dyn_status build_step(int method, double dt, int* S_out, double* err_t, double* T_final, double* dtr_final) {
        const size_t n0 = n;
        const double T0 = t1[n0 - 1];
        const double prev = n0 >= 2 ? T0 - t1[n0 - 2] : 0.0;
        int S;
        std::vector<double> Tn;  // time written by stage s
        std::memset(stages_h, 0, sizeof(StageDev) * SMAX);
        if (method == DYN_RK54 || method == DYN_SSPRK104) {
            const bool ssp = method == DYN_SSPRK104;
            S = ssp ? 10 : 7;
            auto A = [&](int r, int c) { return ssp ? ssp_a(r, c) : RK54_A[r][c]; };
            const double* B = ssp ? SSP_B : RK54_B;
            const double* B2 = ssp ? SSP_B2 : RK54_B2;
            for (int s = 0; s < S; ++s) {
                StageDev& sp = stages_h[s];
                sp.kind = KIND_TABLEAU;
                sp.ncoef = s + 1;
                double gt;
                if (s == 0) {
                    gt = T0 + dt * A(1, 0) * 1.0;  // runge_kutta.cpp:201
                    sp.coef[0] = dt * A(1, 0);
                } else if (s == S - 1) {
                    gt = T0;
                    for (int j = 0; j < S; ++j) { gt += dt * B[j] * 1.0; sp.coef[j] = dt * B[j]; }
                    for (int j = 0; j < S; ++j) sp.coef_e[j] = dt * B2[j];
                } else {
                    gt = T0;
                    for (int j = 0; j <= s; ++j) { gt += dt * A(s + 1, j) * 1.0; sp.coef[j] = dt * A(s + 1, j); }
                }
                Tn.push_back(gt);
                // SSPRK(10,4) reuses the positions of stages 2..4 at stages 5..7
                // (runge_kutta.cpp:60-80)
                sp.b2_save = (ssp && s >= 2 && s <= 4) ? s - 2 : -1;
                sp.b2_reuse = (ssp && s >= 5 && s <= 7) ? s - 5 : -1;
                const int nx = s + 1;
                sp.pos_save = (ssp && nx >= 2 && nx <= 4) ? nx - 2 : -1;
                sp.pos_reuse = (ssp && nx >= 5 && nx <= 7) ? nx - 5 : -1;
                sp.nb2_save = sp.pos_save;
                sp.nb2_reuse = sp.pos_reuse;
            }
            double gte = T0;
            for (int j = 0; j < S; ++j) gte += dt * B2[j] * 1.0;
            *err_t = std::fabs(Tn[S - 1] - gte);
        } else {
            const int q = 2 * (method - 2);
            if (q < 1 || 2 * q > SMAX) return fail(DYN_ERR_INVALID, "SERK2 order out of range");
            S = 2 * q;
            const std::vector<double> b = serk_coeffs(q);
            const double alpha = 1.0 / (4 * q);
            double gt = T0, gte = T0;
            for (int s = 0; s < S; ++s) {
                StageDev& sp = stages_h[s];
                sp.kind = KIND_SERK;
                sp.serk_c = dt * alpha;
                sp.serk_c2 = 2 * dt * alpha;
                sp.serk_b0 = b[0];
                sp.serk_bnext = b[s + 1];
                sp.b2_save = sp.b2_reuse = sp.pos_save = sp.pos_reuse = sp.nb2_save = sp.nb2_reuse = -1;
                if (s == 0) {
                    sp.serk_mode = 0;
                    gt = T0 + dt * alpha * 1.0;
                } else if (s % 2 == 0) {
                    sp.serk_mode = 1;
                    gt += dt * alpha * 1.0;
                } else {
                    sp.serk_mode = 2;
                    gt = 2 * gt - gte + 2 * dt * alpha * 1.0;
                    gte = gt;
                }
                Tn.push_back(gt);
            }
            *err_t = std::fabs((T0 + dt) - gt);
        }
        for (int s = 0; s < S; ++s) {
            StageDev& sp = stages_h[s];
            sp.s = s;
            sp.last = s == S - 1;
            sp.n0 = (int)n0;
            sp.nrows = s == 0 ? (int)n0 : (int)n0 + 1;
            set_clamps(sp);
            sp.nrows_next = (int)n0 + 1;
            sp.T = s == 0 ? T0 : Tn[s - 1];
            sp.T_next = Tn[s];
            sp.tdiff = Tn[s] - T0;
            sp.dtr_new = n0 >= 2 ? sp.tdiff / prev : 0.0;  // time_steps.cpp:58-67,142-149
        }
        *S_out = S;
        *T_final = Tn[S - 1];
        *dtr_final = stages_h[S - 1].dtr_new;
        return DYN_OK;
    }

    dyn_status enqueue_step(int S) {
        CK(cudaMemcpyAsync(d.stages, stages_h, sizeof(StageDev) * S, cudaMemcpyHostToDevice, st));
        for (int s = 0; s < S; ++s) CK(launch_stage(d, s, st));
        CK(cudaMemcpyAsync(slots_h, d.slots, sizeof(Slots), cudaMemcpyDeviceToHost, st));
        return DYN_OK;
    }

    dyn_status step(int method, double dt, dyn_step_result* res) {
        if (n == 0) return fail(DYN_ERR_STATE, "no state: call dyn_state_init or dyn_state_upload");
        dyn_status s = ensure_rows(n + 1);
        if (s) return s;
        int S;
        double err_t, Tf, dtrf;
        if ((s = build_step(method, dt, &S, &err_t, &Tf, &dtrf))) return s;
        if (cfg.use_graph && warm[method] > 0) {
            auto it = graphs.find(method);
            if (it == graphs.end()) {
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                dyn_status es = enqueue_step(S);
                cudaError_t ce = cudaStreamEndCapture(st, &g);
                if (es) return es;
                CK(ce);
                cudaGraphExec_t ge;
                CK(cudaGraphInstantiate(&ge, g, 0));
                cudaGraphDestroy(g);
                it = graphs.emplace(method, ge).first;
            }
            CK(cudaGraphLaunch(it->second, st));
        } else {
            if ((s = enqueue_step(S))) return s;
            warm[method]++;
        }
        CK(cudaStreamSynchronize(st));
        t1.push_back(Tf);
        dtr.push_back(dtrf);
        n += 1;
        gen++;
        if (res) {
            res->delta = slots_h->res_err + err_t;
            res->t = Tf;
            res->r = slots_h->res_r;
            res->energy = slots_h->res_energy;
            res->qk0 = slots_h->res_qk0;
            res->dr = slots_h->res_dr;
        }
        return DYN_OK;
    }

    // ---------------------------------------------------------- adjoint
    dyn_status adjoint_alloc() {
        if (ad_cap == cap && ad.HKR) return DYN_OK;
        release_adjoint();
        const size_t Lz = L;
        dyn_status s;
        if ((s = dalloc(&ad.HKR, cap * Lz)) || (s = dalloc(&ad.HdKR, cap * Lz)) || (s = dalloc(&ad.Hr, cap)) ||
            (s = dalloc(&ad.Hdr, cap)) || (s = dalloc(&ad.Gsave, (size_t)SMAX * Lz)) ||
            (s = dalloc(&ad.Dsave, (size_t)SMAX * Lz)) || (s = dalloc(&ad.rsave, SMAX)) || (s = dalloc(&ad.drsave, SMAX)) ||
            (s = dalloc(&ad.Psave, (size_t)SMAX * Lz)) || (s = dalloc(&ad.hbar, (size_t)SMAX * Lz)) ||
            (s = dalloc(&ad.g0bar, Lz)) || (s = dalloc(&ad.Gbar, Lz)) || (s = dalloc(&ad.Dbar, Lz)) ||
            (s = dalloc(&ad.abar, 8 * Lz)) || (s = dalloc(&ad.lbar_part, Lz * Lz)) || (s = dalloc(&ad.abarA, 2 * Lz * Lz)) || (s = dalloc(&ad.sc, 16)) ||
            (s = dalloc(&ad.b2pk, Lz * Lz)) || (s = dalloc(&ad.b2rank, Lz * Lz)) ||
            (s = dalloc(&ad.rec, (size_t)SMAX * Lz * Lz)) || (s = dalloc(&ad.lrW, 2 * Lz * Lz * (size_t)d.m)) ||
            (s = dalloc(&ad.lrS, 2 * Lz * Lz * (size_t)d.m)) || (s = dalloc(&ad.lrC, Lz * (Lz + 1))) ||
            (s = dalloc(&ad_ck, 4 * Lz)) || (s = dalloc(&snap_KR, cap * Lz)) || (s = dalloc(&snap_dKR, cap * Lz)) ||
            (s = dalloc(&snap_time, 5 * cap))) {
            release_adjoint();
            return s;
        }
        CK(adj_targets_smem_attr(L, d.m));
        {
            // static orders of the transposed gathers (the tables never change)
            const size_t L2 = Lz * Lz;
            std::vector<double> ph(L2);
            std::vector<long long> iA(2 * L2), iB(L2);
            CK(cudaMemcpy(ph.data(), d.phi2, L2 * sizeof(double), cudaMemcpyDeviceToHost));
            std::vector<int> i32(L2);
            for (int t = 0; t < 3; ++t) {
                CK(cudaMemcpy(i32.data(), t == 0 ? d.iA1 : t == 1 ? d.iA2 : d.iB2, L2 * sizeof(int),
                              cudaMemcpyDeviceToHost));
                long long* dst = t < 2 ? iA.data() + t * L2 : iB.data();
                for (size_t e = 0; e < L2; ++e) dst[e] = i32[e];
            }
            std::vector<int> ord(L2), rank(L2);
            for (size_t e = 0; e < L2; ++e) ord[e] = (int)e;
            std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
                return iB[x] != iB[y] ? iB[x] < iB[y] : ph[x] < ph[y];
            });
            for (size_t q = 0; q < L2; ++q) rank[ord[q]] = (int)q;
            CK(cudaMemcpy(ad.b2rank, rank.data(), L2 * sizeof(int), cudaMemcpyHostToDevice));
            // A1/A2 of each row as a column-sorted sparse matrix (counting sort by column)
            const size_t mz = d.m, E = 2 * Lz * mz;
            std::vector<double> wA(2 * L2 * mz), lw(Lz * E);
            CK(cudaMemcpy(wA.data(), d.wA1, L2 * mz * sizeof(double), cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(wA.data() + L2 * mz, d.wA2, L2 * mz * sizeof(double), cudaMemcpyDeviceToHost));
            std::vector<int> ls(Lz * E), lc(Lz * (Lz + 1));
            for (size_t i = 0; i < Lz; ++i) {
                int* cs = lc.data() + i * (Lz + 1);
                std::fill(cs, cs + Lz + 1, 0);
                for (int t = 0; t < 2; ++t)
                    for (size_t j = 0; j < Lz; ++j)
                        for (size_t dd = 0; dd < mz; ++dd) ++cs[iA[t * L2 + i * Lz + j] + dd + 1];
                for (size_t k = 0; k < Lz; ++k) cs[k + 1] += cs[k];
                std::vector<int> fill(cs, cs + Lz);
                for (int t = 0; t < 2; ++t)
                    for (size_t j = 0; j < Lz; ++j)
                        for (size_t dd = 0; dd < mz; ++dd) {
                            const size_t col = iA[t * L2 + i * Lz + j] + dd, p = i * E + fill[col]++;
                            lw[p] = wA[t * L2 * mz + (i * Lz + j) * mz + dd];
                            ls[p] = (int)(2 * j + t);
                        }
            }
            CK(cudaMemcpy(ad.lrW, lw.data(), Lz * E * sizeof(double), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(ad.lrS, ls.data(), Lz * E * sizeof(int), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(ad.lrC, lc.data(), Lz * (Lz + 1) * sizeof(int), cudaMemcpyHostToDevice));
        }
        ad_cap = cap;
        return DYN_OK;
    }

    size_t adjoint_bytes() const {
        const size_t Lz = L;
        return (cap * Lz * 2 * sizeof(double2)) * 2 + cap * 2 * sizeof(double) + 5 * cap * sizeof(double) +
               (size_t)SMAX * Lz * (3 * sizeof(double2) + sizeof(double)) + 3 * Lz * Lz * sizeof(double2) +
               Lz * Lz * (sizeof(AdjDev::B2Packet) + sizeof(int) + SMAX * sizeof(GatherRec)) +
               2 * Lz * Lz * (size_t)d.m * (sizeof(double) + sizeof(int)) + Lz * (Lz + 1) * sizeof(int) +
               Lz * (3 * sizeof(double2) + 9 * sizeof(double)) + 2 * SMAX * sizeof(double) + 16 * sizeof(double);
    }

    // Step n0 -> n0 + 1 again from the history prefix (same kernels, same
    // stage descriptors as the forward), keeping what the reverse sweep needs
    // of each stage: the B1 positions it read and row n0 after it.
    dyn_status recompute_step(int method, double dt, int* S_out) {
        // stages_h is the source of an asynchronous copy: the previous step's
        // copy must have run before the records are rewritten
        if (!stages_copied) CK(cudaEventCreateWithFlags(&stages_copied, cudaEventDisableTiming));
        else CK(cudaEventSynchronize(stages_copied));
        int S;
        double err_t, Tf, dtrf;
        dyn_status s = build_step(method, dt, &S, &err_t, &Tf, &dtrf);
        if (s) return s;
        const size_t n0 = n, Lz = L;
        CK(launch_pos_init(d, (int)n0, st));
        CK(cudaMemcpyAsync(d.stages, stages_h, sizeof(StageDev) * S, cudaMemcpyHostToDevice, st));
        CK(cudaEventRecord(stages_copied, st));
        for (int k = 0; k < S; ++k) {
            CK(cudaMemcpyAsync(ad.Psave + k * Lz, d.posB1x, Lz * sizeof(double), cudaMemcpyDeviceToDevice, st));
            DevCtx dr = d;
            dr.rec = ad.rec + (size_t)k * Lz * Lz;  // k_main records its gathers for the reverse stage
            CK(launch_stage(dr, k, st));
            CK(cudaMemcpyAsync(ad.Gsave + k * Lz, d.KR + n0 * Lz, Lz * sizeof(double2), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(ad.Dsave + k * Lz, d.dKR + n0 * Lz, Lz * sizeof(double2), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(ad.rsave + k, d.rvec + n0, sizeof(double), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(ad.drsave + k, d.drvec + n0, sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
        t1.push_back(Tf);
        dtr.push_back(dtrf);
        n += 1;
        *S_out = S;
        return DYN_OK;
    }

    dyn_status snapshot(bool restore) {
        const size_t rows = n, Lz = L;
        auto cp = [&](void* dst, const void* src, size_t bytes) {
            return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
        };
        double* tv[5] = {d.t1grid, d.dtr, d.inv_dtr, d.rvec, d.drvec};
        if (!restore) {
            CK(cp(snap_KR, d.KR, rows * Lz * sizeof(double2)));
            CK(cp(snap_dKR, d.dKR, rows * Lz * sizeof(double2)));
            for (int k = 0; k < 5; ++k) CK(cp(snap_time + k * cap, tv[k], rows * sizeof(double)));
        } else {
            CK(cp(d.KR, snap_KR, rows * Lz * sizeof(double2)));
            CK(cp(d.dKR, snap_dKR, rows * Lz * sizeof(double2)));
            for (int k = 0; k < 5; ++k) CK(cp(tv[k], snap_time + k * cap, rows * sizeof(double)));
        }
        return DYN_OK;
    }
};

Ctx* C(void* p) { return static_cast<Ctx*>(p); }

}  // namespace

namespace dyn {
void set_last_error(const std::string& msg) { g_err = msg; }

// The checks every table set passes before it reaches the device: theta
// non-decreasing on [0, 1] with theta[L-1] == 1, phi2 in [0, 1] ending at 1
// (these make the largest search position the last row, so the B1/B2 clamps
// are known on the host), stencil starts in [0, L-m]; the starts come back
// as int32.
bool check_tables(size_t L, size_t m, const dyn_tables* tb, std::vector<int> i32[3], std::string& why) {
    if (!tb->theta || !tb->phi2 || !tb->integ || !tb->indsA1y || !tb->indsA2y || !tb->indsB2y || !tb->weightsA1y ||
        !tb->weightsA2y || !tb->weightsB2y) {
        why = "missing table";
        return false;
    }
    for (size_t i = 1; i < L; ++i)
        if (!(tb->theta[i] >= tb->theta[i - 1])) { why = "theta must be non-decreasing"; return false; }
    if (tb->theta[0] < 0.0 || tb->theta[L - 1] != 1.0) { why = "theta must span [0, 1]"; return false; }
    const size_t L2 = L * L;
    const int64_t* src[3] = {tb->indsA1y, tb->indsA2y, tb->indsB2y};
    for (int k = 0; k < 3; ++k) {
        i32[k].resize(L2);
        for (size_t e = 0; e < L2; ++e) {
            const int64_t v = src[k][e];
            if (v < 0 || (size_t)v + m > L) { why = "stencil start out of range [0, len-depth]"; return false; }
            i32[k][e] = (int)v;
        }
    }
    for (size_t e = 0; e < L2; ++e)
        if (!(tb->phi2[e] >= 0.0 && tb->phi2[e] <= 1.0)) { why = "phi2 outside [0, 1]"; return false; }
    // phi2[i][j] = theta_i + (1 - theta_i) theta_j grows along a row; the mixed gathers
    // bracket their interval searches on that
    for (size_t i = 0; i < L; ++i)
        for (size_t j = 1; j < L; ++j)
            if (tb->phi2[i * L + j] < tb->phi2[i * L + j - 1]) { why = "phi2 rows must be non-decreasing"; return false; }
    if (tb->phi2[L2 - 1] != 1.0) { why = "phi2 must end at 1"; return false; }
    for (size_t i = 0; i < L; ++i)
        if (!std::isfinite(tb->integ[i])) { why = "int.dat holds a non-finite weight"; return false; }
    const double* w[3] = {tb->weightsA1y, tb->weightsA2y, tb->weightsB2y};
    for (int k = 0; k < 3; ++k)
        for (size_t e = 0; e < L2 * m; ++e)
            if (!std::isfinite(w[k][e])) { why = "a stencil weight is not finite"; return false; }
    return true;
}

// The model parameters the kernels can evaluate: f'(q), f''(q), f'''(q) with
// integer exponents, 1/T0, and a finite bath temperature.
bool check_model(int p_, int p2_, double lambda, double T0, double Gamma, std::string& why) {
    if (p_ < 0 || p2_ < 0 || p_ > 64 || p2_ > 64) { why = "exponents p, p2 must be in [0, 64]"; return false; }
    if (!std::isfinite(lambda)) { why = "lambda must be finite"; return false; }
    if (!(T0 > 0.0)) { why = "T0 must be positive (1e50 for an infinite-temperature start)"; return false; }
    if (!std::isfinite(Gamma)) { why = "Gamma must be finite"; return false; }
    return true;
}

int sparsify_block_sweeps(int requested) {
    if (requested >= 0) return std::min(10, requested);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 1;
    const double total_mb = (double)(total_b >> 20), used_mb = (double)((total_b - free_b) >> 20);
    return (total_mb > 0 && used_mb > total_mb * 0.5) ? 2 : 1;
}

// SERK2 coefficients (runge_kutta.cu:202-272), long double solve
static long double chebT(int n, long double x) {
    if (n == 0) return 1.0L;
    if (n == 1) return x;
    long double t0 = 1.0L, t1 = x;
    for (int i = 2; i <= n; ++i) { long double t2 = 2.0L * x * t1 - t0; t0 = t1; t1 = t2; }
    return t1;
}
static long double chebU(int n, long double x) {
    if (n == 0) return 1.0L;
    if (n == 1) return 2.0L * x;
    long double u0 = 1.0L, u1 = 2.0L * x;
    for (int i = 2; i <= n; ++i) { long double u2 = 2.0L * x * u1 - u0; u0 = u1; u1 = u2; }
    return u1;
}
std::vector<double> serk_coeffs(int q) {
    const int mm = 2, s = mm * q, N = s + 1;
    const long double mup = 19.0L / 20.0L;
    const long double a2 = (long double)q / ((long double)s * s);
    const long double w0 = 1.0L + mup / ((long double)s * s);
    const long double w1 = chebT(s, w0) / ((long double)s * chebU(s - 1, w0));
    std::vector<std::vector<long double>> A(N, std::vector<long double>(N + 1, 0.0L));
    for (int zi = 0; zi < N; ++zi) {
        const long double z = (long double)(zi + 1);
        A[zi][N] = chebT(s, w0 + w1 * z) / chebT(s, w0);
        A[zi][0] = chebT(0, 1.0L + a2 * z);
        for (int j = 1; j <= q; ++j) {
            const long double tmj = std::pow(chebT(mm, 1.0L + a2 * z), j - 1);
            for (int i = 1; i <= mm; ++i) A[zi][i + mm * (j - 1)] = chebT(i, 1.0L + a2 * z) * tmj;
        }
    }
    for (int i = 0; i < N; ++i) {
        int mx = i;
        for (int k = i + 1; k < N; ++k) if (std::fabs(A[k][i]) > std::fabs(A[mx][i])) mx = k;
        std::swap(A[i], A[mx]);
        for (int k = i + 1; k < N; ++k) {
            const long double f = A[k][i] / A[i][i];
            for (int j = i; j <= N; ++j) A[k][j] -= f * A[i][j];
        }
    }
    std::vector<long double> x(N);
    for (int i = N - 1; i >= 0; --i) {
        x[i] = A[i][N];
        for (int j = i + 1; j < N; ++j) x[i] -= A[i][j] * x[j];
        x[i] /= A[i][i];
    }
    std::vector<double> out(N);
    for (int i = 0; i < N; ++i) out[i] = (double)x[i];
    return out;
}

}

namespace dyn {
// Keep list of one sparsify pass from the per-node flags (bit 1: evaluated,
// bit 2: below the threshold, bit 4: kept by the GPU variant): the index logic
// of each variant (sparsify_utils.cpp:14-97, .cu:38-113, .cu:154-290), the
// derivative rows and their time rescaling (.cu:74-86, :230-265), and the new
// t1grid / delta_t_ratio (.cpp:76-96, .cu:99-110).  False when variant 0
// erases nothing (the reference leaves the state untouched).
bool sparsify_indices(const unsigned char* fl, size_t n, int variant, const std::vector<double>& t1,
                      const std::vector<double>& dtr, std::vector<int>& inds, std::vector<int>& indsD,
                      std::vector<double>& tfac, std::vector<double>& t1n, std::vector<double>& dtrn) {
    inds.clear();
    bool erased = false;
    if (variant == 0) {
        inds.push_back(0);
        for (size_t i = 2; i + 1 < n; ++i) {
            if (fl[i] & 2) erased = true; else inds.push_back((int)i);
        }
        inds.push_back((int)n - 1);
        if (!erased) return false;
    } else if (variant == 1) {
        int loop = 0;
        inds.push_back(0);
        for (size_t i = 2; i + 1 < n; ++i) {
            if ((fl[i] & 2) && !erased) { erased = true; ++loop; }
            else { erased = false; ++loop; inds.push_back(loop); }
        }
        inds.push_back((int)n - 2);
        inds.push_back((int)n - 1);
    } else {
        for (size_t i = 0; i < n; ++i) if (!(fl[i] & 1) || (fl[i] & 4)) inds.push_back((int)i);
    }
    const int k = (int)inds.size();
    indsD.assign(k, 0);
    tfac.assign(k, 1.0);
    if (variant == 0) {
        indsD = inds;
    } else {
        for (int i = 0; i + 1 < k; ++i) indsD[i + 1] = inds[i] + 1;
        for (int i = 1; i < k; ++i) {
            const double num = t1[inds[i]] - t1[inds[i - 1]];
            const double den = t1[indsD[i]] - t1[indsD[i] - 1];
            tfac[i] = variant == 2 ? (den != 0.0 ? num / den : 1.0) : num / den;
        }
    }
    t1n.assign(k, 0.0);
    for (int i = 0; i < k; ++i) t1n[i] = t1[inds[i]];
    if (variant == 0) {
        dtrn.assign(k, 0.0);
        for (int i = 0; i < k; ++i) dtrn[i] = dtr[inds[i]];
    } else {
        dtrn = dtr;
        dtrn.resize(k);
        std::vector<double> dg(k, 0.0);
        for (int i = 1; i < k; ++i) dg[i] = t1n[i] - t1n[i - 1];
        for (int i = 2; i < k; ++i) dtrn[i] = dg[i] / dg[i - 1];
    }
    return true;
}
// The tail fit's state starts as the reference's statics do (tail_fit.cpp:81-85)
static dyn_status tail_reset(Ctx* c) {
    if (!c->tail && dalloc(&c->tail, 1)) return DYN_ERR_NOMEM;
    TailState t{};
    t.prev_off = -1;
    t.prev_n = 0;
    t.alpha = 0.0;
    t.last_rb = -1000;
    cudaError_t e = cudaMemcpyAsync(c->tail, &t, sizeof t, cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) return fail(DYN_ERR_CUDA, cudaGetErrorString(e));
    return DYN_OK;
}

// The fit edits the FP64 master row; the mixed forms' FP32 mirrors of that row follow.
static dyn_status tail_fit(Ctx* c, int rollback_loop) {
    if (c->n == 0) return fail(DYN_ERR_STATE, "no state: call dyn_state_init or dyn_state_upload");
    dyn_status s;
    if (!c->tail && (s = tail_reset(c))) return s;
    DevCtx& d = c->d;
    const size_t row = (c->n - 1) * (size_t)c->L;
    cudaError_t e = launch_tail_fit(d, (int)c->n, rollback_loop, c->cfg.delta_max, c->tail, c->st);
    if (e == cudaSuccess && d.mixed) e = launch_mirror_rows(d.KR + row, d.KRf + row, c->L, c->st);
    if (e == cudaSuccess && d.KRl) e = launch_mirror_lo(d.KR + row, d.KRl + row, c->L, c->st);
    if (e != cudaSuccess) return fail(DYN_ERR_CUDA, cudaGetErrorString(e));
    c->gen++;  // the newest row may have changed
    return DYN_OK;
}

}  // namespace dyn

extern "C" {

int dyn_abi_version(void) { return DYN_ABI_VERSION; }
const char* dyn_last_error(void) { return g_err.c_str(); }

dyn_status dyn_check_tables(size_t len, size_t depth, const dyn_tables* tb) {
    if (!tb) return fail(DYN_ERR_INVALID, "null argument");
    if (len < 4 || len > 4096 || depth < 2 || depth > len)
        return fail(DYN_ERR_INVALID, "len must be in [4, 4096] and 2 <= depth <= len");
    std::vector<int> i32[3];
    std::string why;
    if (!check_tables(len, depth, tb, i32, why)) return fail(DYN_ERR_INVALID, why);
    return DYN_OK;
}

dyn_status dyn_ctx_create(const dyn_config* cfg, const dyn_tables* tb, void** out) {
    if (!cfg || !tb || !out) return fail(DYN_ERR_INVALID, "null argument");
    *out = nullptr;
    const size_t L = cfg->len, m = cfg->depth;
    if (L < 4 || L > 4096 || m < 2 || m > L) return fail(DYN_ERR_INVALID, "len must be in [4, 4096] and 2 <= depth <= len");
    if (cfg->precision != DYN_FP64 && cfg->precision != DYN_MIXED && cfg->precision != DYN_MIXED_DF)
        return fail(DYN_ERR_INVALID, "unknown precision");
    if (cfg->log_response != 0 && cfg->log_response != 1) return fail(DYN_ERR_INVALID, "log_response must be 0 or 1");
    if (cfg->log_response && cfg->precision != DYN_FP64)
        return fail(DYN_ERR_UNSUPPORTED, "log-space response runs on the FP64 form");
    const size_t L2 = L * L;
    std::vector<int> i32[3];
    {
        std::string why;
        if (!check_model(cfg->p, cfg->p2, cfg->lambda, cfg->T0, cfg->Gamma, why)) return fail(DYN_ERR_INVALID, why);
        if (!check_tables(L, m, tb, i32, why)) return fail(DYN_ERR_INVALID, why);
    }

    Ctx* c = new Ctx();
    c->cfg = *cfg;
    c->L = (int)L;
    c->m = (int)m;
    c->L2 = L2;
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) { delete c; return fail(DYN_ERR_CUDA, cudaGetErrorString(e)); }
    if (cfg->stream) {
        c->st = (cudaStream_t)cfg->stream;
    } else {
        e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete c; return fail(DYN_ERR_CUDA, cudaGetErrorString(e)); }
        c->own_stream = true;
    }
    DevCtx& d = c->d;
    d.L = (int)L;
    d.m = (int)m;
    d.search = cfg->search;
    d.logr = cfg->log_response;
    d.mixed = cfg->precision == DYN_MIXED ? 1 : cfg->precision == DYN_MIXED_DF ? 2 : 0;
    // tile shape: threads per CTA x targets per thread.  FP64: few wide CTAs
    // amortize the FP64 reduction; mixed: one target per thread keeps more
    // warps in flight for the latency-bound gathers.
    d.tpb = d.mixed ? 128 : 64;
    d.kpt = d.mixed ? 1 : (L >= 512 ? 4 : (L >= 256 ? 2 : 1));
    d.nch = (int)((L + (size_t)d.tpb * d.kpt - 1) / ((size_t)d.tpb * d.kpt));
    d.M = make_model(cfg->p, cfg->p2, cfg->lambda, cfg->T0, cfg->Gamma);

    dyn_status s;
    const int G = (int)((L + EPI_ROWS - 1) / EPI_ROWS);
    double *th, *p2, *it, *w1, *w2, *w3;
    int *a1, *a2, *b2;
    if ((s = dalloc(&th, L)) || (s = dalloc(&p2, L2)) || (s = dalloc(&it, L)) || (s = dalloc(&a1, L2)) ||
        (s = dalloc(&a2, L2)) || (s = dalloc(&b2, L2)) || (s = dalloc(&w1, L2 * m)) || (s = dalloc(&w2, L2 * m)) ||
        (s = dalloc(&w3, L2 * m)) || (s = dalloc(&d.posB1x, L)) || (s = dalloc(&d.posB1x_next, L)) || (s = dalloc(&d.posB1x_saved, NSAVE * L)) ||
        (s = dalloc(&d.posB2x, L2)) || (s = dalloc(&d.posB2x_saved, NSAVE * L2)) ||
        (s = dalloc(&d.h, (size_t)SMAX * L)) || (s = dalloc(&d.gS, L)) || (s = dalloc(&d.geS, L)) ||
        (s = dalloc(&d.gfS, L)) || (s = dalloc(&d.part, L * (size_t)d.nch * 8)) || (s = dalloc(&d.rowval, L)) ||
        (s = dalloc(&d.epart, (size_t)G * EP_N)) || (s = dalloc(&d.slots, 1)) || (s = dalloc(&d.stages, SMAX)) ||
        (s = dalloc(&d.rhs_out, L)) || (s = dalloc(&d.rint, L)) || (s = dalloc(&c->scratch_dev, 4 * L + 16))) {
        d.theta = th; d.phi2 = p2; d.integ = it; d.iA1 = a1; d.iA2 = a2; d.iB2 = b2; d.wA1 = w1; d.wA2 = w2; d.wB2 = w3;
        delete c;
        return s;
    }
    d.theta = th; d.phi2 = p2; d.integ = it; d.iA1 = a1; d.iA2 = a2; d.iB2 = b2; d.wA1 = w1; d.wA2 = w2; d.wB2 = w3;
#define UP(dst, srcp, count) \
    if ((e = cudaMemcpy((void*)(dst), (srcp), (count), cudaMemcpyHostToDevice)) != cudaSuccess) { delete c; return fail(DYN_ERR_CUDA, cudaGetErrorString(e)); }
    UP(th, tb->theta, L * sizeof(double));
    UP(p2, tb->phi2, L2 * sizeof(double));
    UP(it, tb->integ, L * sizeof(double));
    UP(a1, i32[0].data(), L2 * sizeof(int));
    UP(a2, i32[1].data(), L2 * sizeof(int));
    UP(b2, i32[2].data(), L2 * sizeof(int));
    UP(w1, tb->weightsA1y, L2 * m * sizeof(double));
    UP(w2, tb->weightsA2y, L2 * m * sizeof(double));
    UP(w3, tb->weightsB2y, L2 * m * sizeof(double));
#undef UP
    cudaMemset(d.slots, 0, sizeof(Slots));
    if (d.mixed) {
        const size_t planes = (m + 1) / 2;
        float2 *f1, *f2, *f3;
        if ((s = dalloc(&f1, planes * L2)) || (s = dalloc(&f2, planes * L2)) || (s = dalloc(&f3, planes * L2))) { delete c; return s; }
        d.wA1f = f1; d.wA2f = f2; d.wB2f = f3;
        float* itf;  // [2L]: int.dat as FP32 (hi, lo) planes
        if ((s = dalloc(&itf, 2 * L))) { delete c; return s; }
        d.integ_f = itf;
        d.integ_l = itf + L;
        {
            std::vector<float> hl(2 * L);
            for (size_t k = 0; k < L; ++k) {
                hl[k] = (float)tb->integ[k];
                hl[L + k] = (float)(tb->integ[k] - (double)hl[k]);
            }
            if (cudaMemcpy(itf, hl.data(), 2 * L * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
                delete c;
                return fail(DYN_ERR_CUDA, "FP32 int.dat copy failed");
            }
        }
        if (launch_weights_tapmajor(w1, f1, L2, (int)m, c->st) != cudaSuccess ||
            launch_weights_tapmajor(w2, f2, L2, (int)m, c->st) != cudaSuccess ||
            launch_weights_tapmajor(w3, f3, L2, (int)m, c->st) != cudaSuccess || cudaStreamSynchronize(c->st) != cudaSuccess) {
            delete c;
            return fail(DYN_ERR_CUDA, "FP32 weight copies failed");
        }
        if (d.mixed == 2) {
            float2 *l1, *l2, *l3;
            if ((s = dalloc(&l1, planes * L2)) || (s = dalloc(&l2, planes * L2)) || (s = dalloc(&l3, planes * L2))) { delete c; return s; }
            d.wA1l = l1; d.wA2l = l2; d.wB2l = l3;
            if (launch_weights_tapmajor_lo(w1, l1, L2, (int)m, c->st) != cudaSuccess ||
                launch_weights_tapmajor_lo(w2, l2, L2, (int)m, c->st) != cudaSuccess ||
                launch_weights_tapmajor_lo(w3, l3, L2, (int)m, c->st) != cudaSuccess ||
                cudaStreamSynchronize(c->st) != cudaSuccess) {
                delete c;
                return fail(DYN_ERR_CUDA, "FP32 weight low parts failed");
            }
        }
    }
    if (cudaMallocHost((void**)&c->stages_h, sizeof(StageDev) * SMAX) != cudaSuccess ||
        cudaMallocHost((void**)&c->slots_h, sizeof(Slots)) != cudaSuccess ||
        cudaMallocHost((void**)&c->rhs_h, sizeof(double2) * L) != cudaSuccess) {
        delete c;
        return fail(DYN_ERR_NOMEM, "cudaMallocHost failed");
    }
    c->specRad = 4 * std::sqrt(c->DDf_h(1));
    if ((s = c->ensure_rows(cfg->history_capacity ? cfg->history_capacity : 4096))) { delete c; return s; }
    *out = c;
    return DYN_OK;
}

dyn_status dyn_ctx_destroy(void* p) {
    if (!p) return DYN_OK;
    Ctx* c = C(p);
    cudaSetDevice(c->cfg.device);
    cudaStreamSynchronize(c->st);
    delete c;
    return DYN_OK;
}

dyn_status dyn_sync(void* p) {
    if (!p) return fail(DYN_ERR_INVALID, "null ctx");
    CK(cudaStreamSynchronize(C(p)->st));
    return DYN_OK;
}

// initialization.cpp:204-222
dyn_status dyn_state_init(void* p, double delta_t) {
    if (!p) return fail(DYN_ERR_INVALID, "null ctx");
    Ctx* c = C(p);
    const int L = c->L;
    const size_t n_old = c->n;
    c->n = 1;
    c->gen++;
    c->t1.assign(1, 0.0);
    c->dtr.assign(1, 0.0);
    std::vector<double2> row(L, make_double2(1.0, 1.0)), zero(L, make_double2(0.0, 0.0));
    CK(cudaMemcpyAsync(c->d.KR, row.data(), L * sizeof(double2), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.dKR, zero.data(), L * sizeof(double2), cudaMemcpyHostToDevice, c->st));
    const double r0 = c->cfg.Gamma + c->Df_h(1) / c->cfg.T0;
    CK(cudaMemcpyAsync(c->d.rvec, &r0, sizeof(double), cudaMemcpyHostToDevice, c->st));
    dyn_status s = c->upload_times();
    if (s) return s;
    CK(launch_rstep_exact(c->d, 1, c->d.drvec, c->st));
    if ((s = c->mirror_all())) return s;
    if ((s = c->clear_tail(n_old))) return s;
    c->ctl.delta_t = delta_t > 0 ? delta_t : c->cfg.delta_t_min;
    c->ctl.loop = 0;
    c->last_rollback_loop = -1000;
    c->ctl.delta = 1;
    c->ctl.delta_old = 0;
    c->ctl.method = c->ctl.delta_t < RMAX[0] / c->specRad ? DYN_RK54 : DYN_SSPRK104;
    if ((s = c->pos_init())) return s;
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_state_upload(void* p, const dyn_state* stt) {
    if (!p || !stt) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    const size_t n = stt->n, L = c->L;
    if (n < 1) return fail(DYN_ERR_INVALID, "state needs at least one row");
    if (!stt->t1grid || !stt->delta_t_ratio || !stt->QK || !stt->QR || !stt->dQK || !stt->dQR || !stt->rvec || !stt->drvec)
        return fail(DYN_ERR_INVALID, "missing state array");
    for (size_t k = 0; k < n; ++k) {
        if (!(stt->t1grid[k] >= 0.0) || !std::isfinite(stt->t1grid[k]))
            return fail(DYN_ERR_INVALID, "t1grid must be finite and non-negative");
        if (k && !(stt->t1grid[k] >= stt->t1grid[k - 1])) return fail(DYN_ERR_INVALID, "t1grid must be non-decreasing");
        if (!std::isfinite(stt->delta_t_ratio[k]) || !std::isfinite(stt->rvec[k]) || !std::isfinite(stt->drvec[k]))
            return fail(DYN_ERR_INVALID, "delta_t_ratio, rvec and drvec must be finite");
    }
    for (size_t e = 0; e < n * L; ++e)
        if (!std::isfinite(stt->QK[e]) || !std::isfinite(stt->QR[e]) || !std::isfinite(stt->dQK[e]) ||
            !std::isfinite(stt->dQR[e]))
            return fail(DYN_ERR_INVALID, "QK, QR, dQK and dQR must be finite");
    c->drop_graphs();
    c->gen++;
    const size_t n_old = c->n;
    c->n = 0;
    dyn_status s = c->ensure_rows(n + 1);
    if (s) return s;
    std::vector<double2> kr(n * L), dkr(n * L);
    for (size_t e = 0; e < n * L; ++e) {
        kr[e] = make_double2(stt->QK[e], stt->QR[e]);
        dkr[e] = make_double2(stt->dQK[e], stt->dQR[e]);
    }
    CK(cudaMemcpyAsync(c->d.KR, kr.data(), n * L * sizeof(double2), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.dKR, dkr.data(), n * L * sizeof(double2), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.rvec, stt->rvec, n * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.drvec, stt->drvec, n * sizeof(double), cudaMemcpyHostToDevice, c->st));
    c->n = n;
    c->t1.assign(stt->t1grid, stt->t1grid + n);
    c->dtr.assign(stt->delta_t_ratio, stt->delta_t_ratio + n);
    if ((s = c->mirror_all())) return s;
    if ((s = c->clear_tail(n_old))) return s;
    if ((s = c->upload_times())) return s;
    if ((s = c->pos_init())) return s;
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_state_rows(void* p, size_t* n) {
    if (!p || !n) return fail(DYN_ERR_INVALID, "null argument");
    *n = C(p)->n;
    return DYN_OK;
}

dyn_status dyn_state_time(void* p, double* t) {
    if (!p || !t) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    *t = c->n ? c->t1[c->n - 1] : 0.0;
    return DYN_OK;
}

dyn_status dyn_state_download(void* p, dyn_state* stt) {
    if (!p || !stt) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    const size_t n = c->n, L = c->L;
    if (stt->n < n) return fail(DYN_ERR_INVALID, "state buffers hold fewer rows than the history");
    stt->n = n;
    std::vector<double2> kr(n * L), dkr(n * L);
    CK(cudaMemcpyAsync(kr.data(), c->d.KR, n * L * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(dkr.data(), c->d.dKR, n * L * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    if (stt->rvec) CK(cudaMemcpyAsync(stt->rvec, c->d.rvec, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    if (stt->drvec) CK(cudaMemcpyAsync(stt->drvec, c->d.drvec, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (size_t e = 0; e < n * L; ++e) {
        if (stt->QK) stt->QK[e] = kr[e].x;
        if (stt->QR) stt->QR[e] = kr[e].y;
        if (stt->dQK) stt->dQK[e] = dkr[e].x;
        if (stt->dQR) stt->dQR[e] = dkr[e].y;
    }
    if (stt->t1grid) std::memcpy(stt->t1grid, c->t1.data(), n * sizeof(double));
    if (stt->delta_t_ratio) std::memcpy(stt->delta_t_ratio, c->dtr.data(), n * sizeof(double));
    return DYN_OK;
}

dyn_status dyn_controller_get(void* p, dyn_controller* ctl) {
    if (!p || !ctl) return fail(DYN_ERR_INVALID, "null argument");
    *ctl = C(p)->ctl;
    return DYN_OK;
}

dyn_status dyn_controller_set(void* p, const dyn_controller* ctl) {
    if (!p || !ctl) return fail(DYN_ERR_INVALID, "null argument");
    C(p)->ctl = *ctl;
    return DYN_OK;
}

dyn_status dyn_interpolate(void* p, const double* posB1x, const double* posB2x) {
    if (!p) return fail(DYN_ERR_INVALID, "null ctx");
    Ctx* c = C(p);
    if (c->n == 0) return fail(DYN_ERR_STATE, "no state");
    if (!c->interp_alloc) {
        dyn_status s = dalloc(&c->d.ip, 16 * c->L2);
        if (s) return s;
        c->interp_alloc = true;
    }
    double *p1 = nullptr, *p2 = nullptr;
    if (posB1x) {
        if (dalloc(&p1, c->L)) return DYN_ERR_NOMEM;
        CK(cudaMemcpyAsync(p1, posB1x, c->L * sizeof(double), cudaMemcpyHostToDevice, c->st));
    }
    if (posB2x) {
        if (dalloc(&p2, c->L2)) { cudaFree(p1); return DYN_ERR_NOMEM; }
        CK(cudaMemcpyAsync(p2, posB2x, c->L2 * sizeof(double), cudaMemcpyHostToDevice, c->st));
    }
    cudaError_t e = launch_interp_exact(c->d, (int)c->n, p1, p2, c->st);
    cudaError_t e2 = cudaStreamSynchronize(c->st);
    if (p1) cudaFree(p1);
    if (p2) cudaFree(p2);
    CK(e);
    CK(e2);
    return DYN_OK;
}

dyn_status dyn_get_interp(void* p, int which, double* out) {
    if (!p || !out) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    const double* src;
    size_t count;
    if (which >= 0 && which < 16) {
        if (!c->interp_alloc) return fail(DYN_ERR_STATE, "call dyn_interpolate first");
        src = c->d.ip + (size_t)which * c->L2;
        count = c->L2;
    } else if (which == DYN_RINT) { src = c->d.rint; count = c->L; }
    else if (which == DYN_POSB1X) { src = c->d.posB1x; count = c->L; }
    else if (which == DYN_POSB2X) { src = c->d.posB2x; count = c->L2; }
    else return fail(DYN_ERR_INVALID, "unknown array");
    CK(cudaMemcpyAsync(out, src, count * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_get_interp_dev(void* p, int which, double* out) {
    if (!p || !out) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    const double* src;
    size_t count;
    if (which >= 0 && which < 16) {
        if (!c->interp_alloc) return fail(DYN_ERR_STATE, "call dyn_interpolate first");
        src = c->d.ip + (size_t)which * c->L2;
        count = c->L2;
    } else if (which == DYN_RINT) { src = c->d.rint; count = c->L; }
    else if (which == DYN_POSB1X) { src = c->d.posB1x; count = c->L; }
    else if (which == DYN_POSB2X) { src = c->d.posB2x; count = c->L2; }
    else return fail(DYN_ERR_INVALID, "unknown array");
    CK(cudaMemcpyAsync(out, src, count * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_interp_b1_dev(void* p, double* qk, double* qr) {
    if (!p || !qk || !qr) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    if (c->n == 0) return fail(DYN_ERR_STATE, "no state");
    CK(launch_b1_exact(c->d, (int)c->n, qk, qr, c->st));
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

static bool state_dev_complete(const dyn_state_dev* s) {
    return s && s->t1grid && s->delta_t_ratio && s->QK && s->QR && s->dQK && s->dQR && s->rvec && s->drvec;
}

dyn_status dyn_state_upload_dev(void* p, const dyn_state_dev* stt) {
    if (!p || !state_dev_complete(stt)) return fail(DYN_ERR_INVALID, "null argument or missing state array");
    Ctx* c = C(p);
    const size_t n = stt->n, L = c->L;
    if (n < 1) return fail(DYN_ERR_INVALID, "state needs at least one row");
    std::vector<double> t1(n), dtr(n);
    CK(cudaMemcpyAsync(t1.data(), stt->t1grid, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(dtr.data(), stt->delta_t_ratio, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (size_t k = 0; k < n; ++k) {
        if (!(t1[k] >= 0.0) || !std::isfinite(t1[k])) return fail(DYN_ERR_INVALID, "t1grid must be finite and non-negative");
        if (k && !(t1[k] >= t1[k - 1])) return fail(DYN_ERR_INVALID, "t1grid must be non-decreasing");
        if (!std::isfinite(dtr[k])) return fail(DYN_ERR_INVALID, "delta_t_ratio must be finite");
    }
    c->drop_graphs();
    c->gen++;
    const size_t n_old = c->n;
    c->n = 0;
    dyn_status s = c->ensure_rows(n + 1);
    if (s) return s;
    CK(launch_pack_rows(stt->QK, stt->QR, c->d.KR, n * L, c->st));
    CK(launch_pack_rows(stt->dQK, stt->dQR, c->d.dKR, n * L, c->st));
    CK(cudaMemcpyAsync(c->d.rvec, stt->rvec, n * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.drvec, stt->drvec, n * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
    c->n = n;
    c->t1 = std::move(t1);
    c->dtr = std::move(dtr);
    if ((s = c->mirror_all())) return s;
    if ((s = c->clear_tail(n_old))) return s;
    if ((s = c->upload_times())) return s;
    if ((s = c->pos_init())) return s;
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_state_rows_load_dev(void* p, size_t row0, size_t nrows, const dyn_state_dev* src) {
    if (!p || !state_dev_complete(src)) return fail(DYN_ERR_INVALID, "null argument or missing state array");
    Ctx* c = C(p);
    const size_t L = c->L;
    if (nrows == 0 || row0 + nrows > c->n) return fail(DYN_ERR_INVALID, "rows outside the history");
    const size_t o = row0 * L, cnt = nrows * L;
    CK(launch_pack_rows(src->QK + o, src->QR + o, c->d.KR + o, cnt, c->st));
    CK(launch_pack_rows(src->dQK + o, src->dQR + o, c->d.dKR + o, cnt, c->st));
    CK(cudaMemcpyAsync(c->d.rvec + row0, src->rvec + row0, nrows * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.drvec + row0, src->drvec + row0, nrows * sizeof(double), cudaMemcpyDeviceToDevice,
                       c->st));
    if (c->d.mixed) {
        CK(launch_mirror_rows(c->d.KR + o, c->d.KRf + o, cnt, c->st));
        CK(launch_mirror_rows(c->d.dKR + o, c->d.dKRf + o, cnt, c->st));
        if (c->d.KRl) CK(launch_mirror_lo(c->d.KR + o, c->d.KRl + o, cnt, c->st));
    }
    c->gen++;
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_state_rows_store_dev(void* p, size_t row0, size_t nrows, const dyn_state_dev* dst) {
    if (!p || !state_dev_complete(dst)) return fail(DYN_ERR_INVALID, "null argument or missing state array");
    Ctx* c = C(p);
    const size_t L = c->L;
    if (nrows == 0 || row0 + nrows > c->n) return fail(DYN_ERR_INVALID, "rows outside the history");
    const size_t o = row0 * L, cnt = nrows * L;
    CK(launch_unpack_rows(c->d.KR + o, dst->QK + o, dst->QR + o, cnt, c->st));
    CK(launch_unpack_rows(c->d.dKR + o, dst->dQK + o, dst->dQR + o, cnt, c->st));
    CK(cudaMemcpyAsync(dst->t1grid + row0, c->t1.data() + row0, nrows * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(dst->delta_t_ratio + row0, c->dtr.data() + row0, nrows * sizeof(double),
                       cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(dst->rvec + row0, c->d.rvec + row0, nrows * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(dst->drvec + row0, c->d.drvec + row0, nrows * sizeof(double), cudaMemcpyDeviceToDevice,
                       c->st));
    CK(cudaStreamSynchronize(c->st));  // the host time mirrors are the copies' sources
    return DYN_OK;
}

dyn_status dyn_qkr_step(void* p, double* hK, double* hR) {
    if (!p || !hK || !hR) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    if (!c->interp_alloc) return fail(DYN_ERR_STATE, "call dyn_interpolate first");
    CK(launch_qkr_exact(c->d, (int)c->n, c->d.rhs_out, c->st));
    CK(cudaMemcpyAsync(c->rhs_h, c->d.rhs_out, c->L * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (int i = 0; i < c->L; ++i) { hK[i] = c->rhs_h[i].x; hR[i] = c->rhs_h[i].y; }
    return DYN_OK;
}

dyn_status dyn_rhs(void* p, double* hK, double* hR) {
    if (!p || !hK || !hR) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    if (c->n == 0) return fail(DYN_ERR_STATE, "no state");
    std::memset(c->stages_h, 0, sizeof(StageDev));
    StageDev& sp = c->stages_h[0];
    sp.kind = KIND_RHS;
    sp.nrows = (int)c->n;
    sp.n0 = (int)c->n;
    sp.T = c->t1[c->n - 1];
    Ctx::set_clamps(sp);
    sp.b2_save = NSAVE;  // keep posB2x of the current state readable
    sp.b2_reuse = sp.pos_save = sp.pos_reuse = sp.nb2_save = sp.nb2_reuse = -1;
    dyn_status s = c->pos_init();
    if (s) return s;
    CK(cudaMemcpyAsync(c->d.stages, c->stages_h, sizeof(StageDev), cudaMemcpyHostToDevice, c->st));
    CK(launch_stage(c->d, 0, c->st));
    CK(cudaMemcpyAsync(c->rhs_h, c->d.rhs_out, c->L * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (int i = 0; i < c->L; ++i) { hK[i] = c->rhs_h[i].x; hR[i] = c->rhs_h[i].y; }
    return DYN_OK;
}

dyn_status dyn_rstep(void* p, double* r) {
    if (!p || !r) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    CK(launch_rstep_exact(c->d, (int)c->n, c->scratch_dev, c->st));
    CK(cudaMemcpyAsync(r, c->scratch_dev, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_drstep2(void* p, const double* qK, const double* qR, const double* dqK, const double* dqR, double t,
                       double* dr) {
    if (!p || !qK || !qR || !dqK || !dqR || !dr) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    const int L = c->L;
    double* buf = c->scratch_dev;
    CK(cudaMemcpyAsync(buf, qK, L * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(buf + L, qR, L * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(buf + 2 * L, dqK, L * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(buf + 3 * L, dqR, L * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(launch_drstep2_exact(c->d, buf, buf + L, buf + 2 * L, buf + 3 * L, t, buf + 4 * L, c->st));
    CK(cudaMemcpyAsync(dr, buf + 4 * L, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_energy(void* p, double* e) {
    if (!p || !e) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    CK(launch_energy_exact(c->d, (int)c->n, c->scratch_dev, c->st));
    CK(cudaMemcpyAsync(e, c->scratch_dev, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_tail_fit(void* p, int last_rollback_loop, dyn_tail_info* info) {
    if (!p) return fail(DYN_ERR_INVALID, "null ctx");
    Ctx* c = C(p);
    TraceRange tr("dyn_tail_fit");
    dyn_status s = tail_fit(c, last_rollback_loop);
    if (s || !info) return s;
    TailState t;
    CK(cudaMemcpyAsync(&t, c->tail, sizeof t, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    info->alpha_raw = t.alpha_raw;
    info->alpha = t.alpha;
    info->j0 = t.j0;
    info->applied = t.applied;
    return DYN_OK;
}

dyn_status dyn_tail_fit_reset(void* p) {
    if (!p) return fail(DYN_ERR_INVALID, "null ctx");
    return tail_reset(C(p));
}

dyn_status dyn_energy_history(void* p, double* e, size_t n_rows) {
    if (!p || !e) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    if (n_rows != c->n) return fail(DYN_ERR_INVALID, "n_rows must equal the history rows");
    double* buf;
    if (dalloc(&buf, n_rows)) return DYN_ERR_NOMEM;
    cudaError_t err = launch_energy_history(c->d, (int)n_rows, buf, c->st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(e, buf, n_rows * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(c->st);
    cudaFree(buf);
    CK(err);
    return DYN_OK;
}

dyn_status dyn_conv_dev(void* p, int kind, const double* f, const double* g, size_t n, double t, double* out) {
    if (!p || !f || !g || !out) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    if (n != (size_t)c->L && n != c->L2) return fail(DYN_ERR_INVALID, "n must be len or len*len");
    CK(launch_conv_exact(c->d, kind, f, g, n, t, out, c->st));
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_search_dev(void* p, const double* list, size_t nlist, const double* elem, size_t nelem, double* out) {
    if (!p || !list || !elem || !out || nlist == 0) return fail(DYN_ERR_INVALID, "bad argument");
    Ctx* c = C(p);
    CK(launch_search(c->d, list, nlist, elem, nelem, out, c->st));
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_update(void* p, int method, double delta_t, dyn_step_result* res) {
    if (!p) return fail(DYN_ERR_INVALID, "null ctx");
    if (method < 1) return fail(DYN_ERR_INVALID, "unknown method");
    if (!(delta_t > 0.0)) return fail(DYN_ERR_INVALID, "delta_t must be positive");
    TraceRange tr("dyn_update");
    return C(p)->step(method, delta_t, res);
}

// simulation_runner.cpp:125-304 for a fixed number of iterations
dyn_status dyn_run(void* p, const dyn_run_params* rp, dyn_step_result* last) {
    if (!p || !rp) return fail(DYN_ERR_INVALID, "null argument");
    TraceRange tr("dyn_run");
    Ctx* c = C(p);
    dyn_controller& k = c->ctl;
    const double dmax = c->cfg.delta_max, dmin = c->cfg.delta_t_min;
    if (!rp->dt_schedule && (k.method < 1 || !(k.delta_t > 0.0)))
        return fail(DYN_ERR_STATE, "no step size or method: call dyn_controller_set after dyn_state_upload");
    dyn_step_result r{};
    for (int it = 0; it < rp->nsteps; ++it) {
        if (rp->tmax > 0 && c->t1[c->n - 1] >= rp->tmax) break;
        if (rp->dt_schedule) {
            k.delta_t = rp->dt_schedule[it];
            k.method = rp->method_schedule ? rp->method_schedule[it] : k.method;
        }
        const double t = c->t1[c->n - 1] + k.delta_t;
        TraceRange ts("dyn_run step");
        if (rp->out_dt) rp->out_dt[it] = k.delta_t;
        if (rp->out_method) rp->out_method[it] = k.method;
        k.delta_old = k.delta;
        dyn_status s = c->step(k.method, k.delta_t, &r);
        if (s) return s;
        if (!std::isfinite(r.delta)) {
            // the state holds non-finite values: stop before the controller acts on them
            if (rp->out_delta) rp->out_delta[it] = r.delta;
            if (rp->out_t) rp->out_t[it] = t;
            if (rp->out_energy) rp->out_energy[it] = r.energy;
            if (rp->out_qk0) rp->out_qk0[it] = r.qk0;
            if (rp->out_r) rp->out_r[it] = r.r;
            if (last) *last = r;
            return fail(DYN_ERR_NONFINITE, "dyn_run: non-finite error estimate at iteration " + std::to_string(it));
        }
        k.delta = r.delta;
        if (rp->tail_fit) {  // simulation_runner.cpp:135-141
            if ((s = tail_fit(c, c->last_rollback_loop))) return s;
            if (rp->out_energy && (s = dyn_energy(p, &r.energy))) return s;  // of the fitted row
        }
        k.loop++;
        if (rp->sparsify_every > 0 && k.loop % rp->sparsify_every == 0) {
            // simulation_runner.cpp:148-237: sweeps while the history shrinks, then
            // (outside a replayed schedule) the step halving
            size_t prev = c->n;
            const int sweeps = sparsify_block_sweeps(rp->sparsify_sweeps);
            for (int sw = 0; sw < sweeps; ++sw) {
                size_t nn = prev;
                if ((s = dyn_sparsify(p, dmax, rp->sparsify_variant, &nn))) return s;
                if (nn >= prev) break;
                prev = nn;
            }
            if (!rp->dt_schedule && k.delta < dmax / 2 && k.loop - c->last_rollback_loop > 1000) {
                k.delta_t *= 0.5;
                if (k.method == DYN_RK54) k.method = DYN_SSPRK104;
                else if (rp->use_serk2 && k.method < 2 + SMAX / 4) k.method++;  // init_SERK2(2 (init - 1))
            }
        }
        if (!rp->dt_schedule) {
            const double ratio = c->dtr[c->n - 1];
            if (k.delta < dmax && k.loop > 5 && (k.delta < 1.1 * k.delta_old || k.delta_old < dmax / 1000) &&
                RMAX[k.method - 1] / c->specRad > k.delta_t && ratio == 1.0) {
                k.delta_t *= 1.01;
            } else if (k.delta > 2 * dmax && k.delta_t > dmin) {
                k.delta_t *= 0.9;
            }
            if (k.method == DYN_SSPRK104 && k.delta > dmax && RMAX[0] / c->specRad > k.delta_t) {
                k.method = DYN_RK54;
                k.delta_t *= 0.5;
            }
            if (rp->gpu_rollback && k.delta > 2 * dmax) {
                // simulation_runner.cpp:280-304
                const int nr = std::min(10, std::max(0, (int)c->n - 2));
                if (nr > 0) {
                    if ((s = dyn_rollback(p, nr))) return s;
                    c->last_rollback_loop = k.loop;
                }
                k.delta_t = 0.5 * std::min(std::max(k.delta_t, dmin), RMAX[k.method - 1] / c->specRad);
                k.method = k.method > 3 ? 2 + (2 * (k.method - 3)) / 2 : DYN_SSPRK104;
            }
        }
        if (rp->out_delta) rp->out_delta[it] = k.delta;
        if (rp->out_t) rp->out_t[it] = t;
        if (rp->out_energy) rp->out_energy[it] = r.energy;
        if (rp->out_qk0) rp->out_qk0[it] = r.qk0;
        if (rp->out_r) rp->out_r[it] = r.r;
    }
    if (last) *last = r;
    return DYN_OK;
}

dyn_status dyn_rollback(void* p, int nrows) {
    if (!p) return fail(DYN_ERR_INVALID, "null ctx");
    Ctx* c = C(p);
    if (nrows < 0 || (size_t)nrows >= c->n - 1) return fail(DYN_ERR_INVALID, "cannot roll back that many rows");
    const size_t target = c->n - nrows, n_old = c->n;
    c->n = target;
    c->gen++;
    if (dyn_status cs = c->clear_tail(n_old)) return cs;
    c->t1.resize(target);
    c->dtr.resize(target);
    c->ctl.delta_t = c->t1[target - 1] - c->t1[target - 2];
    c->ctl.loop -= nrows;
    dyn_status s = c->pos_init();
    if (s) return s;
    CK(cudaStreamSynchronize(c->st));
    return DYN_OK;
}

dyn_status dyn_last_row(void* p, double* qK, double* qR) {
    if (!p || !qK || !qR) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    if (c->n == 0) return fail(DYN_ERR_STATE, "no state");
    CK(cudaMemcpyAsync(c->rhs_h, c->d.KR + (c->n - 1) * c->L, c->L * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (int i = 0; i < c->L; ++i) { qK[i] = c->rhs_h[i].x; qR[i] = c->rhs_h[i].y; }
    return DYN_OK;
}

dyn_status dyn_profile_stage(void* p, int reps, float* ms_main, float* ms_epi) {
    if (!p || !ms_main || !ms_epi || reps < 1) return fail(DYN_ERR_INVALID, "bad argument");
    Ctx* c = C(p);
    if (c->n < 2) return fail(DYN_ERR_STATE, "profile needs a history of at least two rows");
    std::memset(c->stages_h, 0, sizeof(StageDev));
    StageDev& sp = c->stages_h[0];
    sp.kind = KIND_RHS;
    sp.nrows = (int)c->n;
    sp.n0 = (int)c->n;
    sp.T = c->t1[c->n - 1];
    Ctx::set_clamps(sp);
    sp.b2_save = sp.b2_reuse = sp.pos_save = sp.pos_reuse = sp.nb2_save = sp.nb2_reuse = -1;
    dyn_status s = c->pos_init();
    if (s) return s;
    CK(cudaMemcpyAsync(c->d.stages, c->stages_h, sizeof(StageDev), cudaMemcpyHostToDevice, c->st));
    CK(launch_stage(c->d, 0, c->st));  // warm
    cudaEvent_t e0, e1, e2;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventCreate(&e2));
    float tm = 0.f, te = 0.f;
    for (int r = 0; r < reps; ++r) {
        float a, b;
        CK(cudaEventRecord(e0, c->st));
        CK(launch_main_only(c->d, 0, c->st));
        CK(cudaEventRecord(e1, c->st));
        CK(launch_epi_only(c->d, 0, c->st));
        CK(cudaEventRecord(e2, c->st));
        CK(cudaEventSynchronize(e2));
        CK(cudaEventElapsedTime(&a, e0, e1));
        CK(cudaEventElapsedTime(&b, e1, e2));
        tm += a;
        te += b;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    *ms_main = tm / reps;
    *ms_epi = te / reps;
    return DYN_OK;
}

dyn_status dyn_probe_fp64(int device, double* gflops) {
    if (!gflops) return fail(DYN_ERR_INVALID, "null argument");
    CK(cudaSetDevice(device));
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    double* buf;
    if (dalloc(&buf, 1)) return DYN_ERR_NOMEM;
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const int threads = 256, blocks = sms * 8, iters = 4096;
    CK(launch_fp64_probe(buf, blocks, threads, 64, st));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, st));
    CK(launch_fp64_probe(buf, blocks, threads, iters, st));
    CK(cudaEventRecord(b, st));
    CK(cudaEventSynchronize(b));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(st);
    cudaFree(buf);
    *gflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e9;
    return DYN_OK;
}

// sparsifyNscale / sparsifyNscaleGPU: device indicator per node, host index
// logic of the selected variant, one device compaction pass.
// ------------------------------------------------------------------ adjoint
dyn_status dyn_adjoint_forward(void* p, const dyn_run_params* rp, dyn_step_result* last) {
    if (!p || !rp) return fail(DYN_ERR_INVALID, "null argument");
    TraceRange tr("dyn_adjoint_forward");
    Ctx* c = C(p);
    if (c->d.mixed) return fail(DYN_ERR_UNSUPPORTED, "the adjoint runs on the FP64 form");
    if (c->d.logr) return fail(DYN_ERR_UNSUPPORTED, "the adjoint differentiates the linear-domain gathers only");
    if (rp->gpu_rollback || rp->sparsify_every > 0)
        return fail(DYN_ERR_INVALID, "the adjoint needs an append-only history: no rollback, no sparsify");
    if (rp->tail_fit) return fail(DYN_ERR_UNSUPPORTED, "the adjoint has no tail fit");
    if (c->n == 0) return fail(DYN_ERR_STATE, "no state: call dyn_state_init or dyn_state_upload");
    if (rp->nsteps < 0) return fail(DYN_ERR_INVALID, "nsteps must be non-negative");
    const size_t N = (size_t)rp->nsteps;
    std::vector<double> dts(N);
    std::vector<int> ms(N);
    dyn_run_params q = *rp;
    q.out_dt = dts.data();
    q.out_method = ms.data();
    const size_t n_start = c->n;
    c->adj_recorded = false;
    const auto t0 = std::chrono::steady_clock::now();
    dyn_status s = dyn_run(p, &q, last);
    if (s) return s;
    CK(cudaStreamSynchronize(c->st));
    const auto t1 = std::chrono::steady_clock::now();
    const size_t ran = c->n - n_start;
    dts.resize(ran);
    ms.resize(ran);
    if (rp->out_dt) std::memcpy(rp->out_dt, dts.data(), ran * sizeof(double));
    if (rp->out_method) std::memcpy(rp->out_method, ms.data(), ran * sizeof(int));
    c->adj_dt = std::move(dts);
    c->adj_method = std::move(ms);
    c->adj_n_start = n_start;
    c->adj_gen = c->gen;
    c->adj_recorded = true;
    c->adj_ms_forward = std::chrono::duration<double, std::milli>(t1 - t0).count();
    return DYN_OK;
}

dyn_status dyn_adjoint_backward(void* p, const dyn_adjoint_objective* obj, double* grad, dyn_adjoint_stats* stats) {
    if (!p || !obj || !grad) return fail(DYN_ERR_INVALID, "null argument");
    TraceRange tr("dyn_adjoint_backward");
    Ctx* c = C(p);
    if (!c->adj_recorded || c->gen != c->adj_gen)
        return fail(DYN_ERR_STATE, "no recorded forward: call dyn_adjoint_forward (the history changed since)");
    for (int m : c->adj_method)
        if (m != DYN_RK54 && m != DYN_SSPRK104) return fail(DYN_ERR_UNSUPPORTED, "adjoint of SERK2 steps is not built");
    if (c->L > 4096) return fail(DYN_ERR_UNSUPPORTED, "len <= 4096");
    dyn_status s = c->adjoint_alloc();
    if (s) return s;
    const auto t0 = std::chrono::steady_clock::now();
    const size_t n_final = c->n, N = c->adj_dt.size(), L = c->L;
    const std::vector<double> t1_saved = c->t1, dtr_saved = c->dtr;
    if ((s = c->snapshot(false))) return s;
    CK(cudaMemsetAsync(c->ad.HKR, 0, n_final * L * sizeof(double2), c->st));
    CK(cudaMemsetAsync(c->ad.HdKR, 0, n_final * L * sizeof(double2), c->st));
    CK(cudaMemsetAsync(c->ad.Hr, 0, n_final * sizeof(double), c->st));
    CK(cudaMemsetAsync(c->ad.Hdr, 0, n_final * sizeof(double), c->st));
    CK(cudaMemsetAsync(c->ad.sc, 0, 16 * sizeof(double), c->st));
    const AdjModel am{c->cfg.p, c->cfg.p2, c->cfg.lambda, c->cfg.T0, c->cfg.Gamma};
    const double* seeds[4] = {obj->c_K, obj->c_R, obj->c_dK, obj->c_dR};
    const double* dseeds[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int k = 0; k < 4; ++k) {
        if (!seeds[k]) continue;
        CK(cudaMemcpyAsync(c->ad_ck + k * L, seeds[k], L * sizeof(double), cudaMemcpyHostToDevice, c->st));
        dseeds[k] = c->ad_ck + k * L;
    }
    CK(launch_adj_seed(c->d, c->ad, am, (int)n_final - 1, obj->w_energy, obj->w_r, obj->w_dr, dseeds[0], dseeds[1],
                       dseeds[2], dseeds[3], c->st));
    for (size_t k = N; k-- > 0;) {
        const size_t n0 = c->adj_n_start + k;
        c->n = n0;
        c->t1.resize(n0);
        c->dtr.resize(n0);
        int S;
        if ((s = c->recompute_step(c->adj_method[k], c->adj_dt[k], &S))) return s;
        CK(launch_adj_verify(c->d, c->ad, c->snap_KR, c->snap_dKR, c->snap_time + 3 * c->cap, c->snap_time + 4 * c->cap,
                             (int)n0, c->st));
        CK(launch_adj_step(c->d, c->ad, am, S, (int)n0, c->st));
    }
    if (c->adj_n_start == 1) CK(launch_adj_initial(c->ad, am, c->st));
    double sc[16];
    CK(cudaMemcpyAsync(sc, c->ad.sc, sizeof sc, cudaMemcpyDeviceToHost, c->st));
    // the history back as the forward left it
    c->n = n_final;
    c->t1 = t1_saved;
    c->dtr = dtr_saved;
    if ((s = c->snapshot(true))) return s;
    if ((s = c->pos_init())) return s;
    CK(cudaStreamSynchronize(c->st));
    const auto t1 = std::chrono::steady_clock::now();
    grad[0] = sc[3];
    grad[1] = sc[4];
    if (stats) {
        stats->ms_forward = c->adj_ms_forward;
        stats->ms_backward = std::chrono::duration<double, std::milli>(t1 - t0).count();
        stats->device_bytes = c->adjoint_bytes();
        stats->steps = (int)N;
        stats->recompute_mismatch = (long long)sc[15];
    }
    return DYN_OK;
}

dyn_status dyn_adjoint_history_grad(void* p, dyn_state* g) {
    if (!p || !g) return fail(DYN_ERR_INVALID, "null argument");
    Ctx* c = C(p);
    if (!c->ad.HKR || !c->adj_recorded) return fail(DYN_ERR_STATE, "call dyn_adjoint_backward first");
    const size_t n = c->adj_n_start, L = c->L;
    if (g->n < n) return fail(DYN_ERR_INVALID, "gradient buffers hold fewer rows than the initial history");
    g->n = n;
    std::vector<double2> kr(n * L), dkr(n * L);
    CK(cudaMemcpyAsync(kr.data(), c->ad.HKR, n * L * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(dkr.data(), c->ad.HdKR, n * L * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    if (g->rvec) CK(cudaMemcpyAsync(g->rvec, c->ad.Hr, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    if (g->drvec) CK(cudaMemcpyAsync(g->drvec, c->ad.Hdr, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (size_t e = 0; e < n * L; ++e) {
        if (g->QK) g->QK[e] = kr[e].x;
        if (g->QR) g->QR[e] = kr[e].y;
        if (g->dQK) g->dQK[e] = dkr[e].x;
        if (g->dQR) g->dQR[e] = dkr[e].y;
    }
    return DYN_OK;
}

dyn_status dyn_sparsify(void* p, double threshold, int variant, size_t* n_out) {
    if (!p) return fail(DYN_ERR_INVALID, "null ctx");
    if (variant < 0 || variant > 2) return fail(DYN_ERR_INVALID, "unknown sparsify variant");
    TraceRange tr("dyn_sparsify");
    Ctx* c = C(p);
    const size_t n = c->n;
    if (n_out) *n_out = n;
    if (n < 3) return DYN_OK;
    unsigned char* fl_d;
    if (dalloc(&fl_d, n)) return DYN_ERR_NOMEM;
    std::vector<unsigned char> fl(n);
    cudaError_t e = launch_sparsify_flags(c->d, (int)n, variant, threshold, fl_d, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fl.data(), fl_d, n, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    cudaFree(fl_d);
    CK(e);
    std::vector<int> inds, indsD;
    std::vector<double> tfac, t1n, dtrn;
    if (!sparsify_indices(fl.data(), n, variant, c->t1, c->dtr, inds, indsD, tfac, t1n, dtrn)) return DYN_OK;
    const int k = (int)inds.size();
    // new buffers sized like the old capacity
    double2 *KRn, *dKRn;
    double *rn, *drn, *dtmp;
    int* id;
    dyn_status s;
    if ((s = dalloc(&KRn, c->cap * c->L)) || (s = dalloc(&dKRn, c->cap * c->L)) || (s = dalloc(&rn, c->cap)) ||
        (s = dalloc(&drn, c->cap)) || (s = dalloc(&id, 2 * (size_t)k)) || (s = dalloc(&dtmp, (size_t)k)))
        return s;
    CK(cudaMemcpyAsync(id, inds.data(), k * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(id + k, indsD.data(), k * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(dtmp, tfac.data(), k * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(launch_compact(c->d, id, id + k, variant == 0 ? nullptr : dtmp, k, KRn, dKRn, rn, drn, c->st));
    CK(cudaStreamSynchronize(c->st));
    cudaFree(id);
    cudaFree(dtmp);
    cudaFree(c->d.KR); cudaFree(c->d.dKR); cudaFree(c->d.rvec); cudaFree(c->d.drvec);
    c->d.KR = KRn; c->d.dKR = dKRn; c->d.rvec = rn; c->d.drvec = drn;
    c->drop_graphs();
    c->t1 = t1n;
    c->dtr = dtrn;
    const size_t n_old = c->n;
    c->n = k;
    c->gen++;
    if ((s = c->mirror_all())) return s;
    if ((s = c->clear_tail(n_old))) return s;
    if ((s = c->upload_times())) return s;
    if ((s = c->pos_init())) return s;
    CK(cudaStreamSynchronize(c->st));
    if (n_out) *n_out = c->n;
    return DYN_OK;
}

}  // extern "C"
