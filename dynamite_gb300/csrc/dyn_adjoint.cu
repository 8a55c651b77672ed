// Discrete adjoint of the FP64 RK-stepped hot path (fixed step schedule).
//
// The two-time history is append-only: a step reads rows 0..n0-1 and writes
// row n0, so the state before any step is a prefix of the final history.
// The reverse sweep therefore needs no stored checkpoints besides the final
// history itself: for step k (last to first) the host recomputes that one
// step's stages from the prefix with the forward kernels (snapshotting the
// row-n0 state and the B1 positions each stage reads), then runs the stages
// backwards:
//
//   k_adj_rowwrite   row n0 after stage s: r = rstep(G_s) (time_steps.cpp:83-92),
//                    dQK/dQR = tdiff_s h_0, dr = tdiff_s DR and the RK
//                    combination G_s = g0 + sum_j coef_j h_j, transposed;
//   k_adj_drstep     DR = drstep2(g0, h_0) (time_steps.cpp:117-125), transposed;
//   k_adj_restore    puts row n0 back into stage s's input state;
//   k_adj_epi        the RHS epilogue (QKstep/QRstep, time_steps.cpp:27-47,
//                    94-100) transposed: row cotangents of the eight memory
//                    integrals, the direct last-row terms, QK^{B1}[i,0] and
//                    rInt (index_vec.cpp:63-156) scattered to the history;
//   k_adj_targets    per target (i,j): the A1/A2/B1/B2 gathers recomputed,
//                    Sigma and the int.dat products differentiated, and the
//                    gathers transposed (scatter-adds into the cotangent
//                    history; the last-row stencils through shared memory and
//                    a per-row partial, reduced by k_adj_lastreduce).
//
// Parameter derivatives (Gamma, lambda) accumulate in device scalars.
#include <cmath>
#include "dyn_epi.cuh"

namespace dyn {

namespace {

enum { SC_RHO = 0, SC_DELTA = 1, SC_DR = 2, SC_GAMMA = 3, SC_LAMBDA = 4 };

__device__ __forceinline__ double qpow(double q, int e) { return e < 0 ? 0.0 : ipow_r(q, e); }
__device__ __forceinline__ double falpha(int p, int k) {
    double a = 1.0;
    for (int j = 0; j < k; ++j) a *= (double)(p - j);
    return a;
}
// k-th derivative of f(q) = lam q^p + (1-lam) q^p2 and its derivative in lam
__device__ __forceinline__ void fder(const AdjModel& m, int k, double q, double& v, double& vl) {
    const double tp = falpha(m.p, k) * qpow(q, m.p - k), tp2 = falpha(m.p2, k) * qpow(q, m.p2 - k);
    v = m.lam * tp + (1.0 - m.lam) * tp2;
    vl = tp - tp2;
}

// The same with the exponents known at compile time (P < 0: runtime exponents)
template <int P, int K>
__host__ __device__ constexpr double alpha_c() {
    double a = 1.0;
    for (int j = 0; j < K; ++j) a *= (double)(P - j);
    return a;
}
template <int P, int P2, int K>
__device__ __forceinline__ void fder_t(const AdjModel& m, double q, double& v, double& vl);
template <int P, int P2, int K>
__device__ __forceinline__ double fd_t(const AdjModel& m, double q) {
    double v, vl;
    fder_t<P, P2, K>(m, q, v, vl);
    return v;
}
template <int P, int P2, int K>
__device__ __forceinline__ void fder_t(const AdjModel& m, double q, double& v, double& vl) {
    if constexpr (P < 0) {
        fder(m, K, q, v, vl);
    } else {
        constexpr double ap = alpha_c<P, K>(), ap2 = alpha_c<P2, K>();
        const double tp = (P - K >= 0 && ap != 0.0) ? ap * ipow_c<(P - K >= 0 ? P - K : 0)>(q) : 0.0;
        const double tp2 = (P2 - K >= 0 && ap2 != 0.0) ? ap2 * ipow_c<(P2 - K >= 0 ? P2 - K : 0)>(q) : 0.0;
        v = m.lam * tp + (1.0 - m.lam) * tp2;
        vl = tp - tp2;
    }
}

// block-wide sum (blockDim.x a multiple of 32, <= 1024); every thread gets it
__device__ double block_sum(double v) {
    __shared__ double s_w[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) s_w[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int k = 0; k < nw; ++k) t += s_w[k];
    return t;
}

__device__ __forceinline__ void add2(double2* p, double x, double y) {
    atomicAdd(&p->x, x);
    atomicAdd(&p->y, y);
}

// ---------------------------------------------------------------- seeds
// J = wE * E(t_f) + sum_j cK[j] C(t_f, theta_j t_f) + wR * r(t_f) on row nl
template <int P, int P2>
__global__ void __launch_bounds__(256) k_adj_seed(const DevCtx c, const AdjDev a, const AdjModel am, const int nl, const double wE,
                           const double wR, const double wDr, const double* cK, const double* cR, const double* cdK,
                           const double* cdR) {
    const int L = c.L;
    const double tf = c.t1grid[nl];
    double lam = 0.0;
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        const double2 g = c.KR[(size_t)nl * L + j];
        const double w = c.integ[j];
        double f1, f1l, f2, f2l;
        fder_t<P, P2, 1>(am, g.x, f1, f1l);
        fder_t<P, P2, 2>(am, g.x, f2, f2l);
        // E = -(t sum_j w_j f'(K_j) R_j + f'(K_0)/T0)
        double kb = -(tf * w * f2 * g.y) - (j == 0 ? f2 / am.T0 : 0.0);
        const double rb = -(tf * w * f1);
        lam += -(tf * w * f1l * g.y) - (j == 0 ? f1l / am.T0 : 0.0);
        kb *= wE;
        if (cK) kb += cK[j];
        double2* h = a.HKR + (size_t)nl * L + j;
        h->x += kb;
        h->y += wE * rb + (cR ? cR[j] : 0.0);
        double2* hd = a.HdKR + (size_t)nl * L + j;
        hd->x += cdK ? cdK[j] : 0.0;
        hd->y += cdR ? cdR[j] : 0.0;
    }
    lam = block_sum(lam);
    if (threadIdx.x == 0) {
        a.sc[SC_LAMBDA] += wE * lam;
        a.Hr[nl] += wR;
        a.Hdr[nl] += wDr;
    }
}

// cotangents of row n0 (state after the last stage) into the stage buffers
__global__ void k_adj_move(const DevCtx c, const AdjDev a, const int n0) {
    const int L = c.L;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
        a.Gbar[j] = a.HKR[(size_t)n0 * L + j];
        a.Dbar[j] = a.HdKR[(size_t)n0 * L + j];
        a.HKR[(size_t)n0 * L + j] = make_double2(0.0, 0.0);
        a.HdKR[(size_t)n0 * L + j] = make_double2(0.0, 0.0);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.sc[SC_RHO] = a.Hr[n0];
        a.sc[SC_DELTA] = a.Hdr[n0];
        a.Hr[n0] = 0.0;
        a.Hdr[n0] = 0.0;
    }
}

// ------------------------------------------------- row write of stage s
template <int P, int P2>
__global__ void __launch_bounds__(256) k_adj_rowwrite(const DevCtx c, const AdjDev a, const AdjModel am, const int s) {
    const StageDev& sp = c.stages[s];
    const int L = c.L;
    const double tn = sp.T_next, td = sp.tdiff;
    const double rb = a.sc[SC_RHO], db = a.sc[SC_DELTA];
    double lam = 0.0;
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        const double2 G = a.Gsave[(size_t)s * L + j];
        const double w = c.integ[j];
        double f1, f1l, f2, f2l, f3, f3l;
        fder_t<P, P2, 1>(am, G.x, f1, f1l);
        fder_t<P, P2, 2>(am, G.x, f2, f2l);
        fder_t<P, P2, 3>(am, G.x, f3, f3l);
        // r = Gamma + sum_j tn w (f''(K) R K + f'(K) R) + f'(K_0) K_0 / T0
        double dK = tn * w * (f3 * G.y * G.x + 2.0 * f2 * G.y);
        const double dR = tn * w * (f2 * G.x + f1);
        lam += tn * w * (f2l * G.y * G.x + f1l * G.y);
        if (j == 0) {
            dK += (f2 * G.x + f1) / am.T0;
            lam += f1l * G.x / am.T0;
        }
        const double2 gb0 = a.Gbar[j];
        const double2 Gb = make_double2(gb0.x + rb * dK, gb0.y + rb * dR);
        // G_s = g0 + sum_{j<=s} coef_j h_j
        double2 g0b = a.g0bar[j];
        g0b.x += Gb.x;
        g0b.y += Gb.y;
        a.g0bar[j] = g0b;
        for (int q = 0; q < sp.ncoef; ++q) {
            double2 hb = a.hbar[(size_t)q * L + j];
            hb.x += sp.coef[q] * Gb.x;
            hb.y += sp.coef[q] * Gb.y;
            a.hbar[(size_t)q * L + j] = hb;
        }
        // dQK, dQR of row n0 = tdiff_s h_0
        const double2 Db = a.Dbar[j];
        double2 h0b = a.hbar[j];
        h0b.x += td * Db.x;
        h0b.y += td * Db.y;
        a.hbar[j] = h0b;
    }
    lam = block_sum(lam);
    if (threadIdx.x == 0) {
        a.sc[SC_LAMBDA] += rb * lam;
        a.sc[SC_GAMMA] += rb;
        a.sc[SC_DR] += td * db;  // dr of row n0 = tdiff_s DR
    }
}

// DR = drstep2(g0, h_0) at the step start (stage 0 time)
template <int P, int P2>
__global__ void __launch_bounds__(256) k_adj_drstep(const DevCtx c, const AdjDev a, const AdjModel am, const int n0) {
    const int L = c.L;
    const double T = c.stages[0].T, DRb = a.sc[SC_DR];
    double lam = 0.0;
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        const double2 g = c.KR[(size_t)(n0 - 1) * L + j];
        const double2 h = c.h[j];
        const double w = c.integ[j], tw = T * w;
        const double K = g.x, R = g.y, hK = h.x, hR = h.y;
        double f1, f1l, f2, f2l, f3, f3l, f4, f4l;
        fder_t<P, P2, 1>(am, K, f1, f1l);
        fder_t<P, P2, 2>(am, K, f2, f2l);
        fder_t<P, P2, 3>(am, K, f3, f3l);
        fder_t<P, P2, 4>(am, K, f4, f4l);
        double dK = w * (f3 * R * K + 2.0 * f2 * R) + tw * (f4 * R * hK * K + 3.0 * f3 * R * hK + f3 * hR * K + 2.0 * f2 * hR);
        const double dR = w * (f2 * K + f1) + tw * (f3 * hK * K + 2.0 * f2 * hK);
        double dhK = tw * (f3 * R * K + 2.0 * f2 * R);
        const double dhR = tw * (f2 * K + f1);
        double dl = w * (f2l * R * K + f1l * R) + tw * (f3l * R * hK * K + f2l * hR * K + 2.0 * f2l * hK * R + f1l * hR);
        if (j == 0) {
            dK += (f3 * K + 2.0 * f2) * hK / am.T0;
            dhK += (f2 * K + f1) / am.T0;
            dl += (f2l * K + f1l) * hK / am.T0;
        }
        double2 gb = a.g0bar[j];
        gb.x += DRb * dK;
        gb.y += DRb * dR;
        a.g0bar[j] = gb;
        double2 hb = a.hbar[j];
        hb.x += DRb * dhK;
        hb.y += DRb * dhR;
        a.hbar[j] = hb;
        lam += dl;
    }
    lam = block_sum(lam);
    if (threadIdx.x == 0) a.sc[SC_LAMBDA] += DRb * lam;
}

// row n0 back into stage s's input state (the state after stage s-1) and the
// B1 positions stage s read
__global__ void k_adj_restore(const DevCtx c, const AdjDev a, const int s, const int n0) {
    const int L = c.L;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
        c.posB1x[j] = a.Psave[(size_t)s * L + j];
        if (s >= 1) {
            c.KR[(size_t)n0 * L + j] = a.Gsave[(size_t)(s - 1) * L + j];
            c.dKR[(size_t)n0 * L + j] = a.Dsave[(size_t)(s - 1) * L + j];
        }
    }
    if (s >= 1 && blockIdx.x == 0 && threadIdx.x == 0) {
        const StageDev& pv = c.stages[s - 1];
        c.rvec[n0] = a.rsave[s - 1];
        c.drvec[n0] = a.drsave[s - 1];
        c.t1grid[n0] = pv.T_next;
        c.dtr[n0] = pv.dtr_new;
        c.inv_dtr[n0] = pv.dtr_new != 0.0 ? 1.0 / pv.dtr_new : 0.0;
    }
}

// Hermite weights of the B1 interpolation of row i (as k_main's rowval)
struct B1W {
    int F, cubic;
    double c0, c1, c2, c3;
};
__device__ __forceinline__ B1W b1w(const DevCtx& c, const StageDev& sp, int i) {
    const B1Row r = b1_row(c, c.posB1x[i], sp.maxceil, sp.nrows);
    return {r.F, r.cubic, r.c0, r.c1, r.c2, r.c3};
}
__device__ __forceinline__ double rint_of(const DevCtx& c, const B1W& w) {
    double ri = w.c0 * c.rvec[w.F - 1] + w.c1 * c.rvec[w.F] - w.c2 * c.drvec[w.F];
    if (w.cubic) ri -= w.c3 * c.drvec[w.F + 1];
    return ri;
}
__device__ __forceinline__ void scatter_rint(const DevCtx& c, const AdjDev& a, const B1W& w, double rb) {
    atomicAdd(a.Hr + w.F - 1, w.c0 * rb);
    atomicAdd(a.Hr + w.F, w.c1 * rb);
    atomicAdd(a.Hdr + w.F, -w.c2 * rb);
    if (w.cubic) atomicAdd(a.Hdr + w.F + 1, -w.c3 * rb);
}

// --------------------------------------------------------- RHS epilogue
template <int P, int P2>
__global__ void __launch_bounds__(256) k_adj_epi(const DevCtx c, const AdjDev a, const AdjModel am, const int s) {
    const StageDev& sp = c.stages[s];
    const int L = c.L, nrows = sp.nrows, lr = nrows - 1;
    const double t = sp.T;
    const bool live = t > 0.0;
    const double q0 = c.KR[(size_t)lr * L].x;
    double rE;
    B1W wE{};
    if (live) {
        wE = b1w(c, sp, L - 1);
        rE = rint_of(c, wE);
    } else {
        rE = c.rvec[0];
    }
    double f1q0, f1lq0;
    fder_t<P, P2, 1>(am, q0, f1q0, f1lq0);
    const double fac1 = f1q0 / am.T0, fac2 = q0 / am.T0;
    double sE = 0.0, sF1 = 0.0, sF2 = 0.0, lam = 0.0, gam = 0.0;
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        const double2 q = c.KR[(size_t)lr * L + i];
        double qb, ri;
        B1W w{};
        if (live) {
            w = b1w(c, sp, i);
            qb = w.c0 * c.KR[(size_t)(w.F - 1) * L].x + w.c1 * c.KR[(size_t)w.F * L].x - w.c2 * c.dKR[(size_t)w.F * L].x;
            if (w.cubic) qb -= w.c3 * c.dKR[(size_t)(w.F + 1) * L].x;
            ri = rint_of(c, w);
        } else {
            qb = c.KR[0].x;
            ri = c.rvec[0];
        }
        const double th = c.theta[i], tA = t * th, tR = t * (1.0 - th);
        const double2 hb = a.hbar[(size_t)s * L + i];
        // hK = d1 + d2 th;  hR = (R (-rE) + a6 tR) + (R ri - a7 tR) th
        const double d1b = hb.x, d2b = th * hb.x;
        double* ab = a.abar + (size_t)i * 8;
        ab[0] = tR * d1b;
        ab[1] = tA * d1b;
        ab[2] = tA * d1b;
        ab[3] = tR * d2b;
        ab[4] = tA * d2b;
        ab[5] = tA * d2b;
        ab[6] = tR * hb.y;
        ab[7] = -tR * th * hb.y;
        // d1 = qb fac1 - K rE + ...;  d2 = f'(qb) fac2 + 2 Gamma R + ... - K ri
        const double Kb = -rE * d1b - ri * d2b;
        const double Rb = hb.y * (-rE + ri * th) + 2.0 * am.Gamma * d2b;
        add2(a.HKR + (size_t)lr * L + i, Kb, Rb);
        sE += -q.y * hb.y - q.x * d1b;
        const double rib = q.y * th * hb.y - q.x * d2b;
        double f1qb, f1lqb;
        fder_t<P, P2, 1>(am, qb, f1qb, f1lqb);
        const double qbb = fac1 * d1b + fd_t<P, P2, 2>(am, qb) * fac2 * d2b;
        sF1 += qb * d1b;
        sF2 += f1qb * d2b;
        lam += f1lqb * fac2 * d2b;
        gam += 2.0 * q.y * d2b;
        if (live) {
            atomicAdd(&a.HKR[(size_t)(w.F - 1) * L].x, w.c0 * qbb);
            atomicAdd(&a.HKR[(size_t)w.F * L].x, w.c1 * qbb);
            atomicAdd(&a.HdKR[(size_t)w.F * L].x, -w.c2 * qbb);
            if (w.cubic) atomicAdd(&a.HdKR[(size_t)(w.F + 1) * L].x, -w.c3 * qbb);
            scatter_rint(c, a, w, rib);
        } else {
            atomicAdd(&a.HKR[0].x, qbb);
            atomicAdd(a.Hr, rib);
        }
    }
    sE = block_sum(sE);
    sF1 = block_sum(sF1);
    sF2 = block_sum(sF2);
    lam = block_sum(lam);
    gam = block_sum(gam);
    if (threadIdx.x == 0) {
        // rE = rInt of row L-1; q0 = QK of the last row at theta = 0
        if (live) scatter_rint(c, a, wE, sE);
        else atomicAdd(a.Hr, sE);
        const double q0b = sF1 * fd_t<P, P2, 2>(am, q0) / am.T0 + sF2 / am.T0;
        atomicAdd(&a.HKR[(size_t)lr * L].x, q0b);
        atomicAdd(a.sc + SC_LAMBDA, lam + sF1 * f1lq0 / am.T0);
        atomicAdd(a.sc + SC_GAMMA, gam);
    }
}

// ------------------------------------------------------- per-target part
// One thread per target (i, j), 64-thread CTAs over (chunk, row): the
// gathered values recorded by the recompute, Sigma and the int.dat products
// differentiated, the B1 gathers transposed into the cotangent history
// (reductions), the A1/A2 cotangents of the target stored for k_adj_lastrow
// and its B2 packet for k_adj_b2ser.
template <int M, int P, int P2>
__global__ void __launch_bounds__(64) k_adj_targets(const DevCtx c, const AdjDev a, const AdjModel am, const int s) {
    const StageDev& sp = c.stages[s];
    const int L = c.L, i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
    const int nrows = sp.nrows;
    const double t = sp.T;
    if (!(t > 0.0)) return;  // t = 0: the memory integrals carry a factor t, all cotangents vanish
    __shared__ double s_c[4];
    __shared__ int s_bi[2];
    if (threadIdx.x == 0) {
        const B1Row r = b1_row(c, c.posB1x[i], sp.maxceil, nrows);
        s_c[0] = r.c0; s_c[1] = r.c1; s_c[2] = r.c2; s_c[3] = r.c3;
        s_bi[0] = r.F; s_bi[1] = r.cubic;
    }
    __syncthreads();
    double lam = 0.0;
    if (j < L) {
        double ab[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) ab[k] = a.abar[(size_t)i * 8 + k];
        const double bc0 = s_c[0], bc1 = s_c[1], bc2 = s_c[2], bc3 = s_c[3];
        const int F = s_bi[0], cubic1 = s_bi[1];
        const size_t ij = (size_t)i * L + j;
        // ---- forward values, recorded by k_main in the recompute of this stage
        const GatherRec g = a.rec[(size_t)s * L * L + ij];
        const double2 a1 = g.a1, a2 = g.a2, b1 = g.b1, b2 = g.b2;
        const int X = g.X;
        const double x = g.x;
        // ---- Sigma and its derivatives
        double fA1[4], lA1[3], fA2[4], lA2[3], fB1[4], lB1[3], fB2[4], lB2[3];
        fder_t<P, P2, 1>(am, a1.x, fA1[1], lA1[0]);
        fder_t<P, P2, 2>(am, a1.x, fA1[2], lA1[1]);
        fder_t<P, P2, 3>(am, a1.x, fA1[3], lA1[2]);
        fder_t<P, P2, 1>(am, a2.x, fA2[1], lA2[0]);
        fder_t<P, P2, 2>(am, a2.x, fA2[2], lA2[1]);
        fder_t<P, P2, 3>(am, a2.x, fA2[3], lA2[2]);
        fder_t<P, P2, 1>(am, b1.x, fB1[1], lB1[0]);
        fder_t<P, P2, 2>(am, b1.x, fB1[2], lB1[1]);
        fder_t<P, P2, 3>(am, b1.x, fB1[3], lB1[2]);
        fder_t<P, P2, 1>(am, b2.x, fB2[1], lB2[0]);
        fder_t<P, P2, 2>(am, b2.x, fB2[2], lB2[1]);
        fder_t<P, P2, 3>(am, b2.x, fB2[3], lB2[2]);
        const double sKA1 = fA1[1], sRA1 = fA1[2] * a1.y, sRA2 = fA2[2] * a2.y;
        const double sKB1 = fB1[1], sRB1 = fB1[2] * b1.y, sKB2 = fB2[1], sRB2 = fB2[2] * b2.y;
        const double W = c.integ[j];
        // ---- cotangents of the eight products P_k (row sums a_k)
        const double sRA2b = W * (b2.x * ab[0] + b2.y * ab[6]);
        double b2Kb = W * sRA2 * ab[0], b2Rb = W * sRA2 * ab[6];
        const double sRA1b = W * b1.x * ab[1];
        double b1Kb = W * sRA1 * ab[1];
        const double sKA1b = W * b1.y * ab[2];
        double b1Rb = W * sKA1 * ab[2];
        double a2Rb = W * (sKB2 * ab[3] + sRB2 * ab[7]);
        const double sKB2b = W * a2.y * ab[3], sRB2b = W * a2.y * ab[7];
        double a1Rb = W * sKB1 * ab[4];
        const double sKB1b = W * a1.y * ab[4];
        double a1Kb = W * sRB1 * ab[5];
        const double sRB1b = W * a1.x * ab[5];
        // ---- Sigma transposed: sK = f'(K), sR = f''(K) R
        a1Kb += fA1[2] * sKA1b + fA1[3] * a1.y * sRA1b;
        a1Rb += fA1[2] * sRA1b;
        const double a2Kb = fA2[3] * a2.y * sRA2b;
        a2Rb += fA2[2] * sRA2b;
        b1Kb += fB1[2] * sKB1b + fB1[3] * b1.y * sRB1b;
        b1Rb += fB1[2] * sRB1b;
        b2Kb += fB2[2] * sKB2b + fB2[3] * b2.y * sRB2b;
        b2Rb += fB2[2] * sRB2b;
        lam = lA1[0] * sKA1b + lA1[1] * a1.y * sRA1b + lA2[1] * a2.y * sRA2b + lB1[0] * sKB1b + lB1[1] * b1.y * sRB1b +
              lB2[0] * sKB2b + lB2[1] * b2.y * sRB2b;
        // ---- gathers transposed: A1/A2 through k_adj_lastrow, B1/B2 here
        a.abarA[2 * ij] = make_double2(a1Kb, a1Rb);
        a.abarA[2 * ij + 1] = make_double2(a2Kb, a2Rb);
        add2(a.HKR + (size_t)(F - 1) * L + j, bc0 * b1Kb, bc0 * b1Rb);
        add2(a.HKR + (size_t)F * L + j, bc1 * b1Kb, bc1 * b1Rb);
        add2(a.HdKR + (size_t)F * L + j, -bc2 * b1Kb, -bc2 * b1Rb);
        if (cubic1) add2(a.HdKR + (size_t)(F + 1) * L + j, -bc3 * b1Kb, -bc3 * b1Rb);
        // B2 transposed by k_adj_b2ser from the packet in static order
        a.b2pk[__ldg(a.b2rank + ij)] = AdjDev::B2Packet{(int)ij, X, x, b2Kb, b2Rb};
    }
    lam = warp_sum(lam);
    if ((threadIdx.x & 31) == 0 && lam != 0.0) atomicAdd(a.sc + SC_LAMBDA, lam);
}

// A1/A2 gathers of target row i transposed onto the last row: a sparse
// matrix-vector product with the row's static column-sorted matrix (lrW,
// lrS, lrC; 2 L m entries).  Every thread takes an equal run of entries and
// accumulates column by column in registers, adding a column's partial sum to
// shared memory when it leaves the column: two FMAs per entry whatever the
// stencil starts look like (runs of equal starts near theta = 0 or 1 only
// make long columns, split over several threads).  The row goes to
// lbar_part[i] for k_adj_lastreduce.
__global__ void __launch_bounds__(256) k_adj_lastrow(const DevCtx c, const AdjDev a, const int s) {
    const StageDev& sp = c.stages[s];
    if (!(sp.T > 0.0)) return;
    const int L = c.L, i = blockIdx.x, E = 2 * L * c.m;
    extern __shared__ double2 s_acc[];  // [L] row sums, [2L] the row's A1/A2 cotangents (2j+t), int [L+1] column starts
    double2* s_cb = s_acc + L;
    int* s_cs = (int*)(s_acc + 3 * L);
    const size_t row = (size_t)i * L;
    const int* cs = a.lrC + (size_t)i * (L + 1);
    for (int k = threadIdx.x; k < L; k += blockDim.x) s_acc[k] = make_double2(0.0, 0.0);
    for (int k = threadIdx.x; k < 2 * L; k += blockDim.x) s_cb[k] = a.abarA[2 * row + k];
    for (int k = threadIdx.x; k <= L; k += blockDim.x) s_cs[k] = __ldg(cs + k);
    __syncthreads();
    const int per = (E + blockDim.x - 1) / blockDim.x;
    const int p0 = threadIdx.x * per, p1 = min(p0 + per, E);
    if (p0 < p1) {
        const double* w = a.lrW + (size_t)i * E;
        const int* src = a.lrS + (size_t)i * E;
        int lo = 0, hi = L;  // column of entry p0: the last k with cs[k] <= p0
        while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (s_cs[mid] <= p0) lo = mid; else hi = mid; }
        int k = lo, kend = s_cs[k + 1];
        double ax = 0.0, ay = 0.0;
        constexpr int B = 8;  // entries loaded ahead
        for (int pb = p0; pb < p1; pb += B) {
            double u[B];
            int si[B];
#pragma unroll
            for (int q = 0; q < B; ++q) {
                const bool in = pb + q < p1;
                u[q] = in ? __ldg(w + pb + q) : 0.0;
                si[q] = in ? __ldg(src + pb + q) : 0;
            }
#pragma unroll
            for (int q = 0; q < B; ++q) {
                const int p = pb + q;
                if (p >= p1) break;
                if (p >= kend) {
                    atomicAdd(&s_acc[k].x, ax);
                    atomicAdd(&s_acc[k].y, ay);
                    ax = ay = 0.0;
                    do { ++k; kend = s_cs[k + 1]; } while (p >= kend);
                }
                const double2 v = s_cb[si[q]];
                ax = fma(u[q], v.x, ax);
                ay = fma(u[q], v.y, ay);
            }
        }
        atomicAdd(&s_acc[k].x, ax);
        atomicAdd(&s_acc[k].y, ay);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < L; k += blockDim.x) a.lbar_part[row + k] = s_acc[k];
}

// B2 gathers transposed from the packets in static (iB2, phi2) order.  Each
// thread runs over B2_RUN consecutive packets; packets with the same key
// (X, iB2) add into the same 8 m history entries (K rows X-1, X; dK rows X,
// X+1; two components), so the thread accumulates them in registers (8 m
// FMAs per packet) and adds the sums to the history when the key changes or
// the run ends.  A warp whose 32 runs all carry one key (phi2 near 0 or 1)
// sums the runs across the warp first.  No key order is assumed: a key that
// recurs non-contiguously only means more additions.
constexpr int B2_RUN = 8;
__device__ __forceinline__ void b2_coeffs(const DevCtx& c, int X, double x, int nrows, double e[4]) {
    const double x2 = x * x, x3 = x2 * x;
    if (X < nrows - 1) {
        e[0] = 1.0 - 3.0 * x2 + 2.0 * x3;   // K row X-1
        e[1] = 3.0 * x2 - 2.0 * x3;         // K row X
        e[2] = x - 2.0 * x2 + x3;           // dK row X
        e[3] = (x3 - x2) * c.inv_dtr[X + 1];  // dK row X+1
    } else {
        e[0] = 1.0 - x2;
        e[1] = x2;
        e[2] = x - x2;
        e[3] = 0.0;
    }
}
template <int M>
__device__ __forceinline__ void b2_flush(const DevCtx& c, const AdjDev& a, int X, int iB2, bool cubic2,
                                         const double acc[M][8]) {
    const int L = c.L;
    const size_t base = (size_t)(X - 1) * L + iB2;
#pragma unroll
    for (int d = 0; d < M; ++d) {
        add2(a.HKR + base + d, acc[d][0], acc[d][1]);
        add2(a.HKR + base + L + d, acc[d][2], acc[d][3]);
        add2(a.HdKR + base + L + d, acc[d][4], acc[d][5]);
        if (cubic2) add2(a.HdKR + base + 2 * L + d, acc[d][6], acc[d][7]);
    }
}
template <int M>
__global__ void __launch_bounds__(128) k_adj_b2ser(const DevCtx c, const AdjDev a, const int s) {
    const StageDev& sp = c.stages[s];
    if (!(sp.T > 0.0)) return;
    const int L = c.L, nrows = sp.nrows, lane = threadIdx.x & 31;
    const long long NP = (long long)L * L;
    const long long q0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * B2_RUN;
    if (__ballot_sync(0xffffffffu, q0 < NP) == 0u) return;  // whole warp past the end
    double acc[M][8];
#pragma unroll
    for (int d = 0; d < M; ++d)
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[d][k] = 0.0;
    long long key = -1;
    int kX = 1, kB = 0, nkeys = 0;
    for (int r = 0; r < B2_RUN; ++r) {
        const long long q = q0 + r;
        if (q >= NP) break;
        const AdjDev::B2Packet pk = a.b2pk[q];
        const int iB2 = __ldg(c.iB2 + pk.ij);
        const long long kq = ((long long)pk.X << 32) | (unsigned)iB2;
        if (kq != key) {
            if (nkeys > 0) {
                b2_flush<M>(c, a, kX, kB, kX < nrows - 1, acc);
#pragma unroll
                for (int d = 0; d < M; ++d)
#pragma unroll
                    for (int k = 0; k < 8; ++k) acc[d][k] = 0.0;
            }
            key = kq;
            kX = pk.X;
            kB = iB2;
            ++nkeys;
        }
        double e[4];
        b2_coeffs(c, pk.X, pk.x, nrows, e);
        double eg[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            eg[2 * k] = e[k] * pk.gK;
            eg[2 * k + 1] = e[k] * pk.gR;
        }
        const double* w = c.wB2 + (size_t)pk.ij * M;
#pragma unroll
        for (int d = 0; d < M; ++d) {
            const double wd = __ldg(w + d);
#pragma unroll
            for (int k = 0; k < 8; ++k) acc[d][k] = fma(eg[k], wd, acc[d][k]);
        }
    }
    // one key over the whole warp: reduce across the lanes, 8 lanes add
    const long long k0 = __shfl_sync(0xffffffffu, key, 0);
    if (__all_sync(0xffffffffu, nkeys == 1 && key == k0)) {
        const int vi = warp_reduce8_index(lane);
        const bool cubic2 = kX < nrows - 1;
        const size_t base = (size_t)(kX - 1) * L + kB;
        // value vi: {K row X-1, K row X, dK row X, dK row X+1} x component
        double* dst = (double*)((vi >> 1) < 2 ? a.HKR : a.HdKR) +
                      2 * (base + ((vi >> 1) == 0 ? 0 : (vi >> 1) == 3 ? 2 * (size_t)L : (size_t)L)) + (vi & 1);
        const bool writer = (lane & 3) == 0 && ((vi >> 1) != 3 || cubic2);
#pragma unroll
        for (int d = 0; d < M; ++d) {
            const double tot = warp_reduce8(acc[d], lane);
            if (writer) atomicAdd(dst + 2 * d, tot);
        }
        return;
    }
    if (nkeys > 0) b2_flush<M>(c, a, kX, kB, kX < nrows - 1, acc);
}

// B2 transposed for a generic stencil depth: one thread per packet, m taps
// added directly.
__global__ void __launch_bounds__(256) k_adj_b2gen(const DevCtx c, const AdjDev a, const int s) {
    const StageDev& sp = c.stages[s];
    if (!(sp.T > 0.0)) return;
    const int L = c.L, m = c.m, nrows = sp.nrows;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)L * L) return;
    const AdjDev::B2Packet pk = a.b2pk[q];
    const int iB2 = __ldg(c.iB2 + pk.ij);
    double e[4];
    b2_coeffs(c, pk.X, pk.x, nrows, e);
    const bool cubic2 = pk.X < nrows - 1;
    const size_t base = (size_t)(pk.X - 1) * L + iB2;
    const double* w = c.wB2 + (size_t)pk.ij * m;
    for (int d = 0; d < m; ++d) {
        const double wd = __ldg(w + d);
        const double gK = wd * pk.gK, gR = wd * pk.gR;
        add2(a.HKR + base + d, e[0] * gK, e[0] * gR);
        add2(a.HKR + base + L + d, e[1] * gK, e[1] * gR);
        add2(a.HdKR + base + L + d, e[2] * gK, e[2] * gR);
        if (cubic2) add2(a.HdKR + base + 2 * L + d, e[3] * gK, e[3] * gR);
    }
}

// sum over target rows of the last-row stencil cotangents (none at t = 0):
// block (bx, by) sums columns bx*32.. over the row slice by, 8 row lanes
// per column, then adds its column totals to the history cotangent
constexpr int LR_COLS = 32, LR_LANES = 8, LR_SLICES = 16;
__global__ void __launch_bounds__(LR_COLS * LR_LANES) k_adj_lastreduce(const DevCtx c, const AdjDev a, const int s,
                                                                      const int lr) {
    const int L = c.L;
    if (!(c.stages[s].T > 0.0)) return;
    __shared__ double2 s_acc[LR_LANES][LR_COLS];
    const int tx = threadIdx.x % LR_COLS, ty = threadIdx.x / LR_COLS;
    const int k = blockIdx.x * LR_COLS + tx;
    const int rows = (L + LR_SLICES - 1) / LR_SLICES, i0 = blockIdx.y * rows, i1 = min(L, i0 + rows);
    double2 acc = make_double2(0.0, 0.0);
    if (k < L)
        for (int i = i0 + ty; i < i1; i += LR_LANES) {
            const double2 v = a.lbar_part[(size_t)i * L + k];
            acc.x += v.x;
            acc.y += v.y;
        }
    s_acc[ty][tx] = acc;
    __syncthreads();
    if (ty == 0 && k < L) {
        for (int q = 1; q < LR_LANES; ++q) {
            acc.x += s_acc[q][tx].x;
            acc.y += s_acc[q][tx].y;
        }
        add2(a.HKR + (size_t)lr * L + k, acc.x, acc.y);
    }
}

// g0 = row n0-1: its cotangent joins the history's
__global__ void k_adj_finish(const DevCtx c, const AdjDev a, const int n0) {
    const int L = c.L;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
        double2* h = a.HKR + (size_t)(n0 - 1) * L + j;
        const double2 g = a.g0bar[j];
        h->x += g.x;
        h->y += g.y;
    }
}

// t = 0 rows: r(0) = drvec(0) = Gamma + f'(1)/T0 (initialization.cpp:217-222)
__global__ void k_adj_initial(const AdjDev a, const AdjModel am) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double f1, f1l;
    fder(am, 1, 1.0, f1, f1l);
    const double rb = a.Hr[0] + a.Hdr[0];
    a.sc[SC_GAMMA] += rb;
    a.sc[SC_LAMBDA] += rb * f1l / am.T0;
}

// the recomputed row n0 against the forward's (snapshot): mismatching elements
__global__ void k_adj_verify(const DevCtx c, const AdjDev a, const double2* snapKR, const double2* snapdKR,
                             const double* snapr, const double* snapdr, const int n0) {
    const int L = c.L;
    int bad = 0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
        const double2 x = c.KR[(size_t)n0 * L + j], y = snapKR[(size_t)n0 * L + j];
        const double2 dx = c.dKR[(size_t)n0 * L + j], dy = snapdKR[(size_t)n0 * L + j];
        bad += (x.x != y.x) + (x.y != y.y) + (dx.x != dy.x) + (dx.y != dy.y);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) bad += (c.rvec[n0] != snapr[n0]) + (c.drvec[n0] != snapdr[n0]);
    if (bad) atomicAdd(a.sc + 15, (double)bad);
}

}  // namespace

cudaError_t launch_adj_verify(const DevCtx& c, const AdjDev& a, const double2* snapKR, const double2* snapdKR,
                              const double* snapr, const double* snapdr, int n0, cudaStream_t st) {
    k_adj_verify<<<(c.L + 255) / 256, 256, 0, st>>>(c, a, snapKR, snapdKR, snapr, snapdr, n0);
    return cudaGetLastError();
}

// ------------------------------------------------------------- launchers
// (p, p2) pairs with compile-time exponents; anything else takes the runtime ones
#define ADJ_DISPATCH(am, CALL)                                          \
    do {                                                                \
        if ((am).p == 3 && (am).p2 == 4) { constexpr int P = 3, P2 = 4; CALL; } \
        else if ((am).p == 3 && (am).p2 == 0) { constexpr int P = 3, P2 = 0; CALL; } \
        else { constexpr int P = -1, P2 = -1; CALL; }                   \
    } while (0)

cudaError_t launch_adj_seed(const DevCtx& c, const AdjDev& a, const AdjModel& am, int nl, double wE, double wR,
                            double wDr, const double* cK, const double* cR, const double* cdK, const double* cdR,
                            cudaStream_t st) {
    ADJ_DISPATCH(am, (k_adj_seed<P, P2><<<1, 256, 0, st>>>(c, a, am, nl, wE, wR, wDr, cK, cR, cdK, cdR)));
    return cudaGetLastError();
}

// k_adj_lastrow's shared memory: row sums, the row's A1/A2 cotangents and
// the column starts
size_t lastrow_smem(int L, int) { return 3 * (size_t)L * sizeof(double2) + (size_t)(L + 1) * sizeof(int); }

template <int P, int P2>
cudaError_t launch_targets_pp(const DevCtx& c, const AdjDev& a, const AdjModel& am, int s,
                              cudaStream_t st) {
    const dim3 grid((c.L + 63) / 64, c.L);
    const size_t lsm = lastrow_smem(c.L, c.m);
    const size_t NP = (size_t)c.L * c.L;
    if (c.m == 10) {
        k_adj_targets<10, P, P2><<<grid, 64, 0, st>>>(c, a, am, s);
        k_adj_lastrow<<<c.L, 256, lsm, st>>>(c, a, s);
        k_adj_b2ser<10><<<(unsigned)((NP + 128 * B2_RUN - 1) / (128 * B2_RUN)), 128, 0, st>>>(c, a, s);
    } else {
        k_adj_targets<0, P, P2><<<grid, 64, 0, st>>>(c, a, am, s);
        k_adj_lastrow<<<c.L, 256, lsm, st>>>(c, a, s);
        k_adj_b2gen<<<(unsigned)((NP + 255) / 256), 256, 0, st>>>(c, a, s);
    }
    return cudaGetLastError();
}
cudaError_t launch_targets(const DevCtx& c, const AdjDev& a, const AdjModel& am, int s,
                           cudaStream_t st) {
    if (am.p == 3 && am.p2 == 4) return launch_targets_pp<3, 4>(c, a, am, s, st);
    if (am.p == 3 && am.p2 == 0) return launch_targets_pp<3, 0>(c, a, am, s, st);
    return launch_targets_pp<-1, -1>(c, a, am, s, st);
}

cudaError_t launch_adj_step(const DevCtx& c, const AdjDev& a, const AdjModel& am, int S, int n0, cudaStream_t st) {
    const int L = c.L;
    const int eb = (L + 255) / 256;
    cudaError_t e;
    if ((e = cudaMemsetAsync(a.hbar, 0, (size_t)SMAX * L * sizeof(double2), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(a.g0bar, 0, (size_t)L * sizeof(double2), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(a.sc + SC_DR, 0, sizeof(double), st)) != cudaSuccess) return e;
    k_adj_move<<<eb, 256, 0, st>>>(c, a, n0);
    for (int s = S - 1; s >= 0; --s) {
        ADJ_DISPATCH(am, (k_adj_rowwrite<P, P2><<<1, 256, 0, st>>>(c, a, am, s)));
        if (s == 0) ADJ_DISPATCH(am, (k_adj_drstep<P, P2><<<1, 256, 0, st>>>(c, a, am, n0)));
        k_adj_restore<<<eb, 256, 0, st>>>(c, a, s, n0);
        ADJ_DISPATCH(am, (k_adj_epi<P, P2><<<1, 256, 0, st>>>(c, a, am, s)));
        if ((e = launch_targets(c, a, am, s, st)) != cudaSuccess) return e;
        // the last row of stage s is row n0 (s >= 1) or n0-1 (s = 0)
        k_adj_lastreduce<<<dim3((L + LR_COLS - 1) / LR_COLS, LR_SLICES), LR_COLS * LR_LANES, 0, st>>>(
            c, a, s, s >= 1 ? n0 : n0 - 1);
        if (s >= 1) k_adj_move<<<eb, 256, 0, st>>>(c, a, n0);
    }
    k_adj_finish<<<eb, 256, 0, st>>>(c, a, n0);
    return cudaGetLastError();
}

cudaError_t launch_adj_initial(const AdjDev& a, const AdjModel& am, cudaStream_t st) {
    k_adj_initial<<<1, 32, 0, st>>>(a, am);
    return cudaGetLastError();
}

cudaError_t adj_targets_smem_attr(int L, int m) {
    return cudaFuncSetAttribute(k_adj_lastrow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lastrow_smem(L, m));
}

}  // namespace dyn
