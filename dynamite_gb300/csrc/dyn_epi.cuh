// Stage epilogue of the DYNAMITE hot path as device functions, shared by the
// single-quench kernel k_epi (dyn_kernels.cu) and the batched epilogue
// (dyn_batch.cu): finish the row reductions, form the EOM right-hand side
// (QKstep/QRstep, time_steps.cpp:27-47,94-100), the RK stage combination
// (tableau or SERK2 recurrence, runge_kutta.cpp:19-252, runge_kutta.cu:397-487),
// write the history row (appendAll/replaceAll, time_steps.cpp:49-81,127-162),
// accumulate r(t) (rstep, time_steps.cpp:83-92), dr/dt at stage 0 (drstep2,
// time_steps.cpp:117-125) and, at the last stage, the error norm and the
// energy terms; the last CTA of a stage folds the per-CTA partials.
#pragma once
#include "dyn_kernels.cuh"

namespace dyn {

// Model helpers of the fused kernels (f', f'', f''' with FMA contraction)
template <int P, int P2>
struct Sig {
    __device__ __forceinline__ static void d12(const DModel& M, double q, double& a, double& b) {
        Sigma<P, P2>::eval(M, q, a, b);
    }
    __device__ __forceinline__ static double d1(const DModel& M, double q) {
        if constexpr (P >= 0) return fma(M.cA, ipow_c<P - 1>(q), M.cB * ipow_c<P2 - 1>(q));
        else return fma(M.cA, ipow_r(q, M.p - 1), M.cB * ipow_r(q, M.p2 - 1));
    }
    __device__ __forceinline__ static double d2(const DModel& M, double q) {
        if constexpr (P >= 0) return fma(M.cC, ipow_c<P - 2>(q), M.cD * ipow_c<P2 - 2>(q));
        else return fma(M.cC, ipow_r(q, M.p - 2), M.cD * ipow_r(q, M.p2 - 2));
    }
    __device__ __forceinline__ static double d3(const DModel& M, double q) {
        if constexpr (P >= 0) return fma(M.cE, ipow_c<P - 3>(q), M.cF * ipow_c<P2 - 3>(q));
        else return fma(M.cE, ipow_r(q, M.p - 3), M.cF * ipow_r(q, M.p2 - 3));
    }
};

// ------------------------------------------------------------------------
// FP64 gathers of the fused kernels (k_main, and the adjoint's recompute)
// sum_d w[d] * x[d] for K and R together (x interleaved)
template <int M>
__device__ __forceinline__ double2 dot2g(const double* __restrict__ w, const double2* __restrict__ x, int m) {
    double2 acc = make_double2(0.0, 0.0);
    if constexpr (M > 0 && (M % 2) == 0) {
        const double2* w2 = reinterpret_cast<const double2*>(w);
#pragma unroll
        for (int d = 0; d < M / 2; ++d) {
            const double2 ww = __ldg(w2 + d);
            const double2 xa = __ldg(x + 2 * d), xb = __ldg(x + 2 * d + 1);
            acc.x = fma(ww.x, xa.x, acc.x);
            acc.y = fma(ww.x, xa.y, acc.y);
            acc.x = fma(ww.y, xb.x, acc.x);
            acc.y = fma(ww.y, xb.y, acc.y);
        }
    } else {
        for (int d = 0; d < m; ++d) {
            const double ww = __ldg(w + d);
            const double2 xa = __ldg(x + d);
            acc.x = fma(ww, xa.x, acc.x);
            acc.y = fma(ww, xa.y, acc.y);
        }
    }
    return acc;
}

template <int M>
__device__ __forceinline__ double2 dot2s(const double* __restrict__ w, const double2* x, int m) {
    double2 acc = make_double2(0.0, 0.0);
    if constexpr (M > 0 && (M % 2) == 0) {
        const double2* w2 = reinterpret_cast<const double2*>(w);
#pragma unroll
        for (int d = 0; d < M / 2; ++d) {
            const double2 ww = __ldg(w2 + d);
            const double2 xa = x[2 * d], xb = x[2 * d + 1];
            acc.x = fma(ww.x, xa.x, acc.x);
            acc.y = fma(ww.x, xa.y, acc.y);
            acc.x = fma(ww.y, xb.x, acc.x);
            acc.y = fma(ww.y, xb.y, acc.y);
        }
    } else {
        for (int d = 0; d < m; ++d) {
            const double ww = __ldg(w + d);
            const double2 xa = x[d];
            acc.x = fma(ww, xa.x, acc.x);
            acc.y = fma(ww, xa.y, acc.y);
        }
    }
    return acc;
}

// B1 Hermite coefficients of one target row (index_vec.cu:399-441 form,
// with the per-row division folded into c3).
struct B1Row {
    int F, cubic;
    double c0, c1, c2, c3;
};

__device__ __forceinline__ B1Row b1_row(const DevCtx& c, double pos, int maxceil, int nrows) {
    B1Row r;
    long long F = (long long)floor(pos);
    if (F < 1) F = 1; else if (F > maxceil) F = maxceil;
    r.F = (int)F;
    const double u = (double)F - pos, u2 = u * u, u3 = u2 * u;
    r.cubic = F < nrows - 1;
    if (r.cubic) {
        r.c0 = 1.0 - 3.0 * u2 - 2.0 * u3;
        r.c1 = 3.0 * u2 + 2.0 * u3;
        r.c2 = u + 2.0 * u2 + u3;
        r.c3 = (u2 + u3) * c.inv_dtr[F + 1];
    } else {
        r.c0 = 1.0 - u2;
        r.c1 = u2;
        r.c2 = u + u2;
        r.c3 = 0.0;
    }
    return r;
}

namespace epi {

// Rows blk*EPI_ROWS .. +EPI_ROWS of stage s (one row per lane of a one-warp
// CTA).  Leaves in ep[] the warp sums of the scalars this stage needs:
// [0..2] r(t) terms, [3..9] dr/dt terms (stage 0), [10] error norm,
// [12] C(t,0), [13] f'(C(t,0)) (last stage).
template <int P, int P2, bool MIXED>
__device__ __forceinline__ void rows(const DevCtx& c, const StageDev& sp, const int s, const int blk, double ep[EP_N]) {
    const int L = c.L, tid = threadIdx.x, i = blk * EPI_ROWS + tid;
    const DModel Mo = c.M;
#pragma unroll
    for (int k = 0; k < EP_N; ++k) ep[k] = 0.0;

    if (tid < EPI_ROWS && i < L) {
        double a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = 0.0;
        for (int ch = 0; ch < c.nch; ++ch) {
#pragma unroll
            for (int k = 0; k < 8; ++k) a[k] += c.part[((size_t)i * c.nch + ch) * 8 + k];
        }
        const double t = sp.T, th = c.theta[i];
        const double tA = t * th, tR = t * (1.0 - th);
        const double2 q = c.KR[(size_t)(sp.nrows - 1) * L + i];
        const double2 rv = c.rowval[i];
        const double rE = c.rowval[L - 1].y;
        const double q0 = c.slots->q0;
        const double fac1 = Sig<P, P2>::d1(Mo, q0) / Mo.T0, fac2 = q0 / Mo.T0;
        const double d1 = rv.x * fac1 + q.x * (-rE) + a[0] * tR + a[1] * tA + a[2] * tA;
        const double d2 = Sig<P, P2>::d1(Mo, rv.x) * fac2 + q.y * (2.0 * Mo.Gamma) + a[3] * tR + a[4] * tA +
                          a[5] * tA - q.x * rv.y;
        const double2 hs = make_double2(d1 + d2 * th, (q.y * (-rE) + a[6] * tR) + (q.y * rv.y - a[7] * tR) * th);
        c.h[(size_t)s * L + i] = hs;
        if (sp.kind == KIND_RHS) {
            c.rhs_out[i] = hs;
        } else {
            const double2 g0 = c.KR[(size_t)(sp.n0 - 1) * L + i];
            const double2 h0 = s == 0 ? hs : c.h[i];
            double2 g;
            if (sp.kind == KIND_TABLEAU) {
                g = g0;
                for (int j = 0; j < sp.ncoef; ++j) {
                    const double2 hj = j == s ? hs : c.h[(size_t)j * L + i];
                    g.x = fma(hj.x, sp.coef[j], g.x);
                    g.y = fma(hj.y, sp.coef[j], g.y);
                }
                if (sp.last) {
                    double2 ge = g0;
                    for (int j = 0; j < sp.ncoef; ++j) {
                        const double2 hj = j == s ? hs : c.h[(size_t)j * L + i];
                        ge.x = fma(hj.x, sp.coef_e[j], ge.x);
                        ge.y = fma(hj.y, sp.coef_e[j], ge.y);
                    }
                    ep[10] = fabs(g.x - ge.x) + fabs(g.y - ge.y);
                }
            } else {
                double2 ge, gf;
                if (sp.serk_mode == 0) {
                    g = make_double2(fma(hs.x, sp.serk_c, g0.x), fma(hs.y, sp.serk_c, g0.y));
                    ge = g0;
                    gf = make_double2(g0.x * sp.serk_b0, g0.y * sp.serk_b0);
                } else {
                    g = c.gS[i]; ge = c.geS[i]; gf = c.gfS[i];
                    if (sp.serk_mode == 1) {
                        g.x = fma(hs.x, sp.serk_c, g.x);
                        g.y = fma(hs.y, sp.serk_c, g.y);
                    } else {
                        g.x = fma(hs.x, sp.serk_c2, 2.0 * g.x - ge.x);
                        g.y = fma(hs.y, sp.serk_c2, 2.0 * g.y - ge.y);
                        ge = g;
                    }
                }
                if (sp.serk_bnext != 0.0) {
                    gf.x = fma(g.x, sp.serk_bnext, gf.x);
                    gf.y = fma(g.y, sp.serk_bnext, gf.y);
                }
                c.gS[i] = g; c.geS[i] = ge; c.gfS[i] = gf;
                if (sp.last) ep[10] = fabs(gf.x - g.x) + fabs(gf.y - g.y);
            }
            const double w = c.integ[i];
            if (s == 0) {
                // drstep2 (time_steps.cu:564-639) on the step's base row and h0
                double sk, dd;
                Sig<P, P2>::d12(Mo, g0.x, sk, dd);
                const double sr = dd * g0.y;
                const double dsk = dd * h0.x;
                const double dsr = (Sig<P, P2>::d3(Mo, g0.x) * g0.y) * h0.x + dd * h0.y;
                const double tw = sp.T * w;
                ep[3] = (w * sr) * g0.x;
                ep[4] = (w * sk) * g0.y;
                ep[5] = (tw * dsr) * g0.x;
                ep[6] = (tw * dsk) * g0.y;
                ep[7] = (tw * sr) * h0.x;
                ep[8] = (tw * sk) * h0.y;
                if (i == 0) ep[9] = (dsk * g0.x + sk * h0.x) / Mo.T0;
            }
            const double td = sp.tdiff;
            c.KR[(size_t)sp.n0 * L + i] = g;
            c.dKR[(size_t)sp.n0 * L + i] = make_double2(td * h0.x, td * h0.y);
            if constexpr (MIXED) {
                c.KRf[(size_t)sp.n0 * L + i] = make_float2((float)g.x, (float)g.y);
                if (c.KRl)
                    c.KRl[(size_t)sp.n0 * L + i] =
                        make_float2((float)(g.x - (double)(float)g.x), (float)(g.y - (double)(float)g.y));
                c.dKRf[(size_t)sp.n0 * L + i] = make_float2((float)(td * h0.x), (float)(td * h0.y));
            }
            // rstep (time_steps.cpp:83-92) of the new row at its time
            const double tn = sp.T_next, tw = tn * w;
            double sk, dd;
            Sig<P, P2>::d12(Mo, g.x, sk, dd);
            ep[0] = (tw * (dd * g.y)) * g.x;
            ep[1] = (tw * sk) * g.y;
            if (i == 0) {
                ep[2] = (sk * g.x) / Mo.T0;
                ep[12] = g.x;
                ep[13] = sk;
            }
            // positions of the next stage (searched by the gather kernel)
            const double pos = sp.pos_reuse >= 0 ? c.posB1x_saved[(size_t)sp.pos_reuse * L + i] : c.posB1x_next[i];
            c.posB1x[i] = pos;
            if (sp.pos_save >= 0) c.posB1x_saved[(size_t)sp.pos_save * L + i] = pos;
        }
    }
    // one warp per CTA: fixed butterfly sums of the quantities this stage uses
    // (r(t) always; dr/dt at stage 0; error norm and C(t,0), f'(C(t,0)) at the last)
    if (sp.kind != KIND_RHS) {
#pragma unroll
        for (int k = 0; k < 3; ++k) ep[k] = warp_sum(ep[k]);
        if (s == 0) {
#pragma unroll
            for (int k = 3; k < 10; ++k) ep[k] = warp_sum(ep[k]);
        }
        if (sp.last) {
            ep[10] = warp_sum(ep[10]);
            ep[12] = warp_sum(ep[12]);
            ep[13] = warp_sum(ep[13]);
        }
    }
}

// Publish this CTA's partials (CTA blk of G) and elect the CTA that finishes
// last (atomic ticket on slots->counter, no waiting); true in every thread
// of that CTA only.
__device__ __forceinline__ bool elect_last(const DevCtx& c, const double ep[EP_N], const unsigned blk, const unsigned G) {
    __shared__ int s_is_last;
    const int tid = threadIdx.x;
    if (tid < EP_N) {
        double v = 0.0;
#pragma unroll
        for (int k = 0; k < EP_N; ++k) if (k == tid) v = ep[k];
        c.epart[(size_t)blk * EP_N + tid] = v;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_is_last = atomicAdd(&c.slots->counter, 1u) == G - 1;
    __syncthreads();
    const bool last = s_is_last;
    if (last) __threadfence();
    return last;
}

// Fold of the G CTAs' partials (in CTA order) and the stage's scalar writes
// (thread 0): r of the written row, dr/dt, t1grid, delta_t_ratio and, at the
// last stage, the step result.  Does not reset slots->counter.
template <int P, int P2, bool MIXED>
__device__ __forceinline__ void fold(const DevCtx& c, const StageDev& sp, const int s, const unsigned G) {
    const int tid = threadIdx.x;
    const DModel Mo = c.M;
    double tot = 0.0;
    if (tid < EP_N) {
        for (unsigned b = 0; b < G; b += 4) {
            // four independent loads in flight, summed in block order
            double v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = b + q < G ? __ldcg(c.epart + (size_t)(b + q) * EP_N + tid) : 0.0;
#pragma unroll
            for (int q = 0; q < 4; ++q) tot += v[q];
        }
    }
    __shared__ double s_tot[EP_N];
    if (tid < EP_N) s_tot[tid] = tot;
    __syncthreads();
    if (tid != 0) return;
    Slots* sl = c.slots;
    if (sp.kind != KIND_RHS) {
        const int n0 = sp.n0;
        const double r_new = ((Mo.Gamma + s_tot[0]) + s_tot[1]) + s_tot[2];
        c.rvec[n0] = r_new;
        if (s == 0)
            sl->dr = (((((s_tot[3] + s_tot[4]) + s_tot[5]) + s_tot[6]) + s_tot[7]) + s_tot[8]) + s_tot[9];
        c.drvec[n0] = sp.tdiff * sl->dr;
        c.t1grid[n0] = sp.T_next;
        c.dtr[n0] = sp.dtr_new;
        c.inv_dtr[n0] = sp.dtr_new != 0.0 ? 1.0 / sp.dtr_new : 0.0;
        if constexpr (MIXED) {
            c.inv_dtr_f[n0] = sp.dtr_new != 0.0 ? (float)(1.0 / sp.dtr_new) : 0.0f;
            c.inv_len_f[n0 - 1] = (float)(1.0 / sp.tdiff);
        }
        if (sp.last) {
            sl->res_err = s_tot[10];
            sl->res_energy = -(s_tot[1] + s_tot[13] / Mo.T0);
            sl->res_r = r_new;
            sl->res_qk0 = s_tot[12];
            sl->res_dr = sl->dr;
        }
    }
}

}  // namespace epi
}  // namespace dyn
