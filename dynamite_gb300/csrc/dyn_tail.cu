// QK tail fit of the newest history row near theta -> 1 (the reference's
// --tail-fit, tailFitBlendCPU in tail_fit.cpp:46-262; applied by the driver
// loop after every update, simulation_runner.cpp:135-141).
//
// On the newest row, y_j = (1 - QK_j) / (1 - theta_j)^2 over the second half
// of theta.  The 16-point window of y with the smallest spread (all windows
// on the first call or when no row was added since the last call; otherwise
// the previous window and its two neighbours) gives alpha_raw, which is
// smoothed with a gain that falls as its standard error grows and is reset by
// a rollback.  If the residuals of QK_fit = 1 - alpha (1 - theta)^2 over the
// tail stay within 3 sigma, the window's spread is below sqrt(delta_max) and
// alpha is not zero, QK is blended into QK_fit over an 8- or 16-point ramp.
//
// The row has at most 4096 entries, so one CTA does it all: y and the window
// statistics in parallel (a thread per window, summing in the reference's
// order), the choice and the residual sums in order by one thread, the blend
// in parallel.
// Every operation is written with round-to-nearest intrinsics (no FMA
// contraction), so results match the reference's scalar CPU arithmetic.
#include <cmath>
#include "dyn_kernels.cuh"

namespace dyn {

namespace {

__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

constexpr int TF_W = 16;           // window length (tail_fit.cpp:62)
constexpr int TF_MAXWIN = 2048 / TF_W;  // windows of the second half of a 4096-point row

// 1 - alpha (1 - theta)^2
__device__ __forceinline__ double qk_fit(double alpha, double th) {
    const double one_m = sub(1.0, th);
    return sub(1.0, mul(mul(alpha, one_m), one_m));
}

__global__ void __launch_bounds__(256) k_tail_fit(const DevCtx c, const int nrows, const int rollback_loop,
                                                  const double delta_max, TailState* ts) {
    const int L = c.L, start = L / 2, N = L - start, tid = threadIdx.x, nt = blockDim.x;
    extern __shared__ double s_y[];  // [N]: y, then the residuals
    __shared__ double s_mean[TF_MAXWIN], s_sse[TF_MAXWIN];
    __shared__ double s_alpha;
    __shared__ int s_j0, s_apply, s_ramp;
    double2* row = c.KR + (size_t)(nrows - 1) * L;

    for (int j = tid; j < N; j += nt) {
        const double one_m = sub(1.0, c.theta[start + j]), den = mul(one_m, one_m);
        s_y[j] = dvd(sub(1.0, row[start + j].x), den > 0.0 ? den : 1e-300);
    }
    __syncthreads();
    const int wc = (N - TF_W) / TF_W + 1;
    for (int w = tid; w < wc; w += nt) {
        // window_mean_sse (tail_fit.cpp:20-45): its `omp simd` sums run as two
        // interleaved partial sums (even and odd k) added at the end
        const double* y = s_y + w * TF_W;
        double s0 = 0.0, s1 = 0.0, e0 = 0.0, e1 = 0.0;
        for (int k = 0; k < TF_W; k += 2) {
            s0 = add(s0, y[k]);
            s1 = add(s1, y[k + 1]);
        }
        const double mean = dvd(add(s0, s1), (double)TF_W);
        for (int k = 0; k < TF_W; k += 2) {
            const double d0 = sub(y[k], mean), d1 = sub(y[k + 1], mean);
            e0 = add(e0, mul(d0, d0));
            e1 = add(e1, mul(d1, d1));
        }
        s_mean[w] = mean;
        s_sse[w] = add(e0, e1);
    }
    __syncthreads();

    double best_sse = __longlong_as_double(0x7ff0000000000000LL);  // +inf
    if (tid == 0) {
        TailState t = *ts;
        const bool new_step = t.prev_n != nrows;
        long long best_off = 0;
        double best_mean = 0.0;
        if (t.prev_off < 0 || !new_step) {
            for (int w = 0; w < wc; ++w)
                if (s_sse[w] < best_sse) { best_sse = s_sse[w]; best_off = (long long)w * TF_W; best_mean = s_mean[w]; }
        } else {
            // the previous window and its neighbours, in ascending order (tail_fit.cpp:115-129)
            const long long prev = t.prev_off;
            const long long cand[3] = {prev - TF_W, prev, prev + TF_W};
            const bool ok[3] = {prev >= TF_W, true, prev + 2 * TF_W <= N};
            for (int k = 0; k < 3; ++k) {
                const long long off = cand[k];
                if (!ok[k] || off + TF_W > N) continue;
                const int w = (int)(off / TF_W);
                if (s_sse[w] < best_sse) { best_sse = s_sse[w]; best_off = off; best_mean = s_mean[w]; }
            }
        }
        t.prev_off = best_off;
        t.prev_n = nrows;
        const double alpha_raw = best_mean;
        // smoothing (tail_fit.cpp:136-176)
        const double var = dvd(best_sse, (double)(TF_W - 1));
        const double se = sqrt(dvd(var < 0.0 ? 0.0 : var, (double)TF_W));  // std::max(var, 0.0)
        const bool rollback = rollback_loop != t.last_rb;
        if (rollback) {
            t.last_rb = rollback_loop;
            if (alpha_raw != 0.0) t.alpha = alpha_raw;
        }
        const double rel = fabs(alpha_raw) > 1e-12 ? dvd(se, fabs(alpha_raw)) : 1.0;
        double gain = dvd(0.50, add(1.0, mul(2.0, rel)));
        gain = 0.50 < gain ? 0.50 : gain;  // std::max(0.10, std::min(gain, 0.50)), NaN -> 0.10
        gain = 0.10 < gain ? gain : 0.10;
        if (!(t.alpha == t.alpha) || (alpha_raw == 0.0 && rollback)) {
            if (alpha_raw != 0.0) t.alpha = alpha_raw;
            else if (!(t.alpha == t.alpha)) t.alpha = 0.0;
        } else if (alpha_raw != 0.0) {
            t.alpha = add(mul(sub(1.0, gain), t.alpha), mul(gain, alpha_raw));
        }
        t.alpha_raw = alpha_raw;
        t.j0 = (int)(start + best_off);
        *ts = t;
        s_alpha = t.alpha;
        s_j0 = t.j0;
    }
    __syncthreads();
    const double alpha = s_alpha;
    const int j0 = s_j0, nr = L - j0;
    for (int j = j0 + tid; j < L; j += nt) s_y[j - j0] = sub(qk_fit(alpha, c.theta[j]), row[j].x);
    __syncthreads();
    if (tid == 0) {
        // residual statistics and the gate (tail_fit.cpp:178-218)
        double mabs = 0.0, mres = 0.0, rvar = 0.0;
        for (int k = 0; k < nr; ++k) mabs = add(mabs, fabs(s_y[k]));
        mabs = dvd(mabs, (double)nr);
        for (int k = 0; k < nr; ++k) mres = add(mres, s_y[k]);
        mres = dvd(mres, (double)nr);
        for (int k = 0; k < nr; ++k) {
            const double d = sub(s_y[k], mres);
            rvar = add(rvar, mul(d, d));
        }
        const double dn = sub((double)nr, 1.0);
        rvar = dvd(rvar, dn > 1.0 ? dn : 1.0);
        const double rstd = sqrt(rvar > 0.0 ? rvar : 0.0);
        const bool apply = mabs <= mul(3.0, rstd) && best_sse <= sqrt(delta_max) && fabs(alpha) > 1e-14;
        const double a_raw = ts->alpha_raw;
        const double ach = dvd(fabs(sub(a_raw, alpha)), fabs(alpha) < 1e-12 ? 1e-12 : fabs(alpha));
        s_ramp = ach < 0.005 ? 8 : 16;
        s_apply = apply;
        ts->applied = apply;
    }
    __syncthreads();
    if (!s_apply) return;
    const int ramp = s_ramp;
    for (int j = j0 + tid; j < L; j += nt) {
        const double w = j < j0 + ramp ? dvd((double)(j - j0), (double)ramp) : 1.0;
        const double q = row[j].x;
        row[j].x = add(mul(sub(1.0, w), q), mul(w, qk_fit(alpha, c.theta[j])));
    }
}

}  // namespace

cudaError_t launch_tail_fit(const DevCtx& c, int nrows, int rollback_loop, double delta_max, TailState* ts,
                            cudaStream_t st) {
    if (c.L < 32 || c.L > 4096 || nrows < 1) return cudaSuccess;  // tail_fit.cpp:47-58
    const size_t smem = (size_t)(c.L - c.L / 2) * sizeof(double);
    k_tail_fit<<<1, 256, smem, st>>>(c, nrows, rollback_loop, delta_max, ts);
    return cudaGetLastError();
}

}  // namespace dyn
