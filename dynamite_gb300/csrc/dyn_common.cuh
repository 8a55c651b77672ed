// Shared device code for the GB300-native DYNAMITE hot path.
//
// Layout in HBM (one context, FP64 form):
//   KR  [cap][L] double2  (QK, QR)   — history rows, row-major, K and R interleaved
//   dKR [cap][L] double2  (dQK, dQR) — staggered derivative rows
//   t1grid/dtr/inv_dtr/rvec/drvec [cap] double
//   tables: iA1/iA2/iB2 [L*L] int32 (stencil starts), wA1/wA2/wB2 [L*L][m] double
// Interleaving K and R makes every history gather one 16-byte load.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dyn {

// Model coefficients in the reference's evaluation order (math_ops.cpp:27-37):
// f'(q)   = (lambda*p) q^(p-1) + ((1-lambda)*p2) q^(p2-1)
// f''(q)  = ((lambda*p)*(p-1)) q^(p-2) + ...
// f'''(q) = (((lambda*p)*(p-1))*(p-2)) q^(p-3) + ...
struct DModel {
    int p, p2;
    double cA, cB, cC, cD, cE, cF;
    double T0, Gamma;
};

// pow_int (math_ops.cpp:7-21), same multiplication order, no contraction.
__device__ __forceinline__ double pow_int_x(double b, int e) {
    if (e == 0) return 1.0;
    if (e == 1) return b;
    if (e == 2) return __dmul_rn(b, b);
    if (e == 3) return __dmul_rn(__dmul_rn(b, b), b);
    if (e == 4) { double sq = __dmul_rn(b, b); return __dmul_rn(sq, sq); }
    double r = 1.0, c = b;
    while (e > 0) {
        if (e & 1) r = __dmul_rn(r, c);
        c = __dmul_rn(c, c);
        e >>= 1;
    }
    return r;
}

// Exact (reference-order) f', f'', f'''.
__device__ __forceinline__ double Df_x(const DModel& M, double q) {
    return __dadd_rn(__dmul_rn(M.cA, pow_int_x(q, M.p - 1)), __dmul_rn(M.cB, pow_int_x(q, M.p2 - 1)));
}
__device__ __forceinline__ double DDf_x(const DModel& M, double q) {
    return __dadd_rn(__dmul_rn(M.cC, pow_int_x(q, M.p - 2)), __dmul_rn(M.cD, pow_int_x(q, M.p2 - 2)));
}
__device__ __forceinline__ double DDDf_x(const DModel& M, double q) {
    return __dadd_rn(__dmul_rn(M.cE, pow_int_x(q, M.p - 3)), __dmul_rn(M.cF, pow_int_x(q, M.p2 - 3)));
}

// Fast f'/f'' for the fused kernels: powers by repeated multiplication with
// exponents known at compile time where possible (P < 0: runtime exponents).
template <int E>
__device__ __forceinline__ double ipow_c(double q) {
    if constexpr (E <= 0) return 1.0;
    else if constexpr (E == 1) return q;
    else if constexpr (E == 2) return q * q;
    else if constexpr (E == 3) return (q * q) * q;
    else if constexpr (E == 4) { double s = q * q; return s * s; }
    else { double s = ipow_c<E / 2>(q); s = s * s; if constexpr (E & 1) s = s * q; return s; }
}
__device__ __forceinline__ double ipow_r(double q, int e) {
    double r = 1.0, c = q;
    while (e > 0) { if (e & 1) r *= c; c *= c; e >>= 1; }
    return r;
}

template <int P, int P2>
struct Sigma {
    // returns f'(q) and f''(q)
    __device__ __forceinline__ static void eval(const DModel& M, double q, double& d1, double& d2) {
        if constexpr (P >= 0) {
            d1 = fma(M.cA, ipow_c<P - 1>(q), M.cB * ipow_c<P2 - 1>(q));
            d2 = fma(M.cC, ipow_c<P - 2>(q), M.cD * ipow_c<P2 - 2>(q));
        } else {
            d1 = fma(M.cA, ipow_r(q, M.p - 1), M.cB * ipow_r(q, M.p2 - 1));
            d2 = fma(M.cC, ipow_r(q, M.p - 2), M.cD * ipow_r(q, M.p2 - 2));
        }
    }
    __device__ __forceinline__ static double d1(const DModel& M, double q) {
        double a, b;
        eval(M, q, a, b);
        return a;
    }
};

// Non-negative doubles order like their bit patterns; the searches compare
// in the integer pipe and leave the (slow on this part) FP64 pipe to the math.
__device__ __forceinline__ long long okey(double v) { return __double_as_longlong(v); }

// t1grid with the last entry optionally replaced (the value a stage is about
// to write), so positions for the next stage can be computed before the
// replacement lands in memory.
struct ListView {
    const double* p;
    int n;
    double vlast;
    __device__ __forceinline__ double at(int k) const { return k == n - 1 ? vlast : __ldg(p + k); }
};

// bsearchPosSorted for one element (search_utils.cpp:13-61): same probe
// sequence, same final formula, so the returned position is bit-identical.
__device__ __forceinline__ double pos_binary(const ListView& L, double El) {
    int n0 = 1, n1 = L.n, m = 1;
    double Lm = 0.0;
    const long long kE = okey(El);
    if (okey(L.at(0)) < kE) {
        while (n0 <= n1) {
            m = (n0 + n1) >> 1;
            Lm = L.at(m - 1);
            const long long k = okey(Lm);
            if (k == kE) { n0 = m; break; }
            if (k < kE) n0 = m + 1; else n1 = m - 1;
        }
    }
    if (okey(Lm) <= kE) {
        if (m == L.n) return (double)m;
        return __dadd_rn((double)m, __ddiv_rn(__dsub_rn(El, Lm), __dsub_rn(L.at(m), Lm)));
    }
    if (m > 1) return __dsub_rn((double)m, __ddiv_rn(__dsub_rn(El, Lm), __dsub_rn(L.at(m - 2), Lm)));
    return (double)m;
}

// bsearch_interp_kernel for one element (search_utils.cu:71-112): lower
// bound, then interpolation inside [list[m-1], list[m]].
__device__ __forceinline__ double pos_lower_bound(const ListView& L, double El) {
    int left = 0, right = L.n;
    const long long kE = okey(El);
    while (left < right) {
        int mid = (left + right) >> 1;
        if (okey(L.at(mid)) < kE) left = mid + 1; else right = mid;
    }
    const int m = left;
    if (m == 0) return 1.0;
    if (m == L.n) return (double)m;
    const double a = L.at(m - 1), b = L.at(m);
    const double den = __dsub_rn(b, a);
    return den == 0.0 ? (double)m + 1 : __dadd_rn((double)m, __ddiv_rn(__dsub_rn(El, a), den));
}

__device__ __forceinline__ double search_pos(int mode, const ListView& L, double El) {
    return mode == 1 ? pos_lower_bound(L, El) : pos_binary(L, El);
}

// Reduce-scatter of 8 per-lane values over a warp: afterwards lane l with
// (l & 3) == 0 holds the warp total of value index ((l>>4)&1)*4+((l>>3)&1)*2+((l>>2)&1).
// 9 adds per lane instead of 40 for eight independent butterflies.
__device__ __forceinline__ double warp_reduce8(const double v[8], int lane) {
    double w[4];
    const bool b16 = lane & 16;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double send = b16 ? v[k] : v[k + 4];
        double keep = b16 ? v[k + 4] : v[k];
        w[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
    const bool b8 = lane & 8;
    double x[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        double send = b8 ? w[k] : w[k + 2];
        double keep = b8 ? w[k + 2] : w[k];
        x[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    const bool b4 = lane & 4;
    double send = b4 ? x[0] : x[1];
    double y = (b4 ? x[1] : x[0]) + __shfl_xor_sync(0xffffffffu, send, 4);
    y += __shfl_xor_sync(0xffffffffu, y, 2);
    y += __shfl_xor_sync(0xffffffffu, y, 1);
    return y;
}
__device__ __forceinline__ int warp_reduce8_index(int lane) {
    return ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization starts while its predecessor drains; this waits until the
// predecessor has finished and its writes are visible.  Without a
// programmatic edge it returns at once.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace dyn
