// Device functions of the mixed-precision stage (FP32 gathers and
// convolutions with compensated sums, FP64 row constants and positions),
// shared by the single-quench kernel (dyn_mixed.cu) and the batched
// persistent kernel (dyn_batch.cu) so that both run the same arithmetic.
#pragma once
#include "dyn_kernels.cuh"

namespace dyn {
namespace mixed {

struct FModel {
    int p, p2;
    float cA, cB, cC, cD;
};

// Packed FP32x2 arithmetic (fma.rn.f32x2 / mul.rn.f32x2 of the sm_100 family): one
// instruction for the (QK, QR) pair, each half rounded exactly as fmaf / __fmul_rn.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
// w * x + c for both halves of x and c
__device__ __forceinline__ float2 ffma2s(float w, float2 x, float2 c) { return ffma2(make_float2(w, w), x, c); }
__device__ __forceinline__ float2 fmul2s(float w, float2 x) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %2};\n\tmov.b64 rb, {%3, %4};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(w), "f"(x.x), "f"(x.y));
    return d;
}
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

template <int E>
__device__ __forceinline__ float fpow_c(float q) {
    if constexpr (E <= 0) return 1.0f;
    else if constexpr (E == 1) return q;
    else if constexpr (E == 2) return q * q;
    else if constexpr (E == 3) return (q * q) * q;
    else if constexpr (E == 4) { float s = q * q; return s * s; }
    else { float s = fpow_c<E / 2>(q); s = s * s; if constexpr (E & 1) s = s * q; return s; }
}
__device__ __forceinline__ float fpow_r(float q, int e) {
    float r = 1.0f, c = q;
    while (e > 0) { if (e & 1) r *= c; c *= c; e >>= 1; }
    return r;
}

template <int P, int P2>
struct SigF {
    __device__ __forceinline__ static void d12(const FModel& M, float q, float& a, float& b) {
        if constexpr (P >= 0) {
            a = fmaf(M.cA, fpow_c<P - 1>(q), M.cB * fpow_c<P2 - 1>(q));
            b = fmaf(M.cC, fpow_c<P - 2>(q), M.cD * fpow_c<P2 - 2>(q));
        } else {
            a = fmaf(M.cA, fpow_r(q, M.p - 1), M.cB * fpow_r(q, M.p2 - 1));
            b = fmaf(M.cC, fpow_r(q, M.p - 2), M.cD * fpow_r(q, M.p2 - 2));
        }
    }
    __device__ __forceinline__ static float d2(const FModel& M, float q) {
        if constexpr (P >= 0) return fmaf(M.cC, fpow_c<P - 2>(q), M.cD * fpow_c<P2 - 2>(q));
        else return fmaf(M.cC, fpow_r(q, M.p - 2), M.cD * fpow_r(q, M.p2 - 2));
    }
};

// FP32 stencil weights are tap-major: plane p holds the tap pair (2p, 2p+1)
// of every target (float2, the second tap zero for an odd depth), so the
// lanes of a warp, handling consecutive targets, read consecutive words.
// sum_d w[d] * x[d] over the m taps of target ij, taps in order.
__device__ __forceinline__ float2 dotfT(const float2* __restrict__ w, size_t L2, size_t ij,
                                        const float2* __restrict__ x, int m, bool ldg) {
    float2 acc = make_float2(0.f, 0.f);
    for (int d = 0; d < m; d += 2) {
        const float2 ww = __ldg(w + (size_t)(d >> 1) * L2 + ij);
        const float2 xa = ldg ? __ldg(x + d) : x[d];
        acc = ffma2s(ww.x, xa, acc);
        if (d + 1 < m) {
            const float2 xb = ldg ? __ldg(x + d + 1) : x[d + 1];
            acc = ffma2s(ww.y, xb, acc);
        }
    }
    return acc;
}

// sum_d w[d] * x[b + d] for a 10-tap segment read as six 16-byte loads from
// the even element at or below b, each tap selecting its element (the select
// form; the same sums as seg11 with shifted weights, up to the sign of an
// exact zero, with fewer live registers)
__device__ __forceinline__ float2 seg10(const float w[10], const float2* __restrict__ arr, size_t b) {
    const size_t a = b & ~(size_t)1;
    const bool sh = b & 1;
    const float4* p = reinterpret_cast<const float4*>(arr + a);
    float2 e[12];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float4 v = __ldg(p + k);
        e[2 * k] = make_float2(v.x, v.y);
        e[2 * k + 1] = make_float2(v.z, v.w);
    }
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int d = 0; d < 10; ++d) acc = ffma2s(w[d], sh ? e[d + 1] : e[d], acc);
    return acc;
}
__device__ __forceinline__ float2 seg10s(const float w[10], const float2* arr, int b) {
    const int a = b & ~1;
    const bool sh = b & 1;
    const float4* p = reinterpret_cast<const float4*>(arr + a);
    float2 e[12];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float4 v = p[k];
        e[2 * k] = make_float2(v.x, v.y);
        e[2 * k + 1] = make_float2(v.z, v.w);
    }
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int d = 0; d < 10; ++d) acc = ffma2s(w[d], sh ? e[d + 1] : e[d], acc);
    return acc;
}

// The ten stencil weights laid over the element pairs that start at the even
// element a = b & ~1 at or below the stencil start b: w11[k] = w[k - (b & 1)]
// (zero outside 0..9).  A segment sum then needs no per-element select, and
// one shift serves every segment whose start has the same parity.
__device__ __forceinline__ void shift_w(const float w[10], const bool sh, float w11[11]) {
    w11[0] = sh ? 0.f : w[0];
#pragma unroll
    for (int k = 1; k < 10; ++k) w11[k] = sh ? w[k - 1] : w[k];
    w11[10] = sh ? w[9] : 0.f;
}

// sum_k w11[k] * arr[a + k], k = 0..10, a even: five 16-byte loads and one
// 8-byte load, taps in order.  The zero tap leaves the sum of the ten others
// unchanged, so arr[a .. a+10] must be finite (history mirrors and the staged
// row are zero-filled past what has been written).
__device__ __forceinline__ float2 seg11(const float w11[11], const float2* __restrict__ arr, size_t a) {
    const float4* p = reinterpret_cast<const float4*>(arr + a);
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const float4 v = __ldg(p + q);
        acc = ffma2s(w11[2 * q], make_float2(v.x, v.y), acc);
        acc = ffma2s(w11[2 * q + 1], make_float2(v.z, v.w), acc);
    }
    return ffma2s(w11[10], __ldg(arr + a + 10), acc);
}

// The same segment from shared memory (the staged last row)
__device__ __forceinline__ float2 seg11s(const float w11[11], const float2* arr, int a) {
    const float4* p = reinterpret_cast<const float4*>(arr + a);
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const float4 v = p[q];
        acc = ffma2s(w11[2 * q], make_float2(v.x, v.y), acc);
        acc = ffma2s(w11[2 * q + 1], make_float2(v.z, v.w), acc);
    }
    return ffma2s(w11[10], arr[a + 10], acc);
}

// the ten taps of target ij from the tap-major planes
__device__ __forceinline__ void load_w10(const float2* __restrict__ w, size_t L2, size_t ij, float wv[10]) {
#pragma unroll
    for (int d = 0; d < 5; ++d) {
        const float2 q = __ldg(w + d * L2 + ij);
        wv[2 * d] = q.x;
        wv[2 * d + 1] = q.y;
    }
}

// TwoSum accumulation: s + c carries the sum to about twice FP32 precision
// (round-to-nearest intrinsics: a product passed as v is never fused into the sum)
__device__ __forceinline__ void two_sum_add(float& s, float& c, float v) {
    const float t = __fadd_rn(s, v);
    const float bp = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(v, bp)));
    s = t;
}

// (hi, lo) += (h2, l2) with TwoSum on the high parts
__device__ __forceinline__ void pair_add(float& h, float& l, float h2, float l2) {
    const float t = __fadd_rn(h, h2);
    const float bp = __fsub_rn(t, h);
    l = __fadd_rn(__fadd_rn(l, l2), __fadd_rn(__fsub_rn(h, __fsub_rn(t, bp)), __fsub_rn(h2, bp)));
    h = t;
}

// Reduce-scatter of 8 compensated sums over a warp (as warp_reduce8, in FP32
// pairs): lane l with (l & 3) == 0 ends with the warp total of value index
// warp_reduce8_index(l) as hi + lo.
__device__ __forceinline__ void warp_reduce8_pair(const float hv[8], const float lv[8], int lane, float& H, float& Lo) {
    float wh[4], wl[4];
    const bool b16 = lane & 16;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float sh = b16 ? hv[k] : hv[k + 4], sl = b16 ? lv[k] : lv[k + 4];
        wh[k] = b16 ? hv[k + 4] : hv[k];
        wl[k] = b16 ? lv[k + 4] : lv[k];
        pair_add(wh[k], wl[k], __shfl_xor_sync(0xffffffffu, sh, 16), __shfl_xor_sync(0xffffffffu, sl, 16));
    }
    const bool b8 = lane & 8;
    float xh[2], xl[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float sh = b8 ? wh[k] : wh[k + 2], sl = b8 ? wl[k] : wl[k + 2];
        xh[k] = b8 ? wh[k + 2] : wh[k];
        xl[k] = b8 ? wl[k + 2] : wl[k];
        pair_add(xh[k], xl[k], __shfl_xor_sync(0xffffffffu, sh, 8), __shfl_xor_sync(0xffffffffu, sl, 8));
    }
    const bool b4 = lane & 4;
    float yh = b4 ? xh[1] : xh[0], yl = b4 ? xl[1] : xl[0];
    pair_add(yh, yl, __shfl_xor_sync(0xffffffffu, b4 ? xh[0] : xh[1], 4),
             __shfl_xor_sync(0xffffffffu, b4 ? xl[0] : xl[1], 4));
    pair_add(yh, yl, __shfl_xor_sync(0xffffffffu, yh, 2), __shfl_xor_sync(0xffffffffu, yl, 2));
    pair_add(yh, yl, __shfl_xor_sync(0xffffffffu, yh, 1), __shfl_xor_sync(0xffffffffu, yl, 1));
    H = yh;
    Lo = yl;
}

// The interval of El in the time list: the largest k in [lo, hi] with list[k] <= El
// (exact: integer compares on the bit patterns of the non-negative FP64 times).  The
// caller brackets the answer: list[lo] <= El (or lo = 0) and k(El) <= hi.
__device__ __forceinline__ int floor_index(const ListView& L, double El, int lo, int hi) {
    const long long kE = okey(El);
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (okey(L.at(mid)) <= kE) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The 1-based position of El in the list split into floor X and FP32 offset x from
// its interval k: X = k + 1, x = (El - list[k]) / (list[k+1] - list[k]) with one
// FP64 difference scaled by the stored FP32 inverse length (El at or past the last
// entry: X = n, x = 0).
__device__ __forceinline__ void split_at(const ListView& L, const float* __restrict__ inv_len, double El, int k,
                                         int& X, float& x) {
    if (k >= L.n - 1) { X = L.n; x = 0.f; return; }
    const float f = (float)(El - L.at(k)) * __ldg(inv_len + k);
    if (f >= 1.0f) { X = k + 2; x = f - 1.0f; } else { X = k + 1; x = f; }
}


// Block-shared scratch of one target row
constexpr int RED_CAP = 256;  // per-warp partial sums held between folds (float pairs)
constexpr int MAX_SEG = 4096 / 32;  // 32-target segments of the longest row
struct RowShared {
    int seg[MAX_SEG + 1];  // B2 interval brackets: seg[w] = k(phi2[i][32 w] t), seg[nseg] = k(phi2[i][L-1] t)
    float c[4];            // B1 Hermite constants of the row (FP32)
    int bi[2];             // B1 floor index, cubic flag
    float2 red[RED_CAP];   // [chunk slot][warp][8] partial sums as (hi, lo)
};

// Row set-up for target row i: stages the last history row (FP32 mirror) in
// shared memory and forms the row's B1 Hermite constants in FP64 from the
// master history.  With `first` set (one block per row) it also writes the
// row's QK^{B1}[i,0] and rInt_i, C(t,0) (row 0) and the next stage's B1
// position.  A stage flagged `fresh` searches the row's B1 position itself
// (after a rollback) instead of reading the one the previous stage left.
__device__ __forceinline__ void row_setup(const DevCtx& c, const StageDev& sp, const int i, const bool first,
                                          float2* s_lastf, RowShared& sh, float* clo = nullptr) {
    const int L = c.L, tpb = blockDim.x;
    const int nrows = sp.nrows;
    const double t = sp.T;
    const bool live = t > 0.0;
    const float2* KRl = c.KRf + (size_t)(nrows - 1) * L;
    for (int k = threadIdx.x; k < L; k += tpb) s_lastf[k] = KRl[k];
    if (threadIdx.x == 0) s_lastf[L] = make_float2(0.f, 0.f), s_lastf[L + 1] = make_float2(0.f, 0.f);
    if (threadIdx.x == 0) {
        if (live) {
            const double pos = sp.fresh ? search_pos(c.search, ListView{c.t1grid, nrows, t}, __dmul_rn(c.theta[i], t))
                                        : c.posB1x[i];
            long long F = (long long)floor(pos);
            if (F < 1) F = 1; else if (F > sp.maxceil) F = sp.maxceil;
            const double u = (double)F - pos, u2 = u * u, u3 = u2 * u;
            const int cubic = F < nrows - 1;
            double c0, c1, c2, c3;
            if (cubic) {
                c0 = 1.0 - 3.0 * u2 - 2.0 * u3; c1 = 3.0 * u2 + 2.0 * u3; c2 = u + 2.0 * u2 + u3;
                c3 = (u2 + u3) * c.inv_dtr[F + 1];
            } else {
                c0 = 1.0 - u2; c1 = u2; c2 = u + u2; c3 = 0.0;
            }
            sh.c[0] = (float)c0; sh.c[1] = (float)c1; sh.c[2] = (float)c2; sh.c[3] = (float)c3;
            if (clo) {
                clo[0] = (float)(c0 - (double)sh.c[0]); clo[1] = (float)(c1 - (double)sh.c[1]);
                clo[2] = (float)(c2 - (double)sh.c[2]); clo[3] = (float)(c3 - (double)sh.c[3]);
            }
            sh.bi[0] = (int)F; sh.bi[1] = cubic;
            if (first) {
                const double2 x0 = c.KR[(size_t)(F - 1) * L], x1 = c.KR[(size_t)F * L];
                const double2 d1 = c.dKR[(size_t)F * L];
                double qb = c0 * x0.x + c1 * x1.x - c2 * d1.x;
                double ri = c0 * c.rvec[F - 1] + c1 * c.rvec[F] - c2 * c.drvec[F];
                if (cubic) {
                    qb -= c3 * c.dKR[(size_t)(F + 1) * L].x;
                    ri -= c3 * c.drvec[F + 1];
                }
                c.rowval[i] = make_double2(qb, ri);
            }
        } else {
            sh.bi[0] = 1; sh.bi[1] = 0;
            sh.c[0] = sh.c[1] = sh.c[2] = sh.c[3] = 0.f;
            if (clo) clo[0] = clo[1] = clo[2] = clo[3] = 0.f;
            if (first) c.rowval[i] = make_double2(c.KR[0].x, c.rvec[0]);
        }
        if (i == 0 && first) c.slots->q0 = c.KR[(size_t)(nrows - 1) * L].x;
    }
    // B2 brackets: phi2 is non-decreasing along a row (checked when the tables are
    // loaded), so every target of 32-target segment w has its interval in
    // [seg[w], seg[w + 1]]; one full search per segment, short ones per target
    if (live) {
        const int nseg = (L + 31) >> 5;
        const ListView lv{c.t1grid, nrows, t};
        for (int w = threadIdx.x; w <= nseg; w += tpb) {
            const int j = w < nseg ? (w << 5) : L - 1;
            sh.seg[w] = floor_index(lv, __dmul_rn(c.phi2[(size_t)i * L + j], t), 0, nrows - 1);
        }
    }
    if (threadIdx.x == 32 && first && sp.kind != KIND_RHS && sp.pos_reuse < 0) {
        // next stage's B1 position of this row (the row this stage writes
        // becomes the last list entry)
        const ListView lvn{c.t1grid, sp.nrows_next, sp.T_next};
        c.posB1x_next[i] = search_pos(c.search, lvn, __dmul_rn(c.theta[i], sp.T_next));
    }
}

// One chunk of tpb*K targets of row i: A1/A2 from the staged row, B1 and B2
// from the FP32 history, Sigma, and the eight int.dat-weighted products with
// TwoSum accumulation; each warp's eight sums land in sh.red[slot][warp].
// Call after row_setup and a __syncthreads(); no barrier inside, so a block
// can run several chunks (slots) before one fold.
// SHIFT picks the segment form for depth 10, bit 0 for the A1/A2 gathers and bit 1
// for B2 (set: shifted weights, seg11; clear: per-tap selects, seg10): same
// results, different instruction counts and register footprints.
template <int M, int K, int P, int P2, int SHIFT = 3>
__device__ __forceinline__ void chunk_sums(const DevCtx& c, const StageDev& sp, const int ch, const int slot,
                                           const float2* s_lastf, RowShared& sh, const int i) {
    const int L = c.L, tpb = blockDim.x;
    const size_t L2 = (size_t)L * L;
    const int nrows = sp.nrows;
    const double t = sp.T;
    const bool live = t > 0.0;
    const FModel Mf{c.M.p, c.M.p2, (float)c.M.cA, (float)c.M.cB, (float)c.M.cC, (float)c.M.cD};
    const int m = M > 0 ? M : c.m;
    const float bc0 = sh.c[0], bc1 = sh.c[1], bc2 = sh.c[2], bc3 = sh.c[3];
    const int F = sh.bi[0], cubic1 = sh.bi[1];
    const int maxX = sp.maxX;
    const float2 fill = c.KRf[0];
    const ListView lv{c.t1grid, nrows, t};

    float acc[8], cmp[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) { acc[k] = 0.f; cmp[k] = 0.f; }

#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
        const int j = ch * tpb * K + kk * tpb + threadIdx.x;
        if (j < L) {
            const size_t ij = (size_t)i * L + j;
            float2 a1, a2, b1, b2;
            if (live) {
                if constexpr (M == 10 && (SHIFT & 1)) {
                    float wv[10], w11[11];
                    const int sa1 = __ldg(c.iA1 + ij), sa2 = __ldg(c.iA2 + ij);
                    load_w10(c.wA1f, L2, ij, wv);
                    shift_w(wv, sa1 & 1, w11);
                    a1 = seg11s(w11, s_lastf, sa1 & ~1);
                    load_w10(c.wA2f, L2, ij, wv);
                    shift_w(wv, sa2 & 1, w11);
                    a2 = seg11s(w11, s_lastf, sa2 & ~1);
                } else if constexpr (M == 10) {
                    float wv[10];
                    load_w10(c.wA1f, L2, ij, wv);
                    a1 = seg10s(wv, s_lastf, __ldg(c.iA1 + ij));
                    load_w10(c.wA2f, L2, ij, wv);
                    a2 = seg10s(wv, s_lastf, __ldg(c.iA2 + ij));
                } else {
                    a1 = dotfT(c.wA1f, L2, ij, s_lastf + __ldg(c.iA1 + ij), m, false);
                    a2 = dotfT(c.wA2f, L2, ij, s_lastf + __ldg(c.iA2 + ij), m, false);
                }
                {
                    const float2 x0 = __ldg(c.KRf + (size_t)(F - 1) * L + j);
                    const float2 x1 = __ldg(c.KRf + (size_t)F * L + j);
                    const float2 d1 = __ldg(c.dKRf + (size_t)F * L + j);
                    // c0 x0 + c1 x1 - c2 d1 (- c3 d2), packed over (QK, QR)
                    float2 r = fmul2s(-bc2, d1);
                    if (cubic1) r = ffma2s(-bc3, __ldg(c.dKRf + (size_t)(F + 1) * L + j), r);
                    b1 = ffma2s(bc0, x0, ffma2s(bc1, x1, r));
                }
                {
                    int X;
                    float x;
                    const double El = __dmul_rn(__ldg(c.phi2 + ij), t);
                    split_at(lv, c.inv_len_f, El, floor_index(lv, El, sh.seg[j >> 5], sh.seg[(j >> 5) + 1]), X, x);
                    if (X > maxX) { x += __int2float_rn(X - maxX); X = maxX; }
                    if (X < 1) { x -= __int2float_rn(1 - X); X = 1; }
                    const float x2 = x * x, x3 = x2 * x;
                    const size_t base = (size_t)(X - 1) * (size_t)L + (size_t)__ldg(c.iB2 + ij);
                    const bool cubic2 = X < nrows - 1;
                    // the four 10-tap segments (rows X-1, X of (QK, QR), rows X, X+1 of (dQK, dQR)),
                    // each folded into the Hermite sum as it completes
                    [[maybe_unused]] float w11[11];
                    [[maybe_unused]] float wv[10];
                    if constexpr (M == 10) {
                        // even L (the M == 10 kernels require it): every segment start has base's parity
                        load_w10(c.wB2f, L2, ij, wv);
                        if constexpr ((SHIFT & 2) != 0) shift_w(wv, base & 1, w11);
                    }
                    auto seg = [&](const float2* __restrict__ arr, size_t off) -> float2 {
                        if constexpr (M == 10 && (SHIFT & 2)) return seg11(w11, arr, (base & ~(size_t)1) + off);
                        else if constexpr (M == 10) return seg10(wv, arr, base + off);
                        else return dotfT(c.wB2f, L2, ij, arr + base + off, m, true);
                    };
                    float2 r;
                    float e0;
                    if (cubic2) {
                        e0 = 1.f - 3.f * x2 + 2.f * x3;
                        const float e1 = x - 2.f * x2 + x3, e2 = 3.f * x2 - 2.f * x3;
                        const float e3 = (x3 - x2) * __ldg(c.inv_dtr_f + X + 1);
                        r = fmul2s(e3, seg(c.dKRf, 2 * (size_t)L));
                        r = ffma2s(e2, seg(c.KRf, L), r);
                        r = ffma2s(e1, seg(c.dKRf, L), r);
                    } else {
                        e0 = 1.f - x2;
                        r = fmul2s(x - x2, seg(c.dKRf, L));
                        r = ffma2s(x2, seg(c.KRf, L), r);
                    }
                    b2 = ffma2s(e0, seg(c.KRf, 0), r);
                }
            } else {
                a1 = a2 = b1 = b2 = fill;
            }
            float sKA1, dA1, sKB1, dB1, sKB2, dB2;
            SigF<P, P2>::d12(Mf, a1.x, sKA1, dA1);
            const float sRA1 = dA1 * a1.y;
            const float sRA2 = SigF<P, P2>::d2(Mf, a2.x) * a2.y;
            SigF<P, P2>::d12(Mf, b1.x, sKB1, dB1);
            const float sRB1 = dB1 * b1.y;
            SigF<P, P2>::d12(Mf, b2.x, sKB2, dB2);
            const float sRB2 = dB2 * b2.y;
            const float wj = __ldg(c.integ_f + j);
            const float wRA2 = wj * sRA2, wQRA2 = wj * a2.y;
            const float v[8] = {wRA2 * b2.x, (wj * sRA1) * b1.x, (wj * sKA1) * b1.y, wQRA2 * sKB2,
                                (wj * a1.y) * sKB1, (wj * a1.x) * sRB1, wRA2 * b2.y, wQRA2 * sRB2};
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                // the first term of a TwoSum from zero is exact: (s, c) = (v, 0)
                if (kk == 0) acc[k] = v[k];
                else two_sum_add(acc[k], cmp[k], v[k]);
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float H, Lo;
    warp_reduce8_pair(acc, cmp, lane, H, Lo);
    if ((lane & 3) == 0) sh.red[((slot * (tpb >> 5)) + warp) * 8 + warp_reduce8_index(lane)] = make_float2(H, Lo);
}

// After a __syncthreads() that follows chunk_sums of slots 0..ng-1 (chunks
// ch0..ch0+ng-1): the block sums of each chunk, warps added in order, into
// part[i][ch][0..8).
__device__ __forceinline__ void fold_chunks(const DevCtx& c, const int i, const int nch, const int ch0, const int ng,
                                            const RowShared& sh) {
    const int nw = blockDim.x >> 5;
    for (int t = threadIdx.x; t < 8 * ng; t += blockDim.x) {
        const int g = t >> 3, k = t & 7;
        // warps in order, compensated on the high parts; one conversion at the end
        float h = 0.f, l = 0.f;
        for (int w = 0; w < nw; ++w) {
            const float2 hl = sh.red[(g * nw + w) * 8 + k];
            pair_add(h, l, hl.x, hl.y);
        }
        c.part[((size_t)i * nch + ch0 + g) * 8 + k] = (double)h + (double)l;
    }
}

}  // namespace mixed

// ---------------------------------------------------------------- (hi, lo) form
// Plain FP32 gathers go wrong over long runs through FP32 roundings that repeat
// step after step (the rounded weights and stored history, and the rounding of
// sums over them).  Here the weights and the stored (QK, QR) history carry FP32
// (hi, lo) pairs; the A1/A2 and B2 stencil sums form every term as an exact
// FP32 product plus the cross terms (w_hi x_lo + w_lo x_hi) and add them with
// TwoSum; the gathered values stay (hi, lo) and everything that changes from
// stage to stage -- the B2 interval offset, the Hermite weights, B1, Sigma and
// the eight int.dat products -- runs in double-float (chunk_dd), so the stage
// derivatives carry no stage-to-stage FP32 rounding noise and the embedded error
// estimate sees the method's error, as in the FP64 form.  The derivative rows
// (dQK, dQR), a step's worth of change, stay single FP32.
namespace mdf {
using namespace mixed;

// (s, c) += (wh + wl) * (xh + xl)
__device__ __forceinline__ void add_prod(float& s, float& c, float wh, float wl, float xh, float xl) {
    const float p = __fmul_rn(wh, xh);  // intrinsics: no fusing of the product into the sums
    float e = __fmaf_rn(wh, xh, -p);
    e = __fmaf_rn(wh, xl, e);
    e = __fmaf_rn(wl, xh, e);
    const float t = __fadd_rn(s, p), bp = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp)), e));
    s = t;
}

// sum_d w[d] * x[d] over the m taps of target ij for both components, as
// (s_QK, c_QK, s_QR, c_QR); weights from the tap-major (hi, lo) planes, the
// segment x from the (hi, lo) history arrays (global or shared)
template <int M>
__device__ __forceinline__ float4 gather(const float2* __restrict__ wh, const float2* __restrict__ wl, size_t L2,
                                         size_t ij, const float2* xh, const float2* xl, int m, bool ldg) {
    float sx = 0.f, cx = 0.f, sy = 0.f, cy = 0.f;
    const int mm = M > 0 ? M : m;
#pragma unroll
    for (int d = 0; d < (M > 0 ? M : 1 << 20); d += 2) {
        if (d >= mm) break;
        const float2 ph = __ldg(wh + (size_t)(d >> 1) * L2 + ij), pl = __ldg(wl + (size_t)(d >> 1) * L2 + ij);
        const float2 ah = ldg ? __ldg(xh + d) : xh[d], al = ldg ? __ldg(xl + d) : xl[d];
        add_prod(sx, cx, ph.x, pl.x, ah.x, al.x);
        add_prod(sy, cy, ph.x, pl.x, ah.y, al.y);
        if (d + 1 < mm) {
            const float2 bh = ldg ? __ldg(xh + d + 1) : xh[d + 1], bl = ldg ? __ldg(xl + d + 1) : xl[d + 1];
            add_prod(sx, cx, ph.y, pl.y, bh.x, bl.x);
            add_prod(sy, cy, ph.y, pl.y, bh.y, bl.y);
        }
    }
    return make_float4(sx, cx, sy, cy);
}

// add_prod for both halves of a (QK, QR) pair at once, in packed FP32x2
// instructions, each half rounded exactly as add_prod rounds it: -p is formed as
// (-wh) * xh (round-to-nearest is symmetric), s + p as s - (-p), and p - bp as
// -((-p) + bp), so every intermediate equals add_prod's up to its sign.
__device__ __forceinline__ void add_prod2(float2& s, float2& c, float wh, float wl, float2 xh, float2 xl) {
    const float2 np = fmul2s(-wh, xh);
    float2 e = ffma2s(wh, xh, np);
    e = ffma2s(wh, xl, e);
    e = ffma2s(wl, xh, e);
    const float2 t = fsub2(s, np), bp = fsub2(t, s);
    c = fadd2(c, fadd2(fsub2(fsub2(s, fsub2(t, bp)), fadd2(np, bp)), e));
    s = t;
}

// The depth-10 (hi, lo) gathers, read tap by tap (8-byte loads at any offset:
// no aligned 16-byte window and no per-tap parity selects), taps in order.  Of
// the staged newest row in shared memory:
__device__ __forceinline__ float4 gather10_staged(const float wh[10], const float wl[10], const float2* xh,
                                                  const float2* xl) {
    float2 s = make_float2(0.f, 0.f), c = make_float2(0.f, 0.f);
#pragma unroll
    for (int d = 0; d < 10; ++d) add_prod2(s, c, wh[d], wl[d], xh[d], xl[d]);
    return make_float4(s.x, c.x, s.y, c.y);
}

// of a history segment in global memory (read-only path):
__device__ __forceinline__ float4 gather10_ldg(const float wh[10], const float wl[10], const float2* __restrict__ xh,
                                               const float2* __restrict__ xl) {
    float2 s = make_float2(0.f, 0.f), c = make_float2(0.f, 0.f);
#pragma unroll
    for (int d = 0; d < 10; ++d) add_prod2(s, c, wh[d], wl[d], __ldg(xh + d), __ldg(xl + d));
    return make_float4(s.x, c.x, s.y, c.y);
}
// and the FP32 sum of a derivative-row segment with the high weights:
__device__ __forceinline__ float2 dot10_ldg(const float w[10], const float2* __restrict__ x) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int d = 0; d < 10; ++d) acc = ffma2s(w[d], __ldg(x + d), acc);
    return acc;
}

__device__ __forceinline__ void load_w10_hl(const float2* __restrict__ wh, const float2* __restrict__ wl, size_t L2,
                                            size_t ij, float h[10], float l[10]) {
#pragma unroll
    for (int d = 0; d < 5; ++d) {
        const float2 a = __ldg(wh + d * L2 + ij), b = __ldg(wl + d * L2 + ij);
        h[2 * d] = a.x; h[2 * d + 1] = a.y;
        l[2 * d] = b.x; l[2 * d + 1] = b.y;
    }
}

// ---- double-float arithmetic: an unevaluated sum h + l of two floats, ~44 bits.
// Every operation is a round-to-nearest intrinsic, so the compiler never fuses a
// product into a following sum (which would break the error-free transformations
// and make the result depend on how a kernel was inlined).
struct ff {
    float h, l;
};
__device__ __forceinline__ ff ff_split(double v) {
    const float h = __double2float_rn(v);
    return {h, __double2float_rn(__dsub_rn(v, (double)h))};
}
__device__ __forceinline__ ff ff_fast(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const float s = __fadd_rn(a.h, b.h), bp = __fsub_rn(s, a.h);
    const float e = __fadd_rn(__fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bp)), __fsub_rn(b.h, bp)), __fadd_rn(a.l, b.l));
    return ff_fast(s, e);
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.h, -a.l}; }
// Products are left unnormalized: the low word is the exact rounding error of the
// high product plus the cross terms, at most ~2 ulp of the high word, which every
// later sum (TwoSum on the high words) and product (cross terms) takes as it is.
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return {p, e};
}
__device__ __forceinline__ ff ff_mulf(ff a, float b) {
    const float p = __fmul_rn(a.h, b);
    float e = __fmaf_rn(a.h, b, -p);
    e = __fmaf_rn(a.l, b, e);
    return {p, e};
}
// q^E as the same left-to-right product chain whether E is a template constant
// (the specialized models) or a run-time value (the generic kernel): both forms
// round alike, so a quench gives the same result in either kernel
template <int E>
__device__ __forceinline__ ff ff_pow_c(ff q) {
    if constexpr (E <= 0) {
        return {1.f, 0.f};
    } else {
        ff r = q;
#pragma unroll
        for (int k = 1; k < E; ++k) r = ff_mul(r, q);
        return r;
    }
}
__device__ __forceinline__ ff ff_pow_r(ff q, int e) {
    if (e <= 0) return {1.f, 0.f};
    ff r = q;
    for (int k = 1; k < e; ++k) r = ff_mul(r, q);
    return r;
}
struct FFModel {
    int p, p2;
    ff cA, cB, cC, cD;
};
// f'(q) and f''(q) in double-float
template <int P, int P2>
__device__ __forceinline__ void ff_sigma(const FFModel& M, ff q, ff& d1, ff& d2) {
    if constexpr (P >= 0) {
        d1 = ff_add(ff_mul(M.cA, ff_pow_c<P - 1>(q)), ff_mul(M.cB, ff_pow_c<P2 - 1>(q)));
        d2 = ff_add(ff_mul(M.cC, ff_pow_c<P - 2>(q)), ff_mul(M.cD, ff_pow_c<P2 - 2>(q)));
    } else {
        d1 = ff_add(ff_mul(M.cA, ff_pow_r(q, M.p - 1)), ff_mul(M.cB, ff_pow_r(q, M.p2 - 1)));
        d2 = ff_add(ff_mul(M.cC, ff_pow_r(q, M.p - 2)), ff_mul(M.cD, ff_pow_r(q, M.p2 - 2)));
    }
}

// chunk with everything that changes from stage to stage in double-float: the B2
// interval offset (one FP64 residual), the Hermite weights, the gathered values
// (the compensated sums kept as (hi, lo)), Sigma and the eight int.dat products,
// accumulated as (hi, lo) pairs.  FP32 roundings that differ between the stages of
// one step would otherwise put a noise of ~1e-7 of |h| into every stage derivative,
// which the embedded error estimate sees: with delta_max = 1e-10 the controller
// then keeps the step ~1000x below the FP64 form's.  The roundings of the frozen
// inputs (the (hi, lo) weights and history, the FP32 derivative rows) vary smoothly
// with the stage time and cancel in the estimate.
template <int M, int K, int P, int P2>
__device__ __forceinline__ void chunk_dd(const DevCtx& c, const StageDev& sp, const int ch, const int slot,
                                         const float2* s_hi, const float2* s_lo, const float* clo, RowShared& sh,
                                         const int i) {
    const int L = c.L, tpb = blockDim.x;
    const size_t L2 = (size_t)L * L;
    const int nrows = sp.nrows;
    const double t = sp.T;
    const bool live = t > 0.0;
    const FFModel Mf{c.M.p, c.M.p2, ff_split(c.M.cA), ff_split(c.M.cB), ff_split(c.M.cC), ff_split(c.M.cD)};
    const int m = M > 0 ? M : c.m;
    const ff bc0{sh.c[0], clo[0]}, bc1{sh.c[1], clo[1]}, bc2{sh.c[2], clo[2]}, bc3{sh.c[3], clo[3]};
    const int F = sh.bi[0], cubic1 = sh.bi[1];
    const int maxX = sp.maxX;
    const ListView lv{c.t1grid, nrows, t};
    float acc[8], cmp[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) { acc[k] = 0.f; cmp[k] = 0.f; }
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
        const int j = ch * tpb * K + kk * tpb + threadIdx.x;
        if (j < L) {
            const size_t ij = (size_t)i * L + j;
            ff a1x, a1y, a2x, a2y, b1x, b1y, b2x, b2y;
            if (live) {
                {
                    const int s1 = __ldg(c.iA1 + ij), s2 = __ldg(c.iA2 + ij);
                    float4 g1, g2;
                    if constexpr (M == 10) {
                        float wh[10], wl[10];
                        load_w10_hl(c.wA1f, c.wA1l, L2, ij, wh, wl);
                        g1 = gather10_staged(wh, wl, s_hi + s1, s_lo + s1);
                        load_w10_hl(c.wA2f, c.wA2l, L2, ij, wh, wl);
                        g2 = gather10_staged(wh, wl, s_hi + s2, s_lo + s2);
                    } else {
                        g1 = gather<M>(c.wA1f, c.wA1l, L2, ij, s_hi + s1, s_lo + s1, m, false);
                        g2 = gather<M>(c.wA2f, c.wA2l, L2, ij, s_hi + s2, s_lo + s2, m, false);
                    }
                    a1x = ff_fast(g1.x, g1.y);
                    a1y = ff_fast(g1.z, g1.w);
                    a2x = ff_fast(g2.x, g2.y);
                    a2y = ff_fast(g2.z, g2.w);
                }
                {
                    const size_t r0 = (size_t)(F - 1) * L + j, r1 = (size_t)F * L + j;
                    const float2 x0 = __ldg(c.KRf + r0), x0l = __ldg(c.KRl + r0);
                    const float2 x1 = __ldg(c.KRf + r1), x1l = __ldg(c.KRl + r1);
                    const float2 d1 = __ldg(c.dKRf + r1);
                    const float2 d2 = cubic1 ? __ldg(c.dKRf + (size_t)(F + 1) * L + j) : make_float2(0.f, 0.f);
                    const ff dx = ff_add(ff_mulf(bc2, d1.x), ff_mulf(bc3, d2.x));
                    const ff dy = ff_add(ff_mulf(bc2, d1.y), ff_mulf(bc3, d2.y));
                    b1x = ff_add(ff_add(ff_mul(bc0, ff{x0.x, x0l.x}), ff_mul(bc1, ff{x1.x, x1l.x})), ff_neg(dx));
                    b1y = ff_add(ff_add(ff_mul(bc0, ff{x0.y, x0l.y}), ff_mul(bc1, ff{x1.y, x1l.y})), ff_neg(dy));
                }
                {
                    const double El = __dmul_rn(__ldg(c.phi2 + ij), t);
                    const int k = floor_index(lv, El, sh.seg[j >> 5], sh.seg[(j >> 5) + 1]);
                    // offset in the interval: x = (El - t_k) / (t_{k+1} - t_k) as x_h + x_l, x_h
                    // from the FP32 inverse length, x_l from the FP64 residual
                    int X;
                    ff x{0.f, 0.f};
                    if (k >= lv.n - 1) {
                        X = lv.n;
                    } else {
                        const double lo = lv.at(k), diff = __dsub_rn(El, lo), len = __dsub_rn(lv.at(k + 1), lo);
                        const float il = __ldg(c.inv_len_f + k);
                        const float xh = __fmul_rn(__double2float_rn(diff), il);
                        x = ff{xh, __fmul_rn(__double2float_rn(__fma_rn(-(double)xh, len, diff)), il)};
                        X = k + 1;
                        if (x.h >= 1.0f) { X = k + 2; x = ff_add(x, ff{-1.f, 0.f}); }
                    }
                    if (X > maxX) { x = ff_add(x, ff{__int2float_rn(X - maxX), 0.f}); X = maxX; }
                    if (X < 1) { x = ff_add(x, ff{-__int2float_rn(1 - X), 0.f}); X = 1; }
                    const ff x2 = ff_mul(x, x), x3 = ff_mul(x2, x);
                    const size_t base = (size_t)(X - 1) * (size_t)L + (size_t)__ldg(c.iB2 + ij);
                    const bool cubic2 = X < nrows - 1;
                    float4 S0, S1;
                    float2 D1, D2 = make_float2(0.f, 0.f);
                    if constexpr (M == 10) {
                        // one weight load for the four segments of rows X-1, X, X+1
                        float wh[10], wl[10];
                        load_w10_hl(c.wB2f, c.wB2l, L2, ij, wh, wl);
                        S0 = gather10_ldg(wh, wl, c.KRf + base, c.KRl + base);
                        S1 = gather10_ldg(wh, wl, c.KRf + base + L, c.KRl + base + L);
                        D1 = dot10_ldg(wh, c.dKRf + base + L);
                        if (cubic2) D2 = dot10_ldg(wh, c.dKRf + base + 2 * L);
                    } else {
                        S0 = gather<M>(c.wB2f, c.wB2l, L2, ij, c.KRf + base, c.KRl + base, m, true);
                        S1 = gather<M>(c.wB2f, c.wB2l, L2, ij, c.KRf + base + L, c.KRl + base + L, m, true);
                        D1 = dotfT(c.wB2f, L2, ij, c.dKRf + base + L, m, true);
                        if (cubic2) D2 = dotfT(c.wB2f, L2, ij, c.dKRf + base + 2 * L, m, true);
                    }
                    // S0 + e2 (S1 - S0) + e1 D1 + e3 D2 (e0 = 1 - e2)
                    ff e1, e2, e3{0.f, 0.f};
                    if (cubic2) {
                        e1 = ff_add(ff_add(x, ff_mulf(x2, -2.f)), x3);
                        e2 = ff_add(ff_mulf(x2, 3.f), ff_mulf(x3, -2.f));
                        e3 = ff_mul(ff_add(x3, ff_neg(x2)), ff_split(c.inv_dtr[X + 1]));
                    } else {
                        e1 = ff_add(x, ff_neg(x2));
                        e2 = x2;
                    }
                    const ff dSx = ff_add(ff{S1.x, S1.y}, ff{-S0.x, -S0.y});
                    const ff dSy = ff_add(ff{S1.z, S1.w}, ff{-S0.z, -S0.w});
                    b2x = ff_add(ff_fast(S0.x, S0.y),
                                 ff_add(ff_mul(e2, dSx), ff_add(ff_mulf(e1, D1.x), ff_mulf(e3, D2.x))));
                    b2y = ff_add(ff_fast(S0.z, S0.w),
                                 ff_add(ff_mul(e2, dSy), ff_add(ff_mulf(e1, D1.y), ff_mulf(e3, D2.y))));
                }
            } else {
                const double2 f0 = c.KR[0];
                a1x = a2x = b1x = b2x = ff_split(f0.x);
                a1y = a2y = b1y = b2y = ff_split(f0.y);
            }
            ff sKA1, dA1, sKA2, dA2, sKB1, dB1, sKB2, dB2;
            ff_sigma<P, P2>(Mf, a1x, sKA1, dA1);
            ff_sigma<P, P2>(Mf, a2x, sKA2, dA2);
            ff_sigma<P, P2>(Mf, b1x, sKB1, dB1);
            ff_sigma<P, P2>(Mf, b2x, sKB2, dB2);
            const ff sRA1 = ff_mul(dA1, a1y), sRA2 = ff_mul(dA2, a2y);
            const ff sRB1 = ff_mul(dB1, b1y), sRB2 = ff_mul(dB2, b2y);
            const ff wj{__ldg(c.integ_f + j), __ldg(c.integ_l + j)};
            const ff wRA2 = ff_mul(wj, sRA2), wQRA2 = ff_mul(wj, a2y);
            const ff v[8] = {ff_mul(wRA2, b2x),           ff_mul(ff_mul(wj, sRA1), b1x), ff_mul(ff_mul(wj, sKA1), b1y),
                             ff_mul(wQRA2, sKB2),         ff_mul(ff_mul(wj, a1y), sKB1), ff_mul(ff_mul(wj, a1x), sRB1),
                             ff_mul(wRA2, b2y),           ff_mul(wQRA2, sRB2)};
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                if (kk == 0) { acc[q] = v[q].h; cmp[q] = v[q].l; }
                else pair_add(acc[q], cmp[q], v[q].h, v[q].l);
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float H, Lo;
    warp_reduce8_pair(acc, cmp, lane, H, Lo);
    if ((lane & 3) == 0) sh.red[((slot * (tpb >> 5)) + warp) * 8 + warp_reduce8_index(lane)] = make_float2(H, Lo);
}

// The low parts of the last history row into shared memory (after row_setup
// staged the high parts)
__device__ __forceinline__ void stage_lo(const DevCtx& c, const StageDev& sp, float2* s_lo) {
    const int L = c.L;
    const float2* KRl = c.KRl + (size_t)(sp.nrows - 1) * L;
    for (int k = threadIdx.x; k < L; k += blockDim.x) s_lo[k] = KRl[k];
    if (threadIdx.x == 0) s_lo[L] = make_float2(0.f, 0.f), s_lo[L + 1] = make_float2(0.f, 0.f);
}

}  // namespace mdf

}  // namespace dyn
