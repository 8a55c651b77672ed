// Mixed-precision stage kernel of the DYNAMITE hot path.
//
// Same algorithm as k_main (dyn_kernels.cu), with the O(L^2) work in FP32:
//   * stencil weights are FP32 copies of the FP64 tables;
//   * the history is read from an FP32 mirror (float2 (QK,QR), (dQK,dQR))
//     that the epilogue writes next to the FP64 master rows;
//   * A1/A2/B1/B2 gathers, Sigma and the eight convolution products are FP32;
//     each thread accumulates its products with a compensated (TwoSum) sum,
//     and the cross-lane fold and everything of size L (RHS, RK combination,
//     r(t), dr/dt, C(t,t), the step-error norm, time) stay in FP64.
// The position search is the exact FP64 binary search (integer compares on
// the bit patterns); only the fractional offset inside the located interval
// is formed in FP32 (one FP64 difference scaled by a stored FP32 inverse
// interval length), so interval indices equal the FP64 form's.  FP32 copies
// of int.dat and 1/delta_t_ratio keep conversions off the (slow) FP64 pipe.
#include <cmath>
#include "dyn_mixed.cuh"

namespace dyn {

// 128 threads; the register cap (48 at one target per thread) keeps ten CTAs per SM
template <int M, int K, int P, int P2>
__global__ void __launch_bounds__(128, K == 1 ? 10 : 4) k_main_mixed(const DevCtx c, const int s) {
    wait_prior_grid();
    const StageDev& sp = c.stages[s];
    extern __shared__ float2 s_lastf[];
    __shared__ mixed::RowShared sh;
    const int i = blockIdx.y;
    mixed::row_setup(c, sp, i, blockIdx.x == 0, s_lastf, sh);
    __syncthreads();
    mixed::chunk_sums<M, K, P, P2>(c, sp, blockIdx.x, 0, s_lastf, sh, i);
    __syncthreads();
    mixed::fold_chunks(c, i, gridDim.x, blockIdx.x, 1, sh);
}


// The (hi, lo) form of k_main_mixed (device functions in dyn_mixed.cuh, namespace mdf)
template <int M, int K, int P, int P2>
__global__ void __launch_bounds__(128, K == 1 ? 8 : 4) k_main_df(const DevCtx c, const int s) {
    wait_prior_grid();
    const StageDev& sp = c.stages[s];
    extern __shared__ float2 s_row[];  // [L+2] hi, [L+2] lo of the last history row
    __shared__ mixed::RowShared sh;
    __shared__ float s_clo[4];
    const int i = blockIdx.y;
    float2* s_lo = s_row + (c.L + 2);
    mixed::row_setup(c, sp, i, blockIdx.x == 0, s_row, sh, s_clo);
    mdf::stage_lo(c, sp, s_lo);
    __syncthreads();
    mdf::chunk_dd<M, K, P, P2>(c, sp, blockIdx.x, 0, s_row, s_lo, s_clo, sh, i);
    __syncthreads();
    mixed::fold_chunks(c, i, gridDim.x, blockIdx.x, 1, sh);
}

namespace {

template <int M, int K, int P, int P2>
cudaError_t launch_df(const DevCtx& c, int s, cudaStream_t st) {
    dim3 grid(c.nch, c.L), block(c.tpb);
    const size_t smem = 2 * (size_t)(c.L + 2) * sizeof(float2);  // > 48 KB from L = 3071 on
    static std::atomic<unsigned long long> devs{0};
    const cudaError_t e = raise_smem_limit(k_main_df<M, K, P, P2>, smem, 2 * (4096 + 2) * (int)sizeof(float2), devs);
    if (e != cudaSuccess) return e;
    return launch_pdl(k_main_df<M, K, P, P2>, grid, block, smem, st, c, s);
}

template <int M, int K, int P, int P2>
cudaError_t launch_t(const DevCtx& c, int s, cudaStream_t st) {
    if (c.mixed == 2) return launch_df<M, K, P, P2>(c, s, st);
    dim3 grid(c.nch, c.L), block(c.tpb);
    return launch_pdl(k_main_mixed<M, K, P, P2>, grid, block, (size_t)(c.L + 2) * sizeof(float2), st, c, s);
}

template <int M, int P, int P2>
cudaError_t launch_k(const DevCtx& c, int s, cudaStream_t st) {
    switch (c.kpt) {
        case 1: return launch_t<M, 1, P, P2>(c, s, st);
        case 2: return launch_t<M, 2, P, P2>(c, s, st);
        default: return launch_t<M, 4, P, P2>(c, s, st);
    }
}

template <int P, int P2>
cudaError_t launch_pp(const DevCtx& c, int s, cudaStream_t st) {
    // the depth-10 kernels lay the weights over element pairs: they need an even L
    return (c.m == 10 && c.L % 2 == 0) ? launch_k<10, P, P2>(c, s, st) : launch_k<0, P, P2>(c, s, st);
}

__global__ void k_to_f32(const double2* in, float2* out, size_t count) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const double2 v = in[e];
        out[e] = make_float2((float)v.x, (float)v.y);
    }
}

// low parts: v - (double)(float)v
__global__ void k_to_f32_lo(const double2* in, float2* out, size_t count) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const double2 v = in[e];
        out[e] = make_float2((float)(v.x - (double)(float)v.x), (float)(v.y - (double)(float)v.y));
    }
}

// FP32 inverse interval lengths and inverse step ratios of rows [0, n)
__global__ void k_time_f32(const double* t1, const double* dtr, int n, float* inv_len, float* inv_dtr) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        inv_dtr[k] = dtr[k] != 0.0 ? (float)(1.0 / dtr[k]) : 0.0f;
        inv_len[k] = k + 1 < n ? (float)(1.0 / (t1[k + 1] - t1[k])) : 0.0f;
    }
}

// out[p][e] = (w[e][2p], w[e][2p+1]) in FP32 (second tap 0 past the depth);
// with LO the low parts w - (double)(float)w instead
template <bool LO>
__global__ void k_weights_tapmajor(const double* in, float2* out, size_t targets, int m) {
    auto part = [](double w) { return LO ? (float)(w - (double)(float)w) : (float)w; };
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < targets; e += (size_t)gridDim.x * blockDim.x)
        for (int d = 0; d < m; d += 2)
            out[(size_t)(d >> 1) * targets + e] = make_float2(part(in[e * m + d]), d + 1 < m ? part(in[e * m + d + 1]) : 0.0f);
}

}  // namespace

cudaError_t launch_main_mixed(const DevCtx& c, int s, cudaStream_t st) {
    if (c.M.p == 3 && c.M.p2 == 4) return launch_pp<3, 4>(c, s, st);
    if (c.M.p == 3 && c.M.p2 == 0) return launch_pp<3, 0>(c, s, st);
    return launch_pp<-1, -1>(c, s, st);
}

cudaError_t launch_mirror_rows(const double2* in, float2* out, size_t count, cudaStream_t st) {
    const int blocks = (int)((count + 255) / 256 < 8192 ? (count + 255) / 256 : 8192);
    k_to_f32<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(in, out, count);
    return cudaGetLastError();
}

cudaError_t clear_mirror_rows(const DevCtx& c, size_t r0, size_t r1, cudaStream_t st) {
    if (r1 <= r0) return cudaSuccess;
    const size_t off = r0 * (size_t)c.L, bytes = (r1 - r0) * (size_t)c.L * sizeof(float2);
    for (float2* p : {c.KRf, c.dKRf, c.KRl}) {
        if (!p) continue;
        const cudaError_t e = cudaMemsetAsync(p + off, 0, bytes, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_time_f32(const double* t1, const double* dtr, int n, float* inv_len, float* inv_dtr,
                            cudaStream_t st) {
    k_time_f32<<<(n + 255) / 256, 256, 0, st>>>(t1, dtr, n, inv_len, inv_dtr);
    return cudaGetLastError();
}

cudaError_t launch_weights_tapmajor(const double* in, float2* out, size_t targets, int m, cudaStream_t st) {
    const int blocks = (int)((targets + 255) / 256 < 8192 ? (targets + 255) / 256 : 8192);
    k_weights_tapmajor<false><<<blocks > 0 ? blocks : 1, 256, 0, st>>>(in, out, targets, m);
    return cudaGetLastError();
}

cudaError_t launch_weights_tapmajor_lo(const double* in, float2* out, size_t targets, int m, cudaStream_t st) {
    const int blocks = (int)((targets + 255) / 256 < 8192 ? (targets + 255) / 256 : 8192);
    k_weights_tapmajor<true><<<blocks > 0 ? blocks : 1, 256, 0, st>>>(in, out, targets, m);
    return cudaGetLastError();
}

cudaError_t launch_mirror_lo(const double2* in, float2* out, size_t count, cudaStream_t st) {
    const int blocks = (int)((count + 255) / 256 < 8192 ? (count + 255) / 256 : 8192);
    k_to_f32_lo<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(in, out, count);
    return cudaGetLastError();
}

}  // namespace dyn
