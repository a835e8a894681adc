// ransac.cu — batched RANSAC hypothesis scoring: the step after matching.
//
// The reference's RansacCPU (wslam/src/pose_estimate_cpu/ransac_cpu.cpp)
// fits a fundamental matrix to 8 random matches per iteration and classifies
// every match by its Sampson distance (SampsonDistance, :183-196;
// ClassifyInliers, :198-210).  The fit (an SVD) stays on the host; this file
// scores many hypotheses against all matches at once on the GPU.
//
// Arithmetic: binary64, no contraction (--fmad=false), in this order:
//   Fx  = F xp            component r: (F[r][0] x_p + F[r][1] y_p) + F[r][2]
//   Ftx = F^T xc          component c: (F[0][c] x_c + F[1][c] y_c) + F[2][c]
//   num = (x_c Fx0 + y_c Fx1) + Fx2
//   den = ((Fx0^2 + Fx1^2) + Ftx0^2) + Ftx1^2
//   d   = den < 1e-12 ? +inf : num^2 / den;   inlier iff d < threshold.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <mutex>
#include <string>

#include "runtime_internal.h"

namespace {

constexpr int KR_THREADS = 256;

__device__ __forceinline__ bool sampson_inlier(const double* F, double xp, double yp, double xc, double yc,
                                               double thr) {
    const double fx0 = (F[0] * xp + F[1] * yp) + F[2];
    const double fx1 = (F[3] * xp + F[4] * yp) + F[5];
    const double fx2 = (F[6] * xp + F[7] * yp) + F[8];
    const double ft0 = (F[0] * xc + F[3] * yc) + F[6];
    const double ft1 = (F[1] * xc + F[4] * yc) + F[7];
    const double num = (xc * fx0 + yc * fx1) + fx2;
    const double den = ((fx0 * fx0 + fx1 * fx1) + ft0 * ft0) + ft1 * ft1;
    if (den < 1e-12) return false;  // infinite distance
    return (num * num) / den < thr;
}

// One CTA per hypothesis: count the inliers over all matches (ballot + popc
// per warp), and write the inlier bitmask when asked (bit i of word i / 32).
__global__ void __launch_bounds__(KR_THREADS)
k_sampson(const double* __restrict__ fmats, int n_hyp, const double2* __restrict__ prev,
          const double2* __restrict__ curr, int n, double thr, int* __restrict__ counts,
          uint32_t* __restrict__ masks) {
    __shared__ double s_f[9];
    __shared__ int s_cnt[KR_THREADS / 32];
    for (int h = blockIdx.x; h < n_hyp; h += gridDim.x) {
        if (threadIdx.x < 9) s_f[threadIdx.x] = fmats[(size_t)h * 9 + threadIdx.x];
        __syncthreads();
        double F[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = s_f[k];
        int cnt = 0;
        const int words = (n + 31) / 32;
        for (int i0 = 0; i0 < n; i0 += KR_THREADS) {
            const int i = i0 + threadIdx.x;
            bool in = false;
            if (i < n) {
                const double2 p = prev[i], q = curr[i];
                in = sampson_inlier(F, p.x, p.y, q.x, q.y, thr);
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, in);
            cnt += (threadIdx.x & 31) == 0 ? __popc(bal) : 0;
            if (masks && (threadIdx.x & 31) == 0 && (i >> 5) < words) masks[(size_t)h * words + (i >> 5)] = bal;
        }
        if ((threadIdx.x & 31) == 0) s_cnt[threadIdx.x >> 5] = cnt;
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < KR_THREADS / 32; ++w) t += s_cnt[w];
            counts[h] = t;
        }
        __syncthreads();
    }
}

}  // namespace

extern "C" {

uslam_status uslam_ransac_score(uslam_ctx* ctx, const double* fmats, int n_hyp, const double* prev_xy,
                                const double* curr_xy, int n_matches, double threshold, int* counts,
                                uint32_t* masks) {
    if (!ctx || n_hyp < 0 || n_matches < 0 || !counts || (n_hyp > 0 && !fmats) ||
        (n_matches > 0 && (!prev_xy || !curr_xy)))
        return set_err(ctx ? &ctx->err : nullptr, USLAM_INVALID_ARG, "ransac_score: bad arguments");
    if (n_hyp == 0) return USLAM_OK;
    cudaError_t e = cudaSetDevice(ctx->device);
    const int words = (n_matches + 31) / 32;
    const size_t f_b = uslam_rt::round_up(sizeof(double) * 9 * static_cast<size_t>(n_hyp), 256);
    const size_t m_b = uslam_rt::round_up(sizeof(double) * 2 * static_cast<size_t>(std::max(n_matches, 1)), 256);
    const size_t c_b = uslam_rt::round_up(sizeof(int) * static_cast<size_t>(n_hyp), 256);
    const size_t k_b = masks ? uslam_rt::round_up(sizeof(uint32_t) * words * static_cast<size_t>(n_hyp), 256) : 0;
    const size_t need = f_b + 2 * m_b + c_b + k_b;
    std::lock_guard<std::mutex> lk(ctx->ransac_mu);
    if (e == cudaSuccess && need > ctx->ransac_bytes) {
        if (ctx->ransac_buf) cudaFree(ctx->ransac_buf);
        ctx->ransac_buf = nullptr;
        ctx->ransac_bytes = 0;
        e = cudaMalloc(&ctx->ransac_buf, need);
        if (e == cudaSuccess) ctx->ransac_bytes = need;
    }
    if (e != cudaSuccess) return ctx->cuda_fail(e, "ransac_score: scratch");
    char* base = static_cast<char*>(ctx->ransac_buf);
    double* d_f = reinterpret_cast<double*>(base);
    double2* d_p = reinterpret_cast<double2*>(base + f_b);
    double2* d_q = reinterpret_cast<double2*>(base + f_b + m_b);
    int* d_c = reinterpret_cast<int*>(base + f_b + 2 * m_b);
    uint32_t* d_k = masks ? reinterpret_cast<uint32_t*>(base + f_b + 2 * m_b + c_b) : nullptr;
    e = cudaMemcpy(d_f, fmats, sizeof(double) * 9 * n_hyp, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n_matches > 0)
        e = cudaMemcpy(d_p, prev_xy, sizeof(double) * 2 * n_matches, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n_matches > 0)
        e = cudaMemcpy(d_q, curr_xy, sizeof(double) * 2 * n_matches, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int grid = std::min(n_hyp, std::max(ctx->num_sms, 1) * 8);
        k_sampson<<<grid, KR_THREADS>>>(d_f, n_hyp, d_p, d_q, n_matches, threshold, d_c, d_k);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(counts, d_c, sizeof(int) * n_hyp, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && masks)
        e = cudaMemcpy(masks, d_k, sizeof(uint32_t) * words * static_cast<size_t>(n_hyp), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "ransac_score");
    return USLAM_OK;
}

}  // extern "C"
