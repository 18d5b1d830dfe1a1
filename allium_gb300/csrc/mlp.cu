// Kernels of the per-cell MLP that predicts the next time step's moments (the
// learned initial iterate of the outer solve): a BF16 tensor-core GEMM with
// FP32 accumulation and a fused bias / ReLU epilogue, the ReLU and bias
// gradients, the mean-squared-error gradient and the Adam update.
//
// GEMM: C[M][N] = alpha * A[M][K] B[K][N] (+ beta C) (+ bias[N]) (ReLU), with A
// and B read through arbitrary element strides, so the same kernel computes
// X W (forward), dY W^T (input gradient) and X^T dY (weight gradient).  A block
// of 4 warps owns a 64 x 64 tile of C; tiles of A (64 x 32) and B (32 x 64) are
// staged in shared memory as BF16 and each warp issues mma.sync.m16n8k16 on its
// 32 x 32 quarter (2 x 4 tiles of 16 x 8), FP32 accumulators in registers.
#include <cuda_bf16.h>
#include <cstdint>

#include "allium_sweep.h"

namespace {

constexpr int TM = 64, TN = 64, TK = 32;

struct GemmArgs {
    int M, N, K;
    const __nv_bfloat16* A;
    long long sam, sak;       // A(m, k) = A[m * sam + k * sak]
    const __nv_bfloat16* B;
    long long sbk, sbn;       // B(k, n) = B[k * sbk + n * sbn]
    float* C;                 // [M][ldc] FP32 output (or null)
    long long ldc;
    __nv_bfloat16* Cb;        // [M][ldc] BF16 copy of the output (or null)
    const float* bias;        // [N] or null
    float alpha, beta;
    int relu;
    int ksplit;               // > 1: blockIdx.z takes one of ksplit K ranges, C accumulated atomically
};

__device__ inline uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__global__ void __launch_bounds__(128) k_gemm_bf16(GemmArgs g) {
    __shared__ __nv_bfloat16 As[TM][TK + 8];
    __shared__ __nv_bfloat16 Bs[TK][TN + 8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;   // warp quarter of the tile
    const int gid = lane >> 2, tig = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.0f;
    const __nv_bfloat16 zero = __float2bfloat16(0.0f);
    // K range of this block (whole K unless split)
    const int kchunk = ((g.K + g.ksplit - 1) / g.ksplit + TK - 1) / TK * TK;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(g.K, kbeg + kchunk);

    for (int k0 = kbeg; k0 < kend; k0 += TK) {
        // stage A (64 x 32) and B (32 x 64), zero outside the matrices
        for (int idx = threadIdx.x; idx < TM * TK; idx += blockDim.x) {
            const int r = idx / TK, c = idx % TK;
            const int m = m0 + r, k = k0 + c;
            As[r][c] = (m < g.M && k < kend) ? g.A[(long long)m * g.sam + (long long)k * g.sak] : zero;
        }
        for (int idx = threadIdx.x; idx < TK * TN; idx += blockDim.x) {
            const int r = idx / TN, c = idx % TN;
            const int k = k0 + r, n = n0 + c;
            Bs[r][c] = (k < kend && n < g.N) ? g.B[(long long)k * g.sbk + (long long)n * g.sbn] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                const int r = wm + a * 16 + gid;
                const int c = kk + tig * 2;
                af[a][0] = pack2(As[r][c], As[r][c + 1]);
                af[a][1] = pack2(As[r + 8][c], As[r + 8][c + 1]);
                af[a][2] = pack2(As[r][c + 8], As[r][c + 9]);
                af[a][3] = pack2(As[r + 8][c + 8], As[r + 8][c + 9]);
            }
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int n = wn + b * 8 + gid;
                const int k = kk + tig * 2;
                bf[b][0] = pack2(Bs[k][n], Bs[k + 1][n]);
                bf[b][1] = pack2(Bs[k + 8][n], Bs[k + 9][n]);
            }
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b)
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
                        : "+f"(acc[a][b][0]), "+f"(acc[a][b][1]), "+f"(acc[a][b][2]), "+f"(acc[a][b][3])
                        : "r"(af[a][0]), "r"(af[a][1]), "r"(af[a][2]), "r"(af[a][3]), "r"(bf[b][0]), "r"(bf[b][1]));
        }
        __syncthreads();
    }

    // epilogue: C = alpha acc + beta C + bias, ReLU
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int m = m0 + wm + a * 16 + gid + (c >= 2 ? 8 : 0);
                const int n = n0 + wn + b * 8 + tig * 2 + (c & 1);
                if (m >= g.M || n >= g.N) continue;
                const long long o = (long long)m * g.ldc + n;
                if (g.ksplit > 1) {   // partial sum of one K range (C zeroed beforehand)
                    atomicAdd(g.C + o, g.alpha * acc[a][b][c]);
                    continue;
                }
                float v = g.alpha * acc[a][b][c];
                if (g.beta != 0.0f && g.C) v += g.beta * g.C[o];
                if (g.bias) v += g.bias[n];
                if (g.relu) v = v > 0.0f ? v : 0.0f;
                if (g.C) g.C[o] = v;
                if (g.Cb) g.Cb[o] = __float2bfloat16(v);
            }
}

// dZ = dY * (Z > 0) (ReLU backward on the pre-activation's sign, which the
// forward's ReLU output shares), written as BF16 for the next GEMM and FP32
__global__ void k_relu_backward(long long count, const float* __restrict__ dy, const float* __restrict__ y,
                                float* __restrict__ dz, __nv_bfloat16* __restrict__ dzb) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float v = y[i] > 0.0f ? dy[i] : 0.0f;
    if (dz) dz[i] = v;
    if (dzb) dzb[i] = __float2bfloat16(v);
}

// db[n] = sum_m dY[m][n]: one block per column stripe of 32, rows split over warps
__global__ void k_bias_grad(int M, int N, const float* __restrict__ dy, float* __restrict__ db) {
    __shared__ float part[8][33];
    const int n = blockIdx.x * 32 + (threadIdx.x & 31);
    const int w = threadIdx.x >> 5;
    float s = 0.0f;
    if (n < N)
        for (int m = w; m < M; m += 8) s += dy[(long long)m * N + n];
    part[w][threadIdx.x & 31] = s;
    __syncthreads();
    if (w == 0 && n < N) {
        float t = 0.0f;
        for (int k = 0; k < 8; ++k) t += part[k][threadIdx.x & 31];
        db[n] = t;
    }
}

// dY = 2 (Y - target) / count (mean squared error over all entries); returns
// per-block partial sums of the squared error in loss[blockIdx.x]
__global__ void k_mse_grad(long long count, const float* __restrict__ y, const float* __restrict__ target,
                           float* __restrict__ dy, float* __restrict__ loss) {
    __shared__ float red[256];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float e2 = 0.0f;
    if (i < count) {
        const float d = y[i] - target[i];
        dy[i] = 2.0f * d / (float)count;
        e2 = d * d;
    }
    red[threadIdx.x] = e2;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss[blockIdx.x] = red[0];
}

// Adam (Kingma & Ba) on FP32 master weights, refreshing the BF16 copy
__global__ void k_adam(long long count, float* __restrict__ w, __nv_bfloat16* __restrict__ wb,
                       const float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
}

__global__ void k_to_bf16(long long count, const float* __restrict__ x, __nv_bfloat16* __restrict__ y) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) y[i] = __float2bfloat16(x[i]);
}

inline int grid1(long long n, int b) { return (int)((n + b - 1) / b); }

inline int status_of(cudaError_t e) { return e == cudaSuccess ? ALLIUM_OK : ALLIUM_ERR_CUDA; }

}  // namespace

extern "C" {

int allium_mlp_gemm(int M, int N, int K, const void* A, long long sam, long long sak, const void* B, long long sbk,
                    long long sbn, float* C, long long ldc, void* C_bf16, const float* bias, float alpha, float beta,
                    int relu, void* stream) {
    if (M <= 0 || N <= 0 || K <= 0 || !A || !B || (!C && !C_bf16) || ldc < N) return ALLIUM_ERR_ARG;
    if (beta != 0.0f && !C) return ALLIUM_ERR_ARG;
    GemmArgs g;
    g.M = M; g.N = N; g.K = K;
    g.A = static_cast<const __nv_bfloat16*>(A); g.sam = sam; g.sak = sak;
    g.B = static_cast<const __nv_bfloat16*>(B); g.sbk = sbk; g.sbn = sbn;
    g.C = C; g.ldc = ldc; g.Cb = static_cast<__nv_bfloat16*>(C_bf16); g.bias = bias;
    g.alpha = alpha; g.beta = beta; g.relu = relu;
    g.ksplit = 1;
    const int tiles = ((N + TN - 1) / TN) * ((M + TM - 1) / TM);
    // few output tiles over a long K (the weight gradients X^T dY over a batch):
    // split K across blocks so the GPU fills, partial sums added atomically
    if (tiles < 304 && K >= 8 * TK && C && !C_bf16 && !bias && !relu && beta == 0.0f && ldc == N) {
        g.ksplit = (304 + tiles - 1) / tiles;
        if (g.ksplit > K / (4 * TK)) g.ksplit = K / (4 * TK);
        if (g.ksplit < 1) g.ksplit = 1;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (g.ksplit > 1 && cudaMemsetAsync(C, 0, (size_t)M * N * sizeof(float), st) != cudaSuccess) return ALLIUM_ERR_CUDA;
    dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM, g.ksplit);
    k_gemm_bf16<<<grid, 128, 0, st>>>(g);
    return status_of(cudaGetLastError());
}

int allium_mlp_relu_backward(long long count, const float* dy, const float* y, float* dz, void* dz_bf16, void* stream) {
    if (count <= 0 || !dy || !y || (!dz && !dz_bf16)) return ALLIUM_ERR_ARG;
    k_relu_backward<<<grid1(count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        count, dy, y, dz, static_cast<__nv_bfloat16*>(dz_bf16));
    return status_of(cudaGetLastError());
}

int allium_mlp_bias_grad(int M, int N, const float* dy, float* db, void* stream) {
    if (M <= 0 || N <= 0 || !dy || !db) return ALLIUM_ERR_ARG;
    k_bias_grad<<<(N + 31) / 32, 256, 0, static_cast<cudaStream_t>(stream)>>>(M, N, dy, db);
    return status_of(cudaGetLastError());
}

int allium_mlp_mse_grad(long long count, const float* y, const float* target, float* dy, float* loss_partials,
                        void* stream) {
    if (count <= 0 || !y || !target || !dy || !loss_partials) return ALLIUM_ERR_ARG;
    k_mse_grad<<<grid1(count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(count, y, target, dy, loss_partials);
    return status_of(cudaGetLastError());
}

int allium_mlp_adam(long long count, float* w, void* w_bf16, const float* grad, float* m, float* v, float lr,
                    float beta1, float beta2, float eps, int step, void* stream) {
    if (count <= 0 || !w || !grad || !m || !v || step < 1) return ALLIUM_ERR_ARG;
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_adam<<<grid1(count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        count, w, static_cast<__nv_bfloat16*>(w_bf16), grad, m, v, lr, beta1, beta2, eps, c1, c2);
    return status_of(cudaGetLastError());
}

int allium_mlp_to_bf16(long long count, const float* x, void* y, void* stream) {
    if (count <= 0 || !x || !y) return ALLIUM_ERR_ARG;
    k_to_bf16<<<grid1(count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(count, x,
                                                                                  static_cast<__nv_bfloat16*>(y));
    return status_of(cudaGetLastError());
}

}  // extern "C"
