// BF16 GEMM on the fifth-generation tensor cores for the per-cell MLP:
//     C[M][N] = alpha * A[M][K] B[N][K]^T (+ beta C) (+ bias[N]) (ReLU),
// A and B K-major in global memory (row strides multiples of 8 elements).
//
// One CTA of 128 threads owns a 128 x BN tile of C (BN = 256 when N > 128, else
// 128); its accumulator lives in tensor memory (128 lanes x BN FP32 columns).
// Warp 0's elected lane streams 128 x 64 tiles of A and BN x 64 tiles of B into
// a shared-memory ring (two stages of 48 KB, or three of 32 KB) with
// cp.async.bulk.tensor (128-byte swizzle, out-of-range rows and columns
// zero-filled by the tensor map); warp 1's elected lane issues
// tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = BN, K = 16, four per stage)
// and frees each stage with tcgen05.commit on the stage's mbarrier.  After the
// last commit every warp reads its 32 accumulator lanes with tcgen05.ld and
// applies the epilogue through shared memory (coalesced row stores).  Two CTAs
// share an SM, so one's epilogue overlaps the other's MMAs.  With ksplit > 1,
// blockIdx.z takes one of ksplit K ranges and the partial sums are added
// atomically (C zeroed beforehand).
//
// Every mbarrier wait is bounded; a wait that gives up sets the module's status
// word (allium_mlp_status), and the epilogue waits once more (bounded) for the
// tile's MMAs before it frees its tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "allium_sweep.h"

namespace {

constexpr int TM = 128, TK = 64;
constexpr int TILE_A_BYTES = TM * TK * 2;            // 16 KB
constexpr int kWaitLimit = 1 << 22;

// tile N (128 or 256: the accumulator's FP32 columns in tensor memory) and the
// ring depth; both shapes use 96 KB of shared memory, so that two CTAs share an
// SM (and its 512 tensor-memory columns) and one's epilogue overlaps the other's
// MMAs
template <int BN>
struct TcShape {
    static constexpr int STAGES = BN == 256 ? 2 : 3;
    static constexpr int TILE_B_BYTES = BN * TK * 2;
    static constexpr int STAGE_BYTES = TILE_A_BYTES + TILE_B_BYTES;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;
    // instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, N, M
    static constexpr uint32_t IDESC =
        (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
};

__device__ int g_tc_status = 0;

struct TcArgs {
    int M, N, K;
    float* C;
    long long ldc;
    __nv_bfloat16* Cb;
    long long ldcb;
    const float* bias;
    float alpha, beta;
    int relu, ksplit;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool bar_try(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool bar_wait(unsigned bar, unsigned parity) {
    for (int i = 0; i < kWaitLimit; ++i)
        if (bar_try(bar, parity)) return true;
    atomicOr(&g_tc_status, 1);
    return false;
}

// shared-memory matrix descriptor of a K-major tile written by the tensor map
// with 128-byte swizzle: rows of 128 bytes, 8-row groups 1024 bytes apart
__device__ __forceinline__ uint64_t sw128_desc(unsigned saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                  // leading-dimension offset (unused with this swizzle)
    d |= (uint64_t)(1024 >> 4) << 32;        // stride-dimension offset: next 8-row group
    d |= (uint64_t)1 << 46;                  // descriptor version of this architecture
    d |= (uint64_t)2 << 61;                  // 128-byte swizzle
    return d;
}

template <int BN>
__global__ void __launch_bounds__(128, 2) k_gemm_tc(const __grid_constant__ CUtensorMap tA,
                                                    const __grid_constant__ CUtensorMap tB, TcArgs g) {
    using Sh = TcShape<BN>;
    constexpr int STAGES = Sh::STAGES, STAGE_BYTES = Sh::STAGE_BYTES;
    extern __shared__ unsigned char dsm[];
    __shared__ __align__(8) unsigned long long full[STAGES], empty[STAGES], done;
    __shared__ unsigned tmem_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* ring = dsm + ((1024u - (smem_u32(dsm) & 1023u)) & 1023u);
    const unsigned ring_s = smem_u32(ring);
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * BN;
    const int kt_total = (g.K + TK - 1) / TK;
    const int per = (kt_total + g.ksplit - 1) / g.ksplit;
    const int kt0 = blockIdx.z * per;
    const int nk = max(0, min(kt_total, kt0 + per) - kt0);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_slot;

    if (warp == 0 && lane == 0) {
        // producer: stage kt into slot kt % STAGES once the MMAs of kt - STAGES freed it
        for (int i = 0; i < nk; ++i) {
            const int s = i % STAGES;
            if (i >= STAGES) bar_wait(smem_u32(&empty[s]), (unsigned)((i / STAGES - 1) & 1));
            const unsigned fb = smem_u32(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(STAGE_BYTES) : "memory");
            const int kx = (kt0 + i) * TK;
            const unsigned sa = ring_s + s * STAGE_BYTES;
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                ::"r"(sa), "l"(reinterpret_cast<uint64_t>(&tA)), "r"(kx), "r"(m0), "r"(fb) : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                ::"r"(sa + TILE_A_BYTES), "l"(reinterpret_cast<uint64_t>(&tB)), "r"(kx), "r"(n0), "r"(fb) : "memory");
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        for (int i = 0; i < nk; ++i) {
            const int s = i % STAGES;
            bar_wait(smem_u32(&full[s]), (unsigned)((i / STAGES) & 1));
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned sa = ring_s + s * STAGE_BYTES;
#pragma unroll
            for (int kk = 0; kk < TK / 16; ++kk) {
                const uint64_t da = sw128_desc(sa + kk * 32);
                const uint64_t db = sw128_desc(sa + TILE_A_BYTES + kk * 32);
                const unsigned acc = (i > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                    ::"r"(tmem), "l"(da), "l"(db), "r"(Sh::IDESC), "r"(acc) : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(smem_u32(&empty[s])) : "memory");
        }
        if (nk > 0)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(smem_u32(&done)) : "memory");
        else
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&done)) : "memory");
    }
    __syncwarp();

    // epilogue: warp w reads accumulator lanes 32w..32w+31 (rows of the tile);
    // a wait that gives up waits once more (bounded) for the tile's MMAs
    if (!bar_wait(smem_u32(&done), 0u)) bar_wait(smem_u32(&done), 0u);
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // 32 x 32 blocks go through shared memory (the ring is free once the MMAs are
    // done), so that each store instruction writes 32 consecutive columns of a row
    float* stage = reinterpret_cast<float*>(ring) + warp * 32 * 33;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
        __syncwarp();
        uint32_t r[32];
        const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
            "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        // lane l holds row 32w + l: write it as row l of the block
#pragma unroll
        for (int j = 0; j < 32; ++j) stage[lane * 33 + j] = nk > 0 ? g.alpha * __uint_as_float(r[j]) : 0.0f;
        __syncwarp();
        // lane l now takes column c0 + l of each of the block's 32 rows
        const int n = n0 + c0 + lane;
        const bool col_ok = n < g.N;
        const float bv = (g.bias && col_ok) ? g.bias[n] : 0.0f;
#pragma unroll 4
        for (int rr = 0; rr < 32; ++rr) {
            const int row = m0 + warp * 32 + rr;
            if (row >= g.M || !col_ok) continue;
            float v = stage[rr * 33 + lane];
            const long long o = (long long)row * g.ldc + n;
            if (g.ksplit > 1) {
                atomicAdd(g.C + o, v);
                continue;
            }
            if (g.beta != 0.0f && g.C) v += g.beta * g.C[o];
            v += bv;
            if (g.relu) v = v > 0.0f ? v : 0.0f;
            if (g.C) g.C[o] = v;
            if (g.Cb) g.Cb[(long long)row * g.ldcb + n] = __float2bfloat16(v);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
}

// out[c][r] = in[r][c] for BF16 matrices (32 x 32 tiles through shared memory)
__global__ void k_transpose_bf16(int rows, int cols, const __nv_bfloat16* __restrict__ in, long long ldi,
                                 __nv_bfloat16* __restrict__ out, long long ldo) {
    __shared__ __nv_bfloat16 t[32][33];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[y][threadIdx.x] = in[(long long)r * ldi + c];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int c = c0 + y, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[(long long)c * ldo + r] = t[threadIdx.x][y];
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    // the driver entry point is process-wide; a race here only repeats the lookup
    static std::atomic<PFN_cuTensorMapEncodeTiled_v12000> cached{nullptr};
    PFN_cuTensorMapEncodeTiled_v12000 fn = cached.load();
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess) {
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
            cached.store(fn);
        }
    }
    return fn;
}

// rows x K BF16 matrix, K contiguous, row stride ld elements; boxes of box_rows rows x 64 K
bool make_map(CUtensorMap* m, const void* base, long long rows, long long K, long long ld, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)TK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int status_of(cudaError_t e) { return e == cudaSuccess ? ALLIUM_OK : ALLIUM_ERR_CUDA; }

}  // namespace

extern "C" {

int allium_mlp_gemm_tc(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb, float* C,
                       long long ldc, void* C_bf16, long long ldcb, const float* bias, float alpha, float beta, int relu,
                       int ksplit, void* stream) {
    if (M <= 0 || N <= 0 || K <= 0 || !A || !B || (!C && !C_bf16)) return ALLIUM_ERR_ARG;
    if (lda < K || ldb < K || (lda % 8) || (ldb % 8) || (reinterpret_cast<uintptr_t>(A) & 15) ||
        (reinterpret_cast<uintptr_t>(B) & 15))
        return ALLIUM_ERR_ARG;   // the tensor map needs 16-byte aligned rows
    if ((C && ldc < N) || (C_bf16 && ldcb < N) || (beta != 0.0f && !C)) return ALLIUM_ERR_ARG;
    if (ksplit < 1) ksplit = 1;
    if (ksplit > 1 && (!C || C_bf16 || bias || relu || beta != 0.0f)) return ALLIUM_ERR_ARG;
    // N tiles of 256 when the output is wider than 128 columns
    const int bn = N > 128 ? 256 : 128;
    CUtensorMap ta, tb;
    if (!make_map(&ta, A, M, K, lda, TM) || !make_map(&tb, B, N, K, ldb, bn)) return ALLIUM_ERR_UNSUPPORTED;
    TcArgs g;
    g.M = M; g.N = N; g.K = K;
    g.C = C; g.ldc = ldc; g.Cb = static_cast<__nv_bfloat16*>(C_bf16); g.ldcb = ldcb;
    g.bias = bias; g.alpha = alpha; g.beta = beta; g.relu = relu; g.ksplit = ksplit;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the dynamic shared-memory opt-in is a per-device function attribute
    static std::atomic<unsigned long long> attr_done{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return ALLIUM_ERR_CUDA;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        if (cudaFuncSetAttribute(k_gemm_tc<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<128>::SMEM_BYTES) != cudaSuccess ||
            cudaFuncSetAttribute(k_gemm_tc<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<256>::SMEM_BYTES) != cudaSuccess)
            return ALLIUM_ERR_CUDA;
        attr_done.fetch_or(bit);
    }
    if (ksplit > 1 &&
        cudaMemset2DAsync(C, (size_t)ldc * sizeof(float), 0, (size_t)N * sizeof(float), (size_t)M, st) != cudaSuccess)
        return ALLIUM_ERR_CUDA;
    dim3 grid((N + bn - 1) / bn, (M + TM - 1) / TM, ksplit);
    if (bn == 256)
        k_gemm_tc<256><<<grid, 128, TcShape<256>::SMEM_BYTES, st>>>(ta, tb, g);
    else
        k_gemm_tc<128><<<grid, 128, TcShape<128>::SMEM_BYTES, st>>>(ta, tb, g);
    return status_of(cudaGetLastError());
}

int allium_mlp_transpose_bf16(int rows, int cols, const void* in, long long ldi, void* out, long long ldo,
                              void* stream) {
    if (rows <= 0 || cols <= 0 || !in || !out || ldi < cols || ldo < rows) return ALLIUM_ERR_ARG;
    dim3 grid((cols + 31) / 32, (rows + 31) / 32);
    k_transpose_bf16<<<grid, dim3(32, 8), 0, static_cast<cudaStream_t>(stream)>>>(
        rows, cols, static_cast<const __nv_bfloat16*>(in), ldi, static_cast<__nv_bfloat16*>(out), ldo);
    return status_of(cudaGetLastError());
}

int allium_mlp_status(void* stream) {
    int st = 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyFromSymbolAsync(&st, g_tc_status, sizeof(int), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return ALLIUM_ERR_CUDA;
    if (st) {
        const int zero = 0;
        cudaMemcpyToSymbolAsync(g_tc_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
        return ALLIUM_ERR_TIMEOUT;
    }
    return ALLIUM_OK;
}

}  // extern "C"
