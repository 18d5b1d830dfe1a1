// Fused FP32 inner sweep, its isotropic source, and the double-float transport
// residual: the kernels of the mixed-precision outer solve.
//
// The inner operator of chive's scalar-flux iteration (MomentMethodFixedPointOperator::Mult,
// src/transport_op.hpp:75-90, with the source of exe/chive.cpp:593-599) is
//     phi_out = D L^{-1} (D^T S phi + q).
// Here it is one small kernel and one CUDA graph: k_iso_source forms the
// per-cell source s = (sigma_s M phi) / sum(w) + q_iso once per cell (it is the
// same for every direction), the graph runs k_fused_level once per wavefront
// level and then k_moments_f32 (DiscreteToMoment::Mult, src/transport_op.cpp:3-31)
// over the FP32 psi with double-float sums.  Nothing psi-sized is read besides
// the upwind traces.
//
// Schedule.  A unit is the set of a cell's angles that share the octant (signs
// of Omega) and the face pattern (which faces are inflow and outflow): all of
// them read their upwind traces across the same faces.  The fused sweep orders
// units by the Kahn frontiers of the unit graph (its edges are the node edges
// between units), so a unit's angles share one level.  On a distorted mesh the
// angles of one octant at a cell fall into about ten different node levels
// (runs of ~5 angles per cell and level at the 64^3 +-0.1h S12 workload); as
// units they stay together (runs of ~21), at the price of ~9% more levels.
// If the unit graph had a cycle the node levels are used instead.
//
// k_fused_level work unit: one thread per (cell, angle, group) node of a level.
// Nodes come from a record {cell, angle | face pattern << 16}, sorted within
// each level by (face pattern, unit, angle) and packed so that a warp holds at
// most kSlots units (padding records {-1, 0} close a warp early).  Each warp copies
// the FP32 tables of its units (B_d = G_d + the unit's outflow-face terms
// n_{k,d} F_k, M, [Mt], F_k and the outward face normals, 1.5 KB for a
// trilinear hex) into shared memory with cp.async.bulk and an mbarrier per
// copy, one slot per unit, while its lanes load their
// sources and, after griddepcontrol.wait, their upwind traces (one 32-byte
// neighbour block per inflow face when the face's DOF map is the standard
// one), folded into the right-hand side with the staged face blocks.  Each row of the local
// system is then assembled from shared memory with packed FP32 (f32x2) FMAs,
// eliminated against the rows above and scaled by its pivot's reciprocal, so
// that only the strict upper triangle of a unit-diagonal U stays in registers.
// Consecutive level launches overlap through programmatic dependent launch: a
// level's blocks load their records, tables and sources while the previous
// level drains.  (Factoring before the wait, to overlap the elimination with
// the previous level as well, measured slower: the factors held across the
// wait spill.)
//
// Layout of every psi-sized vector here (the "fused layout"):
//     v[((g * Ne + e) * Nw + a) * n + i],
// group-major, then cell, angle, DOF: a level's angles of one cell and their
// upwind traces are contiguous runs.
//
// k_residual_df computes r = q + D^T S phi - L psi (AdvectionOperator::Mult,
// src/sweep.cpp:1246-1387, applied to psi) to about 1e-14 of |q| in
// double-float arithmetic (pairs of FP32 values, error-free products and sums)
// on the FP32 pipe: GB300 issues FP64 at 1/64 of its FP32 rate, and this
// residual needs about 420 multiply-adds per (cell, angle) node.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>
#include <utility>
#include <vector>

#include "geometry.cuh"
#include "internal.h"

namespace allium {

namespace {

constexpr int fpow(int b, int e) { return e == 0 ? 1 : b * fpow(b, e - 1); }

template <int D, int P>
struct Shape {
    static constexpr int N1 = P + 1;
    static constexpr int N = fpow(N1, D);
    static constexpr int NF = fpow(N1, D - 1);
    static constexpr int NFACE = 2 * D;
};

// FP32 table of one cell for the sweep: G_d (row-major), M, [Mt], F_k, outward
// unit normals of the faces (4 floats each, 16-byte aligned).
template <int D, int P, bool TD>
struct Tab {
    using S = Shape<D, P>;
    static constexpr int oG = 0;
    static constexpr int oM = D * S::N * S::N;
    static constexpr int oMt = oM + S::N * S::N;
    static constexpr int oF = oMt + (TD ? S::N * S::N : 0);
    static constexpr int oNrm = (oF + S::NFACE * S::NF * S::NF + 3) / 4 * 4;
    static constexpr int size = oNrm + S::NFACE * 4;
};

// double-float table of one cell for the residual.  The volume matrices are
// stored transposed (column j of G_d, M, [Mt] contiguous, rows fastest) so that
// a column feeds two rows per packed operation; then F_k row-major.  High
// parts, then the low parts in the same order.
template <int D, int P, bool TD>
struct DTab {
    using S = Shape<D, P>;
    static constexpr int NV = D + 1 + (TD ? 1 : 0);      // volume matrices
    static constexpr int oV = 0;                          // [j][v][i]
    static constexpr int oF = NV * S::N * S::N;           // [k][ii][jj]
    static constexpr int half = (oF + S::NFACE * S::NF * S::NF + 3) / 4 * 4;
    static constexpr int size = 2 * half;
};

constexpr int kFusedBlock = 128;
constexpr int kFusedWarps = kFusedBlock / 32;
// the sweep's level kernel: 64-thread blocks, at most 72 registers (14 blocks
// per SM; 3.14 ms at 64^3 S12 against 3.22 ms at 10 blocks and 96 registers and
// 3.61 ms at 16 blocks and 64); smaller blocks finish a level's last wave sooner
constexpr int kSweepBlock = 64;
constexpr int kSweepWarps = kSweepBlock / 32;
constexpr int kSweepMinBlocks = 14;
// staged unit tables per warp in the sweep: two (2.84 ms at 64^3 S12) rather than
// three (3.06) or four (3.11): less shared memory per block leaves more L1 for the
// record, source and neighbour loads, at the cost of more padding lanes
constexpr int kSlots = 2;
constexpr int kSlotsUpdate = 4;    // staged cell tables per warp and round (residual update)
constexpr int kSlotsDF = 2;        // staged cell tables per warp and round (residual)
constexpr int kWaitLimit = 1 << 20;
constexpr int kMaxUnits = 64;      // units per cell the schedule setup handles

__host__ __device__ inline long long fused_index(int ne, int Nw, int N, int g, int e, int a) {
    return (((long long)g * ne + e) * Nw + a) * N;
}

// local DOF i's position in the DOF list of face k, or -1
constexpr int face_pos(int dim, int p, int k, int i) {
    const int nf = fpow(p + 1, dim - 1);
    for (int q = 0; q < nf; ++q)
        if (face_dof(dim, p, k, q) == i) return q;
    return -1;
}

// ---------------------------------------------------------------- mbarrier / bulk copy
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// orders this warp's earlier shared-memory reads before a bulk copy that overwrites them
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for one phase of a copy barrier.  On giving up it records
// kErrTimeout and waits once more (bounded) so that no copy into this warp's
// shared memory is still in flight when the thread goes on.
__device__ __forceinline__ void wait_copy(unsigned long long* bar, unsigned parity, int* status) {
    for (int i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return;
    atomicOr(status, kErrTimeout);
    for (int i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return;
}

// Runs of equal keys among the warp's valid lanes (valid lanes are a prefix):
// this lane's run index; `start` on the first lane of a run.  Initialises the
// warp's SLOTS copy barriers and issues the copies of round 0 (runs 0..SLOTS-1).
template <int SLOTS>
__device__ __forceinline__ int stage_runs(float* wtab, unsigned long long* wbar, const float* gtab, int tab_floats,
                                          bool valid, int key, int cell, bool& start) {
    const int lane = threadIdx.x & 31;
    if (lane < SLOTS) mbar_init(&wbar[lane], 1);
    fence_mbar_init();
    __syncwarp();
    const int prev = __shfl_up_sync(0xffffffffu, key, 1);
    start = valid && (lane == 0 || prev != key);
    const unsigned starts = __ballot_sync(0xffffffffu, start);
    const int run = __popc(starts & (0xffffffffu >> (31 - lane))) - 1;
    if (start && run < SLOTS) {
        const unsigned bytes = (unsigned)tab_floats * 4u;
        mbar_expect_tx(&wbar[run], bytes);
        bulk_g2s(wtab + run * tab_floats, gtab + (size_t)cell * tab_floats, bytes, &wbar[run]);
    }
    return run;
}

// Calls body(shared-window byte address of the lane's table) on every valid
// lane, SLOTS runs per round: round 0's copies come from stage_runs, later
// rounds reuse the slots (the barrier of a slot completes phase r in round r).
// Warp-uniform control flow around the body; the body itself must not use
// warp-collective operations.
template <int SLOTS, typename Body>
__device__ __forceinline__ void for_each_round(float* wtab, unsigned long long* wbar, const float* gtab, int tab_floats,
                                               bool valid, int run, bool start, int cell, int* status, Body&& body) {
    const unsigned bytes = (unsigned)tab_floats * 4u;
    for (int round = 0;; ++round) {
        const int rbase = round * SLOTS;
        const bool mine = valid && run >= rbase && run < rbase + SLOTS;
        if (round > 0 && start && mine) {
            fence_proxy_async();
            mbar_expect_tx(&wbar[run - rbase], bytes);
            bulk_g2s(wtab + (run - rbase) * tab_floats, gtab + (size_t)cell * tab_floats, bytes, &wbar[run - rbase]);
        }
        if (mine) {
            wait_copy(&wbar[run - rbase], (unsigned)(round & 1), status);
            body(smem_u32(wtab + (run - rbase) * tab_floats));
        }
        if (!__any_sync(0xffffffffu, valid && run >= rbase + SLOTS)) break;
        __syncwarp();
    }
}

// Compile-time loop: f(std::integral_constant<int, i>) for i in [B, E), so that
// every index into the register-resident local system is a constant.
template <int B, int E, typename F>
__device__ __forceinline__ void sfor(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        sfor<B + 1, E>(f);
    }
}

// ---------------------------------------------------------------- packed FP32 helpers
__device__ __forceinline__ float2 f2(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b with one rounding (b * -1 is exact)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// element j of a row stored as float2 pairs (j a compile-time constant)
template <int NP>
__device__ __forceinline__ float get(const float2 (&row)[NP], int j) {
    return (j & 1) ? row[j >> 1].y : row[j >> 1].x;
}

template <int N>
__device__ __forceinline__ void ld_vec(const float* p, float (&r)[N]) {
    if constexpr (N % 4 == 0) {
#pragma unroll
        for (int c = 0; c < N / 4; ++c) {
            const float4 v = reinterpret_cast<const float4*>(p)[c];
            r[4 * c] = v.x; r[4 * c + 1] = v.y; r[4 * c + 2] = v.z; r[4 * c + 3] = v.w;
        }
    } else if constexpr (N == 2) {
        const float2 v = *reinterpret_cast<const float2*>(p);
        r[0] = v.x; r[1] = v.y;
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) r[i] = p[i];
    }
}

template <int N>
__device__ __forceinline__ void st_vec(float* p, const float (&r)[N]) {
    if constexpr (N % 4 == 0) {
#pragma unroll
        for (int c = 0; c < N / 4; ++c)
            reinterpret_cast<float4*>(p)[c] = make_float4(r[4 * c], r[4 * c + 1], r[4 * c + 2], r[4 * c + 3]);
    } else if constexpr (N == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(r[0], r[1]);
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) p[i] = r[i];
    }
}

// the same through the L2 only (data written by other SMs in an earlier launch)
template <int N>
__device__ __forceinline__ void ld_vec_cg(const float* p, float (&r)[N]) {
    if constexpr (N % 4 == 0) {
#pragma unroll
        for (int c = 0; c < N / 4; ++c) {
            const float4 v = __ldcg(reinterpret_cast<const float4*>(p) + c);
            r[4 * c] = v.x; r[4 * c + 1] = v.y; r[4 * c + 2] = v.z; r[4 * c + 3] = v.w;
        }
    } else if constexpr (N == 2) {
        const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
        r[0] = v.x; r[1] = v.y;
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) r[i] = __ldcg(p + i);
    }
}

// explicit shared-memory loads at a shared-window byte address (cell tables
// staged by cp.async.bulk): always LDS, whatever the compiler infers about a pointer
__device__ __forceinline__ float4 lds4(unsigned a) {
    float4 v;
    asm("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
    return v;
}
__device__ __forceinline__ float2 lds2(unsigned a) {
    float2 v;
    asm("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}
__device__ __forceinline__ float lds1(unsigned a) {
    float v;
    asm("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}

// a row of n floats at shared address a (16-byte aligned) as float2 pairs
template <int N>
__device__ __forceinline__ void lds_row(unsigned a, float2 (&r)[(N + 1) / 2]) {
    if constexpr (N % 4 == 0) {
#pragma unroll
        for (int c = 0; c < N / 4; ++c) {
            const float4 v = lds4(a + 16u * c);
            r[2 * c] = make_float2(v.x, v.y);
            r[2 * c + 1] = make_float2(v.z, v.w);
        }
    } else if constexpr (N == 2) {
        r[0] = lds2(a);
    } else {
        r[0] = make_float2(lds1(a), 0.f);
    }
}

template <int N>
__device__ __forceinline__ void lds_vec(unsigned a, float (&r)[N]) {
    if constexpr (N % 4 == 0) {
#pragma unroll
        for (int c = 0; c < N / 4; ++c) {
            const float4 v = lds4(a + 16u * c);
            r[4 * c] = v.x; r[4 * c + 1] = v.y; r[4 * c + 2] = v.z; r[4 * c + 3] = v.w;
        }
    } else if constexpr (N == 2) {
        const float2 v = lds2(a);
        r[0] = v.x; r[1] = v.y;
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) r[i] = lds1(a + 4u * i);
    }
}

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// programmatic dependent launch: let the next launch in the stream start its
// blocks now / wait here until the previous launch has finished and its writes
// are visible (no-ops for launches without the programmatic attribute)
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ---------------------------------------------------------------- double-float helpers
// A value hi + lo with |lo| <= ulp(hi)/2 after dd_norm.  Error-free transforms
// use the _rn intrinsics, which the compiler never contracts into FMAs.
struct dd {
    float hi, lo;
};

// a * b to about 2^-46 relative (exact product of the high parts plus both
// cross terms), not normalised
__device__ __forceinline__ dd dd_prod(dd a, dd b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return {p, e};
}

// s += p: TwoSum of the high parts, low parts and the rounding error summed
__device__ __forceinline__ void dd_acc(dd& s, dd p) {
    const float t = __fadd_rn(s.hi, p.hi);
    const float bv = __fsub_rn(t, s.hi);
    const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, bv)), __fsub_rn(p.hi, bv));
    s.hi = t;
    s.lo = __fadd_rn(s.lo, __fadd_rn(err, p.lo));
}

__device__ __forceinline__ dd dd_norm(dd s) {
    const float h = __fadd_rn(s.hi, s.lo);
    return {h, __fsub_rn(s.lo, __fsub_rn(h, s.hi))};
}

// two double-float numbers (rows i, i + 1) in packed registers
struct dd2 {
    float2 hi, lo;
};

// a (two rows) times a broadcast scalar b
__device__ __forceinline__ dd2 dd2_prod(dd2 a, dd b) {
    const float2 bh = f2(b.hi);
    const float2 p = mul2(a.hi, bh);
    float2 e = fma2(a.hi, bh, make_float2(-p.x, -p.y));
    e = fma2(a.hi, f2(b.lo), e);
    e = fma2(a.lo, bh, e);
    return {p, e};
}

__device__ __forceinline__ void dd2_acc(dd2& s, dd2 p) {
    const float2 t = add2(s.hi, p.hi);
    const float2 bv = sub2(t, s.hi);
    const float2 err = add2(sub2(s.hi, sub2(t, bv)), sub2(p.hi, bv));
    s.hi = t;
    s.lo = add2(s.lo, add2(err, p.lo));
}

__device__ __forceinline__ dd2 dd2_norm(dd2 s) {
    const float2 h = add2(s.hi, s.lo);
    return {h, sub2(s.lo, sub2(h, s.hi))};
}

__device__ __forceinline__ dd dd_half(const dd2& v, int which) {
    return which ? dd{v.hi.y, v.lo.y} : dd{v.hi.x, v.lo.x};
}

}  // namespace

// ---------------------------------------------------------------- state of the fused path
struct FusedState {
    int2* nodes = nullptr;           // [ne * Nw] fused order: {e, a | pattern << 16}
    int* nbr = nullptr;              // [ne][2 dim] 2 * neighbour + (face DOF map is the standard one)
    unsigned* map = nullptr;         // [ne][2 dim] neighbour DOF of each face DOF, 8 bits each
    float4* omega = nullptr;         // [Nw] FP32 directions
    float* w = nullptr;              // [Nw] FP32 weights
    float* tab = nullptr;            // [ne][Tab::size]
    int tab_td = -1;                 // time mass included in tab (-1: not built)
    // per-unit tables for the sweep: the cell's table with G_d replaced by
    // B_d = G_d + sum over the unit's outflow faces k of n_{k,d} F_k
    float* utab = nullptr;           // [nunits][Tab::size]
    int utab_td = -1;
    int nunits = 0;
    int* unit_cell = nullptr;        // [nunits] cell of each unit
    int* unit_pat = nullptr;         // [nunits] face pattern of each unit
    int* rec_unit = nullptr;         // [records] unit of each record (-1 on padding)
    float* dtab = nullptr;           // [ne][DTab::size]
    int dtab_td = -1;
    float2* ddots = nullptr;         // [nfaces][Nw] double-float Omega . n
    float2* domega = nullptr;        // [Nw][dim] double-float directions
    float2* dw = nullptr;            // [Nw] double-float weights
    float2* dsigma = nullptr;        // [G][ne] double-float sigma_t (refreshed per residual)
    int pdl = 1;                     // programmatic dependent launch between level launches
    // the fused sweep's own wavefront levels over the node records
    int num_levels = 0;
    std::vector<int> level_offsets;  // [num_levels + 1]
    bool unit_levels = false;        // levels of (cell, octant, face pattern) units, not of single nodes
    struct Graph {
        const void* key[7] = {};
        cudaGraphExec_t exec = nullptr;
    };
    static constexpr int kGraphs = 16;
    Graph graphs[kGraphs];
    int next = 0;
};

namespace {

// ---------------------------------------------------------------- setup kernels
// node record {e, a | pattern << 16}; the face codes of the level order:
// 1 outflow, 2 inflow from a neighbour, 3 reflective inflow, 0 none (inflow
// boundary, or Omega.n = 0)
__device__ inline int face_pattern(int e, int a, int Nw, int nface, const double* __restrict__ dots,
                                   const Slot* __restrict__ slots, int* ninflow) {
    int pat = 0, c = 0;
    for (int k = 0; k < nface; ++k) {
        const Slot s = slots[(size_t)e * nface + k];
        const double d1 = dots[(size_t)s.face * Nw + a];
        const double dk = s.side ? -d1 : d1;
        const int code = dk > 0.0 ? 1 : (dk < 0.0 ? (s.nbr >= 0 ? 2 : (s.nbr <= -2 ? 3 : 0)) : 0);
        pat |= code << (2 * k);
        c += code == 2;
    }
    if (ninflow) *ninflow = c;
    return pat;
}

__global__ void k_fused_nodes(long long n, int Nw, int dim, const double* __restrict__ dots,
                              const Slot* __restrict__ slots, int2* __restrict__ out) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int e = (int)(v / Nw), a = (int)(v % Nw);
    out[v] = make_int2(e, a | (face_pattern(e, a, Nw, 2 * dim, dots, slots, nullptr) << 16));
}

// sort key of a record: (level, cell, face pattern); the sort is stable, so
// each (cell, pattern) keeps its angles in order.  level_of is indexed by unit
// (unit_of_node given) or by node e Nw + a.
// sort key of a node record: (level, unit); units are numbered cell by cell, so
// a level's records come out grouped by cell, then unit, then (stable) angle
// key = level (bits 36 and up) | face pattern (bits ubits..35, when ubits < 36) | unit:
// within a level the units of one face pattern are adjacent, so the units that
// share a warp fold the same inflow faces (no divergence in the fold)
__global__ void k_fused_keys(long long n, int Nw, const int2* __restrict__ recs, const int* __restrict__ level_of,
                             bool unit_levels, const int* __restrict__ unit_of_node, int ubits,
                             unsigned long long* __restrict__ keys) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int2 r = recs[t];
    const int a = r.y & 0xffff;
    const long long v = (long long)r.x * Nw + a;
    const int u = unit_of_node[v];
    const int lev = unit_levels ? level_of[u] : level_of[v];
    const unsigned long long pat = ubits < 36 ? (unsigned long long)((unsigned)r.y >> 16) << ubits : 0ull;
    keys[t] = ((unsigned long long)lev << 36) | pat | (unsigned long long)(unsigned)u;
}

// cell and face pattern of every unit (all nodes of a unit share both)
__global__ void k_unit_info(long long n, int Nw, const int2* __restrict__ recs, const int* __restrict__ unit_of_node,
                            int* __restrict__ unit_cell, int* __restrict__ unit_pat) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int u = unit_of_node[v];
    unit_cell[u] = recs[v].x;
    unit_pat[u] = (int)((unsigned)recs[v].y >> 16);
}

// per-unit table: the cell's table with each G_d row replaced by
// B_d = G_d + sum_{outflow faces k} n_{k,d} F_k (F_k at the face's DOFs), so that
// A = sum_d Omega_d B_d + sigma M [+ tau Mt] for every angle of the unit
template <int D, int P, bool TD>
__global__ void k_unit_tab(int nu, const int* __restrict__ unit_cell, const int* __restrict__ unit_pat,
                           const float* __restrict__ tab, float* __restrict__ utab) {
    using S = Shape<D, P>;
    using T = Tab<D, P, TD>;
    constexpr int N = S::N, NF = S::NF, NFACE = S::NFACE;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nu * T::size) return;
    const int u = (int)(t / T::size), o = (int)(t % T::size);
    const float* ct = tab + (size_t)unit_cell[u] * T::size;
    float v = ct[o];
    if (o < T::oM) {
        const int d = o / (N * N), i = (o / N) % N, j = o % N;
        const int pat = unit_pat[u];
        for (int k = 0; k < NFACE; ++k) {
            if (((pat >> (2 * k)) & 3) != 1) continue;
            const int ii = face_pos(D, P, k, i), jj = face_pos(D, P, k, j);
            if (ii < 0 || jj < 0) continue;
            v = fmaf(ct[T::oNrm + 4 * k + d], ct[T::oF + (k * NF + ii) * NF + jj], v);
        }
    }
    utab[t] = v;
}

// first record of each level in the sorted keys (level in bits 36 and up)
__global__ void k_level_starts(int nlev, const unsigned long long* __restrict__ keys, long long n,
                               long long* __restrict__ starts) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l > nlev) return;
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) / 2;
        if ((long long)(keys[mid] >> 36) < l) lo = mid + 1; else hi = mid;
    }
    starts[l] = lo;
}

// ---- unit schedule
// per node: unit key (octant << 12 | pattern) and the number of upwind node edges
__global__ void k_unit_keys(long long n, int Nw, int dim, const double* __restrict__ omega,
                            const double* __restrict__ dots, const Slot* __restrict__ slots, int* __restrict__ key,
                            int* __restrict__ nin) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int e = (int)(v / Nw), a = (int)(v % Nw);
    int c = 0, oct = 0;
    const int pat = face_pattern(e, a, Nw, 2 * dim, dots, slots, &c);
    for (int d = 0; d < dim; ++d) oct |= (omega[a * dim + d] > 0.0) << d;
    key[v] = (oct << 12) | pat;
    nin[v] = c;
}

// per cell: local unit index of each angle (first-seen order of its key) and the
// cell's unit count; sets *overflow when a cell has more than kMaxUnits units
__global__ void k_unit_local(int ne, int Nw, const int* __restrict__ key, int* __restrict__ local,
                             int* __restrict__ count, int* __restrict__ overflow) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int seen[kMaxUnits];
    int nu = 0;
    for (int a = 0; a < Nw; ++a) {
        const int k = key[(long long)e * Nw + a];
        int u = -1;
        for (int j = 0; j < nu; ++j)
            if (seen[j] == k) { u = j; break; }
        if (u < 0) {
            if (nu == kMaxUnits) {
                atomicOr(overflow, 1);
                count[e] = 0;
                return;
            }
            seen[nu] = k;
            u = nu++;
        }
        local[(long long)e * Nw + a] = u;
    }
    count[e] = nu;
}

// local unit index -> unit id; per unit: pending upwind edges and node count
__global__ void k_unit_ids(long long n, int Nw, const int* __restrict__ base, const int* __restrict__ nin,
                           int* __restrict__ unit, int* __restrict__ pending, int* __restrict__ usize) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int u = base[v / Nw] + unit[v];
    unit[v] = u;
    if (nin[v]) atomicAdd(&pending[u], nin[v]);
    atomicAdd(&usize[u], 1);
}

__global__ void k_unit_fill(long long n, const int* __restrict__ unit, const int* __restrict__ ustart,
                            int* __restrict__ ufill, int* __restrict__ unodes) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int u = unit[v];
    unodes[ustart[u] + atomicAdd(&ufill[u], 1)] = (int)v;
}

__global__ void k_unit_frontier0(int nu, const int* __restrict__ pending, int* __restrict__ front,
                                 int* __restrict__ fcount) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u < nu && pending[u] == 0) front[atomicAdd(fcount, 1)] = u;
}

// one Kahn frontier of the unit graph: every outflow edge of the frontier's
// nodes releases one pending edge of the downstream unit
__global__ void k_unit_kahn(int Nw, int dim, const int* __restrict__ key, const Slot* __restrict__ slots,
                            const int* __restrict__ unit, const int* __restrict__ ustart, const int* __restrict__ usize,
                            const int* __restrict__ unodes, int* __restrict__ pending, int* __restrict__ ulevel,
                            const int* __restrict__ cur, int ncur, int* __restrict__ next, int* __restrict__ ncount,
                            int lev) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncur) return;
    const int u = cur[t];
    ulevel[u] = lev;
    const int nface = 2 * dim;
    for (int i = 0; i < usize[u]; ++i) {
        const int v = unodes[ustart[u] + i];
        const int e = v / Nw, a = v - e * Nw;
        const int pat = key[v] & 0xfff;
        for (int k = 0; k < nface; ++k) {
            if (((pat >> (2 * k)) & 3) != 1) continue;
            const int nb = slots[(size_t)e * nface + k].nbr;
            if (nb < 0) continue;
            const int u2 = unit[(long long)nb * Nw + a];
            if (atomicSub(&pending[u2], 1) == 1) next[atomicAdd(ncount, 1)] = u2;
        }
    }
}

// Packing of a level's records into warps of 32 lanes that hold at most
// kSlots units (tables) each: a unit's run of records that would be a warp's
// kSlots+1-th starts the next warp instead, and each level is padded to whole
// warps with records {-1, 0}.  Runs (records of one unit within one level,
// consecutive after the sort) are found in parallel; the greedy placement walks
// a level's runs in one thread; the records are then scattered in parallel.
__global__ void k_run_flags(long long n, const unsigned long long* __restrict__ keys, int* __restrict__ flag) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;   // a run: one unit within one level
}

// run_start[r] = first record of run r (flag[i] == 1, ridx[i] its exclusive scan)
__global__ void k_run_starts(long long n, const int* __restrict__ flag, const int* __restrict__ ridx,
                             int* __restrict__ run_start) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) run_start[ridx[i]] = (int)i;
}

// one thread per level: padded position of each of its runs, padded level size
__global__ void k_pack_runs(int nlev, long long n, int nruns, const long long* __restrict__ starts,
                            const int* __restrict__ ridx, const int* __restrict__ run_start, int* __restrict__ run_pos,
                            long long* __restrict__ sizes) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nlev) return;
    if (starts[l] == starts[l + 1]) {
        sizes[l] = 0;
        return;
    }
    const int r0 = ridx[starts[l]];
    const int r1 = starts[l + 1] < n ? ridx[starts[l + 1]] : nruns;
    long long pos = 0;
    int cells = 0;   // runs (units) touching the warp that holds lane pos
    for (int r = r0; r < r1; ++r) {
        const long long len = (long long)(r + 1 < nruns ? run_start[r + 1] : n) - run_start[r];
        if ((pos & 31) == 0) cells = 0;
        if (cells == kSlots) {
            pos = (pos + 31) & ~31LL;
            cells = 0;
        }
        run_pos[r] = (int)pos;
        cells = ((pos + len - 1) >> 5) == (pos >> 5) ? cells + 1 : 1;
        pos += len;
    }
    sizes[l] = (pos + 31) & ~31LL;
}

__global__ void k_pack_fill(long long n, int2* __restrict__ out, int* __restrict__ out_unit) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = make_int2(-1, 0);
    out_unit[i] = -1;
}

__global__ void k_pack_scatter(long long n, const unsigned long long* __restrict__ keys, const int2* __restrict__ recs,
                               const int* __restrict__ ridx, const int* __restrict__ flag,
                               const int* __restrict__ run_start, const int* __restrict__ run_pos,
                               const long long* __restrict__ out_starts, unsigned long long umask,
                               int2* __restrict__ out, int* __restrict__ out_unit) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = ridx[i] + flag[i] - 1;   // run of record i (inclusive scan - 1)
    const int l = (int)(keys[i] >> 36);
    const long long o = out_starts[l] + run_pos[r] + (i - run_start[r]);
    out[o] = recs[i];
    out_unit[o] = (int)(keys[i] & umask);
}

__global__ void k_fused_cells(int ne, int dim, int p, int nf, const Slot* __restrict__ slots,
                              const uint8_t* __restrict__ nbrmap, int* __restrict__ nbr, unsigned* __restrict__ map) {
    const int nface = 2 * dim;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ne * nface) return;
    const int k = t % nface;
    unsigned m = 0;
    bool standard = true;   // the neighbour's face DOFs in the order of face k^1's
    for (int j = 0; j < nf && j < 4; ++j) {
        const int v = nbrmap[(size_t)t * nf + j];
        m |= (unsigned)v << (8 * j);
        standard = standard && (v == face_dof(dim, p, k ^ 1, j));
    }
    map[t] = m;
    const int nb = slots[t].nbr;
    nbr[t] = nb >= 0 ? 2 * nb + (standard ? 1 : 0) : nb;
}

__global__ void k_fused_angles(int Nw, int dim, const double* __restrict__ omega, const double* __restrict__ w,
                               float4* __restrict__ om4, float* __restrict__ w32, float2* __restrict__ dom,
                               float2* __restrict__ dw) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= Nw) return;
    float v[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < dim; ++d) {
        const double x = omega[a * dim + d];
        v[d] = (float)x;
        dom[a * dim + d] = make_float2(v[d], (float)(x - (double)v[d]));
    }
    om4[a] = make_float4(v[0], v[1], v[2], 0.f);
    const float wh = (float)w[a];
    w32[a] = wh;
    dw[a] = make_float2(wh, (float)(w[a] - (double)wh));
}

template <int D, int P, bool TD>
__global__ void k_fused_tab(int ne, const double* __restrict__ Gm, const double* __restrict__ M,
                            const double* __restrict__ Mt, const double* __restrict__ F, const Slot* __restrict__ slots,
                            const double* __restrict__ normals, float* __restrict__ tab) {
    using S = Shape<D, P>;
    using T = Tab<D, P, TD>;
    constexpr int N = S::N, NF = S::NF, NFACE = S::NFACE;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ne * T::size) return;
    const int e = (int)(t / T::size), o = (int)(t % T::size);
    float v = 0.f;
    if (o < T::oM) v = (float)Gm[(size_t)e * D * N * N + o];
    else if (o < T::oMt) v = (float)M[(size_t)e * N * N + (o - T::oM)];
    else if (o < T::oF) v = (float)Mt[(size_t)e * N * N + (o - T::oMt)];
    else if (o < T::oF + NFACE * NF * NF) v = (float)F[(size_t)e * NFACE * NF * NF + (o - T::oF)];
    else if (o >= T::oNrm && (o - T::oNrm) % 4 < D) {
        const int k = (o - T::oNrm) / 4, d = (o - T::oNrm) % 4;
        const Slot s = slots[(size_t)e * NFACE + k];
        const double x = normals[(size_t)s.face * D + d];
        v = (float)(s.side ? -x : x);
    }
    tab[t] = v;
}

template <int D, int P, bool TD>
__global__ void k_df_tab(int ne, const double* __restrict__ Gm, const double* __restrict__ M,
                         const double* __restrict__ Mt, const double* __restrict__ F, float* __restrict__ tab) {
    using S = Shape<D, P>;
    using T = DTab<D, P, TD>;
    constexpr int N = S::N, NF = S::NF, NFACE = S::NFACE;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ne * T::half) return;
    const int e = (int)(t / T::half), o = (int)(t % T::half);
    double x = 0.0;
    if (o < T::oF) {
        // column j of volume matrix v, row i: [j][v][i]
        const int j = o / (T::NV * N), v = (o / N) % T::NV, i = o % N;
        const int rc = i * N + j;
        if (v < D) x = Gm[(size_t)e * D * N * N + v * N * N + rc];
        else if (v == D) x = M[(size_t)e * N * N + rc];
        else x = Mt[(size_t)e * N * N + rc];
    } else if (o < T::oF + NFACE * NF * NF) {
        x = F[(size_t)e * NFACE * NF * NF + (o - T::oF)];
    }
    const float hi = (float)x;
    tab[(size_t)e * T::size + o] = hi;
    tab[(size_t)e * T::size + T::half + o] = (float)(x - (double)hi);
}

__global__ void k_df_split(long long n, const double* __restrict__ x, float2* __restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double v = x[t];
    const float hi = (float)v;
    out[t] = make_float2(hi, (float)(v - (double)hi));
}

// ---------------------------------------------------------------- isotropic source
// s[g][e][i] = (sigma_s[g][e] (Mt phi_{g,e})_i) / sum(w) + q_iso[g][e N + i] in FP64
// (the same expression and order as the node-major scattering source), stored
// as FP32 and/or as a double-float pair.
__global__ void k_iso_source(int ne, int G, int N, double wsum, const double* __restrict__ Mt,
                             const double* __restrict__ sigma_s, const double* __restrict__ phi,
                             const double* __restrict__ q_iso, float* __restrict__ out, float* __restrict__ out_hi,
                             float* __restrict__ out_lo) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long ndof = (long long)ne * N;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    const int e = (int)(s / N), i = (int)(s % N);
    double v = 0.0;
    if (phi) {
        const double* Mr = Mt + (size_t)e * N * N + (size_t)i * N;
        const double* ph = phi + ndof * g + (long long)e * N;
        double acc = 0.0;
        for (int j = 0; j < N; ++j) acc += Mr[j] * ph[j];
        v = (sigma_s[(size_t)g * ne + e] * acc) / wsum;
    }
    if (q_iso) v += q_iso[t];
    const float hi = (float)v;
    if (out) out[t] = hi;
    if (out_hi) {
        out_hi[t] = hi;
        out_lo[t] = (float)(v - (double)hi);
    }
}

// ---------------------------------------------------------------- fused sweep
struct FusedArgs {
    int ne, Nw, G;
    const int2* nodes;
    const int* rec_unit;     // unit of each record
    int nunits;
    const float* tab;        // per-unit tables
    const int* nbr;
    const unsigned* map;
    const float4* omega;
    const float* sigma;      // [G][ne]
    float tau;
    const float* iso;        // [G][ne][N] or null
    const float* src;        // fused-layout psi-sized source or null
    float* psi;              // fused layout
    float* acc_hi;           // fused layout double-float accumulator (+= psi) or null
    float* acc_lo;
    int* status;
};

template <int D, int P, bool TD>
__global__ void __launch_bounds__(kSweepBlock, kSweepMinBlocks) k_fused_level(FusedArgs f, int base, int count) {
    using S = Shape<D, P>;
    using T = Tab<D, P, TD>;
    constexpr int N = S::N, NF = S::NF, NFACE = S::NFACE;
    constexpr int NP = (N + 1) / 2;
    __shared__ __align__(128) float s_tab[kSweepWarps * kSlots * T::size];
    __shared__ __align__(8) unsigned long long s_bar[kSweepWarps * kSlots];
    griddep_launch_dependents();
    const int warp = threadIdx.x >> 5;
    const long long total = (long long)count * f.G;
    const long long t = (long long)blockIdx.x * kSweepBlock + threadIdx.x;
    bool valid = false;
    int g = 0, e = 0, a = 0, pat = 0, u = 0;
    if (t < total) {
        g = (int)(t / count);
        const int ni = (int)(t - (long long)g * count);
        const int2 r = f.nodes[base + ni];
        valid = r.x >= 0;            // padding records close a warp early
        e = valid ? r.x : 0;
        a = r.y & 0xffff;
        pat = (int)((unsigned)r.y >> 16);
        u = valid ? f.rec_unit[base + ni] : 0;
    }
    float* wtab = s_tab + warp * kSlots * T::size;
    unsigned long long* wbar = s_bar + warp * kSlots;
    bool start = false;
    const int run = stage_runs<kSlots>(wtab, wbar, f.tab, T::size, valid, g * f.nunits + u, u, start);

    // loads that do not depend on the previous levels
    float b[N];
#pragma unroll
    for (int i = 0; i < N; ++i) b[i] = 0.f;
    float4 om = make_float4(0.f, 0.f, 0.f, 0.f);
    float sg = 0.f;
    int nb[NFACE];
    const long long idx = fused_index(f.ne, f.Nw, N, g, e, a);
    if (valid) {
        if (f.iso) ld_vec<N>(f.iso + ((long long)g * f.ne + e) * N, b);
        if (f.src) {
            float s[N];
            ld_vec<N>(f.src + idx, s);
#pragma unroll
            for (int i = 0; i < N; ++i) b[i] += s[i];
        }
        om = f.omega[a];
        sg = f.sigma[(size_t)g * f.ne + e];
#pragma unroll
        for (int k = 0; k < NFACE; ++k)
            if (((pat >> (2 * k)) & 3) == 2) nb[k] = f.nbr[(size_t)e * NFACE + k];
    }
    // the upwind traces were written by earlier levels: after the wait, fold each
    // inflow face's term |Omega.n| F_k u_k into b as its trace arrives, the face
    // block and normal read from the unit's staged table.  The schedule packs at
    // most kSlots units into a warp, so every table of the warp was staged by
    // stage_runs.
    griddep_wait();
    const bool staged = valid && run < kSlots;
    if (valid && !staged) atomicOr(f.status, kErrSchedule);
    unsigned tb = 0;
    if (staged) {
        wait_copy(&wbar[run], 0u, f.status);
        tb = smem_u32(wtab + run * T::size);
        sfor<0, NFACE>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            if (((pat >> (2 * k)) & 3) == 2) {
                float u[NF];
                const float* up = f.psi + fused_index(f.ne, f.Nw, N, g, nb[k] >> 1, a);
                if (nb[k] & 1) {
                    // standard DOF map: the neighbour's face k^1 DOFs, picked at compile time
                    float blk[N];
                    ld_vec_cg<N>(up, blk);
                    sfor<0, NF>([&](auto jc) {
                        constexpr int jj = decltype(jc)::value;
                        u[jj] = blk[face_dof(D, P, k ^ 1, jj)];
                    });
                } else {
                    const unsigned m4 = f.map[(size_t)e * NFACE + k];
#pragma unroll
                    for (int jj = 0; jj < NF; ++jj) u[jj] = __ldcg(up + ((m4 >> (8 * jj)) & 0xffu));
                }
                const float4 nr = lds4(tb + 4u * (T::oNrm + 4 * k));
                float d = om.x * nr.x;
                if (D > 1) d = fmaf(om.y, nr.y, d);
                if (D > 2) d = fmaf(om.z, nr.z, d);
                d = fabsf(d);
                sfor<0, NF>([&](auto ic) {
                    constexpr int ii = decltype(ic)::value;
                    float fr[NF];
                    lds_vec<NF>(tb + 4u * (T::oF + (k * NF + ii) * NF), fr);
                    float acc = 0.f;
#pragma unroll
                    for (int jj = 0; jj < NF; ++jj) acc = fmaf(fr[jj], u[jj], acc);
                    constexpr int fi = face_dof(D, P, k, ii);
                    b[fi] = fmaf(d, acc, b[fi]);
                });
            }
        });
    }

    if (staged) {
        const float omv[3] = {om.x, om.y, om.z};
        // rows of A = sum_d Omega_d B_d + sigma M [+ tau Mt], B_d = G_d + sum_{outflow k}
        // n_{k,d} F_k from the unit's table (on an outflow face Omega.n = |Omega.n|),
        // assembled one at a time, eliminated against the rows above (no pivoting)
        // and scaled by their pivot's reciprocal: only the strict upper triangle of
        // the unit-diagonal U (and the scaled right-hand side) stays live
        float2 U[N][NP] = {};
        bool ok = true;
        sfor<0, N>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            float2 ar[NP], tr[NP];
            lds_row<N>(tb + 4u * (T::oG + i * N), tr);
#pragma unroll
            for (int p = 0; p < NP; ++p) ar[p] = mul2(f2(omv[0]), tr[p]);
#pragma unroll
            for (int d = 1; d < D; ++d) {
                lds_row<N>(tb + 4u * (T::oG + d * N * N + i * N), tr);
#pragma unroll
                for (int p = 0; p < NP; ++p) ar[p] = fma2(f2(omv[d]), tr[p], ar[p]);
            }
            lds_row<N>(tb + 4u * (T::oM + i * N), tr);
#pragma unroll
            for (int p = 0; p < NP; ++p) ar[p] = fma2(f2(sg), tr[p], ar[p]);
            if constexpr (TD) {
                lds_row<N>(tb + 4u * (T::oMt + i * N), tr);
#pragma unroll
                for (int p = 0; p < NP; ++p) ar[p] = fma2(f2(f.tau), tr[p], ar[p]);
            }
            float y = b[i];
            sfor<0, i>([&](auto mc) {
                constexpr int m = decltype(mc)::value;
                const float l = get(ar, m);
                sfor<(m + 1) / 2, NP>([&](auto pc) {
                    constexpr int p = decltype(pc)::value;
                    ar[p] = fma2(f2(-l), U[m][p], ar[p]);
                });
                y = fmaf(-l, b[m], y);
            });
            const float piv = get(ar, i);
            ok = ok && (piv != 0.f);
            const float r = rcp_approx(piv);
            b[i] = y * r;
            sfor<(i + 1) / 2, NP>([&](auto pc) {
                constexpr int p = decltype(pc)::value;
                U[i][p] = mul2(f2(r), ar[p]);
            });
        });
        float x[N] = {};
        sfor<0, N>([&](auto kc) {
            constexpr int k = N - 1 - decltype(kc)::value;
            float v = b[k];
            sfor<k + 1, N>([&](auto jc) {
                constexpr int j = decltype(jc)::value;
                v = fmaf(-get(U[k], j), x[j], v);
            });
            x[k] = v;
        });
        if (!ok) atomicOr(f.status, kErrSingular);
        st_vec<N>(f.psi + idx, x);
        if (f.acc_hi) {
            // (hi, lo) += x: TwoSum into hi, the rounding error into lo
            float h[N], l[N];
            ld_vec<N>(f.acc_hi + idx, h);
            ld_vec<N>(f.acc_lo + idx, l);
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const float s = __fadd_rn(h[i], x[i]);
                const float bv = __fsub_rn(s, h[i]);
                const float err = __fadd_rn(__fsub_rn(h[i], __fsub_rn(s, bv)), __fsub_rn(x[i], bv));
                h[i] = s;
                l[i] = __fadd_rn(l[i], err);
            }
            st_vec<N>(f.acc_hi + idx, h);
            st_vec<N>(f.acc_lo + idx, l);
        }
    }
}

// ---------------------------------------------------------------- moments
// phi[g][e N + i] (=, or +=) sum_a w_a psi(g, e, a, i) of an FP32 psi, summed in
// double-float arithmetic and written as FP64.  One thread per (group, cell,
// DOF): a warp reads 32 consecutive floats per angle.
__global__ void k_moments_f32(int ne, int Nw, int G, int N, const float2* __restrict__ w, const float* __restrict__ psi,
                              double* __restrict__ phi, int add) {
    griddep_wait();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long ndof = (long long)ne * N;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    const int e = (int)(s / N), i = (int)(s % N);
    const float* p = psi + fused_index(ne, Nw, N, g, e, 0) + i;
    dd acc = {0.f, 0.f};
    for (int a = 0; a < Nw; ++a) {
        const float2 wa = w[a];
        dd_acc(acc, dd_prod({wa.x, wa.y}, {__ldcg(p + (long long)a * N), 0.f}));
    }
    const double v = (double)acc.hi + (double)acc.lo;
    phi[t] = add ? phi[t] + v : v;
}

// The same sum in plain FP32 (about 1e-6 relative), for the inner operator of
// a Krylov solve whose own tolerance is far looser: one FMA per angle instead
// of an error-free product and a TwoSum.
__global__ void k_moments_f32_fast(int ne, int Nw, int G, int N, const float* __restrict__ w,
                                   const float* __restrict__ psi, double* __restrict__ phi) {
    griddep_wait();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long ndof = (long long)ne * N;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    const int e = (int)(s / N), i = (int)(s % N);
    const float* p = psi + fused_index(ne, Nw, N, g, e, 0) + i;
    float acc0 = 0.f, acc1 = 0.f;   // two chains: half the dependent-FMA latency
    int a = 0;
    for (; a + 1 < Nw; a += 2) {
        acc0 = fmaf(w[a], __ldcg(p + (long long)a * N), acc0);
        acc1 = fmaf(w[a + 1], __ldcg(p + (long long)(a + 1) * N), acc1);
    }
    if (a < Nw) acc0 = fmaf(w[a], __ldcg(p + (long long)a * N), acc0);
    phi[t] = (double)(acc0 + acc1);
}

// the same for a double-float psi (DiscreteToMoment::Mult of hi + lo)
__global__ void k_moments_df(int ne, int Nw, int G, int N, const float2* __restrict__ w, const float* __restrict__ hi,
                             const float* __restrict__ lo, double* __restrict__ phi) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long ndof = (long long)ne * N;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    const int e = (int)(s / N), i = (int)(s % N);
    const long long base = fused_index(ne, Nw, N, g, e, 0) + i;
    dd acc = {0.f, 0.f};
    for (int a = 0; a < Nw; ++a) {
        const float2 wa = w[a];
        const long long k = base + (long long)a * N;
        dd_acc(acc, dd_prod({wa.x, wa.y}, {hi[k], lo[k]}));
    }
    phi[t] = (double)acc.hi + (double)acc.lo;
}

// ---------------------------------------------------------------- double-float residual
struct ResidArgs {
    int ne, Nw, G;
    const float* dtab;
    const Slot* slots;
    const int* nbr;          // 2 * neighbour + standard-map bit (FusedState::nbr)
    const uint8_t* nbrmap;
    const float2* ddots;     // [nfaces][Nw]
    const float2* domega;    // [Nw][D]
    const float2* dsigma;    // [G][ne]
    float tau_hi, tau_lo;
    const float* iso_hi;     // [G][ne][N] isotropic part of q + D^T S phi
    const float* iso_lo;
    const float* q_hi;       // fused-layout psi-sized part of q, or null
    const float* q_lo;
    const float* psi_hi;
    const float* psi_lo;
    float* r;
    int* status;
};

// r = q + D^T S phi - L psi for every (group, cell, angle) node, angle fastest.
// Face terms first (each face's trace loaded where it is used), then the
// volume part y += (sum_d Omega_d G_d + sigma M [+ tau Mt]) psi over the
// columns j: a column's matrix entries are combined with Omega, sigma, tau and
// multiplied by psi_j for two rows per packed operation.  Five 128-thread
// blocks per SM (96 registers, a few spilled) run the 64^3 S12 residual in
// 8.7 ms against 10.0 ms at four blocks (118 registers, no spills).
template <int D, int P, bool TD>
__global__ void __launch_bounds__(kFusedBlock, 5) k_residual_df(ResidArgs f) {
    using S = Shape<D, P>;
    using T = DTab<D, P, TD>;
    constexpr int N = S::N, NF = S::NF, NFACE = S::NFACE;
    constexpr int NV = T::NV;
    constexpr int NP = (N + 1) / 2;
    __shared__ __align__(128) float s_tab[kFusedWarps * kSlotsDF * T::size];
    __shared__ __align__(8) unsigned long long s_bar[kFusedWarps * kSlotsDF];
    const int warp = threadIdx.x >> 5;
    const long long total = (long long)f.G * f.ne * f.Nw;
    const long long t = (long long)blockIdx.x * kFusedBlock + threadIdx.x;
    const bool valid = t < total;
    int g = 0, e = 0, a = 0;
    if (valid) {
        a = (int)(t % f.Nw);
        const long long rr = t / f.Nw;
        e = (int)(rr % f.ne);
        g = (int)(rr / f.ne);
    }
    float* wtab = s_tab + warp * kSlotsDF * T::size;
    unsigned long long* wbar = s_bar + warp * kSlotsDF;
    bool start = false;
    const int run = stage_runs<kSlotsDF>(wtab, wbar, f.dtab, T::size, valid, g * f.ne + e, e, start);

    const long long idx = fused_index(f.ne, f.Nw, N, g, e, a);
    dd x[N];
    dd cf[NV];            // Omega_0..Omega_{D-1}, sigma, [tau]
    if (valid) {
        float xh[N], xl[N];
        ld_vec<N>(f.psi_hi + idx, xh);
        ld_vec<N>(f.psi_lo + idx, xl);
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] = {xh[i], xl[i]};
#pragma unroll
        for (int d = 0; d < D; ++d) cf[d] = {f.domega[a * D + d].x, f.domega[a * D + d].y};
        cf[D] = {f.dsigma[(size_t)g * f.ne + e].x, f.dsigma[(size_t)g * f.ne + e].y};
        if constexpr (TD) cf[D + 1] = {f.tau_hi, f.tau_lo};
    }

    for_each_round<kSlotsDF>(wtab, wbar, f.dtab, T::size, valid, run, start, e, f.status, [&](unsigned th) {
        const unsigned tl = th + 4u * T::half;   // low parts
        dd yr[N];
#pragma unroll
        for (int i = 0; i < N; ++i) yr[i] = {0.f, 0.f};
        // outflow faces on the cell's own trace, inflow faces on the upwind trace
        sfor<0, NFACE>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            const Slot q = f.slots[(size_t)e * NFACE + k];
            const float2 d1 = f.ddots[(size_t)q.face * f.Nw + a];
            const dd dk = q.side ? dd{-d1.x, -d1.y} : dd{d1.x, d1.y};
            const int code = dk.hi > 0.f ? 1 : ((dk.hi < 0.f && q.nbr >= 0) ? 2 : 0);
            if (code == 0) return;
            dd u[NF];
            if (code == 1) {
                sfor<0, NF>([&](auto jc) {
                    constexpr int jj = decltype(jc)::value;
                    u[jj] = x[face_dof(D, P, k, jj)];
                });
            } else {
                const int nbv = f.nbr[(size_t)e * NFACE + k];
                const long long up = fused_index(f.ne, f.Nw, N, g, nbv >> 1, a);
                if (nbv & 1) {
                    float bh[N], bl[N];
                    ld_vec<N>(f.psi_hi + up, bh);
                    ld_vec<N>(f.psi_lo + up, bl);
                    sfor<0, NF>([&](auto jc) {
                        constexpr int jj = decltype(jc)::value;
                        constexpr int m = face_dof(D, P, k ^ 1, jj);
                        u[jj] = {bh[m], bl[m]};
                    });
                } else {
                    const uint8_t* map = f.nbrmap + ((size_t)e * NFACE + k) * NF;
#pragma unroll
                    for (int jj = 0; jj < NF; ++jj) {
                        const int m = map[jj];
                        u[jj] = {f.psi_hi[up + m], f.psi_lo[up + m]};
                    }
                }
            }
            sfor<0, NF>([&](auto ic) {
                constexpr int ii = decltype(ic)::value;
                dd fu = {0.f, 0.f};
                sfor<0, NF>([&](auto jc) {
                    constexpr int jj = decltype(jc)::value;
                    constexpr unsigned o = 4u * (T::oF + (k * NF + ii) * NF + jj);
                    dd_acc(fu, dd_prod({lds1(th + o), lds1(tl + o)}, u[jj]));
                });
                constexpr int fi = face_dof(D, P, k, ii);
                dd_acc(yr[fi], dd_prod(dk, dd_norm(fu)));
            });
        });
        // volume part, two rows per packed operation
        dd2 y[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p)
            y[p] = {make_float2(yr[2 * p].hi, 2 * p + 1 < N ? yr[2 * p + 1].hi : 0.f),
                    make_float2(yr[2 * p].lo, 2 * p + 1 < N ? yr[2 * p + 1].lo : 0.f)};
        // a rolled loop over the columns (psi_j re-read from L1): the unrolled
        // double-float body would not fit the instruction cache
#pragma unroll 1
        for (int j = 0; j < N; ++j) {
            const dd xj = {f.psi_hi[idx + j], f.psi_lo[idx + j]};
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                dd2 c = {f2(0.f), f2(0.f)};
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    const unsigned o = 4u * (T::oV + (j * NV + v) * N + 2 * p);
                    const dd2 m = {lds2(th + o), lds2(tl + o)};
                    dd2_acc(c, dd2_prod(m, cf[v]));
                }
                dd2_acc(y[p], dd2_prod(dd2_norm(c), xj));
            }
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            yr[2 * p] = dd_half(y[p], 0);
            if (2 * p + 1 < N) yr[2 * p + 1] = dd_half(y[p], 1);
        }
        // r = iso (+ q) - y
        const long long ci = ((long long)g * f.ne + e) * N;
        float rv[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            dd r = {f.iso_hi[ci + i], f.iso_lo[ci + i]};
            if (f.q_hi) dd_acc(r, {f.q_hi[idx + i], f.q_lo[idx + i]});
            dd_acc(r, {-yr[i].hi, -yr[i].lo});
            rv[i] = __fadd_rn(r.hi, r.lo);
        }
        float* out = f.r + idx;
        if constexpr (N % 4 == 0) {
#pragma unroll
            for (int i = 0; i < N; i += 4) *reinterpret_cast<float4*>(out + i) = make_float4(rv[i], rv[i + 1], rv[i + 2], rv[i + 3]);
        } else {
#pragma unroll
            for (int i = 0; i < N; ++i) out[i] = rv[i];
        }
    });
}

// ---------------------------------------------------------------- FP32 residual update
struct UpdateArgs {
    int ne, Nw, G;
    const float* tab;        // the sweep's FP32 cell tables
    const Slot* slots;
    const int* nbr;          // 2 * neighbour + standard-map bit
    const unsigned* map;
    const float* dots;       // [nfaces][Nw] FP32 Omega . n (sign of the FP64 value)
    const float4* omega;
    const float* sigma;      // [G][ne]
    float tau;
    const float* iso;        // [G][ne][N]: (S D x) / sum(w)
    const float* x;          // fused layout
    float* r;                // fused layout, r += iso - L x
    int* status;
};

// r += iso - L x in FP32 for every (group, cell, angle) node, angle fastest:
// the residual of psi + x from the residual r of psi, for a correction x small
// against psi (its FP32 rounding is then small against r).
template <int D, int P, bool TD>
__global__ void __launch_bounds__(kFusedBlock) k_residual_update_f32(UpdateArgs f) {
    using S = Shape<D, P>;
    using T = Tab<D, P, TD>;
    constexpr int N = S::N, NF = S::NF, NFACE = S::NFACE;
    constexpr int NP = (N + 1) / 2;
    __shared__ __align__(128) float s_tab[kFusedWarps * kSlotsUpdate * T::size];
    __shared__ __align__(8) unsigned long long s_bar[kFusedWarps * kSlotsUpdate];
    const int warp = threadIdx.x >> 5;
    const long long total = (long long)f.G * f.ne * f.Nw;
    const long long t = (long long)blockIdx.x * kFusedBlock + threadIdx.x;
    const bool valid = t < total;
    int g = 0, e = 0, a = 0;
    if (valid) {
        a = (int)(t % f.Nw);
        const long long rr = t / f.Nw;
        e = (int)(rr % f.ne);
        g = (int)(rr / f.ne);
    }
    float* wtab = s_tab + warp * kSlotsUpdate * T::size;
    unsigned long long* wbar = s_bar + warp * kSlotsUpdate;
    bool start = false;
    const int run = stage_runs<kSlotsUpdate>(wtab, wbar, f.tab, T::size, valid, g * f.ne + e, e, start);
    const long long idx = fused_index(f.ne, f.Nw, N, g, e, a);
    float x[N], y[N];
    float4 om = make_float4(0.f, 0.f, 0.f, 0.f);
    float sg = 0.f;
    if (valid) {
        ld_vec<N>(f.x + idx, x);
        om = f.omega[a];
        sg = f.sigma[(size_t)g * f.ne + e];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) y[i] = 0.f;
    for_each_round<kSlotsUpdate>(wtab, wbar, f.tab, T::size, valid, run, start, e, f.status, [&](unsigned tb) {
        const float omv[3] = {om.x, om.y, om.z};
        // volume part: row i of (sum_d Omega_d G_d + sigma M [+ tau Mt]) dotted with x
        float2 xp[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) xp[p] = make_float2(x[2 * p], 2 * p + 1 < N ? x[2 * p + 1] : 0.f);
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float2 ar[NP], tr[NP];
            lds_row<N>(tb + 4u * (T::oG + i * N), tr);
#pragma unroll
            for (int p = 0; p < NP; ++p) ar[p] = mul2(f2(omv[0]), tr[p]);
#pragma unroll
            for (int d = 1; d < D; ++d) {
                lds_row<N>(tb + 4u * (T::oG + d * N * N + i * N), tr);
#pragma unroll
                for (int p = 0; p < NP; ++p) ar[p] = fma2(f2(omv[d]), tr[p], ar[p]);
            }
            lds_row<N>(tb + 4u * (T::oM + i * N), tr);
#pragma unroll
            for (int p = 0; p < NP; ++p) ar[p] = fma2(f2(sg), tr[p], ar[p]);
            if constexpr (TD) {
                lds_row<N>(tb + 4u * (T::oMt + i * N), tr);
#pragma unroll
                for (int p = 0; p < NP; ++p) ar[p] = fma2(f2(f.tau), tr[p], ar[p]);
            }
            float2 acc = mul2(ar[0], xp[0]);
#pragma unroll
            for (int p = 1; p < NP; ++p) acc = fma2(ar[p], xp[p], acc);
            y[i] = acc.x + acc.y;
        }
        // face terms with Omega.n of the FP64 sign: outflow on x's own trace, inflow on the upwind x
        sfor<0, NFACE>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            const Slot q = f.slots[(size_t)e * NFACE + k];
            const float d1 = f.dots[(size_t)q.face * f.Nw + a];
            const float dk = q.side ? -d1 : d1;
            const bool out = dk > 0.f, in = dk < 0.f && q.nbr >= 0;
            if (!out && !in) return;
            float u[NF];
            if (out) {
                sfor<0, NF>([&](auto jc) {
                    constexpr int jj = decltype(jc)::value;
                    u[jj] = x[face_dof(D, P, k, jj)];
                });
            } else {
                const int nbv = f.nbr[(size_t)e * NFACE + k];
                const float* up = f.x + fused_index(f.ne, f.Nw, N, g, nbv >> 1, a);
                if (nbv & 1) {
                    float blk[N];
                    ld_vec<N>(up, blk);
                    sfor<0, NF>([&](auto jc) {
                        constexpr int jj = decltype(jc)::value;
                        u[jj] = blk[face_dof(D, P, k ^ 1, jj)];
                    });
                } else {
                    const unsigned m4 = f.map[(size_t)e * NFACE + k];
#pragma unroll
                    for (int jj = 0; jj < NF; ++jj) u[jj] = up[(m4 >> (8 * jj)) & 0xffu];
                }
            }
            sfor<0, NF>([&](auto ic) {
                constexpr int ii = decltype(ic)::value;
                float fr[NF];
                lds_vec<NF>(tb + 4u * (T::oF + (k * NF + ii) * NF), fr);
                float acc = 0.f;
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) acc = fmaf(fr[jj], u[jj], acc);
                constexpr int fi = face_dof(D, P, k, ii);
                y[fi] = fmaf(dk, acc, y[fi]);
            });
        });
        float r[N], s[N];
        ld_vec<N>(f.r + idx, r);
        ld_vec<N>(f.iso + ((long long)g * f.ne + e) * N, s);
#pragma unroll
        for (int i = 0; i < N; ++i) r[i] += s[i] - y[i];
        st_vec<N>(f.r + idx, r);
    });
}

// ---------------------------------------------------------------- layout conversions
// RIGHT FP64 psi(g, a, i) <-> fused layout as FP32 (hi) and its remainder (lo)
__global__ void k_right_to_fused(int ne, int Nw, int G, int N, const double* __restrict__ in, float* __restrict__ hi,
                                 float* __restrict__ lo) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // fused index
    const long long ndof = (long long)ne * N;
    if (t >= (long long)G * Nw * ndof) return;
    const int i = (int)(t % N);
    long long r = t / N;
    const int a = (int)(r % Nw);
    r /= Nw;
    const int e = (int)(r % ne), g = (int)(r / ne);
    const double v = in[psi_index(ndof, Nw, g, a, (long long)e * N + i)];
    const float h = (float)v;
    hi[t] = h;
    if (lo) lo[t] = (float)(v - (double)h);
}

__global__ void k_fused_to_right(int ne, int Nw, int G, int N, const float* __restrict__ hi, const float* __restrict__ lo,
                                 double* __restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // RIGHT index
    const long long ndof = (long long)ne * N;
    if (t >= (long long)G * Nw * ndof) return;
    const long long s = t % ndof;
    const long long r = t / ndof;
    const int a = (int)(r % Nw), g = (int)(r / Nw);
    const int e = (int)(s / N), i = (int)(s % N);
    const long long k = fused_index(ne, Nw, N, g, e, a) + i;
    double v = (double)hi[k];
    if (lo) v += (double)lo[k];
    out[t] = v;
}

#define FCK(x)                                  \
    do {                                        \
        cudaError_t _e = (x);                   \
        if (_e != cudaSuccess) return _e;       \
    } while (0)

inline unsigned blocks(long long n, int b) { return (unsigned)((n + b - 1) / b); }

template <int D, int P, bool TD>
cudaError_t build_tab(Handle& h, FusedState& fs) {
    using T = Tab<D, P, TD>;
    if (fs.tab) { cudaFree(fs.tab); fs.tab = nullptr; }
    FCK(cudaMalloc(&fs.tab, (size_t)h.ne * T::size * sizeof(float)));
    const long long n = (long long)h.ne * T::size;
    k_fused_tab<D, P, TD><<<blocks(n, 256), 256, 0, h.stream>>>(h.ne, h.d_G, h.d_M, h.d_Mt, h.d_F, h.d_slots,
                                                                   h.d_normals, fs.tab);
    FCK(cudaGetLastError());
    fs.tab_td = TD ? 1 : 0;
    return cudaSuccess;
}

template <int D, int P, bool TD>
cudaError_t build_dtab(Handle& h, FusedState& fs) {
    using T = DTab<D, P, TD>;
    if (fs.dtab) { cudaFree(fs.dtab); fs.dtab = nullptr; }
    FCK(cudaMalloc(&fs.dtab, (size_t)h.ne * T::size * sizeof(float)));
    FCK(cudaMemsetAsync(fs.dtab, 0, (size_t)h.ne * T::size * sizeof(float), h.stream));
    const long long n = (long long)h.ne * T::half;
    k_df_tab<D, P, TD><<<blocks(n, 256), 256, 0, h.stream>>>(h.ne, h.d_G, h.d_M, h.d_Mt, h.d_F, fs.dtab);
    FCK(cudaGetLastError());
    fs.dtab_td = TD ? 1 : 0;
    return cudaSuccess;
}

template <int D, int P, bool TD>
cudaError_t build_utab(Handle& h, FusedState& fs) {
    using T = Tab<D, P, TD>;
    if (fs.utab) { cudaFree(fs.utab); fs.utab = nullptr; }
    FCK(cudaMalloc(&fs.utab, (size_t)fs.nunits * T::size * sizeof(float)));
    const long long n = (long long)fs.nunits * T::size;
    k_unit_tab<D, P, TD><<<blocks(n, 256), 256, 0, h.stream>>>(fs.nunits, fs.unit_cell, fs.unit_pat, fs.tab, fs.utab);
    FCK(cudaGetLastError());
    fs.utab_td = TD ? 1 : 0;
    return cudaSuccess;
}

cudaError_t dispatch_utab(Handle& h, FusedState& fs) {
    const bool td = h.time_dependent;
#define UTAB_CASE(D_, P_) \
    case D_ * 10 + P_: return td ? build_utab<D_, P_, true>(h, fs) : build_utab<D_, P_, false>(h, fs);
    switch (h.dim * 10 + h.p) {
        UTAB_CASE(1, 0) UTAB_CASE(1, 1) UTAB_CASE(2, 0) UTAB_CASE(2, 1) UTAB_CASE(3, 0) UTAB_CASE(3, 1)
        default: return cudaErrorNotSupported;
    }
#undef UTAB_CASE
}

template <bool DF>
cudaError_t dispatch_tab(Handle& h, FusedState& fs) {
    const bool td = h.time_dependent;
#define TAB_CASE(D_, P_)                                                                              \
    case D_ * 10 + P_:                                                                                \
        if (DF) return td ? build_dtab<D_, P_, true>(h, fs) : build_dtab<D_, P_, false>(h, fs);       \
        return td ? build_tab<D_, P_, true>(h, fs) : build_tab<D_, P_, false>(h, fs);
    switch (h.dim * 10 + h.p) {
        TAB_CASE(1, 0) TAB_CASE(1, 1) TAB_CASE(2, 0) TAB_CASE(2, 1) TAB_CASE(3, 0) TAB_CASE(3, 1)
        default: return cudaErrorNotSupported;
    }
#undef TAB_CASE
}

// Unit levels: unit of every node (*nunits units, 0 when a cell has more than
// kMaxUnits units) and level of every unit, or *nlev = -1 when there are no
// units or the unit graph has a cycle (the caller then keeps the node levels).
cudaError_t unit_levels(Handle& h, int** unit_of_node, int** level_of_unit, int* nlev, int* nunits) {
    const long long N = (long long)h.ne * h.Nw;
    *nlev = -1;
    *nunits = 0;
    *unit_of_node = nullptr;
    *level_of_unit = nullptr;
    int *key = nullptr, *nin = nullptr, *unit = nullptr, *cnt = nullptr, *base = nullptr, *flag = nullptr;
    int *pending = nullptr, *usize = nullptr, *ustart = nullptr, *ufill = nullptr, *unodes = nullptr, *ulevel = nullptr;
    int *fa = nullptr, *fb = nullptr, *fc = nullptr;
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
    auto finish = [&](cudaError_t e) {
        void* bufs[] = {key, nin, cnt, base, flag, pending, usize, ustart, ufill, unodes, fa, fb, fc, tmp};
        for (void* b : bufs)
            if (b) cudaFree(b);
        if (e != cudaSuccess || *nunits == 0) {
            *nlev = -1;
            *nunits = 0;
            cudaFree(unit);
            cudaFree(ulevel);
            return e;
        }
        *unit_of_node = unit;
        if (*nlev < 0) {
            cudaFree(ulevel);
        } else {
            *level_of_unit = ulevel;
        }
        return e;
    };
#define UCK(x)                                      \
    do {                                            \
        cudaError_t _u = (x);                       \
        if (_u != cudaSuccess) return finish(_u);   \
    } while (0)
    UCK(cudaMalloc(&key, N * sizeof(int)));
    UCK(cudaMalloc(&nin, N * sizeof(int)));
    UCK(cudaMalloc(&unit, N * sizeof(int)));
    UCK(cudaMalloc(&cnt, (size_t)h.ne * sizeof(int)));
    UCK(cudaMalloc(&base, (size_t)h.ne * sizeof(int)));
    UCK(cudaMalloc(&flag, sizeof(int)));
    UCK(cudaMemsetAsync(flag, 0, sizeof(int), h.stream));
    k_unit_keys<<<blocks(N, 256), 256, 0, h.stream>>>(N, h.Nw, h.dim, h.d_omega, h.d_dots, h.d_slots, key, nin);
    k_unit_local<<<blocks(h.ne, 128), 128, 0, h.stream>>>(h.ne, h.Nw, key, unit, cnt, flag);
    UCK(cudaGetLastError());
    UCK(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, cnt, base, h.ne, h.stream));
    UCK(cudaMalloc(&tmp, tmp_bytes));
    UCK(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, cnt, base, h.ne, h.stream));
    int host[3] = {0, 0, 0};
    UCK(cudaMemcpyAsync(host, flag, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    UCK(cudaMemcpyAsync(host + 1, base + h.ne - 1, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    UCK(cudaMemcpyAsync(host + 2, cnt + h.ne - 1, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    UCK(cudaStreamSynchronize(h.stream));
    if (host[0]) return finish(cudaSuccess);   // too many units in a cell
    const int nu = host[1] + host[2];
    *nunits = nu;
    UCK(cudaMalloc(&pending, (size_t)nu * sizeof(int)));
    UCK(cudaMalloc(&usize, (size_t)nu * sizeof(int)));
    UCK(cudaMalloc(&ustart, (size_t)nu * sizeof(int)));
    UCK(cudaMalloc(&ufill, (size_t)nu * sizeof(int)));
    UCK(cudaMalloc(&ulevel, (size_t)nu * sizeof(int)));
    UCK(cudaMalloc(&unodes, N * sizeof(int)));
    UCK(cudaMalloc(&fa, (size_t)nu * sizeof(int)));
    UCK(cudaMalloc(&fb, (size_t)nu * sizeof(int)));
    UCK(cudaMalloc(&fc, 2 * sizeof(int)));
    UCK(cudaMemsetAsync(pending, 0, (size_t)nu * sizeof(int), h.stream));
    UCK(cudaMemsetAsync(usize, 0, (size_t)nu * sizeof(int), h.stream));
    UCK(cudaMemsetAsync(ufill, 0, (size_t)nu * sizeof(int), h.stream));
    UCK(cudaMemsetAsync(fc, 0, 2 * sizeof(int), h.stream));
    k_unit_ids<<<blocks(N, 256), 256, 0, h.stream>>>(N, h.Nw, base, nin, unit, pending, usize);
    UCK(cudaGetLastError());
    size_t need = 0;
    UCK(cub::DeviceScan::ExclusiveSum(nullptr, need, usize, ustart, nu, h.stream));
    if (need > tmp_bytes) {
        cudaFree(tmp);
        tmp = nullptr;
        tmp_bytes = need;
        UCK(cudaMalloc(&tmp, tmp_bytes));
    }
    UCK(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, usize, ustart, nu, h.stream));
    k_unit_fill<<<blocks(N, 256), 256, 0, h.stream>>>(N, unit, ustart, ufill, unodes);
    k_unit_frontier0<<<blocks(nu, 256), 256, 0, h.stream>>>(nu, pending, fa, fc);
    UCK(cudaGetLastError());
    int ncur = 0;
    UCK(cudaMemcpyAsync(&ncur, fc, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    UCK(cudaStreamSynchronize(h.stream));
    long long done = 0;
    int lev = 0;
    while (ncur > 0) {
        done += ncur;
        UCK(cudaMemsetAsync(fc + 1, 0, sizeof(int), h.stream));
        k_unit_kahn<<<blocks(ncur, 128), 128, 0, h.stream>>>(h.Nw, h.dim, key, h.d_slots, unit, ustart, usize, unodes,
                                                             pending, ulevel, fa, ncur, fb, fc + 1, lev);
        UCK(cudaGetLastError());
        UCK(cudaMemcpyAsync(&ncur, fc + 1, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
        UCK(cudaStreamSynchronize(h.stream));
        std::swap(fa, fb);
        ++lev;
    }
    if (done == nu) *nlev = lev;   // else: a cycle among units
#undef UCK
    return finish(cudaSuccess);
}

// Node records, cell neighbour data and FP32 angles: geometry only, built once.
// Levels are the unit levels when the unit graph allows (else the node levels);
// within each level the records are ordered (face pattern, cell, angle): a
// unit's angles are adjacent, so a warp spans few units (one table copy each),
// and the units of a warp fold the same inflow faces.
cudaError_t prepare_common(Handle& h, FusedState& fs) {
    if (fs.nodes) return cudaSuccess;
    const long long N = (long long)h.ne * h.Nw;
    if (h.ne >= (1 << 24) || h.num_levels >= (1 << 27) || N > 0x7fffffffLL) return cudaErrorInvalidValue;
    int* unit = nullptr;
    int* ulevel = nullptr;
    int nlev = -1, nunits = 0;
    FCK(unit_levels(h, &unit, &ulevel, &nlev, &nunits));
    if (nunits == 0 || (long long)h.G * nunits >= (1LL << 31)) {   // more than kMaxUnits units in a cell
        cudaFree(unit);
        cudaFree(ulevel);
        return cudaErrorNotSupported;
    }
    const int* level_of = ulevel;
    fs.unit_levels = nlev >= 0 && nlev < (1 << 27);
    if (!fs.unit_levels) {
        nlev = h.num_levels;
        level_of = h.d_level;
    }
    cudaError_t err = cudaSuccess;
    int2* recs = nullptr;
    unsigned long long *keys = nullptr, *keys_out = nullptr;
    long long* starts = nullptr;
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
    int lev_bits = 1;
    while ((1 << lev_bits) < nlev + 1) ++lev_bits;
    const int end_bit = 36 + lev_bits;
    // the face pattern (at most 12 bits) sits between the level and the unit
    // when the unit ids fit in 24 bits
    const int ubits = nunits <= (1 << 24) ? 24 : 36;
    std::vector<long long> hs(nlev + 1);
    auto step = [&](cudaError_t e) { if (err == cudaSuccess) err = e; };
    int2* sorted = nullptr;
    long long *psize = nullptr, *pstart = nullptr;
    int *flag = nullptr, *ridx = nullptr, *run_start = nullptr, *run_pos = nullptr;
    void* scan_tmp = nullptr;
    size_t scan_bytes = 0;
    int nruns = 0;
    std::vector<long long> ps(nlev + 1, 0);
    step(cudaMalloc(&sorted, N * sizeof(int2)));
    step(cudaMalloc(&psize, (nlev + 1) * sizeof(long long)));
    step(cudaMalloc(&pstart, (nlev + 1) * sizeof(long long)));
    step(cudaMalloc(&flag, N * sizeof(int)));
    step(cudaMalloc(&ridx, N * sizeof(int)));
    step(cudaMalloc(&fs.nbr, (size_t)h.ne * h.nface * sizeof(int)));
    step(cudaMalloc(&fs.map, (size_t)h.ne * h.nface * sizeof(unsigned)));
    step(cudaMalloc(&fs.omega, (size_t)h.Nw * sizeof(float4)));
    step(cudaMalloc(&fs.w, (size_t)h.Nw * sizeof(float)));
    step(cudaMalloc(&fs.domega, (size_t)h.Nw * h.dim * sizeof(float2)));
    step(cudaMalloc(&fs.dw, (size_t)h.Nw * sizeof(float2)));
    step(cudaMalloc(&recs, N * sizeof(int2)));
    step(cudaMalloc(&keys, N * sizeof(unsigned long long)));
    step(cudaMalloc(&keys_out, N * sizeof(unsigned long long)));
    step(cudaMalloc(&starts, (nlev + 1) * sizeof(long long)));
    if (err == cudaSuccess) {
        k_fused_nodes<<<blocks(N, 256), 256, 0, h.stream>>>(N, h.Nw, h.dim, h.d_dots, h.d_slots, recs);
        k_fused_keys<<<blocks(N, 256), 256, 0, h.stream>>>(N, h.Nw, recs, level_of, fs.unit_levels, unit, ubits,
                                                          keys);
        step(cudaGetLastError());
    }
    step(cudaMalloc(&fs.unit_cell, (size_t)nunits * sizeof(int)));
    step(cudaMalloc(&fs.unit_pat, (size_t)nunits * sizeof(int)));
    if (err == cudaSuccess) {
        k_unit_info<<<blocks(N, 256), 256, 0, h.stream>>>(N, h.Nw, recs, unit, fs.unit_cell, fs.unit_pat);
        step(cudaGetLastError());
    }
    if (err == cudaSuccess)
        step(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys_out, recs, sorted, (int)N, 0, end_bit,
                                             h.stream));
    if (err == cudaSuccess) step(cudaMalloc(&tmp, tmp_bytes));
    if (err == cudaSuccess)
        step(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys_out, recs, sorted, (int)N, 0, end_bit,
                                             h.stream));
    if (err == cudaSuccess) {
        k_level_starts<<<blocks(nlev + 1, 128), 128, 0, h.stream>>>(nlev, keys_out, N, starts);
        step(cudaGetLastError());
    }
    // warps of at most kSlots units: runs, their padded positions, level sizes, records
    if (err == cudaSuccess) {
        k_run_flags<<<blocks(N, 256), 256, 0, h.stream>>>(N, keys_out, flag);
        step(cudaGetLastError());
    }
    if (err == cudaSuccess) step(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, flag, ridx, (int)N, h.stream));
    if (err == cudaSuccess) step(cudaMalloc(&scan_tmp, scan_bytes));
    if (err == cudaSuccess) step(cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, flag, ridx, (int)N, h.stream));
    if (err == cudaSuccess) {
        int last[2] = {0, 0};
        step(cudaMemcpyAsync(&last[0], ridx + N - 1, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
        step(cudaMemcpyAsync(&last[1], flag + N - 1, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
        step(cudaStreamSynchronize(h.stream));
        nruns = last[0] + last[1];
    }
    if (err == cudaSuccess) step(cudaMalloc(&run_start, (size_t)(nruns + 1) * sizeof(int)));
    if (err == cudaSuccess) step(cudaMalloc(&run_pos, (size_t)(nruns + 1) * sizeof(int)));
    if (err == cudaSuccess) {
        k_run_starts<<<blocks(N, 256), 256, 0, h.stream>>>(N, flag, ridx, run_start);
        k_pack_runs<<<blocks(nlev, 64), 64, 0, h.stream>>>(nlev, N, nruns, starts, ridx, run_start, run_pos, psize);
        step(cudaGetLastError());
    }
    if (err == cudaSuccess)
        step(cudaMemcpyAsync(hs.data(), psize, nlev * sizeof(long long), cudaMemcpyDeviceToHost, h.stream));
    if (err == cudaSuccess) step(cudaStreamSynchronize(h.stream));
    if (err == cudaSuccess) {
        for (int l = 0; l < nlev; ++l) ps[l + 1] = ps[l] + hs[l];
        if (ps[nlev] > 0x7fffffffLL) err = cudaErrorInvalidValue;
    }
    if (err == cudaSuccess) step(cudaMalloc(&fs.nodes, (size_t)ps[nlev] * sizeof(int2)));
    if (err == cudaSuccess) step(cudaMalloc(&fs.rec_unit, (size_t)ps[nlev] * sizeof(int)));
    if (err == cudaSuccess)
        step(cudaMemcpyAsync(pstart, ps.data(), (nlev + 1) * sizeof(long long), cudaMemcpyHostToDevice, h.stream));
    if (err == cudaSuccess) {
        k_pack_fill<<<blocks(ps[nlev], 256), 256, 0, h.stream>>>(ps[nlev], fs.nodes, fs.rec_unit);
        k_pack_scatter<<<blocks(N, 256), 256, 0, h.stream>>>(N, keys_out, sorted, ridx, flag, run_start, run_pos,
                                                             pstart, (1ull << ubits) - 1, fs.nodes, fs.rec_unit);
        step(cudaGetLastError());
    }
    if (err == cudaSuccess) step(cudaStreamSynchronize(h.stream));
    cudaFree(tmp); cudaFree(starts); cudaFree(keys_out); cudaFree(keys); cudaFree(recs);
    cudaFree(sorted); cudaFree(psize); cudaFree(pstart); cudaFree(flag); cudaFree(ridx); cudaFree(scan_tmp);
    cudaFree(run_start); cudaFree(run_pos);
    cudaFree(unit); cudaFree(ulevel);
    if (err == cudaSuccess) {
        k_fused_cells<<<blocks((long long)h.ne * h.nface, 256), 256, 0, h.stream>>>(h.ne, h.dim, h.p, h.nf, h.d_slots,
                                                                                    h.d_nbrmap, fs.nbr, fs.map);
        k_fused_angles<<<blocks(h.Nw, 128), 128, 0, h.stream>>>(h.Nw, h.dim, h.d_omega, h.d_weights, fs.omega, fs.w,
                                                                fs.domega, fs.dw);
        step(cudaGetLastError());
    }
    if (err != cudaSuccess) {
        void* bufs[] = {fs.nodes, fs.nbr, fs.map, fs.omega, fs.w, fs.domega, fs.dw, fs.rec_unit, fs.unit_cell,
                        fs.unit_pat};
        for (void* b : bufs)
            if (b) cudaFree(b);
        fs.nodes = nullptr; fs.nbr = nullptr; fs.map = nullptr; fs.omega = nullptr; fs.w = nullptr;
        fs.domega = nullptr; fs.dw = nullptr; fs.rec_unit = nullptr; fs.unit_cell = nullptr; fs.unit_pat = nullptr;
        return err;
    }
    fs.nunits = nunits;
    fs.num_levels = nlev;
    fs.level_offsets.assign(nlev + 1, 0);
    for (int l = 0; l <= nlev; ++l) fs.level_offsets[l] = (int)ps[l];
    return cudaSuccess;
}

cudaLaunchAttribute pdl_attr() {
    cudaLaunchAttribute at;
    at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at.val.programmaticStreamSerializationAllowed = 1;
    return at;
}

template <int D, int P, bool TD>
cudaError_t sweep_body(Handle& h, FusedState& fs, const FusedArgs& a, double* phi, int phi_mode, cudaStream_t st) {
    const bool pdl = fs.pdl != 0;
    bool first = true;
    cudaLaunchAttribute attr[1] = {pdl_attr()};
    for (int l = 0; l < fs.num_levels; ++l) {
        const int off = fs.level_offsets[l];
        const int count = fs.level_offsets[l + 1] - off;
        if (count == 0) continue;
        const long long threads = (long long)count * h.G;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(blocks(threads, kSweepBlock));
        cfg.blockDim = dim3(kSweepBlock);
        cfg.stream = st;
        // every level after the first may start its blocks while the previous
        // level drains; they wait (griddepcontrol.wait) before reading upwind traces
        cfg.attrs = attr;
        cfg.numAttrs = (pdl && !first) ? 1 : 0;
        FCK(cudaLaunchKernelEx(&cfg, k_fused_level<D, P, TD>, a, off, count));
        first = false;
    }
    if (phi_mode) {
        const long long total = (long long)h.G * h.ndof;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(blocks(total, 256));
        cfg.blockDim = dim3(256);
        cfg.stream = st;
        cfg.attrs = attr;
        cfg.numAttrs = pdl ? 1 : 0;
        if (phi_mode == 3)
            FCK(cudaLaunchKernelEx(&cfg, k_moments_f32_fast, h.ne, h.Nw, h.G, h.n, (const float*)fs.w,
                                   (const float*)a.psi, phi));
        else
            FCK(cudaLaunchKernelEx(&cfg, k_moments_f32, h.ne, h.Nw, h.G, h.n, (const float2*)fs.dw,
                                   (const float*)a.psi, phi, phi_mode == 2 ? 1 : 0));
    }
    return cudaGetLastError();
}

template <int D, int P, bool TD>
cudaError_t residual_body(Handle& h, const ResidArgs& a, cudaStream_t st) {
    const long long total = (long long)h.G * h.ne * h.Nw;
    k_residual_df<D, P, TD><<<blocks(total, kFusedBlock), kFusedBlock, 0, st>>>(a);
    return cudaGetLastError();
}

// Replay of the fused sweep's level launches through a CUDA graph keyed by
// every vector it touches (captured once per key on a private stream).
template <typename Body>
cudaError_t fused_graph(Handle& h, FusedState& fs, const void* const (&key)[7], Body&& body) {
    if (!h.use_graphs) return body(h.stream);
    for (auto& gr : fs.graphs) {
        if (!gr.exec) continue;
        bool same = true;
        for (int i = 0; i < 7; ++i) same = same && gr.key[i] == key[i];
        if (same) return cudaGraphLaunch(gr.exec, h.stream);
    }
    if (!h.capture_stream) FCK(cudaStreamCreateWithFlags(&h.capture_stream, cudaStreamNonBlocking));
    FCK(cudaStreamBeginCapture(h.capture_stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t be = body(h.capture_stream);
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(h.capture_stream, &graph);
    if (be != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return be;
    }
    FCK(ee);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    FCK(ie);
    auto& slot = fs.graphs[fs.next];
    fs.next = (fs.next + 1) % FusedState::kGraphs;
    if (slot.exec) cudaGraphExecDestroy(slot.exec);
    for (int i = 0; i < 7; ++i) slot.key[i] = key[i];
    slot.exec = exec;
    return cudaGraphLaunch(exec, h.stream);
}

}  // namespace

FusedState* fused_state(Handle& h) {
    if (!h.fused) h.fused = new FusedState();
    return h.fused;
}

bool fused_supported(const Handle& h) { return h.p <= 1 && h.nrefl == 0 && h.Nw < 65536 && h.nf <= 4; }

cudaError_t fused_levels(Handle& h, int* num_levels, int* unit_levels) {
    FusedState& fs = *fused_state(h);
    FCK(prepare_common(h, fs));
    *num_levels = fs.num_levels;
    *unit_levels = fs.unit_levels ? 1 : 0;
    return cudaSuccess;
}

void set_fused_pdl(Handle& h, int on) {
    drop_fused_graphs(h);
    fused_state(h)->pdl = on ? 1 : 0;
}

void drop_fused_graphs(Handle& h) {
    if (!h.fused) return;
    for (auto& gr : h.fused->graphs) {
        if (gr.exec) cudaGraphExecDestroy(gr.exec);
        gr = FusedState::Graph{};
    }
}

void free_fused(Handle& h) {
    if (!h.fused) return;
    drop_fused_graphs(h);
    FusedState& fs = *h.fused;
    void* bufs[] = {fs.nodes, fs.nbr, fs.map, fs.omega, fs.w, fs.tab, fs.dtab, fs.ddots, fs.domega, fs.dw, fs.dsigma,
                    fs.utab, fs.unit_cell, fs.unit_pat, fs.rec_unit};
    for (void* b : bufs)
        if (b) cudaFree(b);
    delete h.fused;
    h.fused = nullptr;
}

cudaError_t launch_fused_sweep(Handle& h, const float* iso, const float* src, float* psi, double* phi, int phi_mode,
                               float* acc_hi, float* acc_lo) {
    FusedState& fs = *fused_state(h);
    FCK(prepare_common(h, fs));
    if (!h.fp32_ready) FCK(make_fp32_copies(h));
    const int td = h.time_dependent ? 1 : 0;
    if (fs.tab_td != td) {
        drop_fused_graphs(h);
        FCK(dispatch_tab<false>(h, fs));
    }
    if (fs.utab_td != td) {
        drop_fused_graphs(h);
        FCK(dispatch_utab(h, fs));
    }
    FusedArgs a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G;
    a.nodes = fs.nodes; a.tab = fs.utab; a.nbr = fs.nbr; a.map = fs.map;
    a.rec_unit = fs.rec_unit; a.nunits = fs.nunits;
    a.omega = fs.omega; a.sigma = h.f_sigma; a.tau = (float)h.tau;
    a.iso = iso; a.src = src; a.psi = psi;
    a.acc_hi = acc_hi; a.acc_lo = acc_hi ? acc_lo : nullptr;
    a.status = h.d_status;
    if (!phi) phi_mode = 0;
    const void* const key[7] = {iso, src, psi, phi, acc_hi, acc_lo, (const void*)(intptr_t)(phi_mode + 4 * td)};
    return fused_graph(h, fs, key, [&](cudaStream_t st) -> cudaError_t {
#define SW_CASE(D_, P_)                                                                         \
    case D_ * 10 + P_:                                                                          \
        return td ? sweep_body<D_, P_, true>(h, fs, a, phi, phi_mode, st)                       \
                  : sweep_body<D_, P_, false>(h, fs, a, phi, phi_mode, st);
        switch (h.dim * 10 + h.p) {
            SW_CASE(1, 0) SW_CASE(1, 1) SW_CASE(2, 0) SW_CASE(2, 1) SW_CASE(3, 0) SW_CASE(3, 1)
            default: return cudaErrorNotSupported;
        }
#undef SW_CASE
    });
}

cudaError_t launch_iso_source(Handle& h, const double* sigma_s, const double* phi, const double* q_iso, float* out,
                              float* out_hi, float* out_lo) {
    const long long total = (long long)h.G * h.ndof;
    k_iso_source<<<blocks(total, 256), 256, 0, h.stream>>>(h.ne, h.G, h.n, h.wsum, h.d_Mt, sigma_s, phi, q_iso, out,
                                                           out_hi, out_lo);
    return cudaGetLastError();
}

cudaError_t launch_residual_df(Handle& h, const float* iso_hi, const float* iso_lo, const float* q_hi, const float* q_lo,
                               const float* psi_hi, const float* psi_lo, float* r) {
    FusedState& fs = *fused_state(h);
    FCK(prepare_common(h, fs));
    const int td = h.time_dependent ? 1 : 0;
    if (fs.dtab_td != td) FCK(dispatch_tab<true>(h, fs));
    if (!fs.ddots) {
        FCK(cudaMalloc(&fs.ddots, (size_t)h.nfaces * h.Nw * sizeof(float2)));
        const long long n = (long long)h.nfaces * h.Nw;
        k_df_split<<<blocks(n, 256), 256, 0, h.stream>>>(n, h.d_dots, fs.ddots);
        FCK(cudaGetLastError());
    }
    if (!fs.dsigma) FCK(cudaMalloc(&fs.dsigma, (size_t)h.G * h.ne * sizeof(float2)));
    k_df_split<<<blocks((long long)h.G * h.ne, 256), 256, 0, h.stream>>>((long long)h.G * h.ne, h.d_sigma, fs.dsigma);
    FCK(cudaGetLastError());
    ResidArgs a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G;
    a.dtab = fs.dtab; a.slots = h.d_slots; a.nbr = fs.nbr; a.nbrmap = h.d_nbrmap; a.ddots = fs.ddots;
    a.domega = fs.domega; a.dsigma = fs.dsigma;
    a.tau_hi = (float)h.tau;
    a.tau_lo = (float)(h.tau - (double)a.tau_hi);
    a.iso_hi = iso_hi; a.iso_lo = iso_lo; a.q_hi = q_hi; a.q_lo = q_hi ? q_lo : nullptr;
    a.psi_hi = psi_hi; a.psi_lo = psi_lo; a.r = r; a.status = h.d_status;
#define RS_CASE(D_, P_) \
    case D_ * 10 + P_: return td ? residual_body<D_, P_, true>(h, a, h.stream) : residual_body<D_, P_, false>(h, a, h.stream);
    switch (h.dim * 10 + h.p) {
        RS_CASE(1, 0) RS_CASE(1, 1) RS_CASE(2, 0) RS_CASE(2, 1) RS_CASE(3, 0) RS_CASE(3, 1)
        default: return cudaErrorNotSupported;
    }
#undef RS_CASE
}

cudaError_t launch_residual_update_f32(Handle& h, const float* iso, const float* x, float* r) {
    FusedState& fs = *fused_state(h);
    FCK(prepare_common(h, fs));
    if (!h.fp32_ready) FCK(make_fp32_copies(h));
    const int td = h.time_dependent ? 1 : 0;
    if (fs.tab_td != td) {
        drop_fused_graphs(h);
        FCK(dispatch_tab<false>(h, fs));
    }
    UpdateArgs a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G;
    a.tab = fs.tab; a.slots = h.d_slots; a.nbr = fs.nbr; a.map = fs.map; a.dots = h.f_dots;
    a.omega = fs.omega; a.sigma = h.f_sigma; a.tau = (float)h.tau;
    a.iso = iso; a.x = x; a.r = r; a.status = h.d_status;
    const long long total = (long long)h.G * h.ne * h.Nw;
#define UP_CASE(D_, P_)                                                                                          \
    case D_ * 10 + P_:                                                                                           \
        if (td) k_residual_update_f32<D_, P_, true><<<blocks(total, kFusedBlock), kFusedBlock, 0, h.stream>>>(a);  \
        else k_residual_update_f32<D_, P_, false><<<blocks(total, kFusedBlock), kFusedBlock, 0, h.stream>>>(a);    \
        return cudaGetLastError();
    switch (h.dim * 10 + h.p) {
        UP_CASE(1, 0) UP_CASE(1, 1) UP_CASE(2, 0) UP_CASE(2, 1) UP_CASE(3, 0) UP_CASE(3, 1)
        default: return cudaErrorNotSupported;
    }
#undef UP_CASE
}

cudaError_t launch_moments_df(Handle& h, const float* hi, const float* lo, double* phi) {
    FusedState& fs = *fused_state(h);
    FCK(prepare_common(h, fs));
    const long long total = (long long)h.G * h.ndof;
    k_moments_df<<<blocks(total, 256), 256, 0, h.stream>>>(h.ne, h.Nw, h.G, h.n, fs.dw, hi, lo, phi);
    return cudaGetLastError();
}

cudaError_t launch_fused_layout(Handle& h, int to_fused, const double* right, float* hi, float* lo) {
    const long long total = h.psi_size;
    if (to_fused)
        k_right_to_fused<<<blocks(total, 256), 256, 0, h.stream>>>(h.ne, h.Nw, h.G, h.n, right, hi, lo);
    else
        k_fused_to_right<<<blocks(total, 256), 256, 0, h.stream>>>(h.ne, h.Nw, h.G, h.n, hi, lo, (double*)right);
    return cudaGetLastError();
}

}  // namespace allium
