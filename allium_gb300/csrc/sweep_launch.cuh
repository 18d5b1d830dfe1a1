// Level-by-level launch of the sweep kernel for one arithmetic type.
#pragma once

#include <type_traits>

#include "sweep_kernels.cuh"

namespace allium {

template <int D, int P, typename R, bool PIVOT>
cudaError_t sweep_levels(Handle& h, const SweepArgs<R>& args, cudaStream_t stream) {
    const int kBlock = std::is_same<R, double>::value ? h.block64 : h.block32;
    for (int l = 0; l < h.num_levels; ++l) {
        const int off = h.h_level_offsets[l];
        const int count = h.h_level_offsets[l + 1] - off;
        if (count == 0) continue;
        const long long threads = (long long)count * h.G;
        if (threads > 0x7fffffffLL) return cudaErrorInvalidValue;
        const unsigned grid = (unsigned)((threads + kBlock - 1) / kBlock);
        k_sweep_level<D, P, R, PIVOT><<<grid, kBlock, 0, stream>>>(args, h.d_level_nodes + off, count);
    }
    return cudaGetLastError();
}

template <int D, int P, typename R, bool PIVOT>
cudaError_t sweep_levels_team(Handle& h, const SweepArgs<R>& args, cudaStream_t stream) {
    constexpr int kBlock = 256;
    constexpr int T = team_size(ipow(P + 1, D));
    for (int l = 0; l < h.num_levels; ++l) {
        const int off = h.h_level_offsets[l];
        const int count = h.h_level_offsets[l + 1] - off;
        if (count == 0) continue;
        const long long threads = (long long)count * h.G * T;
        if (threads > 0x7fffffffLL) return cudaErrorInvalidValue;
        const unsigned grid = (unsigned)((threads + kBlock - 1) / kBlock);
        if (args.fix_kind)
            k_sweep_team<D, P, R, PIVOT, true><<<grid, kBlock, 0, stream>>>(args, h.d_level_nodes + off, count);
        else
            k_sweep_team<D, P, R, PIVOT, false><<<grid, kBlock, 0, stream>>>(args, h.d_level_nodes + off, count);
    }
    return cudaGetLastError();
}

template <int D, int P, typename R, bool PIVOT>
cudaError_t sweep_levels_block(Handle& h, const SweepArgs<R>& args, cudaStream_t stream) {
    for (int l = 0; l < h.num_levels; ++l) {
        const int off = h.h_level_offsets[l];
        const int count = h.h_level_offsets[l + 1] - off;
        if (count == 0) continue;
        const long long blocks = (long long)count * h.G;
        if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
        if (args.fix_kind)
            k_sweep_block<D, P, R, PIVOT, true><<<(unsigned)blocks, 64, 0, stream>>>(args, h.d_level_nodes + off);
        else
            k_sweep_block<D, P, R, PIVOT, false><<<(unsigned)blocks, 64, 0, stream>>>(args, h.d_level_nodes + off);
    }
    return cudaGetLastError();
}

// All-node factor pass and the sweep from stored inverses (p = 1).
template <int D, int P>
cudaError_t factor_all(Handle& h, const SweepArgs<double>& args) {
    constexpr int kBlock = 128;
    const long long total = (long long)h.G * h.ne * h.Nw;
    const unsigned grid = (unsigned)((total + kBlock - 1) / kBlock);
    k_factor_all<D, P><<<grid, kBlock, 0, h.stream>>>(args, h.d_level_nodes, total, h.d_inv);
    return cudaGetLastError();
}

template <int D, int P, typename R>
cudaError_t sweep_levels_cached(Handle& h, const SweepArgs<R>& args, const R* inv, cudaStream_t stream) {
    const int kBlock = std::is_same<R, double>::value ? h.block64 : h.block32;
    const long long stride = (long long)h.G * h.ne * h.Nw;
    // every level after the first may start its blocks while the previous one
    // drains (programmatic dependent launch); they wait before reading upwind data
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    bool first = true;
    for (int l = 0; l < h.num_levels; ++l) {
        const int off = h.h_level_offsets[l];
        const int count = h.h_level_offsets[l + 1] - off;
        if (count == 0) continue;
        const long long threads = (long long)count * h.G;
        if (threads > 0x7fffffffLL) return cudaErrorInvalidValue;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)((threads + kBlock - 1) / kBlock));
        cfg.blockDim = dim3(kBlock);
        cfg.stream = stream;
        cfg.attrs = attr;
        cfg.numAttrs = (h.pdl_levels && !first) ? 1 : 0;
        cudaError_t e = cudaLaunchKernelEx(&cfg, k_sweep_cached_level<D, P, R, false>, args,
                                           (const int*)(h.d_level_nodes + off), count, inv, stride,
                                           (long long)off * h.G, (const int*)nullptr);
        if (e != cudaSuccess) return e;
        first = false;
    }
    return cudaGetLastError();
}

// One angle chunk of the sweep: the chunk's nodes in (level, face pattern, cell, angle)
// order (h.d_chunk_nodes), its own level ranges; the stored inverses found
// through each node's position in the full level order.
template <int D, int P>
cudaError_t sweep_chunk(Handle& h, const SweepArgs<double>& args, int c, cudaStream_t stream) {
    const int kBlock = h.block64;
    const long long stride = (long long)h.G * h.ne * h.Nw;
    const int* offs = h.h_chunk_offsets.data() + (size_t)c * (h.num_levels + 1);
    for (int l = 0; l < h.num_levels; ++l) {
        const int off = offs[l];
        const int count = offs[l + 1] - off;
        if (count == 0) continue;
        const long long threads = (long long)count * h.G;
        if (threads > 0x7fffffffLL) return cudaErrorInvalidValue;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)((threads + kBlock - 1) / kBlock));
        cfg.blockDim = dim3(kBlock);
        cfg.stream = stream;
        // no programmatic dependent launch here: the chunks' level chains run on
        // several compute streams at once, and blocks waiting early would hold SM
        // slots that another chain's ready level could use (the one run with it
        // had a median host-buffer call of 23.6 ms, the runs without 22.0-22.2)
        cudaError_t e = cudaLaunchKernelEx(&cfg, k_sweep_cached_level<D, P, double, true>, args,
                                           (const int*)(h.d_chunk_nodes + off), count, (const double*)h.d_inv, stride,
                                           0LL, (const int*)(h.d_chunk_pos + off));
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

template <typename R>
cudaError_t cached_dispatch(Handle& h, const SweepArgs<R>& a, const R* inv, cudaStream_t st) {
    switch (h.dim * 10 + h.p) {
        case 11: return sweep_levels_cached<1, 1, R>(h, a, inv, st);
        case 21: return sweep_levels_cached<2, 1, R>(h, a, inv, st);
        case 31: return sweep_levels_cached<3, 1, R>(h, a, inv, st);
        default: return cudaErrorNotSupported;
    }
}

// Dataflow launch: epoch bump + counter reset, then one persistent grid sized
// to the blocks that fit the GPU at once.
template <typename Kernel, typename... Args>
cudaError_t launch_flow(Handle& h, cudaStream_t stream, Kernel kernel, size_t smem, Args... args) {
    static int max_blocks = 0;   // per kernel instantiation
    if (max_blocks == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTile, smem);
        if (e != cudaSuccess) return e;
        max_blocks = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
    }
    k_flow_begin<<<1, 1, 0, stream>>>(h.d_flow_words, h.d_flow_words + 1);
    const int grid = h.ntiles < max_blocks ? h.ntiles : max_blocks;
    kernel<<<grid > 0 ? grid : 1, kTile, smem, stream>>>(args...);
    return cudaGetLastError();
}

inline FlowArgs flow_args(Handle& h) {
    FlowArgs f;
    f.flags = h.d_flags;
    f.epoch = h.d_flow_words;
    f.counter = h.d_flow_words + 1;
    f.tile_start = h.d_tile_start;
    f.tile_count = h.d_tile_count;
    f.ntiles = h.ntiles;
    return f;
}

template <int MODE, typename R>
cudaError_t flow_dispatch(Handle& h, const SweepArgs<R>& a, const R* inv, cudaStream_t st) {
    const long long stride = (long long)h.G * h.ne * h.Nw;
    const FlowArgs f = flow_args(h);
    switch (h.dim * 10 + h.p) {
        case 10: return launch_flow(h, st, k_flow<1, 0, R, MODE>, 0, a, f, h.d_level_nodes, inv, stride);
        case 11: return launch_flow(h, st, k_flow<1, 1, R, MODE>, 0, a, f, h.d_level_nodes, inv, stride);
        case 20: return launch_flow(h, st, k_flow<2, 0, R, MODE>, 0, a, f, h.d_level_nodes, inv, stride);
        case 21: return launch_flow(h, st, k_flow<2, 1, R, MODE>, 0, a, f, h.d_level_nodes, inv, stride);
        case 30: return launch_flow(h, st, k_flow<3, 0, R, MODE>, 0, a, f, h.d_level_nodes, inv, stride);
        case 31: return launch_flow(h, st, k_flow<3, 1, R, MODE>, 0, a, f, h.d_level_nodes, inv, stride);
        default: return cudaErrorNotSupported;
    }
}

// Thread per node while the local system fits a thread's registers (N <= 8):
// fewest instructions per node, and every lane busy on the FP64 pipe.  Team
// kernel (lane per row) for the larger systems, which would spill; block per
// node (shared-memory system) for 3D p = 3, wider than a warp.
template <typename R, bool PIVOT>
cudaError_t sweep_dispatch(Handle& h, const SweepArgs<R>& a, cudaStream_t st) {
    switch (h.dim * 10 + h.p) {
        case 10: return sweep_levels<1, 0, R, PIVOT>(h, a, st);
        case 11: return sweep_levels<1, 1, R, PIVOT>(h, a, st);
        case 12: return sweep_levels<1, 2, R, PIVOT>(h, a, st);
        case 13: return sweep_levels<1, 3, R, PIVOT>(h, a, st);
        case 20: return sweep_levels<2, 0, R, PIVOT>(h, a, st);
        case 21: return sweep_levels<2, 1, R, PIVOT>(h, a, st);
        case 22: return sweep_levels_team<2, 2, R, PIVOT>(h, a, st);
        case 23: return sweep_levels_team<2, 3, R, PIVOT>(h, a, st);
        case 30: return sweep_levels<3, 0, R, PIVOT>(h, a, st);
        case 31: return sweep_levels<3, 1, R, PIVOT>(h, a, st);
        case 32: return sweep_levels_team<3, 2, R, PIVOT>(h, a, st);
        case 33: return sweep_levels_block<3, 3, R, PIVOT>(h, a, st);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace allium
