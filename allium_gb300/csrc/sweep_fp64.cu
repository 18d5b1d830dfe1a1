// FP64 sweep (partially pivoted local LU) and the FP64 forward operator.
#include <vector>

#include "sweep_launch.cuh"

namespace allium {

// Tile table (tiles never span two levels), completion flags and the
// epoch/counter words of the dataflow schedule.
cudaError_t prepare_flow(Handle& h) {
    if (h.d_flags) return cudaSuccess;
    std::vector<int> start, count;
    for (int l = 0; l < h.num_levels; ++l) {
        const long long first = (long long)h.h_level_offsets[l] * h.G;
        const long long ng = (long long)(h.h_level_offsets[l + 1] - h.h_level_offsets[l]) * h.G;
        for (long long k = 0; k < ng; k += kTile) {
            start.push_back((int)(first + k));
            count.push_back((int)(ng - k < kTile ? ng - k : kTile));
        }
    }
    h.ntiles = (int)start.size();
    const size_t nflags = (size_t)h.ne * h.Nw * h.G;
    cudaError_t e;
    if ((e = cudaMalloc(&h.d_tile_start, start.size() * sizeof(int))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&h.d_tile_count, count.size() * sizeof(int))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&h.d_flow_words, 2 * sizeof(unsigned))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&h.d_flags, nflags * sizeof(unsigned))) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(h.d_tile_start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice, h.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(h.d_tile_count, count.data(), count.size() * sizeof(int), cudaMemcpyHostToDevice, h.stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(h.d_flow_words, 0, 2 * sizeof(unsigned), h.stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(h.d_flags, 0, nflags * sizeof(unsigned), h.stream)) != cudaSuccess) return e;
    return cudaStreamSynchronize(h.stream);   // host vectors go out of scope
}

cudaError_t launch_wait_probe(Handle& h, int limit) {
    cudaError_t e = prepare_flow(h);
    if (e != cudaSuccess) return e;
    // flags of this handle never hold the value ~0u: the wait can only give up
    k_wait_probe<<<1, 1, 0, h.stream>>>(h.d_flags, ~0u, limit, h.d_status);
    return cudaGetLastError();
}

// (Re)compute the stored inverses when they are stale: FP64, and the FP32
// copy when that buffer exists.
cudaError_t ensure_factors(Handle& h) {
    if (h.inv_valid) return cudaSuccess;
    SweepArgs<double> a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G; a.ndof = h.ndof;
    a.omega = h.d_omega; a.dots = h.d_dots; a.slots = h.d_slots; a.nbrmap = h.d_nbrmap;
    a.Gm = h.d_G; a.M = h.d_M; a.Mt = h.d_Mt; a.F = h.d_F; a.sigma = h.d_sigma;
    a.tau = h.tau; a.td = h.time_dependent ? 1 : 0;
    a.src = nullptr; a.psi = nullptr; a.status = h.d_status; a.refl = h.d_refl;
    a.fix_kind = 0; a.fix_min = 0.0; a.fix_counts = nullptr;
    cudaError_t e;
    switch (h.dim * 10 + h.p) {
        case 11: e = factor_all<1, 1>(h, a); break;
        case 21: e = factor_all<2, 1>(h, a); break;
        case 31: e = factor_all<3, 1>(h, a); break;
        default: e = cudaErrorNotSupported;
    }
    if (e == cudaSuccess) {
        h.inv_valid = true;
        h.f_inv_valid = false;   // the FP32 copy follows the FP64 inverses
    }
    return e;
}

cudaError_t launch_sweep_fp64(Handle& h, const double* src, double* psi) {
    SweepArgs<double> a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G; a.ndof = h.ndof;
    a.omega = h.d_omega; a.dots = h.d_dots; a.slots = h.d_slots; a.nbrmap = h.d_nbrmap;
    a.Gm = h.d_G; a.M = h.d_M; a.Mt = h.d_Mt; a.F = h.d_F; a.sigma = h.d_sigma;
    a.tau = h.tau; a.td = h.time_dependent ? 1 : 0;
    a.src = src; a.psi = psi; a.status = h.d_status; a.refl = h.d_refl;
    a.fix_kind = h.fix_kind; a.fix_min = (double)h.fix_min; a.fix_counts = h.d_fix_counts;
    if (h.fix_kind)   // the fixup needs the local matrix: rebuild and factor, level by level
        return run_graph(h, 21, src, psi, [&](cudaStream_t st) { return sweep_dispatch<double, true>(h, a, st); });
    const bool flow = h.schedule == 1 && h.p <= 1 && h.nrefl == 0;
    if (flow) {
        cudaError_t e = prepare_flow(h);
        if (e != cudaSuccess) return e;
    }
    if (h.d_inv) {
        cudaError_t e = ensure_factors(h);
        if (e != cudaSuccess) return e;
        if (flow)
            return run_graph(h, 12, src, psi, [&](cudaStream_t st) { return flow_dispatch<0, double>(h, a, h.d_inv, st); });
        return run_graph(h, 2, src, psi, [&](cudaStream_t st) { return cached_dispatch<double>(h, a, h.d_inv, st); });
    }
    if (flow)
        return run_graph(h, 11, src, psi, [&](cudaStream_t st) { return flow_dispatch<1, double>(h, a, nullptr, st); });
    return run_graph(h, 1, src, psi, [&](cudaStream_t st) { return sweep_dispatch<double, true>(h, a, st); });
}

// One angle chunk of the FP64 sweep from stored inverses, in place on the
// staging buffer, on `stream` (graph kinds 40 + c)
cudaError_t launch_sweep_chunk(Handle& h, double* stage, int c, cudaStream_t stream) {
    SweepArgs<double> a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G; a.ndof = h.ndof;
    a.omega = h.d_omega; a.dots = h.d_dots; a.slots = h.d_slots; a.nbrmap = h.d_nbrmap;
    a.Gm = h.d_G; a.M = h.d_M; a.Mt = h.d_Mt; a.F = h.d_F; a.sigma = h.d_sigma;
    a.tau = h.tau; a.td = h.time_dependent ? 1 : 0;
    a.src = stage; a.psi = stage; a.status = h.d_status; a.refl = h.d_refl;
    a.fix_kind = 0; a.fix_min = 0.0; a.fix_counts = nullptr;
    return run_graph_on(h, 40 + c, stage, stage, stream, [&](cudaStream_t st) -> cudaError_t {
        switch (h.dim) {
            case 1: return sweep_chunk<1, 1>(h, a, c, st);
            case 2: return sweep_chunk<2, 1>(h, a, c, st);
            case 3: return sweep_chunk<3, 1>(h, a, c, st);
            default: return cudaErrorNotSupported;
        }
    });
}

bool factor_cache_supported(const Handle& h) { return h.p == 1 && h.dim >= 1 && h.dim <= 3; }

template <int D, int P>
cudaError_t apply_L_launch(Handle& h, const ApplyArgs& a) {
    constexpr int kBlock = 128;
    const long long total = (long long)h.G * h.ne * h.Nw;
    const unsigned grid = (unsigned)((total + kBlock - 1) / kBlock);
    k_apply_L<D, P><<<grid, kBlock, 0, h.stream>>>(a);
    return cudaGetLastError();
}

template <int D, int P>
cudaError_t apply_L_rows_launch(Handle& h, const ApplyArgs& a) {
    constexpr int kBlock = 128;
    const long long total = (long long)h.G * h.ne * h.Nw * ipow(P + 1, D);
    const unsigned grid = (unsigned)((total + kBlock - 1) / kBlock);
    k_apply_L_rows<D, P><<<grid, kBlock, 0, h.stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_apply_L_fp64(Handle& h, const double* x, double* y) {
    ApplyArgs a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G; a.ndof = h.ndof;
    a.omega = h.d_omega; a.dots = h.d_dots; a.slots = h.d_slots; a.nbrmap = h.d_nbrmap;
    a.Gm = h.d_G; a.M = h.d_M; a.Mt = h.d_Mt; a.F = h.d_F; a.sigma = h.d_sigma;
    a.tau = h.tau; a.td = h.time_dependent ? 1 : 0;
    a.x = x; a.y = y;
    switch (h.dim * 10 + h.p) {
        case 10: return apply_L_launch<1, 0>(h, a);
        case 11: return apply_L_launch<1, 1>(h, a);
        case 12: return apply_L_launch<1, 2>(h, a);
        case 13: return apply_L_launch<1, 3>(h, a);
        case 20: return apply_L_launch<2, 0>(h, a);
        case 21: return apply_L_launch<2, 1>(h, a);
        case 22: return apply_L_launch<2, 2>(h, a);
        case 23: return apply_L_launch<2, 3>(h, a);
        case 30: return apply_L_launch<3, 0>(h, a);
        case 31: return apply_L_launch<3, 1>(h, a);
        case 32: return apply_L_launch<3, 2>(h, a);
        case 33: return apply_L_rows_launch<3, 3>(h, a);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace allium
