// FP32 sweep: FP32 storage and unpivoted FP32 local elimination.
#include "sweep_launch.cuh"

namespace allium {

cudaError_t launch_sweep_fp32(Handle& h, const float* src, float* psi) {
    SweepArgs<float> a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G; a.ndof = h.ndof;
    a.omega = h.d_omega; a.dots = h.f_dots; a.slots = h.d_slots; a.nbrmap = h.d_nbrmap;
    a.Gm = h.f_G; a.M = h.f_M; a.Mt = h.f_Mt; a.F = h.f_F; a.sigma = h.f_sigma;
    a.tau = (float)h.tau; a.td = h.time_dependent ? 1 : 0;
    a.src = src; a.psi = psi; a.status = h.d_status; a.refl = h.d_refl;
    a.fix_kind = h.fix_kind; a.fix_min = (float)h.fix_min; a.fix_counts = h.d_fix_counts;
    if (h.schedule == 1 && h.p <= 1 && !h.fix_kind && h.nrefl == 0) {
        cudaError_t e = prepare_flow(h);
        if (e != cudaSuccess) return e;
        return run_graph(h, 13, src, psi, [&](cudaStream_t st) { return flow_dispatch<2, float>(h, a, nullptr, st); });
    }
    return run_graph(h, 3, src, psi, [&](cudaStream_t st) { return sweep_dispatch<float, false>(h, a, st); });
}

template <int D, int P>
cudaError_t sweep_levels_nodes(Handle& h, const SweepArgs<float>& args, cudaStream_t stream) {
    const int kBlock = h.block32;
    for (int l = 0; l < h.num_levels; ++l) {
        const int off = h.h_level_offsets[l];
        const int count = h.h_level_offsets[l + 1] - off;
        if (count == 0) continue;
        const long long threads = (long long)count * h.G;
        if (threads > 0x7fffffffLL) return cudaErrorInvalidValue;
        const unsigned grid = (unsigned)((threads + kBlock - 1) / kBlock);
        k_sweep_nodes<D, P><<<grid, kBlock, 0, stream>>>(args, h.d_level_nodes + off, count);
    }
    return cudaGetLastError();
}

template <int D, int P>
cudaError_t sweep_levels_nodes_cached(Handle& h, const SweepArgs<float>& args, cudaStream_t stream) {
    const int kBlock = h.block32;
    for (int l = 0; l < h.num_levels; ++l) {
        const int off = h.h_level_offsets[l];
        const int count = h.h_level_offsets[l + 1] - off;
        if (count == 0) continue;
        const long long threads = (long long)count * h.G;
        if (threads > 0x7fffffffLL) return cudaErrorInvalidValue;
        const unsigned grid = (unsigned)((threads + kBlock - 1) / kBlock);
        const long long stride = (long long)h.G * h.ne * h.Nw;
        if (h.f_inv_entry_major)
            k_sweep_nodes_cached<D, P, true><<<grid, kBlock, 0, stream>>>(args, h.d_level_nodes + off, count,
                                                                          h.f_inv_nodes, (long long)off * h.G, stride);
        else
            k_sweep_nodes_cached<D, P, false><<<grid, kBlock, 0, stream>>>(args, h.d_level_nodes + off, count,
                                                                           h.f_inv_nodes, (long long)off * h.G, stride);
    }
    return cudaGetLastError();
}

// FP32 copy of the stored FP64 inverses (allocated on first use; if it does
// not fit, the node-major sweep keeps rebuilding its local systems)
static bool ensure_f32_inverses(Handle& h) {
    if (!h.d_inv || h.f_inv_failed) return false;
    if (ensure_factors(h) != cudaSuccess) return false;
    if (h.f_inv_valid) return true;
    const int NN = h.n * h.n;
    const long long total = (long long)h.G * h.ne * h.Nw;
    if (!h.f_inv_nodes) {
        std::lock_guard<std::mutex> lock(cache_lock());
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        const size_t need = (size_t)total * NN * sizeof(float);
        if (need > free_b / 2 || cudaMalloc(&h.f_inv_nodes, need) != cudaSuccess) {
            cudaGetLastError();
            h.f_inv_nodes = nullptr;
            h.f_inv_failed = true;
            return false;
        }
    }
    if (h.f_inv_entry_major) {
        const long long n = total * NN;
        k_inv_to_f32_entries<<<(unsigned)((n + 255) / 256), 256, 0, h.stream>>>(n, h.d_inv, h.f_inv_nodes);
        if (cudaGetLastError() != cudaSuccess) return false;
        h.f_inv_valid = true;
        return true;
    }
    const long long work = total * h.n;
    const unsigned grid = (unsigned)((work + 255) / 256);
    switch (h.n) {
        case 2: k_inv_to_f32<2><<<grid, 256, 0, h.stream>>>(total, total, h.d_inv, h.f_inv_nodes); break;
        case 4: k_inv_to_f32<4><<<grid, 256, 0, h.stream>>>(total, total, h.d_inv, h.f_inv_nodes); break;
        case 8: k_inv_to_f32<8><<<grid, 256, 0, h.stream>>>(total, total, h.d_inv, h.f_inv_nodes); break;
        default: return false;
    }
    if (cudaGetLastError() != cudaSuccess) return false;
    h.f_inv_valid = true;
    return true;
}

cudaError_t launch_sweep_nodes_f32(Handle& h, const float* src, float* psi) {
    if (h.nrefl) return cudaErrorNotSupported;   // node layout: inflow/vacuum boundaries only
    SweepArgs<float> a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G; a.ndof = h.ndof;
    a.omega = h.d_omega; a.dots = h.f_dots; a.slots = h.d_slots; a.nbrmap = h.d_nbrmap;
    a.Gm = h.f_G; a.M = h.f_M; a.Mt = h.f_Mt; a.F = h.f_F; a.sigma = h.f_sigma;
    a.tau = (float)h.tau; a.td = h.time_dependent ? 1 : 0;
    a.src = src; a.psi = psi; a.status = h.d_status; a.refl = h.d_refl;
    a.fix_kind = h.fix_kind; a.fix_min = (float)h.fix_min; a.fix_counts = h.d_fix_counts;
    // with stored inverses (factor cache on) every schedule applies them
    if (h.p == 1 && ensure_f32_inverses(h))
        return run_graph(h, 6, src, psi, [&](cudaStream_t st) -> cudaError_t {
            switch (h.dim) {
                case 1: return sweep_levels_nodes_cached<1, 1>(h, a, st);
                case 2: return sweep_levels_nodes_cached<2, 1>(h, a, st);
                case 3: return sweep_levels_nodes_cached<3, 1>(h, a, st);
                default: return cudaErrorNotSupported;
            }
        });
    if (h.schedule == 1) {
        cudaError_t e = prepare_flow(h);
        if (e != cudaSuccess) return e;
        const FlowArgs f = flow_args(h);
        return run_graph(h, 15, src, psi, [&](cudaStream_t st) -> cudaError_t {
            switch (h.dim * 10 + h.p) {
                case 10: return launch_flow(h, st, k_flow_nodes<1, 0>, 0, a, f, h.d_level_nodes);
                case 20: return launch_flow(h, st, k_flow_nodes<2, 0>, 0, a, f, h.d_level_nodes);
                case 30: return launch_flow(h, st, k_flow_nodes<3, 0>, 0, a, f, h.d_level_nodes);
                case 11: return launch_flow(h, st, k_flow_nodes<1, 1>, 0, a, f, h.d_level_nodes);
                case 21: return launch_flow(h, st, k_flow_nodes<2, 1>, 0, a, f, h.d_level_nodes);
                case 31: return launch_flow(h, st, k_flow_nodes<3, 1>, 0, a, f, h.d_level_nodes);
                default: return cudaErrorNotSupported;
            }
        });
    }
    return run_graph(h, 5, src, psi, [&](cudaStream_t st) -> cudaError_t {
        switch (h.dim * 10 + h.p) {
            case 10: return sweep_levels_nodes<1, 0>(h, a, st);
            case 20: return sweep_levels_nodes<2, 0>(h, a, st);
            case 30: return sweep_levels_nodes<3, 0>(h, a, st);
            case 11: return sweep_levels_nodes<1, 1>(h, a, st);
            case 21: return sweep_levels_nodes<2, 1>(h, a, st);
            case 31: return sweep_levels_nodes<3, 1>(h, a, st);
            default: return cudaErrorNotSupported;
        }
    });
}

cudaError_t launch_layout(Handle& h, int to_nodes, const void* in, void* out) {
    const long long total = h.psi_size;
    const int b = 256;
    const unsigned grid = (unsigned)((total + b - 1) / b);
    if (to_nodes)
        k_right_to_nodes<<<grid, b, 0, h.stream>>>(h.ne, h.Nw, h.G, h.n, h.ndof, (const double*)in, (float*)out);
    else
        k_nodes_to_right<<<grid, b, 0, h.stream>>>(h.ne, h.Nw, h.G, h.n, h.ndof, (const float*)in, (double*)out);
    return cudaGetLastError();
}

cudaError_t launch_scatter_nodes(Handle& h, const double* sigma_s, const double* phi, const float* qn, float* out) {
    const long long total = (long long)h.G * h.ndof;
    const int b = 256;
    k_scatter_nodes<<<(unsigned)((total + b - 1) / b), b, 0, h.stream>>>(h.ne, h.Nw, h.G, h.n, h.ndof, h.wsum, h.d_Mt,
                                                                        sigma_s, phi, qn, out);
    return cudaGetLastError();
}

cudaError_t launch_moments_nodes(Handle& h, const float* psi, double* phi) {
    const long long total = (long long)h.G * h.ndof;
    const int b = 256;
    k_moments_nodes<<<(unsigned)((total + b - 1) / b), b, 0, h.stream>>>(h.ne, h.Nw, h.G, h.n, h.ndof, h.d_weights, psi, phi);
    return cudaGetLastError();
}

}  // namespace allium
