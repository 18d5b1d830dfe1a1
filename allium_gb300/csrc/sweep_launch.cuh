// Level-by-level launch of the sweep kernel for one arithmetic type.
#pragma once

#include "sweep_kernels.cuh"

namespace allium {

template <int D, int P, typename R, bool PIVOT>
cudaError_t sweep_levels(Handle& h, const SweepArgs<R>& args) {
    constexpr int kBlock = 128;
    for (int l = 0; l < h.num_levels; ++l) {
        const int off = h.h_level_offsets[l];
        const int count = h.h_level_offsets[l + 1] - off;
        if (count == 0) continue;
        const long long threads = (long long)count * h.G;
        const unsigned grid = (unsigned)((threads + kBlock - 1) / kBlock);
        k_sweep_level<D, P, R, PIVOT><<<grid, kBlock, 0, h.stream>>>(args, h.d_level_nodes + off, count);
    }
    return cudaGetLastError();
}

template <typename R, bool PIVOT>
cudaError_t sweep_dispatch(Handle& h, const SweepArgs<R>& a) {
    switch (h.dim * 10 + h.p) {
        case 10: return sweep_levels<1, 0, R, PIVOT>(h, a);
        case 11: return sweep_levels<1, 1, R, PIVOT>(h, a);
        case 12: return sweep_levels<1, 2, R, PIVOT>(h, a);
        case 13: return sweep_levels<1, 3, R, PIVOT>(h, a);
        case 20: return sweep_levels<2, 0, R, PIVOT>(h, a);
        case 21: return sweep_levels<2, 1, R, PIVOT>(h, a);
        case 22: return sweep_levels<2, 2, R, PIVOT>(h, a);
        case 23: return sweep_levels<2, 3, R, PIVOT>(h, a);
        case 30: return sweep_levels<3, 0, R, PIVOT>(h, a);
        case 31: return sweep_levels<3, 1, R, PIVOT>(h, a);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace allium
