// FP32 sweep: FP32 storage and unpivoted FP32 local elimination.
#include "sweep_launch.cuh"

namespace allium {

cudaError_t launch_sweep_fp32(Handle& h, const float* src, float* psi) {
    SweepArgs<float> a;
    a.ne = h.ne; a.Nw = h.Nw; a.G = h.G; a.ndof = h.ndof;
    a.omega = h.d_omega; a.dots = h.f_dots; a.slots = h.d_slots; a.nbrmap = h.d_nbrmap;
    a.Gm = h.f_G; a.M = h.f_M; a.Mt = h.f_Mt; a.F = h.f_F; a.sigma = h.f_sigma;
    a.tau = (float)h.tau; a.td = h.time_dependent ? 1 : 0;
    a.src = src; a.psi = psi; a.status = h.d_status;
    if (h.f_inv) {
        cudaError_t e = ensure_factors(h);
        if (e != cudaSuccess) return e;
        return run_graph(h, 4, src, psi, [&](cudaStream_t st) { return cached_dispatch<float>(h, a, h.f_inv, st); });
    }
    return run_graph(h, 3, src, psi, [&](cudaStream_t st) { return sweep_dispatch<float, false>(h, a, st); });
}

}  // namespace allium
