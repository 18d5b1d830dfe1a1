// Thermal radiative transfer pieces around the sweep: multigroup Planck
// emission and its temperature gradient, the gray material energy balance with
// the inverse of its gradient, the absorption collapse sum_g M_sigma_g phi_g,
// block-diagonal products, the time source of backward Euler and a power-law
// opacity.  These are the operators LinearizedTRTOperator::Mult
// (src/trt_linearized.cpp:230-312) applies between sweeps.
#include "geometry.cuh"
#include "planck.cuh"

namespace allium {

namespace {

constexpr int kTrtMaxN = 16;     // local DOFs (1D/2D p <= 3, 3D p <= 1)
constexpr int kTrtMaxQ = 27;     // points of the (p + 2)^dim rule: 2D p <= 3 -> 25, 3D p = 1 -> 27

struct EmissionArgs {
    RefTables t;
    int ne, G;
    long long ndof;
    const double* corners;
    const double* T;         // [Ndof]
    const double* sigma;     // [G][Ne] absorption opacity per cell
    const double* bounds;    // [G + 1]
    double K;                // a c ("StefanBoltzmann" of src/constants.hpp)
    double cv_dt;            // heat capacity / time step
    const double* Mt;        // [Ne][n][n] MassIntegrator matrices
    double* emission;        // [G][Ndof] or null
    double* dB;              // [G][Ne][n][n] or null
    double* bt;              // [Ndof] or null
    double* bt_inv;          // [Ne][n][n] or null
    int* status;
};

// Planck and Rosseland fractions of group g at temperature T for the lanes of a
// warp holding groups g = base + lane: F(E_{g+1}/T) - F(E_g/T) with F = 0 below
// the first group and F = 1 above the last (EvalSpectrum, src/planck.hpp:207-222).
// All 32 lanes call it; lanes past the last group pass g = G - 1.
__device__ inline void group_fractions(const double* bounds, int G, int g, double T, double& bp, double& br) {
    const int lane = threadIdx.x & 31;
    double fp_hi = 1.0, fr_hi = 1.0;
    if (g < G - 1) {
        const double x = bounds[g + 1] / T;
        fp_hi = planck_fraction(x);
        fr_hi = rosseland_from_planck(x, fp_hi);
    }
    double fp_lo = __shfl_up_sync(0xffffffffu, fp_hi, 1);
    double fr_lo = __shfl_up_sync(0xffffffffu, fr_hi, 1);
    if (lane == 0) {
        if (g == 0) {
            fp_lo = 0.0;
            fr_lo = 0.0;
        } else {
            const double x = bounds[g] / T;
            fp_lo = planck_fraction(x);
            fr_lo = rosseland_from_planck(x, fp_lo);
        }
    }
    bp = fp_hi - fp_lo;
    br = fr_hi - fr_lo;
}

__device__ inline double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Basis values and reference weights of rule r at its tensor points (shared by
// every cell of the block).  Returns the number of points.
__device__ inline int rule_table(const RefTables& t, int r, double (*phi)[kTrtMaxN], double* xq, double* wq) {
    const int m = t.rn[r];
    int nq = 1;
    for (int d = 0; d < t.dim; ++d) nq *= m;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        double xi[3] = {0.0, 0.0, 0.0}, w = 1.0;
        int rq = q;
        for (int d = 0; d < t.dim; ++d) {
            const int id = rq % m;
            rq /= m;
            xi[d] = t.rx[r][id];
            w *= t.rw[r][id];
        }
        double v[3][kMaxOrder + 1];
        for (int d = 0; d < t.dim; ++d) lagrange1d(t.n1, t.nodes, xi[d], v[d], nullptr);
        for (int i = 0; i < t.n; ++i) {
            int id[3];
            dof_index(t.dim, t.n1, i, id);
            double ph = 1.0;
            for (int d = 0; d < t.dim; ++d) ph *= v[d][id[d]];
            phi[q][i] = ph;
        }
        for (int d = 0; d < 3; ++d) xq[q * 3 + d] = xi[d];
        wq[q] = w;
    }
    return nq;
}

// One warp per cell, lanes over groups (32 at a time).
//   pass 1, PlanckEmissionNFI (src/trt_integrators.cpp:56-86, 120-152), rule
//   order 2p + 1: emission_g(i) = int sigma_g K T^4 b_g(T) phi_i and
//   dB_g(i, j) = int sigma_g 4 K T^3 r_g(T) phi_i phi_j;
//   pass 2, GrayPlanckEmissionNFI (:154-208) at order 2p + 2 plus
//   MassIntegrator(c_v / dt) (exe/scallion.cpp:755-765):
//   bt(i) = int (sum_g sigma_g b_g) K T^4 phi_i + c_v/dt (Mt T)_i and its
//   gradient, inverted in registers (one row per lane, Gauss-Jordan with
//   partial pivoting, first largest pivot).
__global__ void __launch_bounds__(128) k_trt_emission(EmissionArgs s) {
    __shared__ double phi6[kTrtMaxQ][kTrtMaxN], phi7[kTrtMaxQ][kTrtMaxN];
    __shared__ double x6[kTrtMaxQ * 3], x7[kTrtMaxQ * 3], w6[kTrtMaxQ], w7[kTrtMaxQ];
    const RefTables& t = s.t;
    const int nq6 = rule_table(t, 6, phi6, x6, w6);
    const int nq7 = rule_table(t, 7, phi7, x7, w7);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int e = blockIdx.x * 4 + warp;
    if (e >= s.ne) return;
    const int dim = t.dim, n = t.n, nc = 1 << dim;
    double X[24];
    for (int q = 0; q < nc * dim; ++q) X[q] = s.corners[(size_t)e * nc * dim + q];
    double Te[kTrtMaxN];
    for (int i = 0; i < n; ++i) Te[i] = s.T[(size_t)e * n + i];

    // ---- pass 1: multigroup emission and its gradient
    if (s.emission || s.dB) {
        for (int base = 0; base < s.G; base += 32) {
            const int g = base + lane;
            const bool on = g < s.G;
            const double sg = on ? s.sigma[(size_t)g * s.ne + e] : 0.0;
            double em[kTrtMaxN], sq[kTrtMaxQ];
            for (int i = 0; i < n; ++i) em[i] = 0.0;
            for (int q = 0; q < nq6; ++q) {
                double J[3][3], A[3][3];
                cell_jacobian(dim, X, x6 + 3 * q, J, nullptr);
                const double wd = adjugate(dim, J, A) * w6[q];
                double Tq = 0.0;
                for (int i = 0; i < n; ++i) Tq += phi6[q][i] * Te[i];
                double bp, br;
                group_fractions(s.bounds, s.G, on ? g : s.G - 1, Tq, bp, br);
                const double T3 = Tq * Tq * Tq;
                const double c = wd * s.K * T3 * Tq * bp * sg;
                for (int i = 0; i < n; ++i) em[i] += c * phi6[q][i];
                sq[q] = wd * 4.0 * s.K * T3 * br * sg;
            }
            if (!on) continue;
            if (s.emission)
                for (int i = 0; i < n; ++i) s.emission[(size_t)g * s.ndof + (size_t)e * n + i] = em[i];
            if (s.dB) {
                double* out = s.dB + ((size_t)g * s.ne + e) * n * n;
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j) {
                        double acc = 0.0;
                        for (int q = 0; q < nq6; ++q) acc += sq[q] * phi6[q][i] * phi6[q][j];
                        out[i * n + j] = acc;
                    }
            }
        }
    }

    // ---- pass 2: gray energy balance residual and inverse gradient
    if (s.bt || s.bt_inv) {
        double res[kTrtMaxN];
        double row[kTrtMaxN];   // lane i < n holds row i of the gradient
        for (int i = 0; i < n; ++i) { res[i] = 0.0; row[i] = 0.0; }
        const int li = lane < n ? lane : 0;
        for (int q = 0; q < nq7; ++q) {
            double J[3][3], A[3][3];
            cell_jacobian(dim, X, x7 + 3 * q, J, nullptr);
            const double wd = adjugate(dim, J, A) * w7[q];
            double Tq = 0.0;
            for (int i = 0; i < n; ++i) Tq += phi7[q][i] * Te[i];
            double sb = 0.0, sr = 0.0;
            for (int base = 0; base < s.G; base += 32) {
                const int g = base + lane;
                const bool on = g < s.G;
                double bp, br;
                group_fractions(s.bounds, s.G, on ? g : s.G - 1, Tq, bp, br);
                const double sg = on ? s.sigma[(size_t)g * s.ne + e] : 0.0;
                if (on) { sb += sg * bp; sr += sg * br; }
            }
            sb = warp_sum(sb);
            sr = warp_sum(sr);
            const double T3 = Tq * Tq * Tq;
            const double c = sb * wd * s.K * T3 * Tq;
            for (int i = 0; i < n; ++i) res[i] += c * phi7[q][i];
            const double cg = sr * 4.0 * s.K * T3 * wd * phi7[q][li];
            for (int j = 0; j < n; ++j) row[j] += cg * phi7[q][j];
        }
        const double* Mt = s.Mt + (size_t)e * n * n;
        if (s.bt && lane == 0)
            for (int i = 0; i < n; ++i) {
                double mt = 0.0;
                for (int j = 0; j < n; ++j) mt += Mt[i * n + j] * Te[j];
                s.bt[(size_t)e * n + i] = res[i] + s.cv_dt * mt;
            }
        if (s.bt_inv) {
            double inv[kTrtMaxN];
            for (int j = 0; j < n; ++j) {
                row[j] += s.cv_dt * Mt[li * n + j];
                inv[j] = (lane == j) ? 1.0 : 0.0;
            }
            bool ok = true;
            for (int k = 0; k < n; ++k) {
                double v = (lane >= k && lane < n) ? fabs(row[k]) : -1.0;
                int who = lane;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
                    const int w2 = __shfl_xor_sync(0xffffffffu, who, o);
                    if (v2 > v || (v2 == v && w2 < who)) { v = v2; who = w2; }
                }
                if (!(v > 0.0)) { ok = false; break; }
                // exchange rows k and who, then eliminate column k
                for (int j = 0; j < n; ++j) {
                    const double ak = __shfl_sync(0xffffffffu, row[j], k), ap = __shfl_sync(0xffffffffu, row[j], who);
                    const double bk = __shfl_sync(0xffffffffu, inv[j], k), bq = __shfl_sync(0xffffffffu, inv[j], who);
                    if (lane == k) { row[j] = ap; inv[j] = bq; }
                    else if (lane == who) { row[j] = ak; inv[j] = bk; }
                }
                const double piv = __shfl_sync(0xffffffffu, row[k], k);
                const double f = row[k] / piv;
                for (int j = 0; j < n; ++j) {
                    const double pk = __shfl_sync(0xffffffffu, row[j], k);
                    const double qk = __shfl_sync(0xffffffffu, inv[j], k);
                    if (lane == k) { row[j] = pk / piv; inv[j] = qk / piv; }
                    else { row[j] -= f * pk; inv[j] -= f * qk; }
                }
            }
            if (!ok) {
                if (lane == 0) atomicOr(s.status, kErrSingular);
            } else if (lane < n) {
                for (int j = 0; j < n; ++j) s.bt_inv[((size_t)e * n + lane) * n + j] = inv[j];
            }
        }
    }
}

// y_b[e] = alpha B_b[e] x_b[e] (+ y) for nb block sets; x shared by all sets
// when x_stride == 0
__global__ void k_block_apply(int ne, int n, int nb, long long ndof, const double* __restrict__ B,
                              const double* __restrict__ x, long long x_stride, double* __restrict__ y,
                              double alpha, int accumulate) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nb * ne * n) return;
    const int i = (int)(t % n);
    const long long be = t / n;
    const int e = (int)(be % ne), b = (int)(be / ne);
    const double* Bm = B + ((size_t)b * ne + e) * n * n + (size_t)i * n;
    const double* xe = x + (size_t)b * x_stride + (size_t)e * n;
    double acc = 0.0;
    for (int j = 0; j < n; ++j) acc += Bm[j] * xe[j];
    double* ye = y + (size_t)b * ndof + (size_t)e * n + i;
    *ye = accumulate ? *ye + alpha * acc : alpha * acc;
}

// sum_g M_{sigma_g} phi_g: MGMassIntegrator(total) collapsed over groups
// (scallion.cpp:786-797, Mtot_collapse)
__global__ void k_absorption(int ne, int n, int G, long long ndof, const double* __restrict__ M,
                             const double* __restrict__ sigma, const double* __restrict__ phi,
                             double* __restrict__ y, double alpha, int accumulate) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ne * n) return;
    const int i = (int)(t % n), e = (int)(t / n);
    const double* Me = M + (size_t)e * n * n + (size_t)i * n;
    double acc = 0.0;
    for (int g = 0; g < G; ++g) {
        const double* pg = phi + (size_t)g * ndof + (size_t)e * n;
        double m = 0.0;
        for (int j = 0; j < n; ++j) m += Me[j] * pg[j];
        acc += sigma[(size_t)g * ne + e] * m;
    }
    y[t] = accumulate ? y[t] + alpha * acc : alpha * acc;
}

// out(g, a, e.) = q(g, a, e.) + tau Mt[e] psi_prev(g, a, e.): SNTimeMassMatrix::Mult
// (src/tvector.cpp:76-95) and the backward-Euler source (exe/scallion.cpp:1358-1359).
// Reads the whole cell block before writing, so out may alias psi_prev or q.
template <int N>
__global__ void k_time_source(int ne, long long blocks, const double* __restrict__ Mt, const double* psi_prev,
                              const double* q, double tau, double* out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= blocks) return;
    const int e = (int)(t % ne);
    const double* M = Mt + (size_t)e * N * N;
    const size_t off = (size_t)t * N;
    double x[N], b[N];
#pragma unroll
    for (int j = 0; j < N; ++j) { x[j] = psi_prev[off + j]; b[j] = q ? q[off + j] : 0.0; }
#pragma unroll
    for (int i = 0; i < N; ++i) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < N; ++j) acc += __ldg(M + i * N + j) * x[j];
        out[off + i] = b[i] + tau * acc;
    }
}

// sigma_g(e) = C nu_g^a T_c^b with T_c the temperature at the cell centre:
// the analytic opacity of src/opacity.cpp:47-63 evaluated at the group's
// geometric midpoint, projected onto piecewise constants (sigma_fe_order = 0)
__global__ void k_powerlaw_opacity(RefTables t, int ne, int G, const double* __restrict__ T, const double* __restrict__ nu,
                                   double C, double a, double b, double* __restrict__ sigma) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double xi[3] = {0.5, 0.5, 0.5}, phi[64];
    double v[3][kMaxOrder + 1];
    for (int d = 0; d < t.dim; ++d) lagrange1d(t.n1, t.nodes, xi[d], v[d], nullptr);
    double Tc = 0.0;
    for (int i = 0; i < t.n; ++i) {
        int id[3];
        dof_index(t.dim, t.n1, i, id);
        double ph = 1.0;
        for (int d = 0; d < t.dim; ++d) ph *= v[d][id[d]];
        phi[i] = ph;
        Tc += ph * T[(size_t)e * t.n + i];
    }
    const double tb = pow(Tc, b);
    for (int g = 0; g < G; ++g) sigma[(size_t)g * ne + e] = C * pow(nu[g], a) * tb;
}

}  // namespace

bool trt_supported(const Handle& h) { return h.n <= kTrtMaxN && h.lump == 0; }

cudaError_t launch_trt_emission(Handle& h, const double* bounds, const double* sigma, const double* T, double K,
                                double cv_dt, double* emission, double* dB, double* bt, double* bt_inv) {
    EmissionArgs a;
    a.t = h.ref; a.ne = h.ne; a.G = h.G; a.ndof = h.ndof;
    a.corners = h.d_corners; a.T = T; a.sigma = sigma; a.bounds = bounds; a.K = K; a.cv_dt = cv_dt;
    a.Mt = h.d_Mt; a.emission = emission; a.dB = dB; a.bt = bt; a.bt_inv = bt_inv; a.status = h.d_status;
    k_trt_emission<<<(h.ne + 3) / 4, 128, 0, h.stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_block_apply(Handle& h, const double* B, int nb, const double* x, long long x_stride, double* y,
                               double alpha, int accumulate) {
    const long long total = (long long)nb * h.ne * h.n;
    k_block_apply<<<(unsigned)((total + 255) / 256), 256, 0, h.stream>>>(h.ne, h.n, nb, h.ndof, B, x, x_stride, y, alpha,
                                                                         accumulate);
    return cudaGetLastError();
}

cudaError_t launch_absorption(Handle& h, const double* sigma, const double* phi, double* y, double alpha, int accumulate) {
    const long long total = (long long)h.ne * h.n;
    k_absorption<<<(unsigned)((total + 255) / 256), 256, 0, h.stream>>>(h.ne, h.n, h.G, h.ndof, h.d_M, sigma, phi, y,
                                                                        alpha, accumulate);
    return cudaGetLastError();
}

cudaError_t launch_time_source(Handle& h, const double* psi_prev, const double* q, double tau, double* out) {
    const long long blocks = (long long)h.G * h.Nw * h.ne;
    const unsigned grid = (unsigned)((blocks + 127) / 128);
#define TS(NN) k_time_source<NN><<<grid, 128, 0, h.stream>>>(h.ne, blocks, h.d_Mt, psi_prev, q, tau, out); break
    switch (h.n) {
        case 1: TS(1);
        case 2: TS(2);
        case 3: TS(3);
        case 4: TS(4);
        case 8: TS(8);
        case 9: TS(9);
        case 16: TS(16);
        case 27: TS(27);
        default: return cudaErrorInvalidValue;
    }
#undef TS
    return cudaGetLastError();
}

cudaError_t launch_powerlaw_opacity(Handle& h, const double* T, const double* nu, double C, double a, double b,
                                    double* sigma) {
    k_powerlaw_opacity<<<(h.ne + 127) / 128, 128, 0, h.stream>>>(h.ref, h.ne, h.G, T, nu, C, a, b, sigma);
    return cudaGetLastError();
}

}  // namespace allium
