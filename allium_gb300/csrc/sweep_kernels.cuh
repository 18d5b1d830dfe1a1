// The upwind sweep node kernel and the forward transport operator, templated
// on dimension D, order P and the arithmetic type R (double or float).
//
// Work unit: one thread per (cell, angle, group) node of one wavefront level.
// Inside a level the nodes are sorted by (cell, angle), so the threads of a
// warp share a cell and its matrices are read once per warp (broadcast).  The
// thread assembles the (P+1)^D local system in registers
//     A = sum_d Omega_d G_d + sum_{outflow faces} (Omega.n) F_self + sigma_g M [+ tau Mt]
//     b = q(g,a,e) + sum_{inflow faces} |Omega.n| F_self u_upwind
// (allium src/sweep.cpp:365-475), factors it in registers and writes psi(g,a,e).
// The upwind trace u_upwind is the neighbour's psi read through the neighbour
// DOF map of the shared face; on Gauss-Lobatto nodes the face coupling block
// F(self, nbr) equals F_self with its columns permuted by that map.
#pragma once

#include "geometry.cuh"

namespace allium {

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

template <typename R>
struct SweepArgs {
    int ne, Nw, G;
    long long ndof;
    const double* omega;
    const double* normals;
    const Slot* slots;
    const uint8_t* nbrmap;
    const R* Gm;      // [ne][D][N][N]
    const R* M;       // [ne][N][N]   unit-coefficient mass
    const R* Mt;      // [ne][N][N]   time mass (when td)
    const R* F;       // [ne][2D][NF][NF]
    const R* sigma;   // [G][ne]
    R tau;
    int td;
    const R* src;
    R* psi;
    int* status;
};

__device__ __forceinline__ double fma_r(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_r(float a, float b, float c) { return fmaf(a, b, c); }

// Gaussian elimination on registers.  PIVOT: partial pivoting on the largest
// magnitude (first one on ties), the order mfem::LUFactors::Factor uses.  The
// right-hand side is eliminated alongside, and back substitution multiplies
// by the stored pivot reciprocals.
template <int N, bool PIVOT, typename R>
__device__ __forceinline__ bool solve_local(R (&A)[N][N], R (&b)[N]) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (PIVOT) {
            R amax = fabs(A[k][k]);
            int piv = k;
#pragma unroll
            for (int i = k + 1; i < N; ++i) {
                const R v = fabs(A[i][k]);
                if (v > amax) { amax = v; piv = i; }
            }
#pragma unroll
            for (int i = k + 1; i < N; ++i) {
                const bool sw = (piv == i);
#pragma unroll
                for (int j = k; j < N; ++j) {
                    const R x = A[k][j], y = A[i][j];
                    A[k][j] = sw ? y : x;
                    A[i][j] = sw ? x : y;
                }
                const R x = b[k], y = b[i];
                b[k] = sw ? y : x;
                b[i] = sw ? x : y;
            }
        }
        const R pk = A[k][k];
        ok = ok && (pk != R(0));
        const R inv = R(1) / pk;
#pragma unroll
        for (int i = k + 1; i < N; ++i) {
            const R l = A[i][k] * inv;
#pragma unroll
            for (int j = k + 1; j < N; ++j) A[i][j] = fma_r(-l, A[k][j], A[i][j]);
            b[i] = fma_r(-l, b[k], b[i]);
        }
        A[k][k] = inv;
    }
#pragma unroll
    for (int k = N - 1; k >= 0; --k) {
        const R x = b[k] * A[k][k];
        b[k] = x;
#pragma unroll
        for (int i = 0; i < k; ++i) b[i] = fma_r(-A[i][k], x, b[i]);
    }
    return ok;
}

template <int D, int P, typename R, bool PIVOT>
__global__ void __launch_bounds__(128) k_sweep_level(SweepArgs<R> s, const int* __restrict__ nodes, int count) {
    constexpr int N1 = P + 1;
    constexpr int N = ipow(N1, D);
    constexpr int NF = ipow(N1, D - 1);
    constexpr int NFACE = 2 * D;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)count * s.G) return;
    const int node = nodes[t / s.G];
    const int g = (int)(t % s.G);
    const int e = node / s.Nw;
    const int a = node - e * s.Nw;

    double om[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < D; ++d) om[d] = s.omega[a * D + d];

    R A[N][N];
    {
        const R* Gm = s.Gm + (size_t)e * D * N * N;
        const R* M = s.M + (size_t)e * N * N;
        const R sg = s.sigma[(size_t)g * s.ne + e];
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = 0; j < N; ++j) {
                R v = R(om[0]) * Gm[i * N + j];
#pragma unroll
                for (int d = 1; d < D; ++d) v = fma_r(R(om[d]), Gm[d * N * N + i * N + j], v);
                A[i][j] = fma_r(sg, M[i * N + j], v);
            }
        if (s.td) {
            const R* Mt = s.Mt + (size_t)e * N * N;
#pragma unroll
            for (int i = 0; i < N; ++i)
#pragma unroll
                for (int j = 0; j < N; ++j) A[i][j] = fma_r(s.tau, Mt[i * N + j], A[i][j]);
        }
    }

    double dots[NFACE];
    int nbrs[NFACE];
#pragma unroll
    for (int k = 0; k < NFACE; ++k) {
        const Slot q = s.slots[(size_t)e * NFACE + k];
        double nr[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < D; ++d) nr[d] = s.normals[(size_t)q.face * D + d];
        const double d1 = dot_exact(D, om, nr);
        const double dk = q.side ? -d1 : d1;
        dots[k] = dk;
        nbrs[k] = q.nbr;
        if (dk > 0.0) {
            const R* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
            const R rd = R(dk);
#pragma unroll
            for (int ii = 0; ii < NF; ++ii)
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) {
                    const int fi = face_dof(D, P, k, ii), fj = face_dof(D, P, k, jj);
                    A[fi][fj] = fma_r(rd, F[ii * NF + jj], A[fi][fj]);
                }
        }
    }

    R b[N];
    {
        const R* src = s.src + psi_index(s.ndof, s.Nw, g, a, (long long)e * N);
#pragma unroll
        for (int i = 0; i < N; ++i) b[i] = src[i];
    }
#pragma unroll
    for (int k = 0; k < NFACE; ++k) {
        if (dots[k] < 0.0 && nbrs[k] >= 0) {
            const uint8_t* map = s.nbrmap + ((size_t)e * NFACE + k) * NF;
            const R* up = s.psi + psi_index(s.ndof, s.Nw, g, a, (long long)nbrs[k] * N);
            R u[NF];
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) u[jj] = up[map[jj]];
            const R* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
            const R rd = R(-dots[k]);
#pragma unroll
            for (int ii = 0; ii < NF; ++ii) {
                R acc = R(0);
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) acc = fma_r(F[ii * NF + jj], u[jj], acc);
                const int fi = face_dof(D, P, k, ii);
                b[fi] = fma_r(rd, acc, b[fi]);
            }
        }
    }

    if (!solve_local<N, PIVOT>(A, b)) atomicOr(s.status, kErrSingular);

    R* out = s.psi + psi_index(s.ndof, s.Nw, g, a, (long long)e * N);
#pragma unroll
    for (int i = 0; i < N; ++i) out[i] = b[i];
}

// y = L x (AdvectionOperator::Mult, src/sweep.cpp:1246-1387) from the cell's
// point of view: y_e = (sigma M + tau Mt + sum_d Omega_d G_d) x_e
//   + sum_{faces, Omega.n > 0} (Omega.n) F_self x_e
//   + sum_{interior faces, Omega.n < 0} (Omega.n) F_self u_upwind(x_nbr).
struct ApplyArgs {
    int ne, Nw, G;
    long long ndof;
    const double* omega;
    const double* normals;
    const Slot* slots;
    const uint8_t* nbrmap;
    const double *Gm, *M, *Mt, *F, *sigma;
    double tau;
    int td;
    const double* x;
    double* y;
};

template <int D, int P>
__global__ void __launch_bounds__(128) k_apply_L(ApplyArgs s) {
    constexpr int N1 = P + 1;
    constexpr int N = ipow(N1, D);
    constexpr int NF = ipow(N1, D - 1);
    constexpr int NFACE = 2 * D;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)s.G * s.ne * s.Nw;
    if (t >= total) return;
    const int a = (int)(t % s.Nw);
    const long long r = t / s.Nw;
    const int e = (int)(r % s.ne);
    const int g = (int)(r / s.ne);
    double om[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < D; ++d) om[d] = s.omega[a * D + d];
    const double* xe = s.x + psi_index(s.ndof, s.Nw, g, a, (long long)e * N);
    double xv[N], y[N];
#pragma unroll
    for (int i = 0; i < N; ++i) xv[i] = xe[i];
    const double* Gm = s.Gm + (size_t)e * D * N * N;
    const double* M = s.M + (size_t)e * N * N;
    const double sg = s.sigma[(size_t)g * s.ne + e];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        double m = 0.0, gr = 0.0, mt = 0.0;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            m = fma(M[i * N + j], xv[j], m);
            double c = om[0] * Gm[i * N + j];
#pragma unroll
            for (int d = 1; d < D; ++d) c = fma(om[d], Gm[d * N * N + i * N + j], c);
            gr = fma(c, xv[j], gr);
        }
        if (s.td) {
            const double* Mt = s.Mt + (size_t)e * N * N;
#pragma unroll
            for (int j = 0; j < N; ++j) mt = fma(Mt[i * N + j], xv[j], mt);
        }
        y[i] = fma(sg, m, fma(s.tau, mt, gr));
    }
#pragma unroll
    for (int k = 0; k < NFACE; ++k) {
        const Slot q = s.slots[(size_t)e * NFACE + k];
        double nr[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < D; ++d) nr[d] = s.normals[(size_t)q.face * D + d];
        const double d1 = dot_exact(D, om, nr);
        const double dk = q.side ? -d1 : d1;
        const double* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
        if (dk > 0.0) {
#pragma unroll
            for (int ii = 0; ii < NF; ++ii) {
                double acc = 0.0;
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) acc = fma(F[ii * NF + jj], xv[face_dof(D, P, k, jj)], acc);
                const int fi = face_dof(D, P, k, ii);
                y[fi] = fma(dk, acc, y[fi]);
            }
        } else if (dk < 0.0 && q.nbr >= 0) {
            const uint8_t* map = s.nbrmap + ((size_t)e * NFACE + k) * NF;
            const double* up = s.x + psi_index(s.ndof, s.Nw, g, a, (long long)q.nbr * N);
            double u[NF];
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) u[jj] = up[map[jj]];
#pragma unroll
            for (int ii = 0; ii < NF; ++ii) {
                double acc = 0.0;
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) acc = fma(F[ii * NF + jj], u[jj], acc);
                const int fi = face_dof(D, P, k, ii);
                y[fi] = fma(dk, acc, y[fi]);
            }
        }
    }
    double* ye = s.y + psi_index(s.ndof, s.Nw, g, a, (long long)e * N);
#pragma unroll
    for (int i = 0; i < N; ++i) ye[i] = y[i];
}

}  // namespace allium
