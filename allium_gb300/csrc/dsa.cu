// Modified-interior-penalty (MIP) diffusion operator for diffusion synthetic
// acceleration, assembled and applied on the GPU.
//
// InteriorPenaltyDiscretization::GetOperator (src/moment_discretization.cpp:
// 73-110) with the "scalar mip" settings of exe/chive.cpp:663-672:
//   K = DiffusionIntegrator(D = 1/(3 sigma_t)) + MassIntegrator(sigma_a)
//     + MIPDiffusionIntegrator(D, sigma = -1, kappa, lower bound) on interior faces
//     + BoundaryMassIntegrator(alpha_bdr) on inflow (Marshak) boundaries
//     (+ tau MassIntegrator for time-dependent problems),
// with the face integrator of src/moment_integrators.cpp:3-200: symmetric
// interior penalty with penalty max(kappa (D1/h1 + D2/h2)/2, lower bound),
// h = det J / |n| per side.
//
// Storage: per (group, cell) the self block and one block per local face
// (the coupling to the neighbour across it; zero on boundary faces), each
// n x n row major.  One thread assembles one row of all blocks of its cell.
#include "geometry.cuh"

namespace allium {

namespace {

constexpr int kDsaMaxN = 16;   // 1D/2D p <= 3, 3D p <= 1

struct DsaArgs {
    RefTables t;
    int ne, G;
    long long ndof;
    const double* corners;
    const Slot* slots;
    const FaceOrient* orient;
    const double* sigma_t;   // [G][Ne]
    const double* sigma_s;   // [G][Ne]
    const double* Mt;        // [Ne][n][n] MassIntegrator mass
    double kappa, penalty_min, alpha_bdr, tau;
    double* blocks;          // [G][Ne][1 + 2 dim][n][n]
};

// basis values and physical gradients of all local DOFs at reference point xi
__device__ inline double basis_grad(const RefTables& t, const double* X, const double* xi, double* phi,
                                    double (*gx)[3], double J[3][3], double A[3][3]) {
    cell_jacobian(t.dim, X, xi, J, nullptr);
    const double det = adjugate(t.dim, J, A);
    double v[3][kMaxOrder + 1], dv[3][kMaxOrder + 1];
    for (int d = 0; d < t.dim; ++d) lagrange1d(t.n1, t.nodes, xi[d], v[d], dv[d]);
    for (int i = 0; i < t.n; ++i) {
        int id[3];
        dof_index(t.dim, t.n1, i, id);
        double ph = 1.0, gr[3];
        for (int q = 0; q < t.dim; ++q) {
            double g = 1.0;
            for (int d = 0; d < t.dim; ++d) g *= (d == q) ? dv[d][id[d]] : v[d][id[d]];
            gr[q] = g;
            ph *= v[q][id[q]];
        }
        phi[i] = ph;
        // grad_x phi = J^{-T} grad_xi phi = A^T grad_xi phi / det
        for (int r = 0; r < t.dim; ++r) {
            double s = 0.0;
            for (int q = 0; q < t.dim; ++q) s += A[q][r] * gr[q];
            gx[i][r] = s / det;
        }
    }
    return det;
}

__global__ void __launch_bounds__(128) k_dsa_assemble(DsaArgs s) {
    const RefTables& t = s.t;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = t.n, dim = t.dim, nface = 2 * dim, nc = 1 << dim;
    if (tid >= (long long)s.G * s.ne * n) return;
    const int i = (int)(tid % n);
    const long long ge = tid / n;
    const int e = (int)(ge % s.ne), g = (int)(ge / s.ne);
    double X[24], Y[24];
    for (int q = 0; q < nc * dim; ++q) X[q] = s.corners[(size_t)e * nc * dim + q];
    const double st = s.sigma_t[(size_t)g * s.ne + e];
    const double De = 1.0 / (3.0 * st);
    const double sa = st - s.sigma_s[(size_t)g * s.ne + e];
    double* out = s.blocks + (((size_t)g * s.ne + e) * (1 + nface)) * n * n + (size_t)i * n;

    double row[kDsaMaxN];
    for (int j = 0; j < n; ++j) row[j] = 0.0;
    double phi[kDsaMaxN], gx[kDsaMaxN][3], J[3][3], A[3][3];

    // volume: int D grad phi_i . grad phi_j (rule 8) + (sigma_a + tau) Mt
    {
        const int m = t.rn[8];
        int nq = 1;
        for (int d = 0; d < dim; ++d) nq *= m;
        for (int q = 0; q < nq; ++q) {
            double xi[3] = {0, 0, 0}, w = 1.0;
            int rq = q;
            for (int d = 0; d < dim; ++d) { const int id = rq % m; rq /= m; xi[d] = t.rx[8][id]; w *= t.rw[8][id]; }
            const double det = basis_grad(t, X, xi, phi, gx, J, A);
            const double c = w * det * De;
            for (int j = 0; j < n; ++j) {
                double dd = 0.0;
                for (int r = 0; r < dim; ++r) dd += gx[i][r] * gx[j][r];
                row[j] += c * dd;
            }
        }
        const double* M = s.Mt + (size_t)e * n * n + (size_t)i * n;
        for (int j = 0; j < n; ++j) row[j] += (sa + s.tau) * M[j];
    }

    // faces (rule 6: p + 1 points per face axis)
    const int mf = t.rn[6];
    int nqf = 1;
    for (int d = 0; d < dim - 1; ++d) nqf *= mf;
    for (int k = 0; k < nface; ++k) {
        const Slot sl = s.slots[(size_t)e * nface + k];
        double nbr_row[kDsaMaxN];
        for (int j = 0; j < n; ++j) nbr_row[j] = 0.0;
        const bool interior = sl.nbr >= 0;
        const bool marshak = sl.nbr == -1;
        if (interior || marshak) {
            FaceOrient fo{};
            double Dm = 0.0;
            if (interior) {
                fo = s.orient[(size_t)e * nface + k];
                for (int q = 0; q < nc * dim; ++q) Y[q] = s.corners[(size_t)sl.nbr * nc * dim + q];
                Dm = 1.0 / (3.0 * s.sigma_t[(size_t)g * s.ne + sl.nbr]);
            }
            const double sg = (k % 2) ? 1.0 : -1.0;
            for (int q = 0; q < nqf; ++q) {
                double tt[2] = {0, 0}, w = 1.0;
                int rq = q;
                for (int d = 0; d < dim - 1; ++d) { const int id = rq % mf; rq /= mf; tt[d] = t.rx[6][id]; w *= t.rw[6][id]; }
                double xi[3];
                face_to_cell(dim, k, tt, xi);
                const double dete = basis_grad(t, X, xi, phi, gx, J, A);
                double nor[3], nn = 0.0;   // scaled outward normal of e: |nor| = face measure factor
                for (int r = 0; r < dim; ++r) { nor[r] = sg * A[k / 2][r]; nn += nor[r] * nor[r]; }
                const double nlen = sqrt(nn);
                if (marshak) {
                    const double c = s.alpha_bdr * w * nlen * phi[i];
                    for (int j = 0; j < n; ++j) row[j] += c * phi[j];
                    continue;
                }
                double dne[kDsaMaxN];
                for (int j = 0; j < n; ++j) {
                    double d = 0.0;
                    for (int r = 0; r < dim; ++r) d += gx[j][r] * nor[r];
                    dne[j] = d;
                }
                const double pe_i = phi[i], dne_i = dne[i];
                double phe[kDsaMaxN];
                for (int j = 0; j < n; ++j) phe[j] = phi[j];
                // the same physical point in the neighbour
                double s2[2] = {0, 0}, xim[3];
                s2[0] = fo.b0 + fo.c00 * tt[0] + fo.c01 * tt[1];
                s2[1] = fo.b1 + fo.c10 * tt[0] + fo.c11 * tt[1];
                face_to_cell(dim, fo.k2, s2, xim);
                double Jm[3][3], Am[3][3];
                const double detm = basis_grad(t, Y, xim, phi, gx, Jm, Am);
                // -{D grad u . n}[v] - {D grad v . n}[u] + kappa_F [u][v], n out of e
                double pen = s.kappa * 0.5 * (De * nn / dete + Dm * nn / detm) * w;
                const double floor_ = s.penalty_min * w * nlen;
                if (pen < floor_) pen = floor_;
                for (int j = 0; j < n; ++j) {
                    row[j] += w * (-0.5 * De * dne[j] * pe_i - 0.5 * De * dne_i * phe[j]) + pen * pe_i * phe[j];
                    double dnm = 0.0;
                    for (int r = 0; r < dim; ++r) dnm += gx[j][r] * nor[r];
                    nbr_row[j] += w * (-0.5 * Dm * dnm * pe_i + 0.5 * De * dne_i * phi[j]) - pen * pe_i * phi[j];
                }
            }
        }
        double* ob = out + (size_t)(1 + k) * n * n;
        for (int j = 0; j < n; ++j) ob[j] = nbr_row[j];
    }
    for (int j = 0; j < n; ++j) out[j] = row[j];
}

// y(g, e, i) = sum_j K_self[i][j] x(g, e, j) + sum_k K_k[i][j] x(g, nbr_k, j)
__global__ void k_dsa_apply(int ne, int G, int n, int nface, long long ndof, const Slot* __restrict__ slots,
                            const double* __restrict__ blocks, const double* __restrict__ x, double* __restrict__ y) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)G * ne * n) return;
    const int i = (int)(tid % n);
    const long long ge = tid / n;
    const int e = (int)(ge % ne), g = (int)(ge / ne);
    const double* B = blocks + ((size_t)ge * (1 + nface)) * n * n + (size_t)i * n;
    const double* xg = x + (size_t)g * ndof;
    double acc = 0.0;
    for (int j = 0; j < n; ++j) acc += B[j] * xg[(size_t)e * n + j];
    for (int k = 0; k < nface; ++k) {
        const int m = slots[(size_t)e * nface + k].nbr;
        if (m < 0) continue;
        const double* Bk = B + (size_t)(1 + k) * n * n;
        for (int j = 0; j < n; ++j) acc += Bk[j] * xg[(size_t)m * n + j];
    }
    y[(size_t)g * ndof + (size_t)e * n + i] = acc;
}

// inverse of each self block (block-Jacobi preconditioner), Gauss-Jordan with
// partial pivoting, one thread per (group, cell)
__global__ void k_dsa_invert(int ne, int G, int n, int nface, const double* __restrict__ blocks,
                             double* __restrict__ inv, int* status) {
    const long long ge = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (ge >= (long long)G * ne) return;
    const double* B = blocks + ((size_t)ge * (1 + nface)) * n * n;
    double a[kDsaMaxN][kDsaMaxN], b[kDsaMaxN][kDsaMaxN];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) { a[i][j] = B[i * n + j]; b[i][j] = (i == j) ? 1.0 : 0.0; }
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int r = k + 1; r < n; ++r)
            if (fabs(a[r][k]) > fabs(a[p][k])) p = r;
        if (!(fabs(a[p][k]) > 0.0)) { atomicOr(status, kErrSingular); return; }
        if (p != k)
            for (int j = 0; j < n; ++j) {
                double tmp = a[k][j]; a[k][j] = a[p][j]; a[p][j] = tmp;
                tmp = b[k][j]; b[k][j] = b[p][j]; b[p][j] = tmp;
            }
        const double piv = a[k][k];
        for (int j = 0; j < n; ++j) { a[k][j] /= piv; b[k][j] /= piv; }
        for (int r = 0; r < n; ++r) {
            if (r == k) continue;
            const double f = a[r][k];
            for (int j = 0; j < n; ++j) { a[r][j] -= f * a[k][j]; b[r][j] -= f * b[k][j]; }
        }
    }
    double* out = inv + (size_t)ge * n * n;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) out[i * n + j] = b[i][j];
}

// y = alpha A x + beta y for a CSR matrix (the coarse levels of the diffusion
// preconditioner), one thread per row
__global__ void k_csr_spmv(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                           const double* __restrict__ val, const double* __restrict__ x, double* __restrict__ y,
                           double alpha, double beta) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double acc = 0.0;
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) acc += val[k] * x[col[k]];
    y[r] = beta == 0.0 ? alpha * acc : alpha * acc + beta * y[r];
}

}  // namespace

bool dsa_supported(const Handle& h) { return h.n <= kDsaMaxN && h.lump == 0; }

cudaError_t launch_dsa_assemble(Handle& h, const double* sigma_s, double kappa, double penalty_min, double alpha_bdr,
                                double tau) {
    const size_t nblk = (size_t)h.G * h.ne * (1 + h.nface) * h.n * h.n;
    cudaError_t e = cudaSuccess;
    if (!h.d_dsa) e = cudaMalloc(&h.d_dsa, nblk * sizeof(double));
    if (e == cudaSuccess && !h.d_dsa_inv) e = cudaMalloc(&h.d_dsa_inv, (size_t)h.G * h.ne * h.n * h.n * sizeof(double));
    if (e != cudaSuccess) return e;
    DsaArgs a;
    a.t = h.ref; a.ne = h.ne; a.G = h.G; a.ndof = h.ndof;
    a.corners = h.d_corners; a.slots = h.d_slots; a.orient = h.d_orient;
    a.sigma_t = h.d_sigma; a.sigma_s = sigma_s; a.Mt = h.d_Mt;
    a.kappa = kappa; a.penalty_min = penalty_min; a.alpha_bdr = alpha_bdr; a.tau = tau;
    a.blocks = h.d_dsa;
    const long long rows = (long long)h.G * h.ne * h.n;
    k_dsa_assemble<<<(unsigned)((rows + 127) / 128), 128, 0, h.stream>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const long long cells = (long long)h.G * h.ne;
    k_dsa_invert<<<(unsigned)((cells + 127) / 128), 128, 0, h.stream>>>(h.ne, h.G, h.n, h.nface, h.d_dsa, h.d_dsa_inv,
                                                                       h.d_status);
    return cudaGetLastError();
}

cudaError_t launch_dsa_apply(Handle& h, const double* x, double* y) {
    const long long rows = (long long)h.G * h.ne * h.n;
    k_dsa_apply<<<(unsigned)((rows + 255) / 256), 256, 0, h.stream>>>(h.ne, h.G, h.n, h.nface, h.ndof, h.d_slots,
                                                                      h.d_dsa, x, y);
    return cudaGetLastError();
}

}  // namespace allium

extern "C" int allium_csr_spmv(int n, const int* rowptr, const int* col, const double* val, const double* x, double* y,
                               double alpha, double beta, void* stream) {
    if (n <= 0 || !rowptr || !col || !val || !x || !y) return ALLIUM_ERR_ARG;
    allium::k_csr_spmv<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(n, rowptr, col, val, x, y, alpha,
                                                                                       beta);
    return cudaGetLastError() == cudaSuccess ? ALLIUM_OK : ALLIUM_ERR_CUDA;
}

// Greedy pairwise aggregation of a CSR matrix (host arrays): rows in order,
// an unaggregated row joins the unaggregated neighbour with the most negative
// coupling (lowest column on ties), or stays alone.  agg[i] receives the
// aggregate of row i; returns the number of aggregates.
extern "C" int allium_pair_aggregates(int n, const int* rowptr, const int* col, const double* val, int* agg) {
    if (n <= 0 || !rowptr || !col || !val || !agg) return -1;
    for (int i = 0; i < n; ++i) agg[i] = -1;
    int nagg = 0;
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        int best = -1;
        double bv = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            const int j = col[k];
            if (j == i || agg[j] >= 0) continue;
            if (val[k] < bv || (val[k] == bv && best >= 0 && j < best)) { bv = val[k]; best = j; }
        }
        agg[i] = nagg;
        if (best >= 0) agg[best] = nagg;
        ++nagg;
    }
    return nagg;
}
