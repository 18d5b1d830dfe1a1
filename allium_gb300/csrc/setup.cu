// Setup-side kernels of the sweep: reference tables, face normals, local
// matrix assembly (AssembleLocalMatrices), device wavefront levels, the
// transport source, the moment operators and the balance reduction.
#include <cub/device/device_radix_sort.cuh>

#include <cmath>
#include <vector>

#include "geometry.cuh"
#include "sweep_kernels.cuh"

namespace allium {

std::mutex& cache_lock() {
    static std::mutex m;
    return m;
}

// ------------------------------------------------------------ host tables
namespace {

double legendre_p(int n, double x, double* dp) {
    double p0 = 1.0, p1 = x;
    if (n == 0) { *dp = 0.0; return 1.0; }
    for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
    }
    *dp = n * (x * p1 - p0) / (x * x - 1.0);
    return p1;
}

// n-point Gauss-Legendre on [0,1] (Newton on P_n from Chebyshev-like guesses)
void gauss_legendre01(int n, double* x, double* w) {
    for (int i = 0; i < (n + 1) / 2; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            const double pz = legendre_p(n, z, &dp);
            const double dz = pz / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        legendre_p(n, z, &dp);
        const double wt = 1.0 / ((1.0 - z * z) * dp * dp);   // half of the [-1,1] weight
        x[n - 1 - i] = 0.5 * (1.0 + z);
        x[i] = 0.5 * (1.0 - z);
        w[i] = w[n - 1 - i] = wt;
    }
    if (n % 2) x[n / 2] = 0.5;
}

void gauss_lobatto01(int p, double* x) {
    if (p == 0) { x[0] = 0.5; return; }
    x[0] = 0.0; x[p] = 1.0;
    for (int i = 1; i < p; ++i) {
        double z = -std::cos(M_PI * i / p);
        for (int it = 0; it < 100; ++it) {
            double dp = 0.0;
            const double pp = legendre_p(p, z, &dp);
            const double d2 = (2.0 * z * dp - p * (p + 1.0) * pp) / (1.0 - z * z);
            const double dz = dp / d2;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        x[i] = 0.5 * (1.0 + z);
    }
}

void set_rule(RefTables& t, int r, int npts, bool vertex) {
    if (vertex) {
        t.rn[r] = 2;
        t.rx[r][0] = 0.0; t.rx[r][1] = 1.0;
        t.rw[r][0] = 0.5; t.rw[r][1] = 0.5;
    } else {
        t.rn[r] = npts;
        gauss_legendre01(npts, t.rx[r], t.rw[r]);
    }
}

}  // namespace

// Integration rules follow the point counts MFEM's IntRules give the
// integrators allium uses (n = order/2 + 1 Gauss-Legendre points per axis):
//   sigma mass (MGMassIntegrator, order 2p, mg_form.cpp:34-37)        p + 1
//   convection (order OrderGrad + Order + p)                          p + 1 (1D, 2D), p + 2 (3D)
//   time mass (MassIntegrator, order 2p + OrderW)                     p + 1 (1D, 2D), p + 2 (3D)
//   face mass (order 2 max(p1, p2), sweep.cpp:1201-1211)              p + 1
//   source domain (DomainLFIntegrator, order 2p)                      p + 1
//   source boundary (BoundaryFlowIntegrator, order OrderW + 2p)       p + 1 (2D), p + 2 (3D)
// Lumped parts use the reference-cell vertices with equal weights
// (LumpedIntegrationRule, lumping.cpp:3-12).
RefTables make_ref_tables(int dim, int p, int lump) {
    RefTables t{};
    t.dim = dim; t.p = p; t.n1 = p + 1;
    t.n = 1; t.nf = 1;
    for (int d = 0; d < dim; ++d) t.n *= t.n1;
    for (int d = 0; d < dim - 1; ++d) t.nf *= t.n1;
    t.nface = 2 * dim;
    gauss_lobatto01(p, t.nodes);
    const int hi = (dim == 3) ? p + 2 : p + 1;
    set_rule(t, 0, p + 1, lump & ALLIUM_LUMP_MASS);
    set_rule(t, 1, hi, lump & ALLIUM_LUMP_GRADIENT);
    set_rule(t, 2, hi, lump & ALLIUM_LUMP_MASS);
    set_rule(t, 3, p + 1, lump & ALLIUM_LUMP_FACE);
    set_rule(t, 4, p + 1, false);
    set_rule(t, 5, hi, false);
    // IntRules.Get(geom, 2p + 1) and (geom, 2p + 2): n = order / 2 + 1 points
    set_rule(t, 6, p + 1, false);
    set_rule(t, 7, p + 2, false);
    // DiffusionIntegrator on tensor elements: order 2p + dim - 1
    set_rule(t, 8, (2 * p + dim - 1) / 2 + 1, false);
    return t;
}

// ------------------------------------------------------------ face normals
// unit normal at the face centre, out of element 1 (sweep.cpp:142-154)
__global__ void k_face_normals(RefTables t, int nfaces, const int* __restrict__ e1k1,
                               const double* __restrict__ corners, double* __restrict__ normals) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfaces) return;
    const int dim = t.dim, nc = 1 << dim;
    const int e = e1k1[2 * f], k = e1k1[2 * f + 1];
    double X[24];
    for (int q = 0; q < nc * dim; ++q) X[q] = corners[(size_t)e * nc * dim + q];
    const double tc[2] = {0.5, 0.5};
    double xi[3], J[3][3], A[3][3];
    face_to_cell(dim, k, tc, xi);
    cell_jacobian(dim, X, xi, J, nullptr);
    adjugate(dim, J, A);
    const int ax = k / 2;
    const double sg = (k % 2) ? 1.0 : -1.0;
    double nr[3], nn = 0.0;
    for (int r = 0; r < dim; ++r) { nr[r] = sg * A[ax][r]; nn += nr[r] * nr[r]; }
    const double inv = 1.0 / sqrt(nn);
    for (int r = 0; r < dim; ++r) normals[(size_t)f * dim + r] = nr[r] * inv;
}

cudaError_t launch_face_normals(Handle& h) {
    const int b = 128;
    k_face_normals<<<(h.nfaces + b - 1) / b, b, 0, h.stream>>>(h.ref, h.nfaces, h.d_face_e1k1, h.d_corners, h.d_normals);
    return cudaGetLastError();
}

// Omega_a . n_f for all (face, angle), rounded exactly as written (no FMA).
// The FP32 copy keeps the sign of the FP64 value even where it would round to
// zero, so FP32 and FP64 sweeps take the same upwind decisions.
__global__ void k_face_dots(int nfaces, int Nw, int dim, const double* __restrict__ omega,
                            const double* __restrict__ normals, double* __restrict__ dots, float* __restrict__ fdots) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nfaces * Nw) return;
    const int f = (int)(t / Nw), a = (int)(t % Nw);
    double om[3] = {0, 0, 0}, nr[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) { om[d] = omega[a * dim + d]; nr[d] = normals[(size_t)f * dim + d]; }
    const double v = dot_exact(dim, om, nr);
    float fv = (float)v;
    if (fv == 0.0f && v != 0.0) fv = v > 0.0 ? 1.401298464e-45f : -1.401298464e-45f;
    dots[t] = v;
    fdots[t] = fv;
}

cudaError_t launch_face_dots(Handle& h) {
    const long long total = (long long)h.nfaces * h.Nw;
    const int b = 256;
    k_face_dots<<<(unsigned)((total + b - 1) / b), b, 0, h.stream>>>(h.nfaces, h.Nw, h.dim, h.d_omega, h.d_normals,
                                                                      h.d_dots, h.f_dots);
    return cudaGetLastError();
}

// ------------------------------------------------------------ reflections
// GetReflectedAngleIndex (src/angular_quadrature.cpp:27-36, GetIndexForAngle
// :8-25) for every angle entering the domain through reflective face c
// (Omega.n < 0 with the face's own dot products): the first direction of the
// set within 1e-14 (Euclidean) of Omega - 2 (Omega.n) n, n the unit
// face-centre normal.  refl = -1 when there is none, -2 for angles that do not
// enter through the face.
__global__ void k_reflect(int nrefl, int Nw, int dim, const int* __restrict__ faces, const double* __restrict__ omega,
                          const double* __restrict__ normals, const double* __restrict__ dots, int* __restrict__ refl) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nrefl * Nw) return;
    const int c = t / Nw, a = t % Nw;
    const int f = faces[c];
    if (!(dots[(size_t)f * Nw + a] < 0.0)) { refl[t] = -2; return; }
    const double* n = normals + (size_t)f * dim;
    double r[3] = {0, 0, 0};
    double dn = 0.0;
    for (int d = 0; d < dim; ++d) dn = __dadd_rn(dn, __dmul_rn(omega[a * dim + d], n[d]));
    for (int d = 0; d < dim; ++d) r[d] = __dsub_rn(omega[a * dim + d], __dmul_rn(2.0 * dn, n[d]));
    int found = -1;
    for (int b = 0; b < Nw && found < 0; ++b) {
        double d2 = 0.0;
        for (int d = 0; d < dim; ++d) { const double x = omega[b * dim + d] - r[d]; d2 += x * x; }
        if (sqrt(d2) < 1e-14) found = b;
    }
    refl[t] = found;
}

// Reflective edges (sweep.cpp:177-195) as two tables over [nrefl][Nw]:
// d_refl[c][a] = reflected angle feeding entering angle a (else negative),
// d_feed[c][b] = the entering angle that angle b feeds (else -1).
int compute_reflections(Handle& h, const std::vector<int>& refl_faces) {
    h.nrefl = (int)refl_faces.size();
    if (h.nrefl == 0) return ALLIUM_OK;
    const size_t total = (size_t)h.nrefl * h.Nw;
    int* d_faces = nullptr;
    cudaError_t e = cudaMalloc(&d_faces, refl_faces.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&h.d_refl, total * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&h.d_feed, total * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_faces, refl_faces.data(), refl_faces.size() * sizeof(int), cudaMemcpyHostToDevice, h.stream);
    if (e == cudaSuccess) {
        k_reflect<<<(int)((total + 127) / 128), 128, 0, h.stream>>>(h.nrefl, h.Nw, h.dim, d_faces, h.d_omega, h.d_normals,
                                                                   h.d_dots, h.d_refl);
        e = cudaGetLastError();
    }
    std::vector<int> refl(total), feed(total, -1);
    if (e == cudaSuccess) e = cudaMemcpyAsync(refl.data(), h.d_refl, total * sizeof(int), cudaMemcpyDeviceToHost, h.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    if (d_faces) cudaFree(d_faces);
    if (e != cudaSuccess) { h.last_error = cudaGetErrorString(e); return ALLIUM_ERR_CUDA; }
    for (int c = 0; c < h.nrefl; ++c)
        for (int a = 0; a < h.Nw; ++a) {
            const int b = refl[(size_t)c * h.Nw + a];
            if (b == -1) { h.last_error = "a reflected direction is not in the angular quadrature"; return ALLIUM_ERR_MESH; }
            if (b < 0) continue;
            int& slot = feed[(size_t)c * h.Nw + b];
            if (slot >= 0) { h.last_error = "two directions reflect onto one"; return ALLIUM_ERR_MESH; }
            slot = a;
        }
    e = cudaMemcpyAsync(h.d_feed, feed.data(), total * sizeof(int), cudaMemcpyHostToDevice, h.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    if (e != cudaSuccess) { h.last_error = cudaGetErrorString(e); return ALLIUM_ERR_CUDA; }
    return ALLIUM_OK;
}

// ------------------------------------------------------------ assembly
// One block per cell.  Geometric factors of each quadrature point are staged
// in shared memory, then the threads share out the matrix entries.
//   G_d(i,j) = - sum_q w_q phi_j(q) grad_ref phi_i(q) . adj(J_q) e_d      (ConservativeConvection)
//   M(i,j)   =   sum_q w_q det(J_q) phi_i(q) phi_j(q)                     (unit mass)
//   F_k(i,j) =   sum_q w_q |J_face(q)| phi_i(q) phi_j(q) over face DOFs   (FaceMassMatrices)
constexpr int kMaxPts = kMaxRule * kMaxRule * kMaxRule;

struct Tab1D {
    double v[kMaxRule][kMaxOrder + 1], d[kMaxRule][kMaxOrder + 1];
};

__device__ void tab_fill(const RefTables& t, int r, Tab1D& tb) {
    for (int q = threadIdx.x; q < t.rn[r]; q += blockDim.x)
        lagrange1d(t.n1, t.nodes, t.rx[r][q], tb.v[q], tb.d[q]);
}

// point index q of a tensor rule with m points per axis -> per-axis indices
__device__ inline void split_point(int dim, int m, int q, int* id) {
    for (int d = 0; d < dim; ++d) { id[d] = q % m; q /= m; }
}

__global__ void __launch_bounds__(128) k_assemble(RefTables t, const double* __restrict__ corners,
                                                  double* __restrict__ Gout, double* __restrict__ Mout,
                                                  double* __restrict__ Fout, int mass_rule, int do_conv) {
    const int e = blockIdx.x;
    const int dim = t.dim, n = t.n, n1 = t.n1, nc = 1 << dim, nf = t.nf, nface = t.nface;
    __shared__ double X[24];
    __shared__ Tab1D tm, tg, tf;
    __shared__ double wdet[kMaxPts];
    __shared__ double wadj[kMaxPts][3][3];
    __shared__ double wface[6][kMaxRule * kMaxRule];
    for (int q = threadIdx.x; q < nc * dim; q += blockDim.x) X[q] = corners[(size_t)e * nc * dim + q];
    tab_fill(t, mass_rule, tm);
    tab_fill(t, 1, tg);
    tab_fill(t, 3, tf);
    __syncthreads();

    const int mm = t.rn[mass_rule], mg = t.rn[1], mf = t.rn[3];
    int npm = 1, npg = 1, npf = 1;
    for (int d = 0; d < dim; ++d) { npm *= mm; npg *= mg; }
    for (int d = 0; d < dim - 1; ++d) npf *= mf;
    for (int q = threadIdx.x; q < npm; q += blockDim.x) {
        int id[3]; split_point(dim, mm, q, id);
        double xi[3], J[3][3], A[3][3], w = 1.0;
        for (int d = 0; d < dim; ++d) { xi[d] = t.rx[mass_rule][id[d]]; w *= t.rw[mass_rule][id[d]]; }
        cell_jacobian(dim, X, xi, J, nullptr);
        wdet[q] = adjugate(dim, J, A) * w;
    }
    if (do_conv) {
        for (int q = threadIdx.x; q < npg; q += blockDim.x) {
            int id[3]; split_point(dim, mg, q, id);
            double xi[3], J[3][3], A[3][3], w = 1.0;
            for (int d = 0; d < dim; ++d) { xi[d] = t.rx[1][id[d]]; w *= t.rw[1][id[d]]; }
            cell_jacobian(dim, X, xi, J, nullptr);
            adjugate(dim, J, A);
            for (int d = 0; d < dim; ++d)
                for (int r = 0; r < dim; ++r) wadj[q][d][r] = -w * A[r][d];
        }
        for (int q = threadIdx.x; q < nface * npf; q += blockDim.x) {
            const int k = q / npf, qq = q % npf;
            int id[3]; split_point(dim - 1, mf, qq, id);
            double tt[2] = {0.0, 0.0}, w = 1.0;
            for (int d = 0; d < dim - 1; ++d) { tt[d] = t.rx[3][id[d]]; w *= t.rw[3][id[d]]; }
            double xi[3], J[3][3], A[3][3];
            face_to_cell(dim, k, tt, xi);
            cell_jacobian(dim, X, xi, J, nullptr);
            adjugate(dim, J, A);
            double jf = 1.0;
            if (dim > 1) {
                double s = 0.0;
                for (int r = 0; r < dim; ++r) s += A[k / 2][r] * A[k / 2][r];
                jf = sqrt(s);
            }
            wface[k][qq] = w * jf;
        }
    }
    __syncthreads();

    // unit mass
    for (int ij = threadIdx.x; ij < n * n; ij += blockDim.x) {
        const int i = ij / n, j = ij % n;
        int ii[3], jj[3];
        dof_index(dim, n1, i, ii);
        dof_index(dim, n1, j, jj);
        double s = 0.0;
        for (int q = 0; q < npm; ++q) {
            int id[3]; split_point(dim, mm, q, id);
            double pi = 1.0, pj = 1.0;
            for (int d = 0; d < dim; ++d) { pi *= tm.v[id[d]][ii[d]]; pj *= tm.v[id[d]][jj[d]]; }
            s += wdet[q] * pi * pj;
        }
        Mout[(size_t)e * n * n + ij] = s;
    }
    if (!do_conv) return;
    // convection
    for (int t3 = threadIdx.x; t3 < dim * n * n; t3 += blockDim.x) {
        const int d = t3 / (n * n), ij = t3 % (n * n), i = ij / n, j = ij % n;
        int ii[3], jj[3];
        dof_index(dim, n1, i, ii);
        dof_index(dim, n1, j, jj);
        double s = 0.0;
        for (int q = 0; q < npg; ++q) {
            int id[3]; split_point(dim, mg, q, id);
            double pj = 1.0, bi = 0.0;
            for (int c = 0; c < dim; ++c) pj *= tg.v[id[c]][jj[c]];
            for (int r = 0; r < dim; ++r) {
                double gr = 1.0;
                for (int c = 0; c < dim; ++c) gr *= (c == r) ? tg.d[id[c]][ii[c]] : tg.v[id[c]][ii[c]];
                bi += gr * wadj[q][d][r];
            }
            s += pj * bi;
        }
        Gout[((size_t)e * dim + d) * n * n + ij] = s;
    }
    // face mass blocks on face DOFs
    for (int t3 = threadIdx.x; t3 < nface * nf * nf; t3 += blockDim.x) {
        const int k = t3 / (nf * nf), r = t3 % (nf * nf), fi = r / nf, fj = r % nf;
        int ti[3], tj[3];
        dof_index(dim - 1, n1, fi, ti);
        dof_index(dim - 1, n1, fj, tj);
        double s = 0.0;
        for (int q = 0; q < npf; ++q) {
            int id[3]; split_point(dim - 1, mf, q, id);
            double pi = 1.0, pj = 1.0;
            for (int c = 0; c < dim - 1; ++c) { pi *= tf.v[id[c]][ti[c]]; pj *= tf.v[id[c]][tj[c]]; }
            s += pi * pj * wface[k][q];
        }
        Fout[((size_t)e * nface + k) * nf * nf + r] = s;
    }
}

cudaError_t launch_assemble(Handle& h) {
    k_assemble<<<h.ne, 128, 0, h.stream>>>(h.ref, h.d_corners, h.d_G, h.d_M, h.d_F, 0, 1);
    return cudaGetLastError();
}

cudaError_t launch_time_mass(Handle& h) {
    k_assemble<<<h.ne, 128, 0, h.stream>>>(h.ref, h.d_corners, nullptr, h.d_Mt, nullptr, 2, 0);
    return cudaGetLastError();
}

// ------------------------------------------------------------ levels
// Edge rule of sweep.cpp:157-175 on one face: element 1 -> element 2 unless
// Omega . n_face < 0 (n_face points out of element 1).
__device__ inline bool forward_edge(const double* __restrict__ dots, int Nw, int face, int a) {
    return !(dots[(size_t)face * Nw + a] < 0.0);
}

__global__ void k_indegree(int ne, int Nw, int dim, const double* __restrict__ dots, const Slot* __restrict__ slots,
                           int* __restrict__ indeg, int* __restrict__ level,
                           int* __restrict__ frontier, int* __restrict__ fcount) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= (long long)ne * Nw) return;
    const int e = (int)(v / Nw), a = (int)(v % Nw), nface = 2 * dim;
    int c = 0;
    for (int k = 0; k < nface; ++k) {
        const Slot s = slots[(size_t)e * nface + k];
        // reflective face: edge (e, reflected a) -> (e, a) when Omega_a . n < 0 (sweep.cpp:181-194)
        if (s.nbr <= -2) { if (dots[(size_t)s.face * Nw + a] < 0.0) ++c; continue; }
        if (s.nbr < 0) continue;
        const bool fwd = forward_edge(dots, Nw, s.face, a);
        if (s.side ? fwd : !fwd) ++c;
    }
    indeg[v] = c;
    if (c == 0) {
        level[v] = 0;
        frontier[atomicAdd(fcount, 1)] = (int)v;
    }
}

__global__ void k_kahn(int Nw, int dim, const double* __restrict__ dots,
                       const Slot* __restrict__ slots, const int* __restrict__ feed, int* __restrict__ indeg,
                       int* __restrict__ level, const int* __restrict__ cur, int ncur, int* __restrict__ next,
                       int* __restrict__ ncount, int lev) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncur) return;
    const int u = cur[t];
    const int e = u / Nw, a = u % Nw, nface = 2 * dim;
    for (int k = 0; k < nface; ++k) {
        const Slot s = slots[(size_t)e * nface + k];
        if (s.nbr <= -2) {
            const int t2 = feed[(size_t)(-2 - s.nbr) * Nw + a];
            if (t2 >= 0) {
                const int v = e * Nw + t2;
                if (atomicSub(&indeg[v], 1) == 1) {
                    level[v] = lev + 1;
                    next[atomicAdd(ncount, 1)] = v;
                }
            }
            continue;
        }
        if (s.nbr < 0) continue;
        const bool fwd = forward_edge(dots, Nw, s.face, a);
        if (!(s.side ? !fwd : fwd)) continue;   // not an out-edge of u
        const int v = s.nbr * Nw + a;
        if (atomicSub(&indeg[v], 1) == 1) {
            level[v] = lev + 1;
            next[atomicAdd(ncount, 1)] = v;
        }
    }
}

// Sort key of node v = (e, a): its level, then the kind of each face (2 bits:
// none, outflow, inflow from a neighbour, reflective inflow; the branches of
// the node kernels).  Nodes of one level that share the pattern run in the
// same warps, so a warp does not issue both sides of a face branch; on the
// FP64 pipe every issued warp instruction costs its full width.
__global__ void k_level_keys(long long n, int Nw, int dim, int pattern_bits, const double* __restrict__ dots,
                             const Slot* __restrict__ slots, const int* __restrict__ level, int* __restrict__ keys) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int e = (int)(v / Nw), a = (int)(v % Nw), nface = 2 * dim;
    int pat = 0;
    if (pattern_bits)
        for (int k = 0; k < nface; ++k) {
            const Slot s = slots[(size_t)e * nface + k];
            const double d1 = dots[(size_t)s.face * Nw + a];
            const double dk = s.side ? -d1 : d1;
            const int code = dk > 0.0 ? 1 : (dk < 0.0 ? (s.nbr >= 0 ? 2 : (s.nbr <= -2 ? 3 : 0)) : 0);
            pat |= code << (2 * k);
        }
    keys[v] = (level[v] << pattern_bits) | pat;
}

__global__ void k_iota(int* x, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = (int)i;
}

__global__ void k_level_hist(const int* __restrict__ level, long long n, int* __restrict__ hist) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&hist[level[i]], 1);
}

// The same histogram with per-block counts in shared memory (nbins ints) and
// one global add per bin and block: a few hundred bins hit by 10^7..10^8
// global atomics serialise on the bins.
__global__ void k_level_hist_shared(const int* __restrict__ level, long long n, int nbins, int* __restrict__ hist) {
    extern __shared__ int counts[];
    for (int k = threadIdx.x; k < nbins; k += blockDim.x) counts[k] = 0;
    __syncthreads();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        atomicAdd(&counts[level[i]], 1);
    __syncthreads();
    for (int k = threadIdx.x; k < nbins; k += blockDim.x)
        if (counts[k]) atomicAdd(&hist[k], counts[k]);
}

// histogram of n values in [0, nbins) into hist (zeroed here)
static cudaError_t level_histogram(Handle& h, const int* values, long long n, int nbins, int* hist) {
    cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)nbins * sizeof(int), h.stream);
    if (e != cudaSuccess) return e;
    const int b = 256;
    if (nbins <= 12288) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        long long grid = (long long)(sms > 0 ? sms : 1) * 8;
        const long long need = (n + b - 1) / b;
        if (grid > need) grid = need > 0 ? need : 1;
        k_level_hist_shared<<<(unsigned)grid, b, (size_t)nbins * sizeof(int), h.stream>>>(values, n, nbins, hist);
    } else {
        k_level_hist<<<(unsigned)((n + b - 1) / b), b, 0, h.stream>>>(values, n, hist);
    }
    return cudaGetLastError();
}

#define CK(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { h.last_error = cudaGetErrorString(_e); return ALLIUM_ERR_CUDA; } } while (0)

int compute_levels(Handle& h) {
    const long long N = (long long)h.ne * h.Nw;
    if (N > 0x7fffffffLL) { h.last_error = "more than 2^31 (cell, angle) nodes"; return ALLIUM_ERR_SIZE; }
    int *d_indeg = nullptr, *d_fa = nullptr, *d_fb = nullptr, *d_cnt = nullptr, *d_keys = nullptr, *d_vals = nullptr;
    CK(cudaMalloc(&d_indeg, N * sizeof(int)));
    CK(cudaMalloc(&d_fa, N * sizeof(int)));
    CK(cudaMalloc(&d_fb, N * sizeof(int)));
    CK(cudaMalloc(&d_cnt, 2 * sizeof(int)));
    CK(cudaMemsetAsync(d_cnt, 0, 2 * sizeof(int), h.stream));
    const int b = 256;
    const unsigned gN = (unsigned)((N + b - 1) / b);
    k_indegree<<<gN, b, 0, h.stream>>>(h.ne, h.Nw, h.dim, h.d_dots, h.d_slots, d_indeg, h.d_level, d_fa, d_cnt);
    CK(cudaGetLastError());
    int ncur = 0;
    CK(cudaMemcpyAsync(&ncur, d_cnt, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    CK(cudaStreamSynchronize(h.stream));
    long long done = 0;
    int lev = 0;
    while (ncur > 0) {
        done += ncur;
        CK(cudaMemsetAsync(d_cnt + 1, 0, sizeof(int), h.stream));
        k_kahn<<<(ncur + b - 1) / b, b, 0, h.stream>>>(h.Nw, h.dim, h.d_dots, h.d_slots, h.d_feed, d_indeg,
                                                        h.d_level, d_fa, ncur, d_fb, d_cnt + 1, lev);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(&ncur, d_cnt + 1, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
        CK(cudaStreamSynchronize(h.stream));
        std::swap(d_fa, d_fb);
        ++lev;
    }
    cudaFree(d_fb); cudaFree(d_fa); cudaFree(d_indeg);
    if (done != N) {
        cudaFree(d_cnt);
        h.last_error = "the upwind graph has a cycle";
        return ALLIUM_ERR_NOT_DAG;
    }
    h.num_levels = lev;
    // nodes sorted by (level, face pattern), stable in node id -> within a
    // level, nodes of one face pattern in (cell, angle) order
    int* d_key_in = nullptr;
    CK(cudaMalloc(&d_key_in, N * sizeof(int)));
    CK(cudaMalloc(&d_keys, N * sizeof(int)));
    CK(cudaMalloc(&d_vals, N * sizeof(int)));
    int level_bits = 1;
    while ((1 << level_bits) <= lev) ++level_bits;
    const int pattern_bits = (level_bits + 4 * h.dim <= 31) ? 4 * h.dim : 0;
    k_level_keys<<<gN, b, 0, h.stream>>>(N, h.Nw, h.dim, pattern_bits, h.d_dots, h.d_slots, h.d_level, d_key_in);
    CK(cudaGetLastError());
    k_iota<<<gN, b, 0, h.stream>>>(d_vals, N);
    CK(cudaGetLastError());
    const int end_bit = level_bits + pattern_bits;
    size_t tmp_bytes = 0;
    CK(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, d_key_in, d_keys, d_vals, h.d_level_nodes, (int)N, 0, end_bit, h.stream));
    void* tmp = nullptr;
    CK(cudaMalloc(&tmp, tmp_bytes));
    CK(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, d_key_in, d_keys, d_vals, h.d_level_nodes, (int)N, 0, end_bit, h.stream));
    int* d_hist = nullptr;
    CK(cudaMalloc(&d_hist, lev * sizeof(int)));
    CK(level_histogram(h, h.d_level, N, lev, d_hist));
    std::vector<int> hist(lev);
    CK(cudaMemcpyAsync(hist.data(), d_hist, lev * sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    CK(cudaStreamSynchronize(h.stream));
    h.h_level_offsets.assign(lev + 1, 0);
    for (int l = 0; l < lev; ++l) h.h_level_offsets[l + 1] = h.h_level_offsets[l] + hist[l];
    cudaFree(d_hist); cudaFree(tmp); cudaFree(d_vals); cudaFree(d_keys); cudaFree(d_key_in); cudaFree(d_cnt);
    return ALLIUM_OK;
}

// ------------------------------------------------------------ angle chunks
// key of level-order position t: chunk(angle) * num_levels + level
__global__ void k_chunk_keys(long long n, int Nw, int nlev, const int* __restrict__ angle_chunk,
                             const int* __restrict__ level_nodes, const int* __restrict__ level, int* __restrict__ keys) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int node = level_nodes[t];
    keys[t] = angle_chunk[node % Nw] * nlev + level[node];
}

__global__ void k_gather_nodes(long long n, const int* __restrict__ pos, const int* __restrict__ level_nodes,
                               int* __restrict__ out) {
    const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (u < n) out[u] = level_nodes[pos[u]];
}

// First angle of each of the nchunk contiguous blocks of angles.  Chunk
// weights 1 except the first and the last, which get 1/2^taper: small end
// chunks shorten the pipeline's fill (the first copy in) and drain (the last
// sweep and copy out).  Every chunk keeps at least one angle.
std::vector<int> chunk_bounds(int Nw, int nchunk, int taper) {
    std::vector<double> w(nchunk, 1.0);
    if (nchunk >= 3) w[0] = w[nchunk - 1] = 1.0 / (1 << taper);
    double W = 0.0;
    for (double x : w) W += x;
    std::vector<int> b(nchunk + 1, 0);
    double run = 0.0;
    for (int c = 1; c < nchunk; ++c) {
        run += w[c - 1];
        int v = (int)std::lround(Nw * run / W);
        if (v < b[c - 1] + 1) v = b[c - 1] + 1;
        if (v > Nw - (nchunk - c)) v = Nw - (nchunk - c);
        b[c] = v;
    }
    b[nchunk] = Nw;
    return b;
}

// Orders for the chunked host-buffer Mult: angles split into nchunk contiguous
// blocks (chunk_bounds); within a chunk the nodes keep the order of the full
// sweep (stable sort on the key).
int build_chunks(Handle& h, int nchunk, int taper) {
    if (h.nchunk == nchunk && h.chunk_taper == taper) return ALLIUM_OK;
    // the captured chunk sweeps (graph kinds 40 + c) hold the old chunk offsets
    CK(cudaStreamSynchronize(h.stream));
    drop_graphs(h);
    const long long N = (long long)h.ne * h.Nw;
    const int L = h.num_levels;
    if ((long long)nchunk * L >= 0x7fffffffLL) { h.last_error = "too many chunk levels"; return ALLIUM_ERR_SIZE; }
    if (h.d_chunk_nodes) { cudaFree(h.d_chunk_nodes); h.d_chunk_nodes = nullptr; }
    if (h.d_chunk_pos) { cudaFree(h.d_chunk_pos); h.d_chunk_pos = nullptr; }
    int *d_keys = nullptr, *d_keys2 = nullptr, *d_vals = nullptr, *d_hist = nullptr;
    void* tmp = nullptr;
    const int b = 256;
    const unsigned gN = (unsigned)((N + b - 1) / b);
    CK(cudaMalloc(&d_keys, N * sizeof(int)));
    CK(cudaMalloc(&d_keys2, N * sizeof(int)));
    CK(cudaMalloc(&d_vals, N * sizeof(int)));
    CK(cudaMalloc(&h.d_chunk_pos, N * sizeof(int)));
    CK(cudaMalloc(&h.d_chunk_nodes, N * sizeof(int)));
    const std::vector<int> bounds = chunk_bounds(h.Nw, nchunk, taper);
    std::vector<int> angle_chunk(h.Nw);
    for (int c = 0; c < nchunk; ++c)
        for (int a = bounds[c]; a < bounds[c + 1]; ++a) angle_chunk[a] = c;
    int* d_angle_chunk = nullptr;
    CK(cudaMalloc(&d_angle_chunk, (size_t)h.Nw * sizeof(int)));
    CK(cudaMemcpyAsync(d_angle_chunk, angle_chunk.data(), (size_t)h.Nw * sizeof(int), cudaMemcpyHostToDevice, h.stream));
    k_chunk_keys<<<gN, b, 0, h.stream>>>(N, h.Nw, L, d_angle_chunk, h.d_level_nodes, h.d_level, d_keys);
    CK(cudaGetLastError());
    k_iota<<<gN, b, 0, h.stream>>>(d_vals, N);
    CK(cudaGetLastError());
    int end_bit = 1;
    while ((1LL << end_bit) <= (long long)nchunk * L) ++end_bit;
    size_t tmp_bytes = 0;
    CK(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, d_keys, d_keys2, d_vals, h.d_chunk_pos, (int)N, 0, end_bit,
                                       h.stream));
    CK(cudaMalloc(&tmp, tmp_bytes));
    CK(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, d_keys, d_keys2, d_vals, h.d_chunk_pos, (int)N, 0, end_bit,
                                       h.stream));
    k_gather_nodes<<<gN, b, 0, h.stream>>>(N, h.d_chunk_pos, h.d_level_nodes, h.d_chunk_nodes);
    CK(cudaGetLastError());
    const int nkeys = nchunk * L;
    CK(cudaMalloc(&d_hist, (size_t)nkeys * sizeof(int)));
    CK(level_histogram(h, d_keys, N, nkeys, d_hist));
    std::vector<int> hist(nkeys);
    CK(cudaMemcpyAsync(hist.data(), d_hist, (size_t)nkeys * sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    CK(cudaStreamSynchronize(h.stream));
    h.h_chunk_offsets.assign((size_t)nchunk * (L + 1), 0);
    int run = 0;
    for (int c = 0; c < nchunk; ++c) {
        int* o = h.h_chunk_offsets.data() + (size_t)c * (L + 1);
        for (int l = 0; l < L; ++l) { o[l] = run; run += hist[(size_t)c * L + l]; }
        o[L] = run;
    }
    h.h_chunk_angle = bounds;
    cudaFree(d_hist); cudaFree(tmp); cudaFree(d_vals); cudaFree(d_keys2); cudaFree(d_keys); cudaFree(d_angle_chunk);
    h.nchunk = nchunk;
    h.chunk_taper = taper;
    return ALLIUM_OK;
}

// ------------------------------------------------------------ source
// FormTransportSource (sweep.cpp:1135-1185) for a piecewise-constant isotropic
// density and an isotropic inflow per boundary attribute:
//   q(g,a,i) = sum_q w_q det J Q_{g,e} phi_i
//            + sum_{bdr faces} sum_q w_q (|Omega.n_q| - Omega.n_q)/2 psi_in phi_i
// with n_q the unnormalised normal (CalcOrtho) at each face point
// (BoundaryFlowIntegrator with alpha = -1, beta = -1/2).
// qpts (optional, replaces qcell): the density at the domain rule's points,
// [G][Ne][points], or [G][Nw][Ne][points] with q_dir, for a coefficient that
// varies inside a cell (and with the direction): the integral
// DomainLFIntegrator forms from a FunctionCoefficient.  angular: inflow is
// [G][Nw][nattr] (a direction-dependent inflow per attribute) instead of
// [G][nattr].
__device__ void source_domain_term(const RefTables& t, const double* X, double Q, const double* Qp, double* acc) {
    const int dim = t.dim, n = t.n, n1 = t.n1, m4 = t.rn[4];
    int np = 1;
    for (int d = 0; d < dim; ++d) np *= m4;
    for (int i = 0; i < n; ++i) acc[i] = 0.0;
    if (!Qp && Q == 0.0) return;
    for (int q = 0; q < np; ++q) {
        int id[3], rq = q;
        double xi[3], w = 1.0;
        for (int d = 0; d < dim; ++d) { id[d] = rq % m4; rq /= m4; xi[d] = t.rx[4][id[d]]; w *= t.rw[4][id[d]]; }
        double J[3][3], A[3][3];
        cell_jacobian(dim, X, xi, J, nullptr);
        const double val = adjugate(dim, J, A) * (Qp ? Qp[q] : Q);
        double v[3][kMaxOrder + 1];
        for (int d = 0; d < dim; ++d) lagrange1d(n1, t.nodes, xi[d], v[d], nullptr);
        for (int i = 0; i < n; ++i) {
            int ii[3]; dof_index(dim, n1, i, ii);
            double ph = 1.0;
            for (int d = 0; d < dim; ++d) ph *= v[d][ii[d]];
            acc[i] += w * val * ph;
        }
    }
}

__global__ void __launch_bounds__(128) k_form_source(RefTables t, int ne, int Nw, int G, long long ndof,
                                                     const double* __restrict__ corners, const double* __restrict__ omega,
                                                     const Slot* __restrict__ slots, const double* __restrict__ qcell,
                                                     const double* __restrict__ qpts, int q_dir,
                                                     const double* __restrict__ inflow, int nattr, int angular,
                                                     double* __restrict__ out) {
    // one thread per (g, e): a direction-independent domain term is
    // integrated once and each angle adds its own boundary terms to a copy
    // (the same sums in the same order as integrating per angle)
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)G * ne) return;
    const int e = (int)(tid % ne);
    const int g = (int)(tid / ne);
    const int dim = t.dim, n = t.n, n1 = t.n1, nc = 1 << dim;
    double X[24];
    for (int q = 0; q < nc * dim; ++q) X[q] = corners[(size_t)e * nc * dim + q];
    int np = 1;
    for (int d = 0; d < dim; ++d) np *= t.rn[4];
    const double Q = qcell ? qcell[(size_t)g * ne + e] : 0.0;
    double vol[64];
    if (!(qpts && q_dir)) source_domain_term(t, X, Q, qpts ? qpts + ((size_t)g * ne + e) * np : nullptr, vol);
    // boundary faces of this cell that may carry inflow
    bool any_inflow = false;
    if (inflow)
        for (int k = 0; k < 2 * dim; ++k) {
            const Slot s = slots[(size_t)e * 2 * dim + k];
            if (s.nbr < 0 && s.attr >= 0 && s.attr < nattr && (angular || inflow[(size_t)g * nattr + s.attr] != 0.0))
                any_inflow = true;
        }
    const int m5 = t.rn[5];
    int npf = 1;
    for (int d = 0; d < dim - 1; ++d) npf *= m5;
    for (int a = 0; a < Nw; ++a) {
        double* o = out + psi_index(ndof, Nw, g, a, (long long)e * n);
        double acc[64];
        if (qpts && q_dir) source_domain_term(t, X, 0.0, qpts + (((size_t)g * Nw + a) * ne + e) * np, acc);
        else for (int i = 0; i < n; ++i) acc[i] = vol[i];
        if (any_inflow) {
            double om[3] = {0, 0, 0};
            for (int d = 0; d < dim; ++d) om[d] = omega[a * dim + d];
            for (int k = 0; k < 2 * dim; ++k) {
                const Slot s = slots[(size_t)e * 2 * dim + k];
                if (s.nbr >= 0 || s.attr < 0 || s.attr >= nattr) continue;
                const double fin = angular ? inflow[((size_t)g * Nw + a) * nattr + s.attr] : inflow[(size_t)g * nattr + s.attr];
                if (fin == 0.0) continue;
                for (int q = 0; q < npf; ++q) {
                    int id[3], rq = q;
                    double tt[2] = {0, 0}, w = 1.0;
                    for (int d = 0; d < dim - 1; ++d) { id[d] = rq % m5; rq /= m5; tt[d] = t.rx[5][id[d]]; w *= t.rw[5][id[d]]; }
                    double xi[3], J[3][3], A[3][3];
                    face_to_cell(dim, k, tt, xi);
                    cell_jacobian(dim, X, xi, J, nullptr);
                    adjugate(dim, J, A);
                    const double sg = (k % 2) ? 1.0 : -1.0;
                    double un = 0.0;
                    for (int d = 0; d < dim; ++d) un += om[d] * (sg * A[k / 2][d]);
                    const double wt = (0.5 * -1.0 * un - (-0.5) * fabs(un)) * (w * fin);
                    double v[3][kMaxOrder + 1];
                    for (int d = 0; d < dim; ++d) lagrange1d(n1, t.nodes, xi[d], v[d], nullptr);
                    for (int i = 0; i < n; ++i) {
                        int ii[3]; dof_index(dim, n1, i, ii);
                        double ph = 1.0;
                        for (int d = 0; d < dim; ++d) ph *= v[d][ii[d]];
                        acc[i] += wt * ph;
                    }
                }
            }
        }
        for (int i = 0; i < n; ++i) o[i] = acc[i];
    }
}

cudaError_t launch_form_source(Handle& h, const double* q_cell, const double* q_points, int q_dir, const double* inflow,
                               int nattr, int angular, double* out) {
    const long long total = (long long)h.G * h.ne;
    const int b = 128;
    k_form_source<<<(unsigned)((total + b - 1) / b), b, 0, h.stream>>>(h.ref, h.ne, h.Nw, h.G, h.ndof, h.d_corners, h.d_omega,
                                                                       h.d_slots, q_cell, q_points, q_dir, inflow, nattr,
                                                                       angular, out);
    return cudaGetLastError();
}

// Physical coordinates of the source rule's points, [Ne][points][dim], in the
// order k_form_source takes their densities.
__global__ void k_source_points(RefTables t, int ne, const double* __restrict__ corners, double* __restrict__ out) {
    const int dim = t.dim, nc = 1 << dim, m4 = t.rn[4];
    int np = 1;
    for (int d = 0; d < dim; ++d) np *= m4;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)ne * np) return;
    const int e = (int)(tid / np), q = (int)(tid % np);
    double X[24];
    for (int c = 0; c < nc * dim; ++c) X[c] = corners[(size_t)e * nc * dim + c];
    int rq = q;
    double xi[3] = {0, 0, 0}, J[3][3], x[3];
    for (int d = 0; d < dim; ++d) { xi[d] = t.rx[4][rq % m4]; rq /= m4; }
    cell_jacobian(dim, X, xi, J, x);
    for (int d = 0; d < dim; ++d) out[tid * dim + d] = x[d];
}

int source_points_per_cell(const Handle& h) {
    int np = 1;
    for (int d = 0; d < h.dim; ++d) np *= h.ref.rn[4];
    return np;
}

cudaError_t launch_source_points(Handle& h, double* out) {
    const long long total = (long long)h.ne * source_points_per_cell(h);
    k_source_points<<<(unsigned)((total + 127) / 128), 128, 0, h.stream>>>(h.ref, h.ne, h.d_corners, out);
    return cudaGetLastError();
}

// ------------------------------------------------------------ moments
// DiscreteToMoment::Mult (transport_op.cpp:3-31).  The sums run over angles in
// order with separate multiply and add roundings, as the reference loop does.
__global__ void k_moments(int Nw, int G, int dim, long long ndof, const double* __restrict__ omega,
                          const double* __restrict__ w, const double* __restrict__ psi, double* __restrict__ phi, int nmom) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    double acc = 0.0;
    for (int a = 0; a < Nw; ++a) acc = __dadd_rn(acc, __dmul_rn(w[a], psi[psi_index(ndof, Nw, g, a, s)]));
    phi[s + ndof * g] = acc;
    for (int m = 0; m + 1 < nmom; ++m) {
        double am = 0.0;
        for (int a = 0; a < Nw; ++a)
            am = __dadd_rn(am, __dmul_rn(__dmul_rn(omega[a * dim + m], w[a]), psi[psi_index(ndof, Nw, g, a, s)]));
        phi[s + ndof * (g + (long long)G * (1 + m))] = am;
    }
}

// MultTranspose / AddMultTranspose (transport_op.cpp:33-89)
__global__ void k_moments_transpose(int Nw, int G, int dim, long long ndof, const double* __restrict__ omega,
                                    double wsum, const double* __restrict__ phi, double* __restrict__ psi,
                                    int nmom, double alpha, int add) {
    // one thread per (g, i): the isotropic term p0 / sum_w does not depend on
    // the angle, so it is divided once and written to every angle (the writes
    // of a warp are contiguous for each angle)
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)G * ndof) return;
    const long long s = t % ndof;
    const int g = (int)(t / ndof);
    const double p0 = phi[s + ndof * g];
    const double q0 = add ? __ddiv_rn(__dmul_rn(alpha, p0), wsum) : __ddiv_rn(p0, wsum);
    for (int a = 0; a < Nw; ++a) {
        double* p = psi + psi_index(ndof, Nw, g, a, s);
        double v = add ? __dadd_rn(*p, q0) : q0;
        for (int m = 0; m + 1 < nmom; ++m) {
            const double ph = phi[s + ndof * (g + (long long)G * (1 + m))];
            const double om = omega[a * dim + m];
            const double c = add ? __dmul_rn(__dmul_rn(__dmul_rn(alpha, 3.0), om), ph) : __dmul_rn(__dmul_rn(3.0, om), ph);
            v = __dadd_rn(v, __ddiv_rn(c, wsum));
        }
        *p = v;
    }
}

cudaError_t launch_moments(Handle& h, const double* psi, double* phi, int nmom) {
    const long long total = (long long)h.G * h.ndof;
    const int b = 256;
    k_moments<<<(unsigned)((total + b - 1) / b), b, 0, h.stream>>>(h.Nw, h.G, h.dim, h.ndof, h.d_omega, h.d_weights, psi, phi, nmom);
    return cudaGetLastError();
}

cudaError_t launch_moments_transpose(Handle& h, const double* phi, double* psi, int nmom, double alpha, int add) {
    const long long total = (long long)h.G * h.ndof;
    const int b = 256;
    k_moments_transpose<<<(unsigned)((total + b - 1) / b), b, 0, h.stream>>>(h.Nw, h.G, h.dim, h.ndof, h.d_omega, h.wsum,
                                                                            phi, psi, nmom, alpha, add);
    return cudaGetLastError();
}

// ------------------------------------------------------------ balance
// ComputeBalance (sweep.cpp:1400-1462): sum over (g, a, e) of
//   w_a * 1^T (sigma M + tau Mt) psi_e   +   leakage of outflow boundary faces
//   w_a * (Omega.n) * 1^T F_self psi_e|face.
// Each block writes one partial sum; a second pass adds them in order, so the
// result does not depend on scheduling.
constexpr int kBalanceBlock = 256;

__global__ void __launch_bounds__(kBalanceBlock) k_balance(RefTables t, int ne, int Nw, int G, long long ndof,
                                                           const double* __restrict__ w,
                                                           const double* __restrict__ dots, const Slot* __restrict__ slots,
                                                           const double* __restrict__ M, const double* __restrict__ Mt,
                                                           const double* __restrict__ F, const double* __restrict__ sigma,
                                                           double tau, int td, const double* __restrict__ psi,
                                                           double* __restrict__ partial) {
    const int dim = t.dim, n = t.n, nf = t.nf, nface = t.nface;
    const long long total = (long long)G * ne * Nw;
    double local = 0.0;
    for (long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x; tid < total;
         tid += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(tid % Nw);
        const long long r = tid / Nw;
        const int e = (int)(r % ne), g = (int)(r / ne);
        const double* x = psi + psi_index(ndof, Nw, g, a, (long long)e * n);
        const double* Me = M + (size_t)e * n * n;
        const double sg = sigma[(size_t)g * ne + e];
        double absb = 0.0;
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int j = 0; j < n; ++j) {
                double m = sg * Me[i * n + j];
                if (td) m += tau * Mt[(size_t)e * n * n + i * n + j];
                s += m * x[j];
            }
            absb += s;
        }
        double contrib = absb * w[a];
        for (int k = 0; k < nface; ++k) {
            const Slot s = slots[(size_t)e * nface + k];
            if (s.nbr >= 0) continue;
            const double dot = dots[(size_t)s.face * Nw + a];
            if (dot < 0.0) continue;
            const double* Fk = F + ((size_t)e * nface + k) * nf * nf;
            double sum = 0.0;
            for (int ii = 0; ii < nf; ++ii) {
                double acc = 0.0;
                for (int jj = 0; jj < nf; ++jj) acc += Fk[ii * nf + jj] * x[face_dof(dim, t.p, k, jj)];
                sum += acc;
            }
            contrib += w[a] * dot * sum;
        }
        local += contrib;
    }
    __shared__ double red[kBalanceBlock];
    red[threadIdx.x] = local;
    __syncthreads();
    for (int s = kBalanceBlock / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_sum_partials(const double* __restrict__ partial, int nparts, double* __restrict__ out) {
    __shared__ double red[kBalanceBlock];
    double s = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += partial[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = kBalanceBlock / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

cudaError_t launch_balance(Handle& h, const double* psi, double* partial, int nblocks_max, int* nblocks) {
    const long long total = (long long)h.G * h.ne * h.Nw;
    long long want = (total + kBalanceBlock - 1) / kBalanceBlock;
    const int nb = (int)(want < nblocks_max ? want : nblocks_max);
    *nblocks = nb < 1 ? 1 : nb;
    k_balance<<<*nblocks, kBalanceBlock, 0, h.stream>>>(h.ref, h.ne, h.Nw, h.G, h.ndof, h.d_weights, h.d_dots,
                                                         h.d_slots, h.d_M, h.d_Mt, h.d_F, h.d_sigma, h.tau,
                                                         h.time_dependent ? 1 : 0, psi, partial);
    return cudaGetLastError();
}

cudaError_t launch_balance_finish(Handle& h, const double* partial, int nparts, double* out) {
    k_sum_partials<<<1, kBalanceBlock, 0, h.stream>>>(partial, nparts, out);
    return cudaGetLastError();
}

// ------------------------------------------------------------ scattering source
// q(g,a,e.) = q_fixed(g,a,e.) + (sigma_s[g][e] Ms_e phi(g,e.)) / sum_w
// with Ms_e the MassIntegrator matrix (rule order 2p + OrderW; vertex rule when
// the mass is lumped): the S.Mult -> D.MultTranspose -> psi += source chain of
// MomentMethodFixedPointOperator::Mult (transport_op.hpp:75-90).
__global__ void k_scatter_source(int ne, int Nw, int G, int n, long long ndof, double wsum,
                                 const double* __restrict__ Ms, const double* __restrict__ sigma_s,
                                 const double* __restrict__ phi, const double* qfix, double* out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    const int e = (int)(s / n), i = (int)(s % n);
    const double* M = Ms + (size_t)e * n * n + (size_t)i * n;
    const double* ph = phi + ndof * g + (long long)e * n;
    double acc = 0.0;
    for (int j = 0; j < n; ++j) acc += M[j] * ph[j];
    const double v = (sigma_s[(size_t)g * ne + e] * acc) / wsum;
    for (int a = 0; a < Nw; ++a) {
        const long long k = psi_index(ndof, Nw, g, a, s);
        out[k] = qfix ? qfix[k] + v : v;
    }
}

cudaError_t launch_scatter_source(Handle& h, const double* sigma_s, const double* phi, const double* qfix, double* out) {
    const long long total = (long long)h.G * h.ndof;
    const int b = 256;
    k_scatter_source<<<(unsigned)((total + b - 1) / b), b, 0, h.stream>>>(h.ne, h.Nw, h.G, h.n, h.ndof, h.wsum, h.d_Mt,
                                                                          sigma_s, phi, qfix, out);
    return cudaGetLastError();
}

// FP32 psi -> FP64 moments (zeroth moment, FP64 accumulation over angles)
__global__ void k_moments_f32(int Nw, int G, long long ndof, const double* __restrict__ w,
                              const float* __restrict__ psi, double* __restrict__ phi) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    double acc = 0.0;
    for (int a = 0; a < Nw; ++a) acc = fma(w[a], (double)psi[psi_index(ndof, Nw, g, a, s)], acc);
    phi[s + ndof * g] = acc;
}

cudaError_t launch_moments_f32(Handle& h, const float* psi, double* phi) {
    const long long total = (long long)h.G * h.ndof;
    const int b = 256;
    k_moments_f32<<<(unsigned)((total + b - 1) / b), b, 0, h.stream>>>(h.Nw, h.G, h.ndof, h.d_weights, psi, phi);
    return cudaGetLastError();
}

// FP32 scattering source: out = (float)(D^T (S phi) + q_fixed), S phi in FP64
__global__ void k_scatter_source_f32(int ne, int Nw, int G, int n, long long ndof, double wsum,
                                     const double* __restrict__ Ms, const double* __restrict__ sigma_s,
                                     const double* __restrict__ phi, const float* qfix, float* out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    const int e = (int)(s / n), i = (int)(s % n);
    const double* M = Ms + (size_t)e * n * n + (size_t)i * n;
    const double* ph = phi + ndof * g + (long long)e * n;
    double acc = 0.0;
    for (int j = 0; j < n; ++j) acc += M[j] * ph[j];
    const double v = (sigma_s[(size_t)g * ne + e] * acc) / wsum;
    for (int a = 0; a < Nw; ++a) {
        const long long k = psi_index(ndof, Nw, g, a, s);
        out[k] = qfix ? (float)((double)qfix[k] + v) : (float)v;
    }
}

cudaError_t launch_scatter_source_f32(Handle& h, const double* sigma_s, const double* phi, const float* qfix, float* out) {
    const long long total = (long long)h.G * h.ndof;
    const int b = 256;
    k_scatter_source_f32<<<(unsigned)((total + b - 1) / b), b, 0, h.stream>>>(h.ne, h.Nw, h.G, h.n, h.ndof, h.wsum, h.d_Mt,
                                                                              sigma_s, phi, qfix, out);
    return cudaGetLastError();
}

// ------------------------------------------------------------ FP32 copies
__global__ void k_to_f32(const double* __restrict__ in, float* __restrict__ out, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

// Transport-vector layouts (tvector.hpp:47-53): RIGHT psi(g,a,i) at
// i + Ndof (a + Nw g), LEFT at g + G (a + Nw i).  With c = g + G a both are a
// (c, i) matrix, row-major one way and column-major the other; one 32 x 32 tile
// per block is staged in shared memory so reads and writes are both coalesced.
__global__ void __launch_bounds__(256) k_relayout(long long ndof, int Nw, int G, const double* __restrict__ in,
                                                  double* __restrict__ out, int to_left) {
    __shared__ double tile[32][33];   // tile[c - c0][i - i0]
    const long long i0 = (long long)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int GN = G * Nw;
    if (to_left) {
        for (int k = ty; k < 32; k += 8) {
            const int c = c0 + k;
            const long long i = i0 + tx;
            if (c < GN && i < ndof) tile[k][tx] = in[i + ndof * ((c / G) + (long long)Nw * (c % G))];
        }
        __syncthreads();
        for (int k = ty; k < 32; k += 8) {
            const int c = c0 + tx;
            const long long i = i0 + k;
            if (c < GN && i < ndof) out[c + (long long)GN * i] = tile[tx][k];
        }
    } else {
        for (int k = ty; k < 32; k += 8) {
            const int c = c0 + tx;
            const long long i = i0 + k;
            if (c < GN && i < ndof) tile[tx][k] = in[c + (long long)GN * i];
        }
        __syncthreads();
        for (int k = ty; k < 32; k += 8) {
            const int c = c0 + k;
            const long long i = i0 + tx;
            if (c < GN && i < ndof) out[i + ndof * ((c / G) + (long long)Nw * (c % G))] = tile[k][tx];
        }
    }
}

cudaError_t launch_relayout(Handle& h, const double* in, double* out, int to_left) {
    const long long tiles_i = (h.ndof + 31) / 32;
    const long long tiles_c = ((long long)h.G * h.Nw + 31) / 32;
    if (tiles_i > 0x7fffffffLL || tiles_c > 65535) return cudaErrorInvalidValue;
    k_relayout<<<dim3((unsigned)tiles_i, (unsigned)tiles_c), 256, 0, h.stream>>>(h.ndof, h.Nw, h.G, in, out, to_left);
    return cudaGetLastError();
}

static cudaError_t to_f32(Handle& h, const double* in, float** out, long long n) {
    if (!in || n == 0) return cudaSuccess;
    if (!*out) {
        cudaError_t e = cudaMalloc(out, n * sizeof(float));
        if (e != cudaSuccess) return e;
    }
    k_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, h.stream>>>(in, *out, n);
    return cudaGetLastError();
}

cudaError_t make_fp32_copies(Handle& h) {
    const long long nn = (long long)h.n * h.n;
    cudaError_t e;
    if ((e = to_f32(h, h.d_G, &h.f_G, (long long)h.ne * h.dim * nn)) != cudaSuccess) return e;
    if ((e = to_f32(h, h.d_M, &h.f_M, (long long)h.ne * nn)) != cudaSuccess) return e;
    if ((e = to_f32(h, h.d_F, &h.f_F, (long long)h.ne * h.nface * h.nf * h.nf)) != cudaSuccess) return e;
    if ((e = to_f32(h, h.d_sigma, &h.f_sigma, (long long)h.G * h.ne)) != cudaSuccess) return e;
    if (h.time_dependent && (e = to_f32(h, h.d_Mt, &h.f_Mt, (long long)h.ne * nn)) != cudaSuccess) return e;
    h.fp32_ready = true;
    return cudaSuccess;
}

}  // namespace allium
