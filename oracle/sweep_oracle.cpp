// CPU ORACLE -- test infrastructure only.
//
// This file is a plain FP64 restatement of allium's upwind DG transport sweep
// and the operators around it.  It exists so the tests, the smoke check and the
// CPU baseline leg of bench.py have something independent to compare the CUDA
// product against.  Nothing in allium_gb300/ links, loads or calls it.
//
// Reference behaviour restated here (paths inside steven-t-walton/allium):
//   src/sweep.cpp:123-208   upwind graph: one edge per (interior face, angle),
//                           direction from sign(Omega . n_face_centre), ties
//                           (dot == 0) keep element1 -> element2
//   src/sweep.cpp:277-669   Mult_Upwind: Kahn frontiers; per node assemble
//                           sum_d Omega_d G_d + outflow faces + M_sigma (+tau M),
//                           subtract upwind face terms, dense LU solve
//   src/sweep.cpp:924-1022  AssembleLocalMatrices / SetTimeAbsorption
//   src/sweep.cpp:1135-1185 FormTransportSource (DomainLF + BoundaryFlow(-1,-0.5))
//   src/sweep.cpp:1187-1244 FaceMassMatricesIntegrator (rule order 2*max(p))
//   src/sweep.cpp:1246-1387 AdvectionOperator::Mult
//   src/sweep.cpp:1400-1462 AdvectionOperator::ComputeBalance
//   src/mg_form.cpp:4-65    MGMassIntegrator (rule order 2p)
//   src/lumping.cpp:3-12    LumpedIntegrationRule (reference-cell vertices)
//   src/transport_op.cpp:3-89 DiscreteToMoment Mult / MultTranspose / AddMultTranspose
//   src/tvector.hpp:47-70   RIGHT layout psi(g,a,i) = i + Ndof*(a + Nw*g),
//                           moments phi(g,m,i) = i + Ndof*(g + G*m)
//   src/sweep.cpp:177-195,432-437, src/angular_quadrature.cpp:8-36
//                           reflective boundaries (mirror angle edges and trace)
//   src/fixup.cpp:3-174     zero, zero-and-scale, local-optimization and Ryosuke negative-flux fixups
//   src/planck.hpp:157-236  Planck / Rosseland group integrals
//   src/trt_integrators.cpp:56-302, exe/scallion.cpp:755-797,1352-1470,
//   src/tvector.cpp:76-95   TRT emission, energy balance, absorption, time source
// Third-party arithmetic the reference takes from MFEM (@171eeb40, not present
// here) is restated from MFEM's published algorithms: L2 Gauss-Lobatto tensor
// basis with lexicographic local DOFs, Gauss-Legendre rules with MFEM's point
// counts (n = order/2 + 1), ConservativeConvectionIntegrator (-(u, Q.grad v)
// with adj(J)), MassIntegrator (order 2p + OrderW), CalcOrtho face normals,
// LUFactors (partial pivoting, reciprocal pivot, divide in back substitution).
//
// Build: oracle/build.py compiles this file with -O2 -fopenmp -ffp-contract=off.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <vector>
#include <omp.h>

namespace {

// ------------------------------------------------------------------ 1D rules
struct Rule1D {
    std::vector<double> x, w;
};

double legendre(int n, double x, double* dp) {
    // P_n(x) on [-1,1] by the three-term recurrence; dp <- P_n'(x)
    double p0 = 1.0, p1 = x;
    if (n == 0) { *dp = 0.0; return 1.0; }
    for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
    }
    *dp = n * (x * p1 - p0) / (x * x - 1.0);
    return p1;
}

Rule1D gauss_legendre(int n) {
    // n-point Gauss-Legendre rule mapped to [0,1]
    Rule1D r; r.x.resize(n); r.w.resize(n);
    for (int i = 0; i < (n + 1) / 2; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p = legendre(n, z, &dp);
            double dz = p / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        legendre(n, z, &dp);
        double w = 2.0 / ((1.0 - z * z) * dp * dp);
        // z is the i-th largest root; store ascending on [0,1]
        r.x[n - 1 - i] = 0.5 * (1.0 + z);
        r.x[i] = 0.5 * (1.0 - z);
        r.w[i] = r.w[n - 1 - i] = 0.5 * w;
    }
    if (n % 2 == 1) r.x[n / 2] = 0.5;
    return r;
}

std::vector<double> gll_nodes(int p) {
    // Gauss-Lobatto nodes on [0,1]: endpoints and roots of P_p'
    if (p == 0) return {0.5};
    std::vector<double> x(p + 1);
    x[0] = 0.0; x[p] = 1.0;
    for (int i = 1; i < p; ++i) {
        double z = -std::cos(M_PI * i / p);
        for (int it = 0; it < 100; ++it) {
            // Newton on q(z) = P_p'(z); q'(z) from the Legendre ODE
            double dp = 0.0;
            double pp = legendre(p, z, &dp);
            double d2 = (2.0 * z * dp - p * (p + 1.0) * pp) / (1.0 - z * z);
            double dz = dp / d2;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        x[i] = 0.5 * (1.0 + z);
    }
    return x;
}

// 1D Lagrange basis on given nodes: values and derivatives at t
void lagrange(const std::vector<double>& nd, double t, double* v, double* dv) {
    const int m = (int)nd.size();
    for (int i = 0; i < m; ++i) {
        double val = 1.0, der = 0.0;
        for (int j = 0; j < m; ++j) {
            if (j == i) continue;
            double f = (t - nd[j]) / (nd[i] - nd[j]);
            der = der * f + val / (nd[i] - nd[j]);
            val *= f;
        }
        v[i] = val;
        if (dv) dv[i] = der;
    }
}

struct QPoint { double xi[3]; double w; };

std::vector<QPoint> tensor_rule(int dim, const Rule1D& r) {
    std::vector<QPoint> q;
    const int m = (int)r.x.size();
    int tot = 1; for (int d = 0; d < dim; ++d) tot *= m;
    for (int k = 0; k < tot; ++k) {
        QPoint p{{0.5, 0.5, 0.5}, 1.0};
        int kk = k;
        for (int d = 0; d < dim; ++d) { int id = kk % m; kk /= m; p.xi[d] = r.x[id]; p.w *= r.w[id]; }
        q.push_back(p);
    }
    return q;
}

Rule1D vertex_rule1d() { Rule1D r; r.x = {0.0, 1.0}; r.w = {0.5, 0.5}; return r; }

// ------------------------------------------------------------------ problem
struct Face {
    int e1, k1, e2, k2;   // e2 < 0 on the boundary
    int attr;
    double nrm[3];        // unit normal at the face centre, out of e1
    int sb[2], sc[2][2];  // e2 face coords s = sb + sc * t (t = e1 face coords)
    std::vector<int> refl;  // reflective boundary: reflected angle of each entering angle, else -1
};

struct Oracle {
    int dim, p, n1, n, ne, nv, G, Nw, lump;
    std::vector<double> X;   // [nv][dim]
    std::vector<int> V;      // [ne][2^dim] corner ordered
    std::vector<Face> faces;
    std::vector<int> efaces; // [ne][2*dim]
    std::vector<double> omega, wq; double wsum;
    std::vector<double> sigma;  // [G][ne]
    bool timedep = false; double tau = 0.0;
    int fix_kind = 0; double fix_min = 0.0;        // negative-flux fixup (fixup.cpp)
    long long fix_unsupported = 0;                  // Ryosuke solves with more than three positive entries
    long long fix_applied = 0, fix_failed = 0;
    std::vector<double> basis_nodes;
    std::vector<double> Ms, Gm, Mt, F;  // see assemble()
    std::vector<int> indeg0;            // in-degree per node
    std::vector<std::pair<int, int>> rout;  // reflective edges (from node, to node), sorted
    long long ndof() const { return (long long)ne * n; }
    long long psi_size() const { return (long long)G * Nw * ndof(); }
};

const int kQuadCorner[4] = {0, 1, 3, 2};           // corner (c0 + 2 c1) -> MFEM vertex
const int kHexCorner[8] = {0, 1, 3, 2, 4, 5, 7, 6};

void shape_geom(int dim, const double* xi, double* N, double (*dN)[3]) {
    const int nc = 1 << dim;
    for (int c = 0; c < nc; ++c) {
        double v = 1.0;
        for (int d = 0; d < dim; ++d) v *= ((c >> d) & 1) ? xi[d] : 1.0 - xi[d];
        N[c] = v;
        for (int q = 0; q < dim; ++q) {
            double g = 1.0;
            for (int d = 0; d < dim; ++d) {
                double f = (d == q) ? (((c >> d) & 1) ? 1.0 : -1.0) : (((c >> d) & 1) ? xi[d] : 1.0 - xi[d]);
                g *= f;
            }
            dN[c][q] = g;
        }
    }
}

// J[r][q] = dx_r / dxi_q ; x = physical point
void geometry(const Oracle& o, int e, const double* xi, double J[3][3], double* x) {
    double N[8], dN[8][3];
    shape_geom(o.dim, xi, N, dN);
    const int nc = 1 << o.dim;
    for (int r = 0; r < o.dim; ++r) {
        double xr = 0.0;
        for (int q = 0; q < o.dim; ++q) J[r][q] = 0.0;
        for (int c = 0; c < nc; ++c) {
            const double X = o.X[(size_t)o.V[(size_t)e * nc + c] * o.dim + r];
            xr += N[c] * X;
            for (int q = 0; q < o.dim; ++q) J[r][q] += dN[c][q] * X;
        }
        if (x) x[r] = xr;
    }
}

double det_adj(int dim, const double J[3][3], double A[3][3]) {
    if (dim == 1) { A[0][0] = 1.0; return J[0][0]; }
    if (dim == 2) {
        A[0][0] = J[1][1]; A[0][1] = -J[0][1];
        A[1][0] = -J[1][0]; A[1][1] = J[0][0];
        return J[0][0] * J[1][1] - J[0][1] * J[1][0];
    }
    // row a of adj(J) = column (a+1) x column (a+2)
    for (int a = 0; a < 3; ++a) {
        int b = (a + 1) % 3, c = (a + 2) % 3;
        A[a][0] = J[1][b] * J[2][c] - J[2][b] * J[1][c];
        A[a][1] = J[2][b] * J[0][c] - J[0][b] * J[2][c];
        A[a][2] = J[0][b] * J[1][c] - J[1][b] * J[0][c];
    }
    return J[0][0] * A[0][0] + J[1][0] * A[0][1] + J[2][0] * A[0][2];
}

// tensor basis values (and reference gradients) at xi
void basis(const Oracle& o, const double* xi, double* phi, double (*dphi)[3]) {
    double v[3][8], dv[3][8];
    for (int d = 0; d < o.dim; ++d) lagrange(o.basis_nodes, xi[d], v[d], dv[d]);
    for (int i = 0; i < o.n; ++i) {
        int id[3] = {0, 0, 0}, r = i;
        for (int d = 0; d < o.dim; ++d) { id[d] = r % o.n1; r /= o.n1; }
        double val = 1.0;
        for (int d = 0; d < o.dim; ++d) val *= v[d][id[d]];
        phi[i] = val;
        if (dphi) {
            for (int q = 0; q < o.dim; ++q) {
                double g = 1.0;
                for (int d = 0; d < o.dim; ++d) g *= (d == q) ? dv[d][id[d]] : v[d][id[d]];
                dphi[i][q] = g;
            }
        }
    }
}

// local face k = 2*axis + side; tangential axes in increasing order
void face_point(int dim, int k, const double* t, double* xi) {
    const int a = k / 2, s = k % 2;
    int j = 0;
    for (int d = 0; d < dim; ++d) {
        if (d == a) xi[d] = s;
        else xi[d] = t[j++];
    }
}

int face_corner_vertex(const Oracle& o, int e, int k, int m) {
    const int a = k / 2, s = k % 2, nc = 1 << o.dim;
    int c = 0, j = 0;
    for (int d = 0; d < o.dim; ++d) {
        int bit = (d == a) ? s : ((m >> j++) & 1);
        c |= bit << d;
    }
    return o.V[(size_t)e * nc + c];
}

void build_topology(Oracle& o, int nbf, const int* bfv, const int* battr) {
    const int nfc = 1 << (o.dim - 1);
    std::map<std::vector<int>, int> key2face;
    o.efaces.assign((size_t)o.ne * 2 * o.dim, -1);
    for (int e = 0; e < o.ne; ++e) {
        for (int k = 0; k < 2 * o.dim; ++k) {
            std::vector<int> key(nfc);
            for (int m = 0; m < nfc; ++m) key[m] = face_corner_vertex(o, e, k, m);
            std::sort(key.begin(), key.end());
            auto it = key2face.find(key);
            if (it == key2face.end()) {
                Face f{}; f.e1 = e; f.k1 = k; f.e2 = -1; f.k2 = -1; f.attr = 0;
                key2face[key] = (int)o.faces.size();
                o.efaces[(size_t)e * 2 * o.dim + k] = (int)o.faces.size();
                o.faces.push_back(f);
            } else {
                Face& f = o.faces[it->second];
                f.e2 = e; f.k2 = k;
                o.efaces[(size_t)e * 2 * o.dim + k] = it->second;
                // e2 face coordinates as an affine image of e1 face coordinates
                int td = o.dim - 1;
                auto corner_in_e2 = [&](int m1) {
                    int v = face_corner_vertex(o, f.e1, f.k1, m1);
                    for (int m2 = 0; m2 < nfc; ++m2)
                        if (face_corner_vertex(o, e, k, m2) == v) return m2;
                    return -1;
                };
                int m0 = corner_in_e2(0);
                for (int j = 0; j < td; ++j) f.sb[j] = (m0 >> j) & 1;
                for (int c = 0; c < td; ++c) {
                    int mc = corner_in_e2(1 << c);
                    for (int j = 0; j < td; ++j) f.sc[j][c] = ((mc >> j) & 1) - f.sb[j];
                }
            }
        }
    }
    for (int b = 0; b < nbf; ++b) {
        std::vector<int> key(bfv + (size_t)b * nfc, bfv + (size_t)(b + 1) * nfc);
        std::sort(key.begin(), key.end());
        auto it = key2face.find(key);
        if (it != key2face.end()) o.faces[it->second].attr = battr[b];
    }
    // unit normal at the face centre, out of e1 (sweep.cpp:142-154)
    for (auto& f : o.faces) {
        double t[2] = {0.5, 0.5}, xi[3], J[3][3], A[3][3];
        face_point(o.dim, f.k1, t, xi);
        geometry(o, f.e1, xi, J, nullptr);
        det_adj(o.dim, J, A);
        const int a = f.k1 / 2; const double sg = (f.k1 % 2) ? 1.0 : -1.0;
        double nn = 0.0;
        for (int r = 0; r < o.dim; ++r) { f.nrm[r] = sg * A[a][r]; nn += f.nrm[r] * f.nrm[r]; }
        const double inv = 1.0 / std::sqrt(nn);
        for (int r = 0; r < o.dim; ++r) f.nrm[r] *= inv;
    }
}

// raw outward normal (magnitude = face Jacobian) at element point xi on face k
void raw_normal(const Oracle& o, int e, int k, const double* xi, double* nr) {
    double J[3][3], A[3][3];
    geometry(o, e, xi, J, nullptr);
    det_adj(o.dim, J, A);
    const int a = k / 2; const double sg = (k % 2) ? 1.0 : -1.0;
    for (int r = 0; r < o.dim; ++r) nr[r] = sg * A[a][r];
}

double norm(int dim, const double* v) {
    double s = 0.0;
    for (int r = 0; r < dim; ++r) s += v[r] * v[r];
    return std::sqrt(s);
}

void e2_face_coords(const Face& f, int td, const double* t, double* s) {
    for (int j = 0; j < td; ++j) {
        double v = f.sb[j];
        for (int c = 0; c < td; ++c) v += f.sc[j][c] * t[c];
        s[j] = v;
    }
}

int conv_points(int dim, int p) { return dim == 3 ? p + 2 : p + 1; }

void assemble(Oracle& o) {
    const int n = o.n, nn = n * n, dim = o.dim;
    o.Ms.assign((size_t)o.G * o.ne * nn, 0.0);
    o.Gm.assign((size_t)dim * o.ne * nn, 0.0);
    const bool lm = o.lump & 1, lg = o.lump & 2, lf = o.lump & 4;
    const auto rule_mass = tensor_rule(dim, lm ? vertex_rule1d() : gauss_legendre(o.p + 1));
    const auto rule_conv = tensor_rule(dim, lg ? vertex_rule1d() : gauss_legendre(conv_points(dim, o.p)));
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o.ne; ++e) {
        std::vector<double> phi(n), uu(nn);
        std::vector<std::array<double, 3>> dphi(n);
        // MGMassIntegrator::AssembleElementMatrices, mg_form.cpp:34-55
        for (const auto& q : rule_mass) {
            double J[3][3], A[3][3];
            geometry(o, e, q.xi, J, nullptr);
            const double w = det_adj(dim, J, A) * q.w;
            basis(o, q.xi, phi.data(), nullptr);
            for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) uu[i * n + j] = phi[i] * phi[j];
            for (int g = 0; g < o.G; ++g) {
                const double s = w * o.sigma[(size_t)g * o.ne + e];
                double* M = &o.Ms[((size_t)g * o.ne + e) * nn];
                for (int k = 0; k < nn; ++k) M[k] += s * uu[k];
            }
        }
        // ConservativeConvectionIntegrator(e_d, 1): G_d(i,j) = -int phi_j d_d phi_i
        for (const auto& q : rule_conv) {
            double J[3][3], A[3][3];
            geometry(o, e, q.xi, J, nullptr);
            det_adj(dim, J, A);
            basis(o, q.xi, phi.data(), reinterpret_cast<double(*)[3]>(dphi.data()));
            for (int d = 0; d < dim; ++d) {
                double v2[3];
                for (int r = 0; r < dim; ++r) v2[r] = A[r][d] * (-1.0 * q.w);
                double* Gd = &o.Gm[((size_t)d * o.ne + e) * nn];
                for (int i = 0; i < n; ++i) {
                    double b = 0.0;
                    for (int r = 0; r < dim; ++r) b += dphi[i][r] * v2[r];
                    for (int j = 0; j < n; ++j) Gd[i * n + j] += phi[j] * b;
                }
            }
        }
    }
    // FaceMassMatricesIntegrator, sweep.cpp:1187-1244 ; blocks [f][s][t] (n x n)
    o.F.assign((size_t)o.faces.size() * 4 * nn, 0.0);
    const int td = dim - 1;
    const auto rule_face = tensor_rule(td, lf ? vertex_rule1d() : gauss_legendre(o.p + 1));
#pragma omp parallel for schedule(static)
    for (int fi = 0; fi < (int)o.faces.size(); ++fi) {
        const Face& f = o.faces[fi];
        std::vector<double> s1(n), s2(n);
        double* F = &o.F[(size_t)fi * 4 * nn];
        for (const auto& q : rule_face) {
            double xi1[3], xi2[3], nr[3], s[2];
            face_point(dim, f.k1, q.xi, xi1);
            raw_normal(o, f.e1, f.k1, xi1, nr);
            const double w = q.w * (dim == 1 ? 1.0 : norm(dim, nr));
            basis(o, xi1, s1.data(), nullptr);
            for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) F[0 * nn + i * n + j] += s1[i] * s1[j] * w;
            if (f.e2 >= 0) {
                e2_face_coords(f, td, q.xi, s);
                face_point(dim, f.k2, s, xi2);
                basis(o, xi2, s2.data(), nullptr);
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j) {
                        const double val = s1[i] * s2[j] * w;
                        F[1 * nn + i * n + j] += val;   // (1,2)
                        F[2 * nn + j * n + i] += val;   // (2,1)
                    }
                for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) F[3 * nn + i * n + j] += s2[i] * s2[j] * w;
            }
        }
    }
}

void assemble_time_mass(Oracle& o) {
    // MassIntegrator without coefficient, order 2p + OrderW (sweep.cpp:1003-1022)
    const int n = o.n, nn = n * n, dim = o.dim;
    o.Mt.assign((size_t)o.ne * nn, 0.0);
    const int npt = (dim == 3) ? o.p + 2 : o.p + 1;
    const auto rule = tensor_rule(dim, (o.lump & 1) ? vertex_rule1d() : gauss_legendre(npt));
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o.ne; ++e) {
        std::vector<double> phi(n);
        double* M = &o.Mt[(size_t)e * nn];
        for (const auto& q : rule) {
            double J[3][3], A[3][3];
            geometry(o, e, q.xi, J, nullptr);
            const double w = det_adj(dim, J, A) * q.w;
            basis(o, q.xi, phi.data(), nullptr);
            for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) M[i * n + j] += w * phi[i] * phi[j];
        }
    }
}

inline double dotv(int dim, const double* a, const double* b) {
    double s = 0.0;
    for (int d = 0; d < dim; ++d) s += a[d] * b[d];
    return s;
}

// edge across interior face f between (e1,a) and (e2,a): true when e1 -> e2
inline bool forward_edge(const Oracle& o, const Face& f, int a) {
    const double dot = dotv(o.dim, &o.omega[(size_t)a * o.dim], f.nrm);
    return !(dot < 0);
}

bool is_in_edge(const Oracle& o, int e, const Face& f, int a) {
    if (f.e2 < 0) return false;
    const bool fwd = forward_edge(o, f, a);
    return (e == f.e2) ? fwd : !fwd;
}

void build_graph(Oracle& o) {
    const int nd = 2 * o.dim;
    o.indeg0.assign((size_t)o.ne * o.Nw, 0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o.ne; ++e)
        for (int a = 0; a < o.Nw; ++a) {
            int c = 0;
            for (int k = 0; k < nd; ++k) {
                const Face& f = o.faces[o.efaces[(size_t)e * nd + k]];
                if (is_in_edge(o, e, f, a)) ++c;
            }
            o.indeg0[(size_t)e * o.Nw + a] = c;
        }
    // reflective boundary faces, sweep.cpp:177-195: for every angle entering
    // the domain, an edge (e, reflected angle) -> (e, angle)
    o.rout.clear();
    for (const Face& f : o.faces) {
        if (f.e2 >= 0 || f.refl.empty()) continue;
        for (int a = 0; a < o.Nw; ++a) {
            if (f.refl[a] < 0) continue;
            o.indeg0[(size_t)f.e1 * o.Nw + a] += 1;
            o.rout.emplace_back(f.e1 * o.Nw + f.refl[a], f.e1 * o.Nw + a);
        }
    }
    std::sort(o.rout.begin(), o.rout.end());
}

// nodes fed by u through reflective faces
template <class Fn>
void for_reflective_out(const Oracle& o, int u, Fn&& fn) {
    auto lo = std::lower_bound(o.rout.begin(), o.rout.end(), std::make_pair(u, -1));
    for (; lo != o.rout.end() && lo->first == u; ++lo) fn(lo->second);
}

// mfem::LUFactors::Factor + Solve restated (partial pivoting, column major)
bool lu_solve(int m, double* A, double* x) {
    std::vector<int> ipiv(m);
    for (int i = 0; i < m; ++i) {
        int piv = i;
        double a = std::fabs(A[piv + i * m]);
        for (int j = i + 1; j < m; ++j) {
            const double b = std::fabs(A[j + i * m]);
            if (b > a) { a = b; piv = j; }
        }
        ipiv[i] = piv;
        if (piv != i)
            for (int j = 0; j < m; ++j) std::swap(A[i + j * m], A[piv + j * m]);
        if (A[i + i * m] == 0.0) return false;
        const double inv = 1.0 / A[i + i * m];
        for (int j = i + 1; j < m; ++j) A[j + i * m] *= inv;
        for (int k = i + 1; k < m; ++k) {
            const double aik = A[i + k * m];
            for (int j = i + 1; j < m; ++j) A[j + k * m] -= aik * A[j + i * m];
        }
    }
    for (int i = 0; i < m; ++i) std::swap(x[i], x[ipiv[i]]);
    for (int j = 0; j < m; ++j) {
        const double xj = x[j];
        for (int i = j + 1; i < m; ++i) x[i] -= A[i + j * m] * xj;
    }
    for (int j = m - 1; j >= 0; --j) {
        const double xj = (x[j] /= A[j + j * m]);
        for (int i = 0; i < j; ++i) x[i] -= A[i + j * m] * xj;
    }
    return true;
}

// mfem::LinearSolve restated: closed forms for n = 1, 2; LU otherwise
// RyosukeFixupOperator::perform_nff (src/fixup.cpp:96-174): entries at or
// below the floor set to it; the others ("positive") solve C y = d with C's
// first row the column sums w of the positive entries, its first column
// -x_k / x_0 below a unit diagonal, d = (sum b, 0, ...), in the reference's
// closed forms for 1, 2, 3 unknowns.  -2 where the reference aborts (more
// than three positive entries).
int fixup_ryosuke(int n, const double* w, double total, double* x, double xmin) {
    std::vector<int> count;
    for (int i = 0; i < n; ++i) {
        if (x[i] <= xmin) x[i] = xmin;
        else count.push_back(i);
    }
    const int pos = (int)count.size();
    if (pos == 0 || pos == n) return 0;
    if (pos > 3) return -2;
    std::vector<double> C((size_t)pos * pos, 0.0);
    for (int i = 0; i < pos; ++i) {
        C[i] = w[count[i]];
        if (i == 0) {
            for (int j = 1; j < pos; ++j) C[(size_t)j * pos] = -x[count[j]] / x[count[0]];
        } else {
            C[(size_t)i * (pos + 1)] = 1.0;
        }
    }
    const double d0 = total;
    if (pos == 1) {
        x[count[0]] = d0 / C[0];
    } else if (pos == 2) {
        double det = C[0] * C[3] - C[1] * C[2];
        det = 1.0 / det;
        x[count[0]] = d0 * C[3] * det;
        x[count[1]] = -d0 * C[2] * det;
    } else {
        double det = C[0] * C[4] * C[8] - C[1] * C[3] * C[8] - C[2] * C[4] * C[6];
        det = 1.0 / det;
        x[count[0]] = d0 * C[4] * C[8] * det;
        x[count[1]] = -d0 * C[3] * C[8] * det;
        x[count[2]] = -d0 * C[4] * C[6] * det;
    }
    for (int k = 0; k < pos; ++k)
        if (x[count[k]] < xmin) {
            for (int j = 0; j < pos; ++j) x[count[j]] = xmin;
            return -1;
        }
    return 1;
}

// LocalOptimizationFixupOperator::Apply (src/fixup.cpp:59-88): argmin
// |x - x0|^2 subject to w . x = sum b and x >= floor (what
// mfem::SLBQPOptimizer iterates towards).  The minimiser is
// x_i = max(x0_i + lam w_i, floor); lam is found exactly by clamping every
// free entry that falls below the floor and recomputing lam on the rest, until
// none does.  Entries with w_i = 0 take max(x0_i, floor).
int fixup_local_opt(int n, const double* w, double total, double* x, double xmin) {
    double lo = x[0];
    for (int i = 1; i < n; ++i) lo = std::min(lo, x[i]);
    if (lo > xmin || total <= xmin) return 0;
    std::vector<char> freev(n);
    for (int i = 0; i < n; ++i) freev[i] = w[i] > 0.0;
    double lam = 0.0;
    bool feasible = false;
    for (int pass = 0; pass <= n; ++pass) {
        double rest = total, ww = 0.0;   // free: w (x0 + lam w); clamped: w * floor; w = 0: nothing
        for (int i = 0; i < n; ++i) {
            if (freev[i]) { rest -= w[i] * x[i]; ww += w[i] * w[i]; }
            else if (w[i] > 0.0) rest -= w[i] * xmin;
        }
        if (!(ww > 0.0)) break;
        lam = rest / ww;
        bool clamped = false;
        for (int i = 0; i < n; ++i)
            if (freev[i] && x[i] + lam * w[i] < xmin) { freev[i] = 0; clamped = true; }
        if (!clamped) { feasible = true; break; }
    }
    if (!feasible) {
        for (int i = 0; i < n; ++i) x[i] = x[i] > xmin ? x[i] : xmin;
        return -1;
    }
    for (int i = 0; i < n; ++i) {
        const double v = freev[i] ? x[i] + lam * w[i] : (w[i] > 0.0 ? xmin : x[i]);
        x[i] = v > xmin ? v : xmin;
    }
    return 1;
}

bool linear_solve(int m, double* A /*column major*/, double* x) {
    if (m == 1) { if (A[0] == 0.0) return false; x[0] /= A[0]; return true; }
    if (m == 2) {
        const double det = A[0] * A[3] - A[2] * A[1];
        if (det == 0.0) return false;
        const double inv = 1.0 / det, b0 = x[0], b1 = x[1];
        x[0] = (A[3] * b0 - A[2] * b1) * inv;
        x[1] = (-A[1] * b0 + A[0] * b1) * inv;
        return true;
    }
    return lu_solve(m, A, x);
}

inline long long pidx(const Oracle& o, int g, int a, long long i) {
    return i + o.ndof() * ((long long)a + (long long)o.Nw * g);
}

// one node (e,a), all groups: sweep.cpp:365-475
bool solve_node(const Oracle& o, int e, int a, const double* src, double* psi,
                std::vector<double>& grad, std::vector<double>& A, std::vector<double>& rhs) {
    const int n = o.n, nn = n * n, dim = o.dim, nd = 2 * dim;
    const double* Om = &o.omega[(size_t)a * dim];
    std::fill(grad.begin(), grad.end(), 0.0);
    for (int d = 0; d < dim; ++d) {
        const double* Gd = &o.Gm[((size_t)d * o.ne + e) * nn];
        for (int k = 0; k < nn; ++k) grad[k] += Om[d] * Gd[k];
    }
    for (int k = 0; k < nd; ++k) {
        const Face& f = o.faces[o.efaces[(size_t)e * nd + k]];
        const bool keep = (e == f.e1);
        double nor[3];
        for (int d = 0; d < dim; ++d) nor[d] = keep ? f.nrm[d] : -f.nrm[d];
        const double dot = dotv(dim, Om, nor);
        const int idx = keep ? 0 : 1;
        if (dot > 0) {
            const double* Fm = &o.F[((size_t)o.efaces[(size_t)e * nd + k] * 4 + idx * 3) * nn];
            for (int q = 0; q < nn; ++q) grad[q] += dot * Fm[q];
        }
    }
    const long long off = (long long)e * n;
    for (int g = 0; g < o.G; ++g) {
        const double* Mg = &o.Ms[((size_t)g * o.ne + e) * nn];
        // column-major copy for the LU
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) A[i + j * n] = grad[i * n + j] + 1.0 * Mg[i * n + j];
        for (int i = 0; i < n; ++i) rhs[i] = src[pidx(o, g, a, off + i)];
        for (int k = 0; k < nd; ++k) {
            const int fid = o.efaces[(size_t)e * nd + k];
            const Face& f = o.faces[fid];
            if (f.e2 < 0 && !f.refl.empty() && f.refl[a] >= 0) {
                // reflection, sweep.cpp:432-437: the same cell's values in the
                // reflected angle through the face block (1,1)
                const double dot = dotv(dim, Om, f.nrm);
                const double* Fm = &o.F[((size_t)fid * 4) * nn];
                for (int i = 0; i < n; ++i) {
                    double s = 0.0;
                    for (int j = 0; j < n; ++j) s += Fm[i * n + j] * psi[pidx(o, g, f.refl[a], off + j)];
                    rhs[i] += -dot * s;
                }
                continue;
            }
            if (!is_in_edge(o, e, f, a)) continue;
            const bool keep = (e == f.e1);
            double nor[3];
            for (int d = 0; d < dim; ++d) nor[d] = keep ? f.nrm[d] : -f.nrm[d];
            const double dot = dotv(dim, Om, nor);
            const int idx = keep ? 0 : 1, nidx = 1 - idx;
            const int nbr = keep ? f.e2 : f.e1;
            const double* Fm = &o.F[((size_t)fid * 4 + idx * 2 + nidx) * nn];
            const long long noff = (long long)nbr * n;
            for (int i = 0; i < n; ++i) {
                double s = 0.0;
                for (int j = 0; j < n; ++j) s += Fm[i * n + j] * psi[pidx(o, g, a, noff + j)];
                rhs[i] += -dot * s;
            }
        }
        if (o.timedep) {
            const double* Mt = &o.Mt[(size_t)e * nn];
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) A[i + j * n] += o.tau * Mt[i * n + j];
        }
        std::vector<double> Acopy, bcopy;
        if (o.fix_kind) { Acopy = A; bcopy = rhs; }
        if (!linear_solve(n, A.data(), rhs.data())) return false;
        if (o.fix_kind) {
            // ZeroFixupOperator / ZeroAndScaleFixupOperator::Apply (fixup.cpp:3-57)
            int applied = 0;
            double lo = rhs[0];
            for (int i = 1; i < n; ++i) lo = std::min(lo, rhs[i]);
            if (o.fix_kind == 1) {
                for (int i = 0; i < n; ++i) if (rhs[i] <= o.fix_min) { rhs[i] = o.fix_min; applied = 1; }
            } else if (o.fix_kind == 3 || o.fix_kind == 4) {
                std::vector<double> w(n, 0.0);
                for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) w[i] += Acopy[j + i * n];
                double total = 0.0;
                for (int i = 0; i < n; ++i) total += bcopy[i];
                applied = o.fix_kind == 3 ? fixup_ryosuke(n, w.data(), total, rhs.data(), o.fix_min)
                                          : fixup_local_opt(n, w.data(), total, rhs.data(), o.fix_min);
                if (applied == -2) {
#pragma omp atomic
                    const_cast<Oracle&>(o).fix_unsupported += 1;
                    applied = -1;
                }
            } else if (!(lo > o.fix_min)) {
                std::vector<double> w(n, 0.0);
                for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) w[i] += Acopy[j + i * n];
                for (int i = 0; i < n; ++i) if (rhs[i] <= o.fix_min) rhs[i] = o.fix_min;
                double orig = 0.0, nb = 0.0;
                for (int i = 0; i < n; ++i) { orig += bcopy[i]; nb += w[i] * rhs[i]; }
                if (orig < 0.0 || nb < 0.0) applied = -1;
                else if (orig == 0.0 || nb == 0.0) { for (int i = 0; i < n; ++i) rhs[i] = 0.0; applied = 1; }
                else { for (int i = 0; i < n; ++i) rhs[i] *= orig / nb; applied = 1; }
            }
            if (applied) {
#pragma omp atomic
                (applied > 0 ? const_cast<Oracle&>(o).fix_applied : const_cast<Oracle&>(o).fix_failed) += 1;
            }
        }
        for (int i = 0; i < n; ++i) psi[pidx(o, g, a, off + i)] = rhs[i];
    }
    return true;
}

}  // namespace

extern "C" {

void* oracle_create(int dim, int nv, const double* verts, int ne, const int* ev,
                    int nbf, const int* bfv, const int* battr,
                    int order, int lump, int Nw, const double* omega, const double* wts,
                    int G, const double* sigma) {
    if (dim < 1 || dim > 3 || order < 0 || order > 3 || Nw < 1 || G < 1) return nullptr;
    Oracle* o = new Oracle;
    o->dim = dim; o->p = order; o->n1 = order + 1; o->ne = ne; o->nv = nv; o->G = G; o->Nw = Nw; o->lump = lump;
    o->n = 1; for (int d = 0; d < dim; ++d) o->n *= o->n1;
    o->X.assign(verts, verts + (size_t)nv * dim);
    const int nc = 1 << dim;
    o->V.resize((size_t)ne * nc);
    for (int e = 0; e < ne; ++e)
        for (int c = 0; c < nc; ++c) {
            const int mv = (dim == 1) ? c : (dim == 2 ? kQuadCorner[c] : kHexCorner[c]);
            o->V[(size_t)e * nc + c] = ev[(size_t)e * nc + mv];
        }
    o->omega.assign(omega, omega + (size_t)Nw * dim);
    o->wq.assign(wts, wts + Nw);
    o->wsum = 0.0; for (double w : o->wq) o->wsum += w;
    o->sigma.assign(sigma, sigma + (size_t)G * ne);
    o->basis_nodes = gll_nodes(order);
    build_topology(*o, nbf, bfv, battr);
    assemble(*o);
    build_graph(*o);
    return o;
}

void oracle_destroy(void* h) { delete static_cast<Oracle*>(h); }

void oracle_set_time_absorption(void* h, double tau) {
    Oracle& o = *static_cast<Oracle*>(h);
    o.tau = tau; o.timedep = true;
    if (o.Mt.empty()) assemble_time_mass(o);
}

// Reflective boundary attributes (BoundaryCondition::REFLECTIVE).  The
// reflected angle is GetReflectedAngleIndex (angular_quadrature.cpp:27-36):
// the first direction within 1e-14 of Omega - 2 (Omega.n) n.  Returns 0, or
// -1 when an entering direction has no reflection in the set.
int oracle_set_reflective(void* h, int num, const int* attrs) {
    Oracle& o = *static_cast<Oracle*>(h);
    const int dim = o.dim;
    int status = 0;
    for (Face& f : o.faces) {
        f.refl.clear();
        if (f.e2 >= 0 || std::find(attrs, attrs + num, f.attr) == attrs + num) continue;
        f.refl.assign(o.Nw, -1);
        for (int a = 0; a < o.Nw; ++a) {
            const double* Om = &o.omega[(size_t)a * dim];
            const double dot = dotv(dim, Om, f.nrm);
            if (!(dot < 0)) continue;
            double r[3];
            for (int d = 0; d < dim; ++d) r[d] = Om[d] - (2 * dot) * f.nrm[d];
            for (int b = 0; b < o.Nw; ++b) {
                double diff = 0.0;
                for (int d = 0; d < dim; ++d) diff += std::pow(o.omega[(size_t)b * dim + d] - r[d], 2);
                if (std::sqrt(diff) < 1e-14) { f.refl[a] = b; break; }
            }
            if (f.refl[a] < 0) status = -1;
        }
    }
    build_graph(o);
    return status;
}

void oracle_set_fixup(void* h, int kind, double minimum) {
    Oracle& o = *static_cast<Oracle*>(h);
    o.fix_kind = kind; o.fix_min = minimum; o.fix_applied = o.fix_failed = 0; o.fix_unsupported = 0;
}

long long oracle_fixup_unsupported(void* h) { return static_cast<Oracle*>(h)->fix_unsupported; }

void oracle_fixup_counts(void* h, long long* applied, long long* failed) {
    const Oracle& o = *static_cast<Oracle*>(h);
    *applied = o.fix_applied; *failed = o.fix_failed;
}

int oracle_num_faces(void* h) { return (int)static_cast<Oracle*>(h)->faces.size(); }

// face f: e1, k1, e2, k2, attr ; normal -> nrm[dim]
void oracle_face_info(void* h, int f, int* info, double* nrm) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const Face& F = o.faces[f];
    info[0] = F.e1; info[1] = F.k1; info[2] = F.e2; info[3] = F.k2; info[4] = F.attr;
    for (int d = 0; d < o.dim; ++d) nrm[d] = F.nrm[d];
}

// element matrices of cell e: G (dim*n*n), M_sigma of group g (n*n); row major
void oracle_element_matrices(void* h, int e, int g, double* Gout, double* Mout) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const size_t nn = (size_t)o.n * o.n;
    for (int d = 0; d < o.dim; ++d)
        std::memcpy(Gout + d * nn, &o.Gm[((size_t)d * o.ne + e) * nn], nn * sizeof(double));
    std::memcpy(Mout, &o.Ms[((size_t)g * o.ne + e) * nn], nn * sizeof(double));
}

void oracle_time_mass(void* h, int e, double* Mout) {
    Oracle& o = *static_cast<Oracle*>(h);
    if (o.Mt.empty()) assemble_time_mass(o);   // assembled on first use
    const size_t nn = (size_t)o.n * o.n;
    std::memcpy(Mout, &o.Mt[(size_t)e * nn], nn * sizeof(double));
}

// face blocks [2][2][n][n] of face f (row major), MFEM FaceMassMatrices ordering
void oracle_face_matrices(void* h, int f, double* out) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const size_t nn = (size_t)o.n * o.n;
    std::memcpy(out, &o.F[(size_t)f * 4 * nn], 4 * nn * sizeof(double));
}

// Kahn frontiers (sweep.cpp:308-322, 477-512); level of node e*Nw + a.
// Returns the number of levels, or -1 if the graph has a cycle.
int oracle_levels(void* h, int* level) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const long long N = (long long)o.ne * o.Nw;
    const int nd = 2 * o.dim;
    std::vector<int> deg(o.indeg0);
    std::vector<int> cur, next;
    for (long long v = 0; v < N; ++v) if (deg[v] == 0) { cur.push_back((int)v); level[v] = 0; }
    long long done = 0; int lev = 0;
    while (!cur.empty()) {
        done += cur.size();
        next.clear();
        for (int u : cur) {
            const int e = u / o.Nw, a = u % o.Nw;
            for (int k = 0; k < nd; ++k) {
                const Face& f = o.faces[o.efaces[(size_t)e * nd + k]];
                if (f.e2 < 0) continue;
                const int nbr = (e == f.e1) ? f.e2 : f.e1;
                if (!is_in_edge(o, nbr, f, a)) continue;
                const int v = nbr * o.Nw + a;
                if (--deg[v] == 0) { next.push_back(v); level[v] = lev + 1; }
            }
            for_reflective_out(o, u, [&](int v) {
                if (--deg[v] == 0) { next.push_back(v); level[v] = lev + 1; }
            });
        }
        std::swap(cur, next);
        ++lev;
    }
    return done == N ? lev : -1;
}

// InverseAdvectionOperator::Mult (upwind).  src may alias psi.  Returns 0 on
// success, 2 on a cycle, 3 on a singular local system.
int oracle_sweep(void* h, const double* src, double* psi, int nthreads) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const long long N = (long long)o.ne * o.Nw;
    const int nd = 2 * o.dim, n = o.n;
    std::vector<int> deg(o.indeg0);
    std::deque<int> local;
    for (long long v = 0; v < N; ++v) if (deg[v] == 0) local.push_back((int)v);
    long long nsweep = 0;
    int status = 0;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
    {
        std::vector<double> grad((size_t)n * n), A((size_t)n * n), rhs(n);
        while (true) {
            // the frontier only changes inside the single block below, whose
            // implicit barrier makes every thread read the same size here
            const long long front = (long long)local.size();
            if (front == 0) break;
#pragma omp for schedule(dynamic, 16)
            for (long long s = 0; s < front; ++s) {
                const int node = local[s];
                if (!solve_node(o, node / o.Nw, node % o.Nw, src, psi, grad, A, rhs)) {
#pragma omp atomic write
                    status = 3;
                }
            }
#pragma omp single
            {
                nsweep += front;
                for (long long s = 0; s < front; ++s) {
                    const int u = local.front(); local.pop_front();
                    const int e = u / o.Nw, a = u % o.Nw;
                    for (int k = 0; k < nd; ++k) {
                        const Face& f = o.faces[o.efaces[(size_t)e * nd + k]];
                        if (f.e2 < 0) continue;
                        const int nbr = (e == f.e1) ? f.e2 : f.e1;
                        if (!is_in_edge(o, nbr, f, a)) continue;
                        const int v = nbr * o.Nw + a;
                        if (--deg[v] == 0) local.push_back(v);
                    }
                    for_reflective_out(o, u, [&](int v) {
                        if (--deg[v] == 0) local.push_back(v);
                    });
                }
            }
        }
    }
    if (status) return status;
    return nsweep == N ? 0 : 2;
}

// AdvectionOperator::Mult (sweep.cpp:1246-1387), single rank
void oracle_apply_L(void* h, const double* x, double* y) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const int n = o.n, nn = n * n, dim = o.dim;
    std::fill(y, y + o.psi_size(), 0.0);
#pragma omp parallel for collapse(2) schedule(static)
    for (int g = 0; g < o.G; ++g)
        for (int a = 0; a < o.Nw; ++a) {
            const double* Om = &o.omega[(size_t)a * dim];
            std::vector<double> grad(nn), yl(n), yl2(n);
            for (int e = 0; e < o.ne; ++e) {
                const long long off = (long long)e * n;
                const double* M = &o.Ms[((size_t)g * o.ne + e) * nn];
                for (int i = 0; i < n; ++i) {
                    double s = 0.0;
                    for (int j = 0; j < n; ++j) s += M[i * n + j] * x[pidx(o, g, a, off + j)];
                    yl[i] = s;
                }
                if (o.timedep) {
                    const double* Mt = &o.Mt[(size_t)e * nn];
                    for (int i = 0; i < n; ++i) {
                        double s = 0.0;
                        for (int j = 0; j < n; ++j) s += Mt[i * n + j] * x[pidx(o, g, a, off + j)];
                        yl[i] += o.tau * s;
                    }
                }
                std::fill(grad.begin(), grad.end(), 0.0);
                for (int d = 0; d < dim; ++d) {
                    const double* Gd = &o.Gm[((size_t)d * o.ne + e) * nn];
                    for (int k = 0; k < nn; ++k) grad[k] += Om[d] * Gd[k];
                }
                for (int i = 0; i < n; ++i) {
                    double s = 0.0;
                    for (int j = 0; j < n; ++j) s += grad[i * n + j] * x[pidx(o, g, a, off + j)];
                    y[pidx(o, g, a, off + i)] += yl[i] + s;
                }
            }
            for (size_t fi = 0; fi < o.faces.size(); ++fi) {
                const Face& f = o.faces[fi];
                const double dot = dotv(dim, Om, f.nrm);
                const double* F = &o.F[fi * 4 * nn];
                const long long o1 = (long long)f.e1 * n;
                std::fill(yl.begin(), yl.end(), 0.0);
                if (f.e2 >= 0) {
                    const long long o2 = (long long)f.e2 * n;
                    std::fill(yl2.begin(), yl2.end(), 0.0);
                    const int src_blk = dot >= 0 ? 0 : 1;
                    const long long os = dot >= 0 ? o1 : o2;
                    for (int i = 0; i < n; ++i) {
                        double s1 = 0.0, s2 = 0.0;
                        for (int j = 0; j < n; ++j) {
                            const double xv = x[pidx(o, g, a, os + j)];
                            s1 += F[(0 * 2 + src_blk) * nn + i * n + j] * xv;
                            s2 += F[(1 * 2 + src_blk) * nn + i * n + j] * xv;
                        }
                        yl[i] += dot * s1;
                        yl2[i] += -dot * s2;
                    }
                    for (int i = 0; i < n; ++i) y[pidx(o, g, a, o2 + i)] += yl2[i];
                } else if (dot >= 0) {
                    for (int i = 0; i < n; ++i) {
                        double s = 0.0;
                        for (int j = 0; j < n; ++j) s += F[i * n + j] * x[pidx(o, g, a, o1 + j)];
                        yl[i] += dot * s;
                    }
                }
                for (int i = 0; i < n; ++i) y[pidx(o, g, a, o1 + i)] += yl[i];
            }
        }
}

// AdvectionOperator::ComputeBalance (sweep.cpp:1400-1462)
double oracle_balance(void* h, const double* psi) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const int n = o.n, nn = n * n, dim = o.dim;
    double absorption = 0.0;
    std::vector<double> M(nn), loc(n);
    for (int e = 0; e < o.ne; ++e) {
        const long long off = (long long)e * n;
        for (int g = 0; g < o.G; ++g) {
            const double* Ms = &o.Ms[((size_t)g * o.ne + e) * nn];
            for (int k = 0; k < nn; ++k) M[k] = Ms[k];
            if (o.timedep) for (int k = 0; k < nn; ++k) M[k] += o.tau * o.Mt[(size_t)e * nn + k];
            for (int a = 0; a < o.Nw; ++a) {
                double sum = 0.0;
                for (int i = 0; i < n; ++i) {
                    double s = 0.0;
                    for (int j = 0; j < n; ++j) s += M[i * n + j] * psi[pidx(o, g, a, off + j)];
                    sum += s;
                }
                absorption += sum * o.wq[a];
            }
        }
    }
    double leakage = 0.0;
    for (size_t fi = 0; fi < o.faces.size(); ++fi) {
        const Face& f = o.faces[fi];
        if (f.e2 >= 0) continue;
        const double* F = &o.F[fi * 4 * nn];
        const long long off = (long long)f.e1 * n;
        for (int a = 0; a < o.Nw; ++a) {
            const double dot = dotv(dim, &o.omega[(size_t)a * dim], f.nrm);
            if (dot >= 0) {
                for (int g = 0; g < o.G; ++g) {
                    double sum = 0.0;
                    for (int i = 0; i < n; ++i) {
                        double s = 0.0;
                        for (int j = 0; j < n; ++j) s += F[i * n + j] * psi[pidx(o, g, a, off + j)];
                        sum += s;
                    }
                    leakage += o.wq[a] * dot * sum;
                }
            }
        }
    }
    return leakage + absorption;
}

// DiscreteToMoment::Mult (transport_op.cpp:3-31); nmom = 1 or dim+1
void oracle_moments(void* h, const double* psi, double* phi, int nmom) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const long long Nd = o.ndof();
    std::fill(phi, phi + (size_t)o.G * nmom * Nd, 0.0);
    for (int g = 0; g < o.G; ++g)
        for (int a = 0; a < o.Nw; ++a)
            for (long long s = 0; s < Nd; ++s)
                phi[s + Nd * g] += o.wq[a] * psi[pidx(o, g, a, s)];
    if (nmom > 1)
        for (int g = 0; g < o.G; ++g)
            for (int a = 0; a < o.Nw; ++a)
                for (long long s = 0; s < Nd; ++s)
                    for (int m = 0; m < o.dim; ++m)
                        phi[s + Nd * (g + (long long)o.G * (1 + m))] +=
                            o.omega[(size_t)a * o.dim + m] * o.wq[a] * psi[pidx(o, g, a, s)];
}

// DiscreteToMoment::MultTranspose / AddMultTranspose (transport_op.cpp:33-89)
void oracle_moments_transpose(void* h, const double* phi, double* psi, int nmom, double alpha, int add) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const long long Nd = o.ndof();
    for (int g = 0; g < o.G; ++g)
        for (int a = 0; a < o.Nw; ++a)
            for (long long s = 0; s < Nd; ++s) {
                if (add) psi[pidx(o, g, a, s)] += alpha * phi[s + Nd * g] / o.wsum;
                else psi[pidx(o, g, a, s)] = phi[s + Nd * g] / o.wsum;
            }
    if (nmom > 1)
        for (int g = 0; g < o.G; ++g)
            for (int a = 0; a < o.Nw; ++a)
                for (long long s = 0; s < Nd; ++s)
                    for (int m = 0; m < o.dim; ++m) {
                        const double om = o.omega[(size_t)a * o.dim + m];
                        const double ph = phi[s + Nd * (g + (long long)o.G * (1 + m))];
                        if (add) psi[pidx(o, g, a, s)] += alpha * 3 * om * ph / o.wsum;
                        else psi[pidx(o, g, a, s)] += 3 * om * ph / o.wsum;
                    }
}

// S.Mult -> D.MultTranspose -> += source (transport_op.hpp:75-90): the scattering
// mass is MassIntegrator(sigma_s) (rule order 2p + OrderW, vertex rule when the
// mass is lumped), applied cell by cell to phi [G][Ndof].
void oracle_scattering_source(void* h, const double* sigma_s, const double* phi, const double* qfix, double* out) {
    Oracle& o = *static_cast<Oracle*>(h);
    if (o.Mt.empty()) assemble_time_mass(o);
    const int n = o.n, nn = n * n;
    const long long Nd = o.ndof();
    std::vector<double> y((size_t)o.G * Nd);
    for (int g = 0; g < o.G; ++g)
        for (int e = 0; e < o.ne; ++e) {
            const double* M = &o.Mt[(size_t)e * nn];
            for (int i = 0; i < n; ++i) {
                double s = 0.0;
                for (int j = 0; j < n; ++j) s += M[i * n + j] * phi[Nd * g + (long long)e * n + j];
                y[Nd * g + (long long)e * n + i] = sigma_s[(size_t)g * o.ne + e] * s;
            }
        }
    for (int g = 0; g < o.G; ++g)
        for (int a = 0; a < o.Nw; ++a)
            for (long long s = 0; s < Nd; ++s) {
                const double v = y[Nd * g + s] / o.wsum;
                out[pidx(o, g, a, s)] = qfix ? qfix[pidx(o, g, a, s)] + v : v;
            }
}

typedef double (*oracle_fn)(const double* x, const double* omega, int g, int attr);

// FormTransportSource (sweep.cpp:1135-1185).  Source density Q(x, Omega, g) is
// either q_cell[g*ne + e] (piecewise constant, isotropic) or qfn; the inflow is
// inflow[g*nattr + attr] per boundary attribute or inflow_fn.
void oracle_form_source(void* h, const double* q_cell, oracle_fn qfn,
                        const double* inflow, int nattr, oracle_fn inflow_fn, double* out) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const int n = o.n, dim = o.dim, td = dim - 1;
    const auto rule_dom = tensor_rule(dim, gauss_legendre(o.p + 1));
    const auto rule_bdr = tensor_rule(td, gauss_legendre(dim == 3 ? o.p + 2 : o.p + 1));
    std::fill(out, out + o.psi_size(), 0.0);
    std::vector<double> phi(n);
    for (int g = 0; g < o.G; ++g)
        for (int a = 0; a < o.Nw; ++a) {
            const double* Om = &o.omega[(size_t)a * dim];
            for (int e = 0; e < o.ne; ++e) {
                const long long off = (long long)e * n;
                for (const auto& q : rule_dom) {
                    double J[3][3], A[3][3], x[3];
                    geometry(o, e, q.xi, J, x);
                    const double Q = qfn ? qfn(x, Om, g, 0) : q_cell[(size_t)g * o.ne + e];
                    const double val = det_adj(dim, J, A) * Q;
                    basis(o, q.xi, phi.data(), nullptr);
                    for (int i = 0; i < n; ++i) out[pidx(o, g, a, off + i)] += q.w * val * phi[i];
                }
            }
            for (const Face& f : o.faces) {
                if (f.e2 >= 0) continue;
                const long long off = (long long)f.e1 * n;
                for (const auto& q : rule_bdr) {
                    double xi[3], nr[3], J[3][3], x[3];
                    face_point(dim, f.k1, q.xi, xi);
                    raw_normal(o, f.e1, f.k1, xi, nr);
                    geometry(o, f.e1, xi, J, x);
                    const double un = dotv(dim, Om, nr);
                    double w = 0.5 * -1.0 * un - (-0.5) * std::fabs(un);
                    const double fin = inflow_fn ? inflow_fn(x, Om, g, f.attr)
                                                 : ((f.attr >= 0 && f.attr < nattr) ? inflow[(size_t)g * nattr + f.attr] : 0.0);
                    w *= q.w * fin;
                    basis(o, xi, phi.data(), nullptr);
                    for (int i = 0; i < n; ++i) out[pidx(o, g, a, off + i)] += w * phi[i];
                }
            }
        }
}

// sum over groups of || u_h(g, a=ang) - u(x) ||_{L2} with the rule MFEM's
// GridFunction::ComputeL2Error uses (order 2p+3).  u_h is one (g, angle) slice.
double oracle_l2_error(void* h, const double* psi, int g, int ang, oracle_fn exact) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const int n = o.n, dim = o.dim;
    const auto rule = tensor_rule(dim, gauss_legendre(o.p + 2));
    std::vector<double> phi(n);
    double err = 0.0;
    for (int e = 0; e < o.ne; ++e) {
        const long long off = (long long)e * n;
        double loc = 0.0;
        for (const auto& q : rule) {
            double J[3][3], A[3][3], x[3];
            geometry(o, e, q.xi, J, x);
            const double w = det_adj(dim, J, A) * q.w;
            basis(o, q.xi, phi.data(), nullptr);
            double uh = 0.0;
            for (int i = 0; i < n; ++i) uh += phi[i] * psi[pidx(o, g, ang, off + i)];
            const double d = uh - exact(x, &o.omega[(size_t)ang * dim], g, 0);
            loc += w * d * d;
        }
        err += loc;
    }
    return std::sqrt(err);
}


// ---------------------------------------------------------------- thermal radiative transfer
// Planck integrals (src/planck.hpp:157-236): b(x) = 15/pi^4 int_0^x t^3/(e^t - 1)
// as min(Taylor through x^21, 9-term polylogarithm), the Rosseland form
// r(x) = b(x) - 15/(4 pi^4) x^4/(e^x - 1), group fractions with F = 0 below the
// first and F = 1 above the last group.  The Taylor coefficients come from
// Bernoulli numbers generated here by their recurrence.
static double oracle_bernoulli_coef(int n) {
    static double c[19];
    static bool ready = false;
    if (!ready) {
        double B[19];
        B[0] = 1.0;
        for (int m = 1; m <= 18; ++m) {
            double s = 0.0, binom = 1.0;   // C(m+1, k)
            for (int k = 0; k < m; ++k) {
                s += binom * B[k];
                binom = binom * (m + 1 - k) / (k + 1);
            }
            B[m] = -s / (m + 1);
        }
        double fact = 1.0;
        for (int k = 0; k <= 18; ++k) {
            if (k > 0) fact *= k;
            c[k] = (k >= 3 && k % 2 == 1) ? 0.0 : B[k] / (fact * (k + 3));
        }
        ready = true;
    }
    return c[n];
}

static double oracle_planck_b(double x) {
    const double pi = 3.14159265358979323846;
    const double norm = 15.0 / (pi * pi * pi * pi);
    if (x > 1e100) return 1.0;
    if (x == 0.0) return 0.0;
    double taylor = 0.0;
    for (int k = 0; k <= 18; ++k) taylor += oracle_bernoulli_coef(k) * std::pow(x, k + 3);
    taylor *= norm;
    double poly = 0.0;
    for (int l = 1; l <= 9; ++l) {
        const double el = std::exp(-l * x), L = l;
        poly += el * (6.0 / (L * L * L * L) + 6.0 * x / (L * L * L) + 3.0 * x * x / (L * L) + x * x * x / L);
    }
    poly = 1.0 - norm * poly;
    return std::min(taylor, poly);
}

static double oracle_rosseland_r(double x, double b) {
    const double pi = 3.14159265358979323846;
    if (x > std::pow(1.7976931348623157e308, 0.25)) return b;
    return b - 0.25 * (15.0 / (pi * pi * pi * pi)) * std::pow(x, 4) / std::expm1(x);
}

static void oracle_spectrum(const double* bounds, int G, double T, int kind, double* out) {
    double prev = 0.0;
    for (int g = 0; g < G - 1; ++g) {
        const double x = bounds[g + 1] / T;
        double f = oracle_planck_b(x);
        if (kind == 1) f = oracle_rosseland_r(x, f);
        out[g] = f - prev;
        prev = f;
    }
    out[G - 1] = 1.0 - prev;
}

void oracle_planck_spectrum(const double* bounds, int G, double T, int kind, double* out) {
    oracle_spectrum(bounds, G, T, kind, out);
}

// PlanckEmissionNonlinearForm::Mult / GetGradient (trt_integrators.cpp:56-152,
// 229-302) at rule order 2p + 1; sigma per cell [G][Ne].
void oracle_planck_emission(void* h, const double* bounds, const double* sigma, const double* T, double K,
                            double* emission, double* grad) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const int n = o.n, dim = o.dim, G = o.G;
    const auto rule = tensor_rule(dim, gauss_legendre(o.p + 1));
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o.ne; ++e) {
        std::vector<double> phi(n), bs(G), rs(G);
        for (int g = 0; g < G; ++g)
            for (int i = 0; i < n; ++i) {
                if (emission) emission[(size_t)g * o.ndof() + (size_t)e * n + i] = 0.0;
                if (grad) for (int j = 0; j < n; ++j) grad[(((size_t)g * o.ne + e) * n + i) * n + j] = 0.0;
            }
        for (const auto& q : rule) {
            double J[3][3], A[3][3];
            geometry(o, e, q.xi, J, nullptr);
            const double w = det_adj(dim, J, A) * q.w;
            basis(o, q.xi, phi.data(), nullptr);
            double Tq = 0.0;
            for (int i = 0; i < n; ++i) Tq += T[(size_t)e * n + i] * phi[i];
            oracle_spectrum(bounds, G, Tq, 0, bs.data());
            oracle_spectrum(bounds, G, Tq, 1, rs.data());
            for (int g = 0; g < G; ++g) {
                const double sg = sigma[(size_t)g * o.ne + e];
                if (emission) {
                    const double c = w * K * std::pow(Tq, 4) * bs[g] * sg;
                    for (int i = 0; i < n; ++i) emission[(size_t)g * o.ndof() + (size_t)e * n + i] += c * phi[i];
                }
                if (grad) {
                    const double c = sg * rs[g] * w * 4.0 * K * std::pow(Tq, 3);
                    for (int i = 0; i < n; ++i)
                        for (int j = 0; j < n; ++j) grad[(((size_t)g * o.ne + e) * n + i) * n + j] += c * phi[i] * phi[j];
                }
            }
        }
    }
}

// meb_form of exe/scallion.cpp:755-765: GrayPlanckEmissionNFI at order 2p + 2
// (trt_integrators.cpp:154-208) plus MassIntegrator(cv_dt); residual and the
// gradient blocks [Ne][n][n].
void oracle_energy_balance(void* h, const double* bounds, const double* sigma, const double* T, double K, double cv_dt,
                           double* residual, double* grad) {
    Oracle& o = *static_cast<Oracle*>(h);
    if (o.Mt.empty()) assemble_time_mass(o);
    const int n = o.n, nn = n * n, dim = o.dim, G = o.G;
    const auto rule = tensor_rule(dim, gauss_legendre(o.p + 2));
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o.ne; ++e) {
        std::vector<double> phi(n), bs(G), rs(G), res(n, 0.0), gr(nn, 0.0);
        const double* Te = T + (size_t)e * n;
        for (const auto& q : rule) {
            double J[3][3], A[3][3];
            geometry(o, e, q.xi, J, nullptr);
            const double w = det_adj(dim, J, A) * q.w;
            basis(o, q.xi, phi.data(), nullptr);
            double Tq = 0.0;
            for (int i = 0; i < n; ++i) Tq += Te[i] * phi[i];
            oracle_spectrum(bounds, G, Tq, 0, bs.data());
            oracle_spectrum(bounds, G, Tq, 1, rs.data());
            double sb = 0.0, sr = 0.0;
            for (int g = 0; g < G; ++g) {
                sb += sigma[(size_t)g * o.ne + e] * bs[g];
                sr += sigma[(size_t)g * o.ne + e] * rs[g];
            }
            for (int i = 0; i < n; ++i) res[i] += w * K * std::pow(Tq, 4) * sb * phi[i];
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) gr[i * n + j] += sr * 4.0 * K * std::pow(Tq, 3) * w * phi[i] * phi[j];
        }
        const double* Mt = &o.Mt[(size_t)e * nn];
        for (int i = 0; i < n; ++i) {
            double m = 0.0;
            for (int j = 0; j < n; ++j) m += Mt[i * n + j] * Te[j];
            if (residual) residual[(size_t)e * n + i] = res[i] + cv_dt * m;
            if (grad)
                for (int j = 0; j < n; ++j) grad[((size_t)e * n + i) * n + j] = gr[i * n + j] + cv_dt * Mt[i * n + j];
        }
    }
}

// out = q + tau Mt psi_prev per (g, a, e) block (tvector.cpp:76-95, scallion.cpp:1358-1359)
void oracle_time_source(void* h, const double* psi_prev, const double* q, double tau, double* out) {
    Oracle& o = *static_cast<Oracle*>(h);
    if (o.Mt.empty()) assemble_time_mass(o);
    const int n = o.n;
    const long long blocks = (long long)o.G * o.Nw * o.ne;
#pragma omp parallel for schedule(static)
    for (long long b = 0; b < blocks; ++b) {
        const int e = (int)(b % o.ne);
        const double* M = &o.Mt[(size_t)e * n * n];
        std::vector<double> x(psi_prev + b * n, psi_prev + (b + 1) * n);
        for (int i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int j = 0; j < n; ++j) acc += M[i * n + j] * x[j];
            out[b * n + i] = (q ? q[b * n + i] : 0.0) + tau * acc;
        }
    }
}

// unit MGMassIntegrator matrix of cell e (rule order 2p), row major
static void oracle_unit_mass_cell(const Oracle& o, int e, double* M) {
    const int n = o.n, dim = o.dim;
    const auto rule = tensor_rule(dim, gauss_legendre(o.p + 1));
    std::vector<double> phi(n);
    for (int k = 0; k < n * n; ++k) M[k] = 0.0;
    for (const auto& q : rule) {
        double J[3][3], A[3][3];
        geometry(o, e, q.xi, J, nullptr);
        const double w = det_adj(dim, J, A) * q.w;
        basis(o, q.xi, phi.data(), nullptr);
        for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) M[i * n + j] += w * phi[i] * phi[j];
    }
}

// which = 1: unit sigma mass, 2: MassIntegrator mass; y = M x per cell (Ndof)
void oracle_mass_apply(void* h, int which, const double* x, double* y) {
    Oracle& o = *static_cast<Oracle*>(h);
    if (which == 2 && o.Mt.empty()) assemble_time_mass(o);
    const int n = o.n;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o.ne; ++e) {
        std::vector<double> Mu(n * n);
        const double* M = &o.Mt[0];
        if (which == 1) { oracle_unit_mass_cell(o, e, Mu.data()); M = Mu.data(); }
        else M = &o.Mt[(size_t)e * n * n];
        for (int i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int j = 0; j < n; ++j) acc += M[i * n + j] * x[(size_t)e * n + j];
            y[(size_t)e * n + i] = acc;
        }
    }
}

// sum_g sigma_g M phi_g (Mtot_collapse, scallion.cpp:786-797)
void oracle_absorption(void* h, const double* sigma, const double* phi, double* y) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const int n = o.n;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o.ne; ++e) {
        std::vector<double> Mu(n * n);
        oracle_unit_mass_cell(o, e, Mu.data());
        for (int i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int g = 0; g < o.G; ++g) {
                double m = 0.0;
                for (int j = 0; j < n; ++j) m += Mu[i * n + j] * phi[(size_t)g * o.ndof() + (size_t)e * n + j];
                acc += sigma[(size_t)g * o.ne + e] * m;
            }
            y[(size_t)e * n + i] = acc;
        }
    }
}

// sigma[g][e] = C nu_g^a T(centre)^b (opacity.cpp:47-63 at the group midpoints, piecewise constant)
void oracle_powerlaw_opacity(void* h, const double* T, const double* nu, double C, double a, double b, double* sigma) {
    const Oracle& o = *static_cast<Oracle*>(h);
    const int n = o.n;
    const double xc[3] = {0.5, 0.5, 0.5};
    std::vector<double> phi(n);
    basis(o, xc, phi.data(), nullptr);
    for (int e = 0; e < o.ne; ++e) {
        double Tc = 0.0;
        for (int i = 0; i < n; ++i) Tc += phi[i] * T[(size_t)e * n + i];
        for (int g = 0; g < o.G; ++g) sigma[(size_t)g * o.ne + e] = C * std::pow(nu[g], a) * std::pow(Tc, b);
    }
}


// ---------------------------------------------------------------- MIP diffusion (DSA)
// InteriorPenaltyDiscretization::GetOperator (moment_discretization.cpp:73-110)
// as a dense matrix [Ndof][Ndof] for group g: DiffusionIntegrator(1/(3 sigma_t))
// at order 2p + dim - 1, MassIntegrator(sigma_a) (+ tau) at the mass rule,
// MIPDiffusionIntegrator face by face as moment_integrators.cpp:3-200 forms it
// (elmat = -A + sigma A^T + J over the 2n x 2n face block, sigma = -1), and
// BoundaryMassIntegrator(alpha_bdr) on non-reflective boundary faces when
// marshak != 0.
void oracle_dsa_matrix(void* h, const double* sigma_s, int g, double kappa, double penalty_min, double alpha_bdr,
                       double tau, int marshak, double* K) {
    Oracle& o = *static_cast<Oracle*>(h);
    if (o.Mt.empty()) assemble_time_mass(o);
    const int n = o.n, dim = o.dim, td = dim - 1;
    const long long N = o.ndof();
    for (long long q = 0; q < N * N; ++q) K[q] = 0.0;
    auto D = [&](int e) { return 1.0 / (3.0 * o.sigma[(size_t)g * o.ne + e]); };
    auto phys_grad = [&](int e, const double* xi, std::vector<double>& phi, std::vector<std::array<double, 3>>& gx) {
        double J[3][3], A[3][3];
        geometry(o, e, xi, J, nullptr);
        const double det = det_adj(dim, J, A);
        std::vector<std::array<double, 3>> dref(n);
        basis(o, xi, phi.data(), reinterpret_cast<double(*)[3]>(dref.data()));
        for (int i = 0; i < n; ++i)
            for (int r = 0; r < dim; ++r) {
                double v = 0.0;
                for (int qq = 0; qq < dim; ++qq) v += A[qq][r] * dref[i][qq];
                gx[i][r] = v / det;
            }
        return det;
    };
    std::vector<double> phi(n), phi2(n);
    std::vector<std::array<double, 3>> gx(n), gx2(n);
    // volume terms
    const auto rule_d = tensor_rule(dim, gauss_legendre((2 * o.p + dim - 1) / 2 + 1));
    for (int e = 0; e < o.ne; ++e) {
        const long long off = (long long)e * n;
        for (const auto& q : rule_d) {
            const double det = phys_grad(e, q.xi, phi, gx);
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) {
                    double d = 0.0;
                    for (int r = 0; r < dim; ++r) d += gx[i][r] * gx[j][r];
                    K[(off + i) * N + off + j] += q.w * det * D(e) * d;
                }
        }
        const double sa = o.sigma[(size_t)g * o.ne + e] - sigma_s[(size_t)g * o.ne + e];
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) K[(off + i) * N + off + j] += (sa + tau) * o.Mt[((size_t)e * n + i) * n + j];
    }
    // faces
    const auto rule_f = tensor_rule(td, gauss_legendre(o.p + 1));
    for (const Face& f : o.faces) {
        if (f.e2 < 0) {
            if (!marshak || !f.refl.empty()) continue;
            const long long off = (long long)f.e1 * n;
            for (const auto& q : rule_f) {
                double xi[3], nr[3];
                face_point(dim, f.k1, q.xi, xi);
                raw_normal(o, f.e1, f.k1, xi, nr);
                const double w = q.w * (dim == 1 ? 1.0 : norm(dim, nr));
                basis(o, xi, phi.data(), nullptr);
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j) K[(off + i) * N + off + j] += alpha_bdr * w * phi[i] * phi[j];
            }
            continue;
        }
        const int n2 = 2 * n;
        std::vector<double> elmat(n2 * n2, 0.0), jmat(n2 * n2, 0.0);
        for (const auto& q : rule_f) {
            double xi1[3], xi2[3], s2[2], nr[3];
            face_point(dim, f.k1, q.xi, xi1);
            e2_face_coords(f, td, q.xi, s2);
            face_point(dim, f.k2, s2, xi2);
            raw_normal(o, f.e1, f.k1, xi1, nr);      // scaled normal out of e1
            const double nn = dotv(dim, nr, nr);
            const double det1 = phys_grad(f.e1, xi1, phi, gx);
            const double det2 = phys_grad(f.e2, xi2, phi2, gx2);
            const double w1 = q.w / 2 * D(f.e1), w2 = q.w / 2 * D(f.e2);
            std::vector<double> dn1(n), dn2(n);
            for (int j = 0; j < n; ++j) {
                dn1[j] = w1 * dotv(dim, gx[j].data(), nr);
                dn2[j] = w2 * dotv(dim, gx2[j].data(), nr);
            }
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) {
                    elmat[i * n2 + j] += phi[i] * dn1[j];
                    elmat[i * n2 + n + j] += phi[i] * dn2[j];
                    elmat[(n + i) * n2 + j] -= phi2[i] * dn1[j];
                    elmat[(n + i) * n2 + n + j] -= phi2[i] * dn2[j];
                }
            double wq = kappa * (w1 * nn / det1 + w2 * nn / det2);
            const double fl = penalty_min * q.w * std::sqrt(nn);
            if (wq < fl) wq = fl;
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) {
                    jmat[i * n2 + j] += wq * phi[i] * phi[j];
                    jmat[i * n2 + n + j] -= wq * phi[i] * phi2[j];
                    jmat[(n + i) * n2 + j] -= wq * phi2[i] * phi[j];
                    jmat[(n + i) * n2 + n + j] += wq * phi2[i] * phi2[j];
                }
        }
        // elmat := -elmat + sigma elmat^T + jmat with sigma = -1
        const long long off[2] = {(long long)f.e1 * n, (long long)f.e2 * n};
        for (int i = 0; i < n2; ++i)
            for (int j = 0; j < n2; ++j) {
                const double v = -elmat[i * n2 + j] - elmat[j * n2 + i] + jmat[i * n2 + j];
                K[(off[i / n] + i % n) * N + off[j / n] + j % n] += v;
            }
    }
}

}  // extern "C"
