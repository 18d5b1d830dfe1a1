// Device helpers for (multi)linear cell geometry and the tensor Gauss-Lobatto
// basis.  Cells are described by their 2^dim corners in corner order
// c = c0 + 2 c1 + 4 c2 (c_d in {0,1} is the reference coordinate of the corner).
// Local faces are k = 2 * axis + side; a face's tangential axes are the other
// axes in increasing order, and face DOFs are ordered lexicographically over
// them (first tangential axis fastest).
#pragma once

#include "internal.h"

namespace allium {

// J[r][q] = d x_r / d xi_q at xi, optionally the physical point x
__host__ __device__ inline void cell_jacobian(int dim, const double* X, const double* xi,
                                              double J[3][3], double* x) {
    const int nc = 1 << dim;
    for (int r = 0; r < dim; ++r) {
        for (int q = 0; q < dim; ++q) J[r][q] = 0.0;
        if (x) x[r] = 0.0;
    }
    for (int c = 0; c < nc; ++c) {
        double f[3], df[3];
        for (int d = 0; d < dim; ++d) {
            const int b = (c >> d) & 1;
            f[d] = b ? xi[d] : 1.0 - xi[d];
            df[d] = b ? 1.0 : -1.0;
        }
        double N = 1.0;
        for (int d = 0; d < dim; ++d) N *= f[d];
        for (int q = 0; q < dim; ++q) {
            double g = df[q];
            for (int d = 0; d < dim; ++d)
                if (d != q) g *= f[d];
            for (int r = 0; r < dim; ++r) J[r][q] += g * X[c * dim + r];
        }
        if (x)
            for (int r = 0; r < dim; ++r) x[r] += N * X[c * dim + r];
    }
}

// adjugate of J (A = det(J) J^{-1}); row a of A is the (unnormalised) normal
// of the reference faces xi_a = const.  Returns det(J).
__host__ __device__ inline double adjugate(int dim, const double J[3][3], double A[3][3]) {
    if (dim == 1) {
        A[0][0] = 1.0;
        return J[0][0];
    }
    if (dim == 2) {
        A[0][0] = J[1][1]; A[0][1] = -J[0][1];
        A[1][0] = -J[1][0]; A[1][1] = J[0][0];
        return J[0][0] * J[1][1] - J[0][1] * J[1][0];
    }
    for (int a = 0; a < 3; ++a) {
        const int b = (a + 1) % 3, c = (a + 2) % 3;
        A[a][0] = J[1][b] * J[2][c] - J[2][b] * J[1][c];
        A[a][1] = J[2][b] * J[0][c] - J[0][b] * J[2][c];
        A[a][2] = J[0][b] * J[1][c] - J[1][b] * J[0][c];
    }
    return J[0][0] * A[0][0] + J[1][0] * A[0][1] + J[2][0] * A[0][2];
}

// 1D Lagrange values (and derivatives) of the n1 nodes at t
__host__ __device__ inline void lagrange1d(int n1, const double* nodes, double t, double* v, double* dv) {
    for (int i = 0; i < n1; ++i) {
        double val = 1.0, der = 0.0;
        for (int j = 0; j < n1; ++j) {
            if (j == i) continue;
            const double inv = 1.0 / (nodes[i] - nodes[j]);
            const double f = (t - nodes[j]) * inv;
            der = der * f + val * inv;
            val *= f;
        }
        v[i] = val;
        if (dv) dv[i] = der;
    }
}

// element point of face-frame point t on local face k
__host__ __device__ inline void face_to_cell(int dim, int k, const double* t, double* xi) {
    const int a = k / 2, s = k % 2;
    int j = 0;
    for (int d = 0; d < dim; ++d) xi[d] = (d == a) ? (double)s : t[j++];
}

// local DOF of face DOF q on local face k (order p)
__host__ __device__ constexpr int face_dof(int dim, int p, int k, int q) {
    int idx = 0, stride = 1, r = q;
    const int n1 = p + 1, a = k / 2, s = k % 2;
    for (int d = 0; d < dim; ++d) {
        int id = 0;
        if (d == a) {
            id = s * p;
        } else {
            id = r % n1;
            r /= n1;
        }
        idx += id * stride;
        stride *= n1;
    }
    return idx;
}

// tensor multi-index of local DOF i (order p)
__host__ __device__ inline void dof_index(int dim, int n1, int i, int* id) {
    for (int d = 0; d < dim; ++d) {
        id[d] = i % n1;
        i /= n1;
    }
}

// psi(g, a, i) in allium's RIGHT layout
__host__ __device__ inline long long psi_index(long long ndof, int Nw, int g, int a, long long i) {
    return i + ndof * ((long long)a + (long long)Nw * g);
}

// Omega . n without fused multiply-add, so the upwind decision is the same
// bit for bit wherever it is evaluated
__device__ inline double dot_exact(int dim, const double* om, const double* nr) {
    double s = __dmul_rn(om[0], nr[0]);
    if (dim > 1) s = __dadd_rn(s, __dmul_rn(om[1], nr[1]));
    if (dim > 2) s = __dadd_rn(s, __dmul_rn(om[2], nr[2]));
    return s;
}

}  // namespace allium
