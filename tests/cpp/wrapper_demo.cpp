// C++ host side through the header-only wrapper: a 2D 12x12 mesh, p = 1,
// sigma_t = 0, unit isotropic inflow on every boundary: psi == 1 everywhere
// (test/test_sweep.cpp:7-43).  Prints "ok <max error>" and exits 0 on success.
#include <cmath>
#include <cstdio>
#include <vector>

#include "allium_sweep.hpp"

int main() {
    const int n = 12, nv = n + 1;
    allium::Mesh mesh;
    mesh.dim = 2;
    for (int j = 0; j < nv; ++j)
        for (int i = 0; i < nv; ++i) {
            mesh.vertices.push_back((double)i / n);
            mesh.vertices.push_back((double)j / n);
        }
    auto v = [&](int i, int j) { return i + nv * j; };
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            int q[4] = {v(i, j), v(i + 1, j), v(i + 1, j + 1), v(i, j + 1)};
            mesh.element_vertices.insert(mesh.element_vertices.end(), q, q + 4);
        }
    for (int i = 0; i < n; ++i) {
        int f[4][2] = {{v(i, 0), v(i + 1, 0)}, {v(n, i), v(n, i + 1)}, {v(i + 1, n), v(i, n)}, {v(0, i + 1), v(0, i)}};
        for (int s = 0; s < 4; ++s) {
            mesh.boundary_face_vertices.push_back(f[s][0]);
            mesh.boundary_face_vertices.push_back(f[s][1]);
            mesh.boundary_attributes.push_back(s + 1);
        }
    }
    // S2 level-symmetric set in 2D: (+-1/sqrt3, +-1/sqrt3), weights pi
    allium::Quadrature quad;
    quad.dim = 2;
    const double mu = 1.0 / std::sqrt(3.0);
    const double sx[4] = {1, -1, 1, -1}, sy[4] = {1, 1, -1, -1};
    for (int a = 0; a < 4; ++a) {
        quad.omega.push_back(sx[a] * mu);
        quad.omega.push_back(sy[a] * mu);
        quad.weights.push_back(M_PI);
    }
    const int ne = n * n;
    std::vector<double> sigma(ne, 0.0);
    allium::InverseAdvectionOperator Linv(mesh, 1, quad, 1, sigma);
    std::vector<double> inflow(5, 1.0), source(Linv.Width()), psi(Linv.Height());
    allium::check(allium_sweep_form_source(Linv.handle(), nullptr, inflow.data(), 5, source.data()), Linv.handle());
    Linv.Mult(source.data(), psi.data());
    double err = 0.0;
    for (double x : psi) err = std::fmax(err, std::fabs(x - 1.0));
    allium::DiscreteToMoment D(Linv);
    std::vector<double> phi(Linv.NumDofs());
    D.Mult(psi.data(), phi.data());
    for (double x : phi) err = std::fmax(err, std::fabs(x / (4 * M_PI) - 1.0));
    // the reference's fixup and PBJ controls (src/sweep.hpp:100-118): with no
    // negative flux the zero fixup changes nothing and counts no application
    Linv.UseParallelBlockJacobi(true);
    Linv.SetNumPBJSweeps(2);
    Linv.Exchange(psi.data());
    Linv.SetFixupOperator(1);
    if (!Linv.IsFixupOn()) return 2;
    Linv.Mult(source.data(), psi.data());
    long long applied = -1, failed = -1;
    Linv.FixupCounts(&applied, &failed, true);
    for (double x : psi) err = std::fmax(err, std::fabs(x - 1.0));
    Linv.UseFixup(false);
    if (Linv.IsFixupOn() || applied != 0 || failed != 0) return 3;
    std::printf("ok %.3e levels %d\n", err, Linv.NumLevels());
    return err < 1e-10 ? 0 : 1;
}
