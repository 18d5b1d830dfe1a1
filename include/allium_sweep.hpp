// allium_sweep.hpp -- header-only C++ host side over the C ABI in allium_sweep.h.
//
// allium::InverseAdvectionOperator mirrors the reference class of the same name
// (src/sweep.hpp:13-130): height = width = G * Nw * Ndof, Mult(source, psi) with
// source == psi allowed, AssembleLocalMatrices, SetTimeAbsorption,
// UseParallelBlockJacobi.  The vector type V only needs V::GetData() returning
// double* (const-qualified overload for const V) and V::Size(), which
// mfem::Vector provides, so an MFEM build can call it directly on its vectors;
// raw pointers work as well.  Failures throw allium::Error (the reference
// aborts through MFEM_ABORT instead).
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "allium_sweep.h"

namespace allium {

class Error : public std::runtime_error {
public:
    Error(int status, const std::string& msg) : std::runtime_error(msg), status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

inline void check(int st, const allium_sweep* h = nullptr) {
    if (st != ALLIUM_OK) {
        std::string msg = allium_status_string(st);
        if (h) msg += std::string(" (") + allium_sweep_last_error(h) + ")";
        throw Error(st, msg);
    }
}

struct Mesh {
    int dim = 0;
    std::vector<double> vertices;              // [nv][dim]
    std::vector<int> element_vertices;         // [ne][2^dim], MFEM local vertex order
    std::vector<int> boundary_face_vertices;   // [nbf][2^(dim-1)]
    std::vector<int> boundary_attributes;      // [nbf]
};

// boundary attribute -> ALLIUM_BC_INFLOW / ALLIUM_BC_REFLECTIVE (BoundaryConditionMap)
struct BoundaryConditions {
    std::vector<int> attributes;
    std::vector<int> kinds;
    void Set(int attribute, int kind) { attributes.push_back(attribute); kinds.push_back(kind); }
};

struct Quadrature {
    int dim = 0;
    std::vector<double> omega;    // [Nw][dim]
    std::vector<double> weights;  // [Nw]
    int Size() const { return (int)weights.size(); }
};

class InverseAdvectionOperator {
public:
    // sigma_t: [G][Ne] piecewise-constant total cross section; lump: allium bit mask
    InverseAdvectionOperator(const Mesh& mesh, int order, const Quadrature& quad, int num_groups,
                             const std::vector<double>& sigma_t, int lump = 0,
                             const BoundaryConditions& bc = BoundaryConditions()) {
        allium_mesh_desc m;
        m.dim = mesh.dim;
        m.num_vertices = (int)(mesh.vertices.size() / mesh.dim);
        m.vertices = mesh.vertices.data();
        m.num_elements = (int)(mesh.element_vertices.size() >> mesh.dim);
        m.element_vertices = mesh.element_vertices.data();
        m.num_boundary_faces = (int)mesh.boundary_attributes.size();
        m.boundary_face_vertices = mesh.boundary_face_vertices.data();
        m.boundary_attributes = mesh.boundary_attributes.data();
        allium_fe_desc fe{order, ALLIUM_BASIS_GAUSS_LOBATTO, lump};
        allium_quad_desc q{quad.dim, quad.Size(), quad.omega.data(), quad.weights.data()};
        allium_bc_desc b{(int)bc.attributes.size(), bc.attributes.data(), bc.kinds.data()};
        check(allium_sweep_create(&m, &fe, &q, num_groups, sigma_t.data(), bc.attributes.empty() ? nullptr : &b, &h_));
        long long n = 0;
        int nl = 0;
        check(allium_sweep_sizes(h_, &n, &ndof_, &nl), h_);
        size_ = n;
        num_levels_ = nl;
    }
    ~InverseAdvectionOperator() { allium_sweep_destroy(h_); }
    InverseAdvectionOperator(const InverseAdvectionOperator&) = delete;
    InverseAdvectionOperator& operator=(const InverseAdvectionOperator&) = delete;

    long long Height() const { return size_; }
    long long Width() const { return size_; }
    long long NumDofs() const { return ndof_; }
    int NumLevels() const { return num_levels_; }

    // psi = L^{-1} source; host or device pointers, source may equal psi.
    // With one GPU owning every cell, the parallel block Jacobi variant has no
    // off-rank data to lag, so any number of PBJ sweeps gives this same result.
    void Mult(const double* source, double* psi) const { check(allium_sweep_mult(h_, source, psi), h_); }
    template <class V>
    void Mult(const V& source, V& psi) const {
        if ((long long)source.Size() != size_ || (long long)psi.Size() != size_)
            throw Error(ALLIUM_ERR_SIZE, "vector size does not match the operator");
        Mult(source.GetData(), psi.GetData());
    }

    void MultF32(const float* source, float* psi) const { check(allium_sweep_mult_f32(h_, source, psi), h_); }

    void AssembleLocalMatrices(const std::vector<double>& sigma_t) { check(allium_sweep_assemble(h_, sigma_t.data()), h_); }
    void SetTimeAbsorption(double tau) {
        tau_ = tau;
        check(allium_sweep_set_time_absorption(h_, tau), h_);
    }
    double GetTimeAbsorption() const { return tau_; }
    void UseParallelBlockJacobi(bool use = true) { pbj_ = use; }
    bool IsParallelBlockJacobi() const { return pbj_; }
    void SetNumPBJSweeps(int n) { num_pbj_sweeps_ = n; }
    // Exchange loads lagged off-rank traces for PBJ (src/sweep.cpp:877-922); one
    // GPU owns every cell, so there is nothing to load.
    void Exchange(const double* /*psi*/) {}
    // message packing of the MPI sweep (src/sweep.hpp:109-110): no messages on one GPU
    void SetSendBufferSize(int s) { send_buffer_size_ = s; }
    void SetMaxSendsPerReceive(int s) { max_sends_per_recv_ = s; }

    // Negative-flux fixup (src/sweep.hpp:112-118): kind 1 ZeroFixupOperator,
    // 2 ZeroAndScaleFixupOperator (src/fixup.cpp:3-57), with its floor.
    void SetFixupOperator(int kind, double minimum = 0.0) {
        fix_kind_ = kind;
        fix_min_ = minimum;
        UseFixup(true);
    }
    void UseFixup(bool use = true) {
        check(allium_sweep_set_fixup(h_, use ? fix_kind_ : 0, fix_min_), h_);
        fix_on_ = use && fix_kind_ != 0;
    }
    bool IsFixupOn() const { return fix_on_; }
    // local solves the fixup changed / could not balance since the last reset
    void FixupCounts(long long* applied, long long* failed, bool reset = false) const {
        check(allium_sweep_fixup_counts(h_, applied, failed, reset ? 1 : 0), h_);
    }
    void Synchronize() const { check(allium_sweep_synchronize(h_), h_); }

    allium_sweep* handle() const { return h_; }

private:
    allium_sweep* h_ = nullptr;
    long long size_ = 0, ndof_ = 0;
    int num_levels_ = 0;
    double tau_ = 0.0;
    bool pbj_ = false;
    int num_pbj_sweeps_ = 1;
    int send_buffer_size_ = 8, max_sends_per_recv_ = 8;
    int fix_kind_ = 0;
    double fix_min_ = 0.0;
    bool fix_on_ = false;
};

// AdvectionOperator (src/sweep.hpp:155-166)
class AdvectionOperator {
public:
    explicit AdvectionOperator(const InverseAdvectionOperator& Linv) : Linv_(Linv) {}
    void Mult(const double* x, double* y) const { check(allium_sweep_apply_L(Linv_.handle(), x, y), Linv_.handle()); }
    double ComputeBalance(const double* psi) const {
        double out = 0.0;
        check(allium_sweep_balance(Linv_.handle(), psi, &out), Linv_.handle());
        return out;
    }

private:
    const InverseAdvectionOperator& Linv_;
};

// DiscreteToMoment (src/transport_op.hpp:97-122)
class DiscreteToMoment {
public:
    DiscreteToMoment(const InverseAdvectionOperator& Linv, int num_moments = 1) : Linv_(Linv), nm_(num_moments) {}
    void Mult(const double* psi, double* phi) const { check(allium_sweep_moments(Linv_.handle(), psi, phi, nm_), Linv_.handle()); }
    void MultTranspose(const double* phi, double* psi) const {
        check(allium_sweep_moments_transpose(Linv_.handle(), phi, psi, nm_, 1.0, 0), Linv_.handle());
    }
    void AddMultTranspose(const double* phi, double* psi, double alpha = 1.0) const {
        check(allium_sweep_moments_transpose(Linv_.handle(), phi, psi, nm_, alpha, 1), Linv_.handle());
    }

private:
    const InverseAdvectionOperator& Linv_;
    int nm_;
};

}  // namespace allium
