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

#include <type_traits>

#include "geometry.cuh"

namespace allium {

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

template <typename R>
struct SweepArgs {
    int ne, Nw, G;
    long long ndof;
    const double* omega;
    const R* dots;    // [nfaces][Nw] Omega_a . n_f, n_f out of element 1
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
    const int* refl;   // [nrefl][Nw] reflected angle at reflective face c (slots with nbr = -2 - c)
    // negative-flux fixup (src/fixup.cpp): 0 none, 1 zero, 2 zero and scale
    int fix_kind;
    R fix_min;
    unsigned long long* fix_counts;   // [0] applied, [1] failed
};

// RyosukeFixupOperator::Apply / perform_nff (src/fixup.cpp:90-174): negative entries
// to the floor, then the remaining ("positive") entries rescaled so that
// w . x equals the source total, by the reference's closed forms for 1, 2 or 3
// positive entries.  Returns 0, 1, -1, or -2 for more than three positive
// entries (where the reference aborts, src/fixup.cpp:155).
template <int N, typename R>
__device__ __noinline__ int fixup_ryosuke(R xmin, const R (&w)[N], R balance, R (&x)[N]) {
    int cnt[N];
    int pos = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if (x[i] <= xmin) x[i] = xmin;
        else cnt[pos++] = i;
    }
    if (pos == 0 || pos == N) return 0;
    if (pos > 3) return -2;
    R xv[3], wv[3];
    for (int k = 0; k < pos; ++k) {
#pragma unroll
        for (int i = 0; i < N; ++i)
            if (i == cnt[k]) { xv[k] = x[i]; wv[k] = w[i]; }
    }
    // C: first row the weights of the positive entries, first column
    // -x_k / x_0 below the diagonal of ones; right-hand side (balance, 0, ..)
    R out[3];
    if (pos == 1) {
        out[0] = balance / wv[0];
    } else if (pos == 2) {
        const R c0 = wv[0], c1 = wv[1], c2 = -xv[1] / xv[0], c3 = R(1);
        R det = c0 * c3 - c1 * c2;
        det = R(1) / det;
        out[0] = balance * c3 * det;
        out[1] = -balance * c2 * det;
    } else {
        const R c0 = wv[0], c1 = wv[1], c2 = wv[2];
        const R c3 = -xv[1] / xv[0], c4 = R(1), c6 = -xv[2] / xv[0], c8 = R(1);
        R det = c0 * c4 * c8 - c1 * c3 * c8 - c2 * c4 * c6;
        det = R(1) / det;
        out[0] = balance * c4 * c8 * det;
        out[1] = -balance * c3 * c8 * det;
        out[2] = -balance * c4 * c6 * det;
    }
    bool fail = false;
    for (int k = 0; k < pos; ++k) fail = fail || out[k] < xmin;
    for (int k = 0; k < pos; ++k) {
#pragma unroll
        for (int i = 0; i < N; ++i)
            if (i == cnt[k]) x[i] = fail ? xmin : out[k];
    }
    return fail ? -1 : 1;
}

// LocalOptimizationFixupOperator::Apply (src/fixup.cpp:59-88): the point
// nearest to the solved x0 with w . x = source total and x >= floor, the
// problem mfem::SLBQPOptimizer solves iteratively (to 1e-12 relative in
// allium's setup, src/io.cpp:879-890).  Here exactly: x_i = max(x0_i +
// lam w_i, floor) with lam from the active set, shrunk until no free entry
// falls below the floor (each pass lowers lam, so a clamped entry stays
// clamped; at most N passes).  Entries with w_i = 0 take max(x0_i, floor).
template <int N, typename R>
__device__ __noinline__ int fixup_local_optimization(R xmin, const R (&w)[N], R balance, R (&x)[N]) {
    R lo = x[0];
#pragma unroll
    for (int i = 1; i < N; ++i) lo = x[i] < lo ? x[i] : lo;
    if (lo > xmin || balance <= xmin) return 0;
    bool freev[N];
#pragma unroll
    for (int i = 0; i < N; ++i) freev[i] = w[i] > R(0);
    R lam = R(0);
    bool feasible = false;
    for (int pass = 0; pass <= N; ++pass) {
        // free entries contribute w (x0 + lam w), clamped ones w * floor,
        // entries with w = 0 nothing
        R rest = balance, ww = R(0);
#pragma unroll
        for (int i = 0; i < N; ++i) {
            if (freev[i]) { rest -= w[i] * x[i]; ww += w[i] * w[i]; }
            else if (w[i] > R(0)) rest -= w[i] * xmin;
        }
        if (!(ww > R(0))) break;
        lam = rest / ww;
        bool clamped = false;
#pragma unroll
        for (int i = 0; i < N; ++i)
            if (freev[i] && x[i] + lam * w[i] < xmin) { freev[i] = false; clamped = true; }
        if (!clamped) { feasible = true; break; }
    }
    if (!feasible) {
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] = x[i] > xmin ? x[i] : xmin;
        return -1;
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const R v = freev[i] ? x[i] + lam * w[i] : (w[i] > R(0) ? xmin : x[i]);
        x[i] = v > xmin ? v : xmin;
    }
    return 1;
}

// ZeroFixupOperator / ZeroAndScaleFixupOperator::Apply (src/fixup.cpp:3-57),
// kinds 1 and 2, and the Ryosuke (3) and local-optimization (4) fixups above,
// on the solved local vector x, with w the column sums of the local matrix and
// balance = sum of the right-hand side.  Returns 0 (untouched), 1, -1, or -2
// (Ryosuke with more than three positive entries).
template <int N, typename R>
__device__ __forceinline__ int apply_fixup(int kind, R xmin, const R (&w)[N], R balance, R (&x)[N]) {
    if (kind == 3) return fixup_ryosuke<N, R>(xmin, w, balance, x);
    if (kind == 4) return fixup_local_optimization<N, R>(xmin, w, balance, x);
    R lo = x[0];
#pragma unroll
    for (int i = 1; i < N; ++i) lo = x[i] < lo ? x[i] : lo;
    if (kind == 1) {
        int applied = 0;
#pragma unroll
        for (int i = 0; i < N; ++i)
            if (x[i] <= xmin) { x[i] = xmin; applied = 1; }
        return applied;
    }
    if (lo > xmin) return 0;
#pragma unroll
    for (int i = 0; i < N; ++i)
        if (x[i] <= xmin) x[i] = xmin;
    R nb = R(0);
#pragma unroll
    for (int i = 0; i < N; ++i) nb += w[i] * x[i];
    if (balance < R(0) || nb < R(0)) return -1;
    if (balance == R(0) || nb == R(0)) {
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] = R(0);
    } else {
        const R sc = balance / nb;
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] *= sc;
    }
    return 1;
}

// The fixup on a solution and column sums held in shared (or any) memory, out
// of line so that the team and block kernels keep their register budget for
// the fixup-free path; counts and the Ryosuke abort status recorded here.
template <int N, typename R>
__device__ __noinline__ void apply_fixup_mem(int kind, R xmin, R* xs, const R* ws, R balance, int* status,
                                             unsigned long long* counts) {
    R x[N], w[N];
    for (int i = 0; i < N; ++i) { x[i] = xs[i]; w[i] = ws[i]; }
    const int res = apply_fixup<N, R>(kind, xmin, w, balance, x);
    if (res == -2) atomicOr(status, kErrFixup);
    if (res) atomicAdd(counts + (res > 0 ? 0 : 1), 1ull);
    for (int i = 0; i < N; ++i) xs[i] = x[i];
}

__device__ __forceinline__ double fma_r(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_r(float a, float b, float c) { return fmaf(a, b, c); }

// Sign tests and sign flips of Omega.n on the bit pattern, on the integer
// pipe: GB300 issues every FP64 compare or negate on its narrow FP64 pipe,
// which the node kernels already fill with FMAs.  below_zero(x) == (x < 0)
// and above_zero(x) == (x > 0) for every non-NaN x (-0.0 is neither);
// negate_if(x, f) == (f ? -x : x) bit for bit.
__device__ __forceinline__ bool below_zero(double x) {
    const long long b = __double_as_longlong(x);
    return b < 0 && (b << 1) != 0;
}
__device__ __forceinline__ bool below_zero(float x) {
    const int b = __float_as_int(x);
    return b < 0 && (b << 1) != 0;
}
__device__ __forceinline__ bool above_zero(double x) { return __double_as_longlong(x) > 0; }
__device__ __forceinline__ bool above_zero(float x) { return __float_as_int(x) > 0; }
__device__ __forceinline__ double negate_if(double x, bool f) {
    return __longlong_as_double((long long)((unsigned long long)__double_as_longlong(x) ^ ((unsigned long long)f << 63)));
}
__device__ __forceinline__ float negate_if(float x, bool f) {
    return __int_as_float((int)((unsigned)__float_as_int(x) ^ ((unsigned)f << 31)));
}

// n contiguous values of one (group, angle, cell) block; 16-byte vectors when
// the block size allows (the API requires 16-byte aligned vectors)
template <int N, typename R>
__device__ __forceinline__ void load_block(const R* p, R (&v)[N]) {
    if constexpr (sizeof(R) == 4 && N % 4 == 0) {
#pragma unroll
        for (int i = 0; i < N / 4; ++i) {
            const float4 x = reinterpret_cast<const float4*>(p)[i];
            v[4 * i] = x.x; v[4 * i + 1] = x.y; v[4 * i + 2] = x.z; v[4 * i + 3] = x.w;
        }
    } else if constexpr (sizeof(R) == 8 && N % 2 == 0) {
#pragma unroll
        for (int i = 0; i < N / 2; ++i) {
            const double2 x = reinterpret_cast<const double2*>(p)[i];
            v[2 * i] = x.x; v[2 * i + 1] = x.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = p[i];
    }
}

template <int N, typename R>
__device__ __forceinline__ void store_block(R* p, const R (&v)[N]) {
    if constexpr (sizeof(R) == 4 && N % 4 == 0) {
#pragma unroll
        for (int i = 0; i < N / 4; ++i)
            reinterpret_cast<float4*>(p)[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    } else if constexpr (sizeof(R) == 8 && N % 2 == 0) {
#pragma unroll
        for (int i = 0; i < N / 2; ++i) reinterpret_cast<double2*>(p)[i] = make_double2(v[2 * i], v[2 * i + 1]);
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) p[i] = v[i];
    }
}

// Compile-time loop: f(std::integral_constant<int, i>) for i in [B, E).  Keeps
// every register-array index a constant, so the local system stays in registers.
template <int B, int E, typename F>
__device__ __forceinline__ void static_for(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

// Gaussian elimination on registers.  PIVOT: partial pivoting on the largest
// magnitude (first one on ties), the order mfem::LUFactors::Factor uses.  The
// right-hand side is eliminated alongside, and back substitution multiplies
// by the stored pivot reciprocals.
template <int N, bool PIVOT, typename R>
__device__ __forceinline__ bool solve_local(R (&A)[N][N], R (&b)[N]) {
    bool ok = true;
    static_for<0, N>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        if constexpr (PIVOT) {
            R amax = fabs(A[k][k]);
            int piv = k;
            static_for<k + 1, N>([&](auto ic) {
                constexpr int i = decltype(ic)::value;
                const R v = fabs(A[i][k]);
                if (v > amax) { amax = v; piv = i; }
            });
            static_for<k + 1, N>([&](auto ic) {
                constexpr int i = decltype(ic)::value;
                const bool sw = (piv == i);
                static_for<k, N>([&](auto jc) {
                    constexpr int j = decltype(jc)::value;
                    const R x = A[k][j], y = A[i][j];
                    A[k][j] = sw ? y : x;
                    A[i][j] = sw ? x : y;
                });
                const R x = b[k], y = b[i];
                b[k] = sw ? y : x;
                b[i] = sw ? x : y;
            });
        }
        const R pk = A[k][k];
        ok = ok && (pk != R(0));
        const R inv = R(1) / pk;
        static_for<k + 1, N>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            const R l = A[i][k] * inv;
            static_for<k + 1, N>([&](auto jc) {
                constexpr int j = decltype(jc)::value;
                A[i][j] = fma_r(-l, A[k][j], A[i][j]);
            });
            b[i] = fma_r(-l, b[k], b[i]);
        });
        A[k][k] = inv;
    });
    static_for<0, N>([&](auto kc) {
        constexpr int k = N - 1 - decltype(kc)::value;
        const R x = b[k] * A[k][k];
        b[k] = x;
        static_for<0, k>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            b[i] = fma_r(-A[i][k], x, b[i]);
        });
    });
    return ok;
}

// In-place inverse by Gauss-Jordan elimination with partial pivoting (row
// swaps undone as column swaps at the end).
template <int N>
__device__ __forceinline__ bool invert_local(double (&A)[N][N]) {
    bool ok = true;
    int perm[N];
    static_for<0, N>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        double amax = fabs(A[k][k]);
        int piv = k;
        static_for<k + 1, N>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            const double v = fabs(A[i][k]);
            if (v > amax) { amax = v; piv = i; }
        });
        perm[k] = piv;
        static_for<k + 1, N>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            const bool sw = (piv == i);
            static_for<0, N>([&](auto jc) {
                constexpr int j = decltype(jc)::value;
                const double x = A[k][j], y = A[i][j];
                A[k][j] = sw ? y : x;
                A[i][j] = sw ? x : y;
            });
        });
        ok = ok && (A[k][k] != 0.0);
        const double inv = 1.0 / A[k][k];
        A[k][k] = 1.0;
        static_for<0, N>([&](auto jc) { A[k][decltype(jc)::value] *= inv; });
        static_for<0, N>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            if constexpr (i != k) {
                const double f = A[i][k];
                A[i][k] = 0.0;
                static_for<0, N>([&](auto jc) {
                    constexpr int j = decltype(jc)::value;
                    A[i][j] = fma(-f, A[k][j], A[i][j]);
                });
            }
        });
    });
    static_for<0, N>([&](auto kc) {
        constexpr int k = N - 1 - decltype(kc)::value;
        static_for<k + 1, N>([&](auto jc) {
            constexpr int j = decltype(jc)::value;
            const bool sw = (perm[k] == j);
            static_for<0, N>([&](auto ic) {
                constexpr int i = decltype(ic)::value;
                const double x = A[i][k], y = A[i][j];
                A[i][k] = sw ? y : x;
                A[i][j] = sw ? x : y;
            });
        });
    });
    return ok;
}

// Local matrix of node (e, a), group g (the assembly part of k_sweep_level).
template <int D, int P, typename R>
__device__ __forceinline__ void assemble_local(const SweepArgs<R>& s, int e, int a, int g,
                                               R (&A)[ipow(P + 1, D)][ipow(P + 1, D)],
                                               R (&dots)[2 * D], int (&nbrs)[2 * D]) {
    constexpr int N = ipow(P + 1, D);
    constexpr int NF = ipow(P + 1, D - 1);
    constexpr int NFACE = 2 * D;
    R om[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int d = 0; d < D; ++d) om[d] = R(s.omega[a * D + d]);
    const R* Gm = s.Gm + (size_t)e * D * N * N;
    const R* M = s.M + (size_t)e * N * N;
    const R sg = s.sigma[(size_t)g * s.ne + e];
    // whole rows per load: the cell's matrices are shared by the warp's threads
#pragma unroll
    for (int i = 0; i < N; ++i) {
        R row[N], mrow[N];
        load_block<N>(Gm + i * N, row);
        load_block<N>(M + i * N, mrow);
#pragma unroll
        for (int j = 0; j < N; ++j) A[i][j] = om[0] * row[j];
#pragma unroll
        for (int d = 1; d < D; ++d) {
            load_block<N>(Gm + d * N * N + i * N, row);
#pragma unroll
            for (int j = 0; j < N; ++j) A[i][j] = fma_r(om[d], row[j], A[i][j]);
        }
#pragma unroll
        for (int j = 0; j < N; ++j) A[i][j] = fma_r(sg, mrow[j], A[i][j]);
    }
    if (s.td) {
        const R* Mt = s.Mt + (size_t)e * N * N;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            R row[N];
            load_block<N>(Mt + i * N, row);
#pragma unroll
            for (int j = 0; j < N; ++j) A[i][j] = fma_r(s.tau, row[j], A[i][j]);
        }
    }
#pragma unroll
    for (int k = 0; k < NFACE; ++k) {
        const Slot q = s.slots[(size_t)e * NFACE + k];
        const R d1 = s.dots[(size_t)q.face * s.Nw + a];
        const R dk = negate_if(d1, q.side);
        dots[k] = dk;
        nbrs[k] = q.nbr;
        if (above_zero(dk)) {
            const R* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
#pragma unroll
            for (int ii = 0; ii < NF; ++ii) {
                R frow[NF];
                load_block<NF>(F + ii * NF, frow);
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) {
                    const int fi = face_dof(D, P, k, ii), fj = face_dof(D, P, k, jj);
                    A[fi][fj] = fma_r(dk, frow[jj], A[fi][fj]);
                }
            }
        }
    }
}

// Right-hand side of node (e, a), group g: q plus the upwind face terms.
template <typename R>
__device__ __forceinline__ R load_upstream(const R* p, bool cg) {
    return cg ? __ldcg(p) : *p;
}

template <int D, int P, typename R, bool CG = false>
__device__ __forceinline__ void assemble_rhs(const SweepArgs<R>& s, int e, int a, int g, const R (&dots)[2 * D],
                                             const int (&nbrs)[2 * D], R (&b)[ipow(P + 1, D)]) {
    constexpr int N = ipow(P + 1, D);
    constexpr int NF = ipow(P + 1, D - 1);
    constexpr int NFACE = 2 * D;
    load_block<N>(s.src + psi_index(s.ndof, s.Nw, g, a, (long long)e * N), b);
#pragma unroll
    for (int k = 0; k < NFACE; ++k) {
        if (below_zero(dots[k]) && nbrs[k] >= 0) {
            const uint8_t* map = s.nbrmap + ((size_t)e * NFACE + k) * NF;
            const R* up = s.psi + psi_index(s.ndof, s.Nw, g, a, (long long)nbrs[k] * N);
            R u[NF];
            if constexpr (NF == 4) {
                // the four map bytes of a face in one 32-bit load (4-byte aligned: NF = 4)
                const unsigned m4 = *reinterpret_cast<const unsigned*>(map);
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) u[jj] = load_upstream(up + ((m4 >> (8 * jj)) & 0xffu), CG);
            } else {
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) u[jj] = load_upstream(up + map[jj], CG);
            }
            const R* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
            const R rd = -dots[k];
#pragma unroll
            for (int ii = 0; ii < NF; ++ii) {
                R frow[NF];
                load_block<NF>(F + ii * NF, frow);
                R acc = R(0);
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) acc = fma_r(frow[jj], u[jj], acc);
                const int fi = face_dof(D, P, k, ii);
                b[fi] = fma_r(rd, acc, b[fi]);
            }
        } else if (below_zero(dots[k]) && nbrs[k] <= -2) {
            // reflective face: the same cell's trace in the reflected direction
            // (sweep.cpp:432-437), face block F(self, self)
            const int ar = s.refl[(size_t)(-2 - nbrs[k]) * s.Nw + a];
            const R* own = s.psi + psi_index(s.ndof, s.Nw, g, ar, (long long)e * N);
            R u[NF];
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) u[jj] = load_upstream(own + face_dof(D, P, k, jj), CG);
            const R* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
            const R rd = -dots[k];
#pragma unroll
            for (int ii = 0; ii < NF; ++ii) {
                R frow[NF];
                load_block<NF>(F + ii * NF, frow);
                R acc = R(0);
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) acc = fma_r(frow[jj], u[jj], acc);
                const int fi = face_dof(D, P, k, ii);
                b[fi] = fma_r(rd, acc, b[fi]);
            }
        }
    }
}

template <int D, int P, typename R, bool PIVOT>
__global__ void __launch_bounds__(128, (sizeof(R) == 4 ? 4 : 1)) k_sweep_level(SweepArgs<R> s, const int* __restrict__ nodes, int count) {
    constexpr int N = ipow(P + 1, D);
    // count * G < 2^31 is checked by the launcher
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count * s.G) return;
    const int ni = t / s.G;
    const int g = t - ni * s.G;
    const int node = nodes[ni];
    const int e = node / s.Nw;
    const int a = node - e * s.Nw;
    R A[N][N], dots[2 * D];
    int nbrs[2 * D];
    assemble_local<D, P, R>(s, e, a, g, A, dots, nbrs);
    R b[N];
    assemble_rhs<D, P, R>(s, e, a, g, dots, nbrs, b);
    R w[N], balance = R(0);
    if (s.fix_kind) {
#pragma unroll
        for (int i = 0; i < N; ++i) {
            R c = R(0);
#pragma unroll
            for (int j = 0; j < N; ++j) c += A[j][i];
            w[i] = c;
            balance += b[i];
        }
    }
    if (!solve_local<N, PIVOT>(A, b)) atomicOr(s.status, kErrSingular);
    if (s.fix_kind) {
        const int r = apply_fixup<N, R>(s.fix_kind, s.fix_min, w, balance, b);
        if (r == -2) atomicOr(s.status, kErrFixup);
        if (r) atomicAdd(s.fix_counts + (r > 0 ? 0 : 1), 1ull);
    }
    store_block<N>(s.psi + psi_index(s.ndof, s.Nw, g, a, (long long)e * N), b);
}


// ---------------------------------------------------------------- team kernel
// One team of T lanes (T = smallest power of two >= N, N <= 32) per (cell,
// angle, group) node; lane r owns row r of the local system.  Rows of the cell
// matrices and of q/psi are read by consecutive lanes (coalesced), elimination
// runs on warp shuffles inside the team, so a lane holds one row (~N + 10
// registers) instead of the whole matrix.  PIVOT: partial pivoting by a team
// argmax (largest magnitude, lowest row on ties) and a row exchange between
// the two lanes.
__host__ __device__ constexpr int team_size(int n) {
    return n <= 1 ? 1 : n <= 2 ? 2 : n <= 4 ? 4 : n <= 8 ? 8 : n <= 16 ? 16 : 32;
}

template <int D, int P, typename R, bool PIVOT, bool FIX = false>
__global__ void __launch_bounds__(256) k_sweep_team(SweepArgs<R> s, const int* __restrict__ nodes, int count) {
    constexpr int N1 = P + 1;
    constexpr int N = ipow(N1, D);
    constexpr int NF = ipow(N1, D - 1);
    constexpr int NFACE = 2 * D;
    constexpr int T = team_size(N);
    static_assert(N <= 32, "team kernel handles local systems up to 32 x 32");
    const int lane = threadIdx.x & 31;
    const int r = lane & (T - 1);
    const unsigned mask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << (lane & ~(T - 1)));
    const int team = (blockIdx.x * blockDim.x + threadIdx.x) / T;
    if (team >= count * s.G) return;   // whole teams leave together
    const bool act = r < N;
    const int ni = team / s.G;
    const int g = team - ni * s.G;
    const int node = nodes[ni];
    const int e = node / s.Nw;
    const int a = node - e * s.Nw;

    // this lane's row: tensor indices of local DOF r
    int rid[3] = {0, 0, 0};
    {
        int q = r;
#pragma unroll
        for (int d = 0; d < D; ++d) { rid[d] = q % N1; q /= N1; }
    }

    R Ar[N];
    R br = R(0);
    {
        R om[3] = {R(0), R(0), R(0)};
#pragma unroll
        for (int d = 0; d < D; ++d) om[d] = R(s.omega[a * D + d]);
        const int rr = act ? r : 0;
        const R* Gm = s.Gm + (size_t)e * D * N * N + rr * N;
        const R* M = s.M + (size_t)e * N * N + rr * N;
        const R sg = s.sigma[(size_t)g * s.ne + e];
        R row[N];
        load_block<N>(Gm, row);
#pragma unroll
        for (int j = 0; j < N; ++j) Ar[j] = om[0] * row[j];
#pragma unroll
        for (int d = 1; d < D; ++d) {
            load_block<N>(Gm + d * N * N, row);
#pragma unroll
            for (int j = 0; j < N; ++j) Ar[j] = fma_r(om[d], row[j], Ar[j]);
        }
        load_block<N>(M, row);
#pragma unroll
        for (int j = 0; j < N; ++j) Ar[j] = fma_r(sg, row[j], Ar[j]);
        if (s.td) {
            load_block<N>(s.Mt + (size_t)e * N * N + rr * N, row);
#pragma unroll
            for (int j = 0; j < N; ++j) Ar[j] = fma_r(s.tau, row[j], Ar[j]);
        }
        if (act) br = s.src[psi_index(s.ndof, s.Nw, g, a, (long long)e * N + r)];
    }

    static_for<0, NFACE>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int ax = k / 2, side = k % 2;
        const Slot q = s.slots[(size_t)e * NFACE + k];
        const R d1 = s.dots[(size_t)q.face * s.Nw + a];
        const R dk = q.side ? -d1 : d1;
        // is row r on face k, and which face DOF is it
        const bool on = act && (rid[ax] == side * P);
        int ii = 0, stride = 1;
#pragma unroll
        for (int d = 0; d < D; ++d)
            if (d != ax) { ii += rid[d] * stride; stride *= N1; }
        const R* F = s.F + ((size_t)e * NFACE + k) * NF * NF + ii * NF;
        if (dk > R(0) && on) {
            R frow[NF];
            load_block<NF>(F, frow);
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) {
                const int fj = face_dof(D, P, k, jj);
                Ar[fj] = fma_r(dk, frow[jj], Ar[fj]);
            }
        }
        if (dk < R(0) && q.nbr >= 0 && on) {
            const uint8_t* map = s.nbrmap + ((size_t)e * NFACE + k) * NF;
            const R* up = s.psi + psi_index(s.ndof, s.Nw, g, a, (long long)q.nbr * N);
            R frow[NF];
            load_block<NF>(F, frow);
            R acc = R(0);
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) acc = fma_r(frow[jj], up[map[jj]], acc);
            br = fma_r(-dk, acc, br);
        }
        if (dk < R(0) && q.nbr <= -2 && on) {
            const int ar = s.refl[(size_t)(-2 - q.nbr) * s.Nw + a];
            const R* own = s.psi + psi_index(s.ndof, s.Nw, g, ar, (long long)e * N);
            R frow[NF];
            load_block<NF>(F, frow);
            R acc = R(0);
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) acc = fma_r(frow[jj], own[face_dof(D, P, k, jj)], acc);
            br = fma_r(-dk, acc, br);
        }
    });

    // fixup inputs, before the elimination overwrites A and b: lane r keeps the
    // column sum w_r = sum_j A[j][r]; bal = sum of the right-hand side
    R wcol = R(0), bal = R(0);
    if constexpr (FIX) {
        static_for<0, N>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            R v = act ? Ar[i] : R(0);
#pragma unroll
            for (int off = T / 2; off > 0; off >>= 1) v += __shfl_xor_sync(mask, v, off, T);
            if (r == i) wcol = v;
        });
        R v = act ? br : R(0);
#pragma unroll
        for (int off = T / 2; off > 0; off >>= 1) v += __shfl_xor_sync(mask, v, off, T);
        bal = v;
    }

    bool ok = true;
    static_for<0, N>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        if constexpr (PIVOT) {
            // team argmax of |A[i][k]| over rows i >= k
            R best = (r >= k && act) ? fabs(Ar[k]) : R(-1);
            int bi = r;
#pragma unroll
            for (int off = T / 2; off > 0; off >>= 1) {
                const R ob = __shfl_xor_sync(mask, best, off, T);
                const int oi = __shfl_xor_sync(mask, bi, off, T);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            const int p = bi;   // same on every lane of the team
            const int src = (r == k) ? p : (r == p ? k : r);
#pragma unroll
            for (int j = k; j < N; ++j) Ar[j] = __shfl_sync(mask, Ar[j], src, T);
            br = __shfl_sync(mask, br, src, T);
        }
        const R akk = __shfl_sync(mask, Ar[k], k, T);
        ok = ok && (akk != R(0));
        const R inv = R(1) / akk;
        const R l = Ar[k] * inv;
        const R bk = __shfl_sync(mask, br, k, T);
#pragma unroll
        for (int j = k + 1; j < N; ++j) {
            const R akj = __shfl_sync(mask, Ar[j], k, T);
            if (r > k) Ar[j] = fma_r(-l, akj, Ar[j]);
        }
        if (r > k) br = fma_r(-l, bk, br);
        if (r == k) Ar[k] = inv;
    });
    static_for<0, N>([&](auto kc) {
        constexpr int k = N - 1 - decltype(kc)::value;
        const R xk = __shfl_sync(mask, br * Ar[k], k, T);
        if (r == k) br = xk;
        if (r < k) br = fma_r(-Ar[k], xk, br);
    });
    if (!ok && r == 0) atomicOr(s.status, kErrSingular);
    if constexpr (FIX) {
        // the team's solution and column sums through shared memory to its
        // first lane, which applies the fixup as the thread-per-node kernel does
        __shared__ R fx[256], fw[256];
        const int base = threadIdx.x - r;
        fx[threadIdx.x] = br;
        fw[threadIdx.x] = wcol;
        __syncwarp(mask);
        if (r == 0) apply_fixup_mem<N, R>(s.fix_kind, s.fix_min, fx + base, fw + base, bal, s.status, s.fix_counts);
        __syncwarp(mask);
        br = fx[threadIdx.x];
    }
    if (act) s.psi[psi_index(s.ndof, s.Nw, g, a, (long long)e * N + r)] = br;
}

// Block per (node, group) for local systems wider than a warp (3D p = 3:
// 64 x 64, 33 KB in FP64).  The system sits in shared memory, one row per
// thread, and is solved by Gaussian elimination with the team kernel's pivot
// rule (largest magnitude, first row on ties) and arithmetic (reciprocal of the
// pivot, multiplier A[i][k] * inv, back substitution by x_k = b_k * inv_k).
template <int D, int P, typename R, bool PIVOT, bool FIX = false>
__global__ void __launch_bounds__(64) k_sweep_block(SweepArgs<R> s, const int* __restrict__ nodes) {
    constexpr int N1 = P + 1;
    constexpr int N = ipow(N1, D);
    constexpr int NF = ipow(N1, D - 1);
    constexpr int NFACE = 2 * D;
    constexpr int LD = N + 1;   // odd row stride: a column walk touches distinct banks
    constexpr int NW = N / 32;
    static_assert(N == 64, "block kernel is laid out for 64 x 64 local systems");
    __shared__ R A[N * LD];
    __shared__ R b[N];
    __shared__ R wbest[NW];
    __shared__ int widx[NW];
    const int r = threadIdx.x;
    const int lane = r & 31, warp = r >> 5;
    const int ni = blockIdx.x / s.G;   // the grid is exactly count * G blocks
    const int g = blockIdx.x - ni * s.G;
    const int node = nodes[ni];
    const int e = node / s.Nw;
    const int a = node - e * s.Nw;

    int rid[3] = {0, 0, 0};
    {
        int q = r;
#pragma unroll
        for (int d = 0; d < D; ++d) { rid[d] = q % N1; q /= N1; }
    }
    R om[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int d = 0; d < D; ++d) om[d] = R(s.omega[a * D + d]);
    {
        const R* Gm = s.Gm + (size_t)e * D * N * N;
        const R* M = s.M + (size_t)e * N * N;
        const R* Mt = s.Mt + (size_t)e * N * N;
        const R sg = s.sigma[(size_t)g * s.ne + e];
        for (int idx = r; idx < N * N; idx += N) {
            R v = om[0] * Gm[idx];
#pragma unroll
            for (int d = 1; d < D; ++d) v = fma_r(om[d], Gm[d * N * N + idx], v);
            v = fma_r(sg, M[idx], v);
            if (s.td) v = fma_r(s.tau, Mt[idx], v);
            A[(idx / N) * LD + idx % N] = v;
        }
    }
    R br = s.src[psi_index(s.ndof, s.Nw, g, a, (long long)e * N + r)];
    __syncthreads();

    static_for<0, NFACE>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int ax = k / 2, side = k % 2;
        const Slot q = s.slots[(size_t)e * NFACE + k];
        const R d1 = s.dots[(size_t)q.face * s.Nw + a];
        const R dk = q.side ? -d1 : d1;
        const R* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
        if (dk > R(0)) {   // outflow face: (Omega.n) F on the face block, one add per entry
            for (int idx = r; idx < NF * NF; idx += N) {
                const int ii = idx / NF, jj = idx - ii * NF;
                R* dst = &A[face_dof(D, P, k, ii) * LD + face_dof(D, P, k, jj)];
                *dst = fma_r(dk, F[idx], *dst);
            }
        }
        const bool on = rid[ax] == side * P;
        int ii = 0, stride = 1;
#pragma unroll
        for (int d = 0; d < D; ++d)
            if (d != ax) { ii += rid[d] * stride; stride *= N1; }
        if (dk < R(0) && q.nbr >= 0 && on) {
            const uint8_t* map = s.nbrmap + ((size_t)e * NFACE + k) * NF;
            const R* up = s.psi + psi_index(s.ndof, s.Nw, g, a, (long long)q.nbr * N);
            R acc = R(0);
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) acc = fma_r(F[ii * NF + jj], up[map[jj]], acc);
            br = fma_r(-dk, acc, br);
        }
        if (dk < R(0) && q.nbr <= -2 && on) {
            const int ar = s.refl[(size_t)(-2 - q.nbr) * s.Nw + a];
            const R* own = s.psi + psi_index(s.ndof, s.Nw, g, ar, (long long)e * N);
            R acc = R(0);
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) acc = fma_r(F[ii * NF + jj], own[face_dof(D, P, k, jj)], acc);
            br = fma_r(-dk, acc, br);
        }
        __syncthreads();   // faces share edge and corner entries: one face at a time
    });
    b[r] = br;
    __syncthreads();
    // fixup inputs before the elimination: column sums of A, the source total
    __shared__ R wsh[N];
    __shared__ R balsh;
    if constexpr (FIX) {
        R c = R(0);
        for (int j = 0; j < N; ++j) c += A[j * LD + r];
        wsh[r] = c;
        if (r == 0) {
            R t = R(0);
            for (int j = 0; j < N; ++j) t += b[j];
            balsh = t;
        }
        __syncthreads();
    }

    bool ok = true;
    R myinv = R(0);
    for (int k = 0; k < N; ++k) {
        if (PIVOT) {
            R best = (r >= k) ? R(fabs(A[r * LD + k])) : R(-1);
            int bi = r;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const R ob = __shfl_xor_sync(0xffffffffu, best, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (lane == 0) { wbest[warp] = best; widx[warp] = bi; }
            __syncthreads();
            best = wbest[0];
            bi = widx[0];
#pragma unroll
            for (int w = 1; w < NW; ++w)
                if (wbest[w] > best || (wbest[w] == best && widx[w] < bi)) { best = wbest[w]; bi = widx[w]; }
            if (bi != k) {   // the same on every thread
                if (r >= k) {
                    const R t = A[k * LD + r];
                    A[k * LD + r] = A[bi * LD + r];
                    A[bi * LD + r] = t;
                }
                if (r == 0) {
                    const R t = b[k];
                    b[k] = b[bi];
                    b[bi] = t;
                }
            }
            __syncthreads();
        }
        const R akk = A[k * LD + k];
        ok = ok && (akk != R(0));
        const R inv = R(1) / akk;
        if (r == k) myinv = inv;
        if (r > k) {
            const R l = A[r * LD + k] * inv;
            for (int j = k + 1; j < N; ++j) A[r * LD + j] = fma_r(-l, A[k * LD + j], A[r * LD + j]);
            b[r] = fma_r(-l, b[k], b[r]);
        }
        __syncthreads();
    }
    // back substitution; b[r] of rows below k is final once row k is reached
    for (int k = N - 1; k >= 0; --k) {
        if (r == k) b[k] = b[k] * myinv;
        __syncthreads();
        if (r < k) b[r] = fma_r(-A[r * LD + k], b[k], b[r]);
    }
    __syncthreads();
    if (!ok && r == 0) atomicOr(s.status, kErrSingular);
    if constexpr (FIX) {
        if (r == 0) apply_fixup_mem<N, R>(s.fix_kind, s.fix_min, b, wsh, balsh, s.status, s.fix_counts);
        __syncthreads();
    }
    s.psi[psi_index(s.ndof, s.Nw, g, a, (long long)e * N + r)] = b[r];
}

// Inverse of every local matrix, in one pass over all node-groups of all levels
// (no level ordering needed: the local matrices do not depend on upstream
// data).  Node-group t of the level-sorted order is stored entry-major,
// inv[(i*N + j) * stride + t], so a warp's loads of one entry are contiguous.
template <int D, int P>
__global__ void __launch_bounds__(128) k_factor_all(SweepArgs<double> s, const int* __restrict__ nodes,
                                                    long long total, double* __restrict__ inv64) {
    constexpr int N = ipow(P + 1, D);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const long long ni = t / s.G;
    const int g = (int)(t - ni * s.G);
    const int node = nodes[ni];
    const int e = node / s.Nw;
    const int a = node - e * s.Nw;
    double A[N][N], dots[2 * D];
    int nbrs[2 * D];
    assemble_local<D, P, double>(s, e, a, g, A, dots, nbrs);
    if (!invert_local<N>(A)) atomicOr(s.status, kErrSingular);
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) inv64[(size_t)(i * N + j) * total + t] = A[i][j];
}

// Sweep with the stored inverses: psi = inv(A) (q + upwind terms).  Launched with
// programmatic dependent launch after the first level: the node's record and its
// face slots and Omega.n come before griddepcontrol.wait (none depends on the
// previous level); the right-hand side, which reads the upwind traces (and q,
// which may alias psi), comes after it.  (An L2 prefetch of the stored inverse
// before the wait measured 12% slower.)
template <int D, int P, typename R, bool POS = false>
__global__ void __launch_bounds__(128) k_sweep_cached_level(SweepArgs<R> s, const int* __restrict__ nodes,
                                                            int count, const R* __restrict__ inv,
                                                            long long stride, long long base,
                                                            const int* __restrict__ pos) {
    constexpr int N = ipow(P + 1, D);
    constexpr int NFACE = 2 * D;
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count * s.G) return;
    const int ni = t / s.G;
    const int g = t - ni * s.G;
    const int node = nodes[ni];
    const int e = node / s.Nw;
    const int a = node - e * s.Nw;
    R dots[NFACE];
    int nbrs[NFACE];
#pragma unroll
    for (int k = 0; k < NFACE; ++k) {
        const Slot q = s.slots[(size_t)e * NFACE + k];
        const R d1 = s.dots[(size_t)q.face * s.Nw + a];
        dots[k] = negate_if(d1, q.side);
        nbrs[k] = q.nbr;
    }
    // stored inverse of this (node, group): level-order position base + t, or,
    // for the angle-chunk orders, the node's level-order position pos[ni]
    const R* in = inv + (POS ? (long long)pos[ni] * s.G + g : base + t);
    asm volatile("griddepcontrol.wait;" ::: "memory");
    R b[N];
    assemble_rhs<D, P, R>(s, e, a, g, dots, nbrs, b);
    R x[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        R acc = R(0);
#pragma unroll
        for (int j = 0; j < N; ++j) acc = fma_r(__ldg(in + (size_t)(i * N + j) * stride), b[j], acc);
        x[i] = acc;
    }
    store_block<N>(s.psi + psi_index(s.ndof, s.Nw, g, a, (long long)e * N), x);
}


// ------------------------------------------------------------ node-major FP32 sweep
// Internal layout for the inner iterations of the FP64 outer solve:
//   v[((e * Nw + a) * G + g) * N + i]
// (cell, angle, group, DOF).  In a wavefront level the threads of a warp hold
// consecutive angles of one cell, so their q/psi blocks and their upwind traces
// (same octant, same upwind neighbour) are contiguous runs.
__host__ __device__ inline long long node_index(int Nw, int G, int N, int e, int a, int g) {
    return (((long long)e * Nw + a) * G + g) * N;
}

template <int D, int P>
__global__ void __launch_bounds__(128, 4) k_sweep_nodes(SweepArgs<float> s, const int* __restrict__ nodes, int count) {
    constexpr int N = ipow(P + 1, D);
    constexpr int NF = ipow(P + 1, D - 1);
    constexpr int NFACE = 2 * D;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count * s.G) return;
    const int ni = t / s.G;
    const int g = t - ni * s.G;
    const int node = nodes[ni];
    const int e = node / s.Nw;
    const int a = node - e * s.Nw;
    float A[N][N], dots[NFACE];
    int nbrs[NFACE];
    assemble_local<D, P, float>(s, e, a, g, A, dots, nbrs);
    float b[N];
    load_block<N>(s.src + node_index(s.Nw, s.G, N, e, a, g), b);
#pragma unroll
    for (int k = 0; k < NFACE; ++k) {
        if (dots[k] < 0.0f && nbrs[k] >= 0) {
            const uint8_t* map = s.nbrmap + ((size_t)e * NFACE + k) * NF;
            float nb[N];
            load_block<N>(s.psi + node_index(s.Nw, s.G, N, nbrs[k], a, g), nb);
            // the neighbour's face values, selected in registers by the DOF map
            float u[NF];
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) {
                const int m = map[jj];
                float v = nb[0];
#pragma unroll
                for (int c = 1; c < N; ++c) v = (m == c) ? nb[c] : v;
                u[jj] = v;
            }
            const float* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
            const float rd = -dots[k];
#pragma unroll
            for (int ii = 0; ii < NF; ++ii) {
                float frow[NF];
                load_block<NF>(F + ii * NF, frow);
                float acc = 0.0f;
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) acc = fmaf(frow[jj], u[jj], acc);
                const int fi = face_dof(D, P, k, ii);
                b[fi] = fmaf(rd, acc, b[fi]);
            }
        }
    }
    if (!solve_local<N, false>(A, b)) atomicOr(s.status, kErrSingular);
    store_block<N>(s.psi + node_index(s.Nw, s.G, N, e, a, g), b);
}

// FP32 copy of the stored FP64 inverses, one contiguous n x n block per
// (level-order node, group): out[t][i][j] = inv64[(i n + j) stride + t].  One
// thread per (t, row i): reads coalesced across t, writes one contiguous row.
template <int N>
__global__ void k_inv_to_f32(long long total, long long stride, const double* __restrict__ inv64,
                             float* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total * N) return;
    const long long t = idx % total;
    const int i = (int)(idx / total);
    float row[N];
#pragma unroll
    for (int j = 0; j < N; ++j) row[j] = (float)inv64[(long long)(i * N + j) * stride + t];
    store_block<N>(out + (t * N + i) * N, row);
}

// The FP64 inverses' entry-major order kept in FP32: out[e * total + t] =
// inv64[e * total + t] for the N*N entries e (one warp load = 32 nodes' entry).
static __global__ void k_inv_to_f32_entries(long long n, const double* __restrict__ inv64, float* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < n) out[idx] = (float)inv64[idx];
}

// Node-major FP32 sweep from the stored FP32 inverses: right-hand side as in
// k_sweep_nodes, then psi = inv(A) b.  ENTRY_MAJOR: entry (i, j) of node-group
// t at inv[(i N + j) stride + t] (coalesced across a warp); otherwise each
// node-group's N x N block is contiguous and read as float4 rows.
template <int D, int P, bool ENTRY_MAJOR = false>
__global__ void __launch_bounds__(128) k_sweep_nodes_cached(SweepArgs<float> s, const int* __restrict__ nodes,
                                                            int count, const float* __restrict__ inv,
                                                            long long base, long long stride) {
    constexpr int N = ipow(P + 1, D);
    constexpr int NF = ipow(P + 1, D - 1);
    constexpr int NFACE = 2 * D;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count * s.G) return;
    const int ni = t / s.G;
    const int g = t - ni * s.G;
    const int node = nodes[ni];
    const int e = node / s.Nw;
    const int a = node - e * s.Nw;
    float b[N];
    load_block<N>(s.src + node_index(s.Nw, s.G, N, e, a, g), b);
#pragma unroll
    for (int k = 0; k < NFACE; ++k) {
        const Slot q = s.slots[(size_t)e * NFACE + k];
        const float d1 = s.dots[(size_t)q.face * s.Nw + a];
        const float dk = q.side ? -d1 : d1;
        if (dk < 0.0f && q.nbr >= 0) {
            const uint8_t* map = s.nbrmap + ((size_t)e * NFACE + k) * NF;
            float nb[N];
            load_block<N>(s.psi + node_index(s.Nw, s.G, N, q.nbr, a, g), nb);
            float u[NF];
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) {
                const int m = map[jj];
                float v = nb[0];
#pragma unroll
                for (int c = 1; c < N; ++c) v = (m == c) ? nb[c] : v;
                u[jj] = v;
            }
            const float* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
            const float rd = -dk;
#pragma unroll
            for (int ii = 0; ii < NF; ++ii) {
                float frow[NF];
                load_block<NF>(F + ii * NF, frow);
                float acc = 0.0f;
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) acc = fmaf(frow[jj], u[jj], acc);
                const int fi = face_dof(D, P, k, ii);
                b[fi] = fmaf(rd, acc, b[fi]);
            }
        }
    }
    float x[N];
    if constexpr (ENTRY_MAJOR) {
        const float* in = inv + base + t;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float acc = 0.0f;
#pragma unroll
            for (int j = 0; j < N; ++j) acc = fmaf(__ldg(in + (long long)(i * N + j) * stride), b[j], acc);
            x[i] = acc;
        }
    } else {
        const float* in = inv + (base + t) * (long long)(N * N);
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float row[N];
            load_block<N>(in + i * N, row);
            float acc = 0.0f;
#pragma unroll
            for (int j = 0; j < N; ++j) acc = fmaf(row[j], b[j], acc);
            x[i] = acc;
        }
    }
    store_block<N>(s.psi + node_index(s.Nw, s.G, N, e, a, g), x);
}

// RIGHT (g, a, i) FP64 <-> node-major FP32, and the node-major scattering source / moments
static __global__ void k_right_to_nodes(int ne, int Nw, int G, int N, long long ndof, const double* __restrict__ in,
                                 float* __restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // node-major index
    if (t >= (long long)ne * Nw * G * N) return;
    const int i = (int)(t % N);
    long long r = t / N;
    const int g = (int)(r % G); r /= G;
    const int a = (int)(r % Nw);
    const int e = (int)(r / Nw);
    out[t] = (float)in[psi_index(ndof, Nw, g, a, (long long)e * N + i)];
}

static __global__ void k_nodes_to_right(int ne, int Nw, int G, int N, long long ndof, const float* __restrict__ in,
                                 double* __restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // RIGHT index
    if (t >= (long long)ne * Nw * G * N) return;
    const long long s = t % ndof;
    const long long r = t / ndof;
    const int a = (int)(r % Nw), g = (int)(r / Nw);
    const int e = (int)(s / N), i = (int)(s % N);
    out[t] = (double)in[node_index(Nw, G, N, e, a, g) + i];
}

// out = (float)(D^T (S phi) + q), node-major; one thread per (cell, group, DOF)
static __global__ void k_scatter_nodes(int ne, int Nw, int G, int N, long long ndof, double wsum,
                                const double* __restrict__ Ms, const double* __restrict__ sigma_s,
                                const double* __restrict__ phi, const float* qn, float* out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    const int e = (int)(s / N), i = (int)(s % N);
    const double* M = Ms + (size_t)e * N * N + (size_t)i * N;
    const double* ph = phi + ndof * g + (long long)e * N;
    double acc = 0.0;
    for (int j = 0; j < N; ++j) acc += M[j] * ph[j];
    const double v = (sigma_s[(size_t)g * ne + e] * acc) / wsum;
    for (int a = 0; a < Nw; ++a) {
        const long long k = node_index(Nw, G, N, e, a, g) + i;
        out[k] = qn ? (float)((double)qn[k] + v) : (float)v;
    }
}

// phi(g, e N + i) = sum_a w_a psi(e, a, g, i), FP64 accumulation
static __global__ void k_moments_nodes(int ne, int Nw, int G, int N, long long ndof, const double* __restrict__ w,
                                const float* __restrict__ psi, double* __restrict__ phi) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)G * ndof) return;
    const int g = (int)(t / ndof);
    const long long s = t % ndof;
    const int e = (int)(s / N), i = (int)(s % N);
    double acc = 0.0;
    for (int a = 0; a < Nw; ++a) acc = fma(w[a], (double)psi[node_index(Nw, G, N, e, a, g) + i], acc);
    phi[t] = acc;
}


// ------------------------------------------------------------ dataflow sweep
// One persistent launch per sweep.  The level-sorted node-groups are cut into
// tiles of at most kTile node-groups that never span two levels; blocks take
// tiles in order from an atomic counter.  A node-group waits only for the
// completion flags of the upwind neighbours it reads, then computes, writes
// psi, fences and publishes its own flag (the sweep's epoch number, so flags
// never need clearing).  Every upwind neighbour lies in an earlier level, hence
// in an earlier tile, which a running block has already taken: by induction
// over the tile index every wait ends.  Waits are bounded anyway: past
// kSpinLimit polls, or once another thread has given up, the thread records
// kErrTimeout and goes on, so the launch always finishes.
constexpr int kSpinLimit = 1 << 22;

struct FlowArgs {
    unsigned* flags;            // [ne * Nw * G] epoch of the last sweep that wrote each node-group
    const unsigned* epoch;      // device word, incremented before each sweep
    unsigned* counter;          // tile counter, zeroed before each sweep
    const int* tile_start;      // [ntiles] first level-sorted node-group of each tile
    const int* tile_count;      // [ntiles]
    int ntiles;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool wait_flag(const unsigned* f, unsigned epoch, int* status, int limit = kSpinLimit) {
    for (int it = 0;; ++it) {
        if (ld_acquire(f) == epoch) return true;
        if (it >= limit || (*reinterpret_cast<volatile int*>(status) & kErrTimeout)) {
            atomicOr(status, kErrTimeout);
            return false;
        }
        __nanosleep(32);
    }
}

// Waits on a flag that nothing sets, with a caller-chosen poll limit: checks
// that a bounded wait gives up and reports kErrTimeout.
static __global__ void k_wait_probe(const unsigned* flag, unsigned epoch, int limit, int* status) {
    wait_flag(flag, epoch, status, limit);
}

static __global__ void k_flow_begin(unsigned* epoch, unsigned* counter) {
    *epoch += 1u;
    *counter = 0u;
}

// Take the next tile: (first sorted node-group, count), or count = 0 when done.
__device__ __forceinline__ void next_tile(const FlowArgs& f, int& start, int& count) {
    __shared__ int s_tile;
    __syncthreads();   // everyone has read the previous tile
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(f.counter, 1u);
    __syncthreads();
    const int t = s_tile;
    if (t >= f.ntiles) { start = 0; count = 0; return; }
    start = f.tile_start[t];
    count = f.tile_count[t];
}

// wait for the upwind neighbours this node-group reads
template <int D, typename R>
__device__ __forceinline__ void wait_upwind(const FlowArgs& f, int Nw, int G, int a, int g, const R (&dots)[2 * D],
                                            const int (&nbrs)[2 * D], unsigned epoch, int* status) {
#pragma unroll
    for (int k = 0; k < 2 * D; ++k)
        if (below_zero(dots[k]) && nbrs[k] >= 0)
            wait_flag(f.flags + ((size_t)nbrs[k] * Nw + a) * G + g, epoch, status);
}

__device__ __forceinline__ void publish(const FlowArgs& f, int Nw, int G, int e, int a, int g, unsigned epoch) {
    __threadfence();
    st_release(f.flags + ((size_t)e * Nw + a) * G + g, epoch);
}

template <int D, typename R>
__device__ __forceinline__ void face_info(const SweepArgs<R>& s, int e, int a, R (&dots)[2 * D], int (&nbrs)[2 * D]) {
#pragma unroll
    for (int k = 0; k < 2 * D; ++k) {
        const Slot q = s.slots[(size_t)e * 2 * D + k];
        const R d1 = s.dots[(size_t)q.face * s.Nw + a];
        dots[k] = negate_if(d1, q.side);
        nbrs[k] = q.nbr;
    }
}

// MODE 0: FP64 from stored inverses; 1: FP64 rebuilt and pivoted LU; 2: FP32 rebuilt (RIGHT layout)
template <int D, int P, typename R, int MODE>
__global__ void __launch_bounds__(kTile) k_flow(SweepArgs<R> s, FlowArgs f, const int* __restrict__ nodes,
                                                const R* __restrict__ inv, long long stride) {
    constexpr int N = ipow(P + 1, D);
    const unsigned epoch = *f.epoch;
    int start, count;
    for (next_tile(f, start, count); count > 0; next_tile(f, start, count)) {
        if ((int)threadIdx.x >= count) continue;
        const int t = start + threadIdx.x;
        const int ni = t / s.G;
        const int g = t - ni * s.G;
        const int node = nodes[ni];
        const int e = node / s.Nw;
        const int a = node - e * s.Nw;
        R dots[2 * D];
        int nbrs[2 * D];
        R b[N];
        if constexpr (MODE == 0) {
            face_info<D, R>(s, e, a, dots, nbrs);
            wait_upwind<D, R>(f, s.Nw, s.G, a, g, dots, nbrs, epoch, s.status);
            assemble_rhs<D, P, R, true>(s, e, a, g, dots, nbrs, b);
            const R* in = inv + t;
            R x[N];
#pragma unroll
            for (int i = 0; i < N; ++i) {
                R acc = R(0);
#pragma unroll
                for (int j = 0; j < N; ++j) acc = fma_r(__ldg(in + (size_t)(i * N + j) * stride), b[j], acc);
                x[i] = acc;
            }
            store_block<N>(s.psi + psi_index(s.ndof, s.Nw, g, a, (long long)e * N), x);
        } else {
            R A[N][N];
            assemble_local<D, P, R>(s, e, a, g, A, dots, nbrs);
            wait_upwind<D, R>(f, s.Nw, s.G, a, g, dots, nbrs, epoch, s.status);
            assemble_rhs<D, P, R, true>(s, e, a, g, dots, nbrs, b);
            if (!solve_local<N, MODE == 1>(A, b)) atomicOr(s.status, kErrSingular);
            store_block<N>(s.psi + psi_index(s.ndof, s.Nw, g, a, (long long)e * N), b);
        }
        publish(f, s.Nw, s.G, e, a, g, epoch);
    }
}

// FP32, node-major layout, local systems rebuilt each sweep
template <int D, int P>
__global__ void __launch_bounds__(kTile, 4) k_flow_nodes(SweepArgs<float> s, FlowArgs f, const int* __restrict__ nodes) {
    constexpr int N = ipow(P + 1, D);
    constexpr int NF = ipow(P + 1, D - 1);
    constexpr int NFACE = 2 * D;
    const unsigned epoch = *f.epoch;
    int start, count;
    for (next_tile(f, start, count); count > 0; next_tile(f, start, count)) {
        if ((int)threadIdx.x >= count) continue;
        const int t = start + threadIdx.x;
        const int ni = t / s.G;
        const int g = t - ni * s.G;
        const int node = nodes[ni];
        const int e = node / s.Nw;
        const int a = node - e * s.Nw;
        float A[N][N], dots[NFACE];
        int nbrs[NFACE];
        assemble_local<D, P, float>(s, e, a, g, A, dots, nbrs);
        float b[N];
        load_block<N>(s.src + node_index(s.Nw, s.G, N, e, a, g), b);
        wait_upwind<D, float>(f, s.Nw, s.G, a, g, dots, nbrs, epoch, s.status);
#pragma unroll
        for (int k = 0; k < NFACE; ++k) {
            if (dots[k] < 0.0f && nbrs[k] >= 0) {
                const uint8_t* map = s.nbrmap + ((size_t)e * NFACE + k) * NF;
                const float* up = s.psi + node_index(s.Nw, s.G, N, nbrs[k], a, g);
                float nb[N];
#pragma unroll
                for (int c = 0; c < N; ++c) nb[c] = __ldcg(up + c);
                float u[NF];
#pragma unroll
                for (int jj = 0; jj < NF; ++jj) {
                    const int m = map[jj];
                    float v = nb[0];
#pragma unroll
                    for (int c = 1; c < N; ++c) v = (m == c) ? nb[c] : v;
                    u[jj] = v;
                }
                const float* F = s.F + ((size_t)e * NFACE + k) * NF * NF;
                const float rd = -dots[k];
#pragma unroll
                for (int ii = 0; ii < NF; ++ii) {
                    float frow[NF];
                    load_block<NF>(F + ii * NF, frow);
                    float acc = 0.0f;
#pragma unroll
                    for (int jj = 0; jj < NF; ++jj) acc = fmaf(frow[jj], u[jj], acc);
                    const int fi = face_dof(D, P, k, ii);
                    b[fi] = fmaf(rd, acc, b[fi]);
                }
            }
        }
        if (!solve_local<N, false>(A, b)) atomicOr(s.status, kErrSingular);
        store_block<N>(s.psi + node_index(s.Nw, s.G, N, e, a, g), b);
        publish(f, s.Nw, s.G, e, a, g, epoch);
    }
}

// y = L x (AdvectionOperator::Mult, src/sweep.cpp:1246-1387) from the cell's
// point of view: y_e = (sigma M + tau Mt + sum_d Omega_d G_d) x_e
//   + sum_{faces, Omega.n > 0} (Omega.n) F_self x_e
//   + sum_{interior faces, Omega.n < 0} (Omega.n) F_self u_upwind(x_nbr).
struct ApplyArgs {
    int ne, Nw, G;
    long long ndof;
    const double* omega;
    const double* dots;
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
        const double d1 = s.dots[(size_t)q.face * s.Nw + a];
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

// The same operator with one thread per row (3D p = 3: a thread per node would
// hold 2 x 64 doubles).  Row i gets the sums of k_apply_L's row i, in its order.
template <int D, int P>
__global__ void __launch_bounds__(128) k_apply_L_rows(ApplyArgs s) {
    constexpr int N1 = P + 1;
    constexpr int N = ipow(N1, D);
    constexpr int NF = ipow(N1, D - 1);
    constexpr int NFACE = 2 * D;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)s.G * s.ne * s.Nw * N;
    if (t >= total) return;
    const int i = (int)(t % N);
    const long long nd = t / N;
    const int a = (int)(nd % s.Nw);
    const long long r = nd / s.Nw;
    const int e = (int)(r % s.ne);
    const int g = (int)(r / s.ne);
    int rid[3] = {0, 0, 0};
    {
        int q = i;
#pragma unroll
        for (int d = 0; d < D; ++d) { rid[d] = q % N1; q /= N1; }
    }
    double om[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < D; ++d) om[d] = s.omega[a * D + d];
    const double* xv = s.x + psi_index(s.ndof, s.Nw, g, a, (long long)e * N);
    const double* Gm = s.Gm + (size_t)e * D * N * N;
    const double* M = s.M + (size_t)e * N * N;
    const double sg = s.sigma[(size_t)g * s.ne + e];
    double m = 0.0, gr = 0.0, mt = 0.0;
    for (int j = 0; j < N; ++j) {
        const double xj = xv[j];
        m = fma(M[i * N + j], xj, m);
        double c = om[0] * Gm[i * N + j];
#pragma unroll
        for (int d = 1; d < D; ++d) c = fma(om[d], Gm[d * N * N + i * N + j], c);
        gr = fma(c, xj, gr);
    }
    if (s.td) {
        const double* Mt = s.Mt + (size_t)e * N * N;
        for (int j = 0; j < N; ++j) mt = fma(Mt[i * N + j], xv[j], mt);
    }
    double y = fma(sg, m, fma(s.tau, mt, gr));
#pragma unroll
    for (int k = 0; k < NFACE; ++k) {
        const int ax = k / 2, side = k % 2;
        if (rid[ax] != side * P) continue;
        int ii = 0, stride = 1;
#pragma unroll
        for (int d = 0; d < D; ++d)
            if (d != ax) { ii += rid[d] * stride; stride *= N1; }
        const Slot q = s.slots[(size_t)e * NFACE + k];
        const double d1 = s.dots[(size_t)q.face * s.Nw + a];
        const double dk = q.side ? -d1 : d1;
        const double* F = s.F + ((size_t)e * NFACE + k) * NF * NF + ii * NF;
        if (dk > 0.0) {
            double acc = 0.0;
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) acc = fma(F[jj], xv[face_dof(D, P, k, jj)], acc);
            y = fma(dk, acc, y);
        } else if (dk < 0.0 && q.nbr >= 0) {
            const uint8_t* map = s.nbrmap + ((size_t)e * NFACE + k) * NF;
            const double* up = s.x + psi_index(s.ndof, s.Nw, g, a, (long long)q.nbr * N);
            double acc = 0.0;
#pragma unroll
            for (int jj = 0; jj < NF; ++jj) acc = fma(F[jj], up[map[jj]], acc);
            y = fma(dk, acc, y);
        }
    }
    s.y[psi_index(s.ndof, s.Nw, g, a, (long long)e * N + i)] = y;
}

}  // namespace allium
