/* allium_sweep.h -- C ABI of the GB300 upwind DG transport sweep.
 *
 * One handle replaces one allium InverseAdvectionOperator (src/sweep.hpp:13-130)
 * together with the AdvectionOperator, DiscreteToMoment and FormTransportSource
 * pieces that sit on either side of it.  All sizes are plain ints, all arrays
 * plain pointers; there are no CUDA or torch types in the signatures (the
 * stream is passed as void*).
 *
 * Vectors use allium's RIGHT transport layout (src/tvector.hpp:47-58):
 *   psi(g, a, i) = psi[i + Ndof * (a + Nw * g)],  i = e * n + local DOF,
 * where the local DOF order of an element is lexicographic (x fastest) over
 * Gauss-Lobatto nodes, exactly as MFEM's L2_FECollection numbers it.
 * Moments use MomentVectorLayout (src/tvector.hpp:68):
 *   phi(g, m, i) = phi[i + Ndof * (g + G * m)].
 *
 * Every array argument may be a host pointer or a device pointer; the library
 * asks the CUDA runtime which one it is.  Calls with host pointers stage the
 * data through device buffers and return when the host result is written.
 * Calls with device pointers are enqueued on the handle's stream and return
 * at once; allium_sweep_synchronize() waits and reports any error raised by a
 * kernel (singular local system, non-finite values).
 *
 * Every function returns an allium status (ALLIUM_OK = 0) and never aborts.
 * allium_sweep_last_error() gives a one-line reason for the last failure.
 * A handle is not thread safe: one host thread and one stream per handle.
 */
#ifndef ALLIUM_SWEEP_H
#define ALLIUM_SWEEP_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct allium_sweep allium_sweep;

enum allium_status {
    ALLIUM_OK = 0,
    ALLIUM_ERR_ARG = 1,          /* bad argument (null pointer, out of range) */
    ALLIUM_ERR_NOT_DAG = 2,      /* upwind graph has a cycle (sweep.cpp:205-208 aborts) */
    ALLIUM_ERR_SIZE = 3,         /* size mismatch or a size above a stated maximum */
    ALLIUM_ERR_TIMEOUT = 4,      /* a bounded device wait gave up */
    ALLIUM_ERR_NAN = 5,          /* non-finite value detected */
    ALLIUM_ERR_CUDA = 6,         /* CUDA runtime error (message in last_error) */
    ALLIUM_ERR_UNSUPPORTED = 7,  /* option not implemented (order, fixup kind, ...) */
    ALLIUM_ERR_MESH = 8,         /* non-conforming or malformed mesh */
    ALLIUM_ERR_SINGULAR = 9      /* zero pivot in a local solve (mfem::LinearSolve fails) */
};

enum allium_bc_kind { ALLIUM_BC_INFLOW = 0, ALLIUM_BC_REFLECTIVE = 1 };  /* src/bdr_conditions.hpp:5-10 */
enum allium_lump { ALLIUM_LUMP_MASS = 1, ALLIUM_LUMP_GRADIENT = 2, ALLIUM_LUMP_FACE = 4 };  /* src/lumping.hpp:10-18 */
enum allium_basis { ALLIUM_BASIS_GAUSS_LOBATTO = 0 };
/* Transport-vector layouts (src/tvector.hpp:47-55, chosen by the reference's
 * TRANSPORT_VECTOR_LAYOUT build option, RIGHT by default):
 * RIGHT psi(g,a,i) at i + Ndof (a + Nw g); LEFT at g + G (a + Nw i). */
enum allium_layout { ALLIUM_LAYOUT_RIGHT = 0, ALLIUM_LAYOUT_LEFT = 1 };

/* Mesh of segments (dim 1), quadrilaterals (dim 2) or hexahedra (dim 3) with
 * (multi)linear geometry.  element_vertices uses MFEM's local vertex order:
 * quad (0,0),(1,0),(1,1),(0,1); hex: bottom quad then top quad.  Boundary faces
 * carry the attributes used by the boundary-condition map and the inflow
 * source; a boundary face not listed gets attribute 0.
 * Replaces the mfem::ParMesh / ParFiniteElementSpace pair the reference
 * constructor takes (src/sweep.hpp:82). */
typedef struct {
    int dim;
    int num_vertices;
    const double* vertices;             /* [num_vertices][dim] */
    int num_elements;
    const int* element_vertices;        /* [num_elements][2^dim] */
    int num_boundary_faces;
    const int* boundary_face_vertices;  /* [num_boundary_faces][2^(dim-1)] */
    const int* boundary_attributes;     /* [num_boundary_faces] */
} allium_mesh_desc;

/* L2 DG space: order p in 0..3, Gauss-Lobatto basis, lumping bit mask
 * (allium's `lump` constructor argument, src/sweep.hpp:83). */
typedef struct {
    int order;
    int basis;
    int lump;
} allium_fe_desc;

/* Angular quadrature: directions [num_angles][dim] and weights
 * (AngularQuadrature, src/angular_quadrature.hpp:4-22). */
typedef struct {
    int dim;
    int num_angles;
    const double* omega;
    const double* weights;
} allium_quad_desc;

/* BoundaryConditionMap (src/bdr_conditions.hpp): attribute -> kind. */
typedef struct {
    int num;
    const int* attributes;
    const int* kinds;
} allium_bc_desc;

/* InverseAdvectionOperator::InverseAdvectionOperator (src/sweep.cpp:10-244):
 * builds the upwind graph, its device wavefront levels and assembles the local
 * matrices.  sigma_t is the piecewise-constant total cross section
 * [num_groups][num_elements] (a MultiGroupCoefficient sampled per cell).
 * bc may be NULL (all INFLOW).  On REFLECTIVE boundaries a direction entering
 * the domain takes the trace of its mirror direction in the same cell
 * (src/sweep.cpp:177-195, 432-437); the mirror must be in the quadrature set
 * (else ALLIUM_ERR_MESH), and mirror loops that close a cycle give
 * ALLIUM_ERR_NOT_DAG as in the reference. */
int allium_sweep_create(const allium_mesh_desc* mesh, const allium_fe_desc* fe,
                        const allium_quad_desc* quad, int num_groups,
                        const double* sigma_t, const allium_bc_desc* bc,
                        allium_sweep** out);

/* ~InverseAdvectionOperator (src/sweep.cpp:246-257). */
void allium_sweep_destroy(allium_sweep* s);

/* Enqueue all further work of the handle on the given cudaStream_t; NULL
 * selects the CUDA default stream.  Until this is called the handle uses a
 * non-blocking stream of its own. */
int allium_sweep_set_stream(allium_sweep* s, void* cuda_stream);

/* Width()/Height() of the operator (src/sweep.cpp:29): psi_size = G*Nw*Ndof. */
int allium_sweep_sizes(const allium_sweep* s, long long* psi_size, long long* num_dofs,
                       int* num_levels);

/* AssembleLocalMatrices (src/sweep.cpp:924-1001) after a change of sigma_t
 * [G][Ne]; as in the reference, the time absorption setting is kept. */
int allium_sweep_assemble(allium_sweep* s, const double* sigma_t);

/* SetTimeAbsorption (src/sweep.cpp:1003-1022): adds tau * M to every local
 * system; the time mass matrix is assembled once. */
int allium_sweep_set_time_absorption(allium_sweep* s, double tau);

/* InverseAdvectionOperator::Mult (src/sweep.cpp:259-669), FP64 throughout,
 * partially pivoted local LU.  source may equal psi (in-place Mult(psi, psi),
 * as transport_op.hpp:28 and chive.cpp:733 call it).  With page-locked host
 * vectors (and the factor cache on, no reflective faces, no fixup) the
 * directions are swept in 8 independent chunks whose host->device copy, sweep
 * and device->host copy overlap those of the other chunks. */
int allium_sweep_mult(allium_sweep* s, const double* source, double* psi);

/* FP64 factor cache (no counterpart in the reference, which refactors every
 * local system on every Mult).  mode 1 (default): on the first FP64 Mult after
 * construction, AssembleLocalMatrices or a new time absorption, the sweep also
 * stores the inverse of every (cell, angle, group) local matrix (G*Nw*Ne*n*n
 * doubles, 22.5 GB for 64^3 cells, p = 1, S12) when that needs at most half of
 * the free device memory; later Mults apply the stored inverses instead of
 * factoring.  mode 0: never cache (frees the cache). */
int allium_sweep_set_factor_cache(allium_sweep* s, int mode);

/* Launch schedule of the sweep (no counterpart in the reference).
 * 0 (default): one launch per wavefront level (the reference's frontier
 * order), replayed as a CUDA graph.
 * 1: one persistent launch per sweep; each (cell, angle, group) waits on
 * completion flags of the upwind neighbours it reads, so later wavefronts
 * start while earlier ones drain (orders p <= 1).  Same results bit for bit. */
int allium_sweep_set_schedule(allium_sweep* s, int mode);

/* The same sweep with FP32 storage and FP32 local solves rebuilt every call (unpivoted
 * elimination; the local upwind matrix has a positive definite symmetric part
 * when sigma_t > 0).  Meant as the inner operator of an FP64 outer iteration. */
int allium_sweep_mult_f32(allium_sweep* s, const float* source, float* psi);

/* Threads per block (32, 64 or 128) of the thread-per-node level kernels of
 * the FP64 (precision 64) or FP32 (32) sweeps; the autotuner's knob (no
 * reference counterpart).  Default 128. */
int allium_sweep_set_block_size(allium_sweep* s, int precision, int threads);

/* Order of the FP32 copy of the stored inverses that the node-major FP32 sweep
 * reads: 0 each node-group's n x n block contiguous (float4 rows, default),
 * 1 entry-major like the FP64 store (one warp load = one entry of 32
 * node-groups).  A tuning knob with no reference counterpart; results do not
 * depend on it. */
int allium_sweep_set_f32_inverse_layout(allium_sweep* s, int entry_major);

/* Shape of the host-buffer pipeline of allium_sweep_mult (pinned host vectors,
 * stored inverses, inflow boundaries): the directions are cut into `chunks`
 * contiguous slices (2..32, at most half the directions), each copied in,
 * swept and copied out on its own, and the sweeps of consecutive slices
 * alternate over `streams` compute streams (1..4).  With taper t (0..3) the
 * first and last slices get 1/2^t of the others' share of directions, which
 * shortens the pipeline's fill and drain.  Default 8, 4, 0.  No reference
 * counterpart (the reference's vectors are host memory).  Results do not
 * depend on the shape. */
int allium_sweep_set_pipeline(allium_sweep* s, int chunks, int streams, int taper);

/* Negative-flux fixup inside the sweep (SetFixupOperator / UseFixup,
 * src/sweep.hpp:108-117, applied at src/sweep.cpp:465-470): kind 0 off,
 * 1 ZeroFixupOperator, 2 ZeroAndScaleFixupOperator (src/fixup.cpp:3-57),
 * 3 RyosukeFixupOperator (src/fixup.cpp:90-174), 4 LocalOptimizationFixupOperator
 * (src/fixup.cpp:59-88; the bound-constrained projection solved exactly instead of
 * by mfem::SLBQPOptimizer's iteration), with the operator's minimum_solution.
 * Where the reference aborts (Ryosuke with more than three positive entries) the
 * sweep returns ALLIUM_ERR_UNSUPPORTED.  Every order is supported.
 * While a fixup is on, Mult rebuilds and factors every local system. */
int allium_sweep_set_fixup(allium_sweep* s, int kind, double minimum);

/* Number of local solves the fixup changed (applied) or could not balance
 * (failed, Apply returned -1) since the last reset; reset != 0 zeroes them. */
int allium_sweep_fixup_counts(allium_sweep* s, long long* applied, long long* failed, int reset);

/* AdvectionOperator::Mult (src/sweep.cpp:1246-1387): y = L x, FP64. x != y. */
int allium_sweep_apply_L(allium_sweep* s, const double* x, double* y);

/* AdvectionOperator::ComputeBalance (src/sweep.cpp:1400-1462): absorption +
 * leakage of psi, written to *out (host or device double). */
int allium_sweep_balance(allium_sweep* s, const double* psi, double* out);

/* The balance of allium_sweep_balance for callers that cannot allocate GPU
 * memory at the time of the call: code running under its own memory pool or
 * in a time-step loop that must not allocate (an allocation there would
 * synchronise the device or break the caller's memory budget), and hosts that
 * hand the library only the vectors it works on.  No counterpart in the
 * reference.  It allocates nothing: psi must be device memory, *out may be
 * device or host memory (a host *out makes the call copy the result to the
 * host and wait for it).  Its partial sums
 * live in a fixed 32 KB array inside the library's device image, held by every
 * GPU that loads the library until the process exits, which limits it to
 * G*Nw*Ne <= 134217728 items (larger problems get ALLIUM_ERR_SIZE).  The first
 * call on each device looks the array up (cudaGetSymbolAddress) with that
 * device current: make it before any stream capture starts.  The address is
 * kept for the rest of the process, so the library assumes one CUDA context
 * per device for its lifetime (no cudaDeviceReset in between).  Calls share the
 * array, so calls whose kernels overlap on the GPU race; results match
 * allium_sweep_balance to rounding (the partial sums are grouped differently). */
int allium_sweep_balance_noalloc(allium_sweep* s, const double* psi, double* out);

/* DiscreteToMoment::Mult (src/transport_op.cpp:3-31); num_moments is 1 or dim+1. */
int allium_sweep_moments(allium_sweep* s, const double* psi, double* phi, int num_moments);

/* Copy a psi-sized FP64 device vector from one transport-vector layout to the
 * other (a tiled device transpose; in and out must not overlap).  Every other
 * entry point takes RIGHT vectors, so a caller built with the LEFT layout
 * converts at this boundary (src/tvector.hpp:47-51). */
int allium_sweep_relayout(allium_sweep* s, const double* in, int in_layout, double* out, int out_layout);

/* DiscreteToMoment::MultTranspose (accumulate = 0) and AddMultTranspose
 * (accumulate = 1, psi += alpha * D^T phi) (src/transport_op.cpp:33-89). */
int allium_sweep_moments_transpose(allium_sweep* s, const double* phi, double* psi,
                                   int num_moments, double alpha, int accumulate);

/* FormTransportSource (src/sweep.cpp:1135-1185) for an isotropic, piecewise
 * constant source density q_cell [G][Ne] (NULL = 0) and an isotropic inflow
 * inflow [G][num_attr] indexed by boundary attribute (NULL = vacuum). */
int allium_sweep_form_source(allium_sweep* s, const double* q_cell, const double* inflow,
                             int num_attr, double* source);

/* FormTransportSource for coefficients that vary inside a cell and with the
 * direction (src/sweep.cpp:1135-1185 with a FunctionCoefficient source and a
 * PhaseSpaceCoefficient inflow constant along each boundary attribute):
 * q_points the density at the P domain-rule points of every cell (their
 * coordinates from allium_sweep_source_points; NULL for none), [G][Ne][P], or
 * [G][Nw][Ne][P] per direction when q_per_direction is 1 (a PhaseSpaceCoefficient
 * source such as the manufactured solutions' of test/test_transport_mms.cpp);
 * inflow_angular [G][Nw][num_attr] the inflow psi of each direction per
 * boundary attribute (NULL for vacuum).  Integrated with the same rules as
 * allium_sweep_form_source, which it equals for constant data. */
int allium_sweep_form_source_general(allium_sweep* s, const double* q_points, int q_per_direction,
                                     const double* inflow_angular, int num_attr, double* source);

/* Points of the source's domain rule (DomainLFIntegrator, order 2p: p + 1
 * Gauss-Legendre points per axis): *points_per_cell = P and, when coords is
 * not NULL, their physical coordinates [Ne][P][dim] (host or device). */
int allium_sweep_source_points(allium_sweep* s, int* points_per_cell, double* coords);

/* Isotropic scattering source around the sweep: out = D^T (S phi) + q_fixed,
 * S = sigma_s [G][Ne] times the MassIntegrator matrix of each cell (within-group
 * scattering), as chive's source iteration and MomentMethodFixedPointOperator::Mult
 * build it (src/transport_op.hpp:75-90, exe/chive.cpp:593-599).  q_fixed may be
 * NULL.  phi is [G][Ndof] (zeroth moment). */
int allium_sweep_scattering_source(allium_sweep* s, const double* sigma_s, const double* phi,
                                   const double* q_fixed, double* out);

/* FP32 companions for the inner iterations of an FP64 outer solve (device
 * vectors only): zeroth moment of an FP32 psi accumulated in FP64, and the
 * scattering source D^T (S phi) + q_fixed computed in FP64 and stored in FP32
 * (q_fixed FP32 or NULL). */
int allium_sweep_moments_f32(allium_sweep* s, const float* psi, double* phi);
int allium_sweep_scattering_source_f32(allium_sweep* s, const double* sigma_s, const double* phi,
                                       const float* q_fixed, float* out);

/* Node-major FP32 companions for inner iterations the caller keeps on the GPU
 * (no counterpart in the reference; device vectors only).  The node-major
 * layout stores v[((e*Nw + a)*G + g)*n + i]: in a wavefront level the
 * consecutive angles of one cell, and their upwind traces, are contiguous.
 * Conversions to/from allium's RIGHT FP64 layout, the FP32 sweep (in place
 * allowed; local systems in FP32, unpivoted, or the FP32 copy of the stored
 * inverses; no negative-flux fixup: it is the linear inner operator of an
 * FP64 outer iteration, as allium switches the fixup off around its linear
 * solves, src/trt_linearized.cpp:237-239), the scattering source
 * D^T (S phi) + q (S phi in FP64) and the FP64-accumulated zeroth moment. */
int allium_sweep_to_node_layout_f32(allium_sweep* s, const double* psi_right, float* out_nodes);
int allium_sweep_from_node_layout_f32(allium_sweep* s, const float* in_nodes, double* psi_right);
int allium_sweep_mult_f32_nodes(allium_sweep* s, const float* source, float* psi);
int allium_sweep_scattering_source_f32_nodes(allium_sweep* s, const double* sigma_s, const double* phi,
                                             const float* q_nodes, float* out);
int allium_sweep_moments_f32_nodes(allium_sweep* s, const float* psi, double* phi);

/* ---- fused FP32 inner operator and the FP64-accurate transport residual ----
 * The pieces of an FP32-inner / FP64-outer solve that never needs an FP64
 * sweep (device vectors only; orders 0 and 1, inflow or vacuum boundaries,
 * else ALLIUM_ERR_UNSUPPORTED).  psi-sized vectors use the fused layout
 *     v[((g*Ne + e)*Nw + a)*n + i]
 * (group, cell, angle, DOF), equal to the node-major layout when G = 1; a
 * "double-float" vector is a pair of FP32 vectors hi, lo whose sum carries
 * about 48 bits (hi = fl32(x), lo = fl32(x - hi)). */

/* Per-cell isotropic source s[g][e n + i] = (sigma_s (M phi))/sum(w) + q_iso: the
 * D^T (S phi) + q of chive's source build (exe/chive.cpp:593-599,
 * MomentMethodFixedPointOperator::Mult, src/transport_op.hpp:75-90) for a source
 * q that is the same in every direction (FormTransportSource of an isotropic
 * density with vacuum boundaries), computed in FP64 and written as FP32 (out)
 * and/or double-float (out_hi, out_lo).  phi and q_iso are [G][Ndof] FP64 and
 * may each be NULL; sigma_s [G][Ne] (host or device) is required with phi the
 * first time, NULL reuses the last one given. */
int allium_sweep_isotropic_source(allium_sweep* s, const double* sigma_s, const double* phi, const double* q_iso,
                                  float* out, float* out_hi, float* out_lo);

/* The inner operator phi = D L^{-1} (iso + source) as one CUDA graph:
 * InverseAdvectionOperator::Mult (src/sweep.cpp:277-669) in FP32, one launch per
 * wavefront level, with the isotropic source read per cell (iso [G][Ndof], or
 * NULL) plus an optional psi-sized FP32 source, followed by
 * DiscreteToMoment::Mult (src/transport_op.cpp:3-31) of the FP32 psi summed in
 * double-float arithmetic: phi_mode 0 leaves phi alone, 1 writes phi = D psi,
 * 2 adds D psi to phi (FP64); 3 writes phi = D psi summed in plain FP32 (about
 * 1e-6 relative, for the inner operator of a Krylov solve).  psi receives the FP32 angular flux;
 * psi_hi/psi_lo (or NULL) is a double-float vector that psi is added to.
 * source may equal psi. */
int allium_sweep_fused_mult_f32(allium_sweep* s, const float* iso, const float* source, float* psi, double* phi,
                                int phi_mode, float* psi_hi, float* psi_lo);

/* Wavefront levels of the fused sweep (no reference counterpart; the reference
 * sweeps node frontiers, src/sweep.cpp:308-322).  The fused sweep orders whole
 * units -- a cell's angles with the same octant and face pattern, which read
 * their upwind traces across the same faces -- by Kahn frontiers of the unit
 * graph, so all of a unit's angles share a level (unit_levels = 1); if that
 * graph has a cycle it keeps the node levels (unit_levels = 0).  Either order
 * sweeps every node after its upwind nodes. */
int allium_sweep_fused_levels(allium_sweep* s, int* num_levels, int* unit_levels);

/* Launch overlap of the fused sweep's level launches (no reference
 * counterpart): 1 (default) lets each level's blocks start while the previous
 * level drains (programmatic dependent launch; they load their records, unit
 * tables and sources, then wait before reading upwind traces), 0 plain
 * stream order.  Results do not depend on it. */
int allium_sweep_set_fused_pdl(allium_sweep* s, int on);

/* The same for the FP64 (and RIGHT-layout FP32) sweep from stored local
 * inverses on device vectors (no reference counterpart): 1 (default) lets each
 * level's blocks read their node records and face data while the previous
 * level drains, 0 plain stream order.  Results do not depend on it. */
int allium_sweep_set_level_pdl(allium_sweep* s, int on);

/* r = q + D^T S phi - L psi for a double-float psi: AdvectionOperator::Mult
 * (src/sweep.cpp:1246-1387) subtracted from the source, evaluated in
 * double-float arithmetic on the FP32 units (error-free products and sums, about
 * 1e-14 of |q|), written as FP32 r.  iso_hi/iso_lo is the per-cell part
 * (allium_sweep_isotropic_source of phi and q_iso), q_hi/q_lo an optional
 * psi-sized part of q. */
int allium_sweep_transport_residual_df(allium_sweep* s, const float* iso_hi, const float* iso_lo, const float* q_hi,
                                       const float* q_lo, const float* psi_hi, const float* psi_lo, float* r);

/* The residual of psi + dpsi from the residual r of psi, in FP32:
 * r += iso - L dpsi (AdvectionOperator::Mult, src/sweep.cpp:1246-1387, of the
 * correction; iso [G][Ndof] is the per-cell (S D dpsi)/sum(w) from
 * allium_sweep_isotropic_source).  Its rounding is about 1e-7 of |L dpsi|, so
 * it keeps r accurate while dpsi is small against psi; fused-layout FP32
 * vectors. */
int allium_sweep_transport_residual_update_f32(allium_sweep* s, const float* iso, const float* dpsi, float* r);

/* DiscreteToMoment::Mult (src/transport_op.cpp:3-31) of a double-float psi in the
 * fused layout, summed in double-float arithmetic: phi[G][Ndof] (FP64) to about
 * 1e-14 of sum_a w_a |psi_a|. */
int allium_sweep_moments_df(allium_sweep* s, const float* psi_hi, const float* psi_lo, double* phi);

/* RIGHT FP64 <-> fused-layout double-float (lo may be NULL: FP32 only) */
int allium_sweep_to_fused_layout(allium_sweep* s, const double* psi_right, float* hi, float* lo);
int allium_sweep_from_fused_layout(allium_sweep* s, const float* hi, const float* lo, double* psi_right);

/* Wavefront level of every (cell, angle) node e*Nw + a (the Kahn frontier
 * index of src/sweep.cpp:308-512), host or device int array [Ne*Nw]. */
int allium_sweep_levels(allium_sweep* s, int* levels);

/* Failure-detection self test (no counterpart in the reference): runs the
 * sweep's bounded device wait on a completion flag that nothing sets, with
 * poll_limit polls (1..2^20); the wait gives up and the call returns
 * ALLIUM_ERR_TIMEOUT with the device still usable. */
int allium_sweep_selftest_wait(allium_sweep* s, int poll_limit);

/* ---- thermal radiative transfer operators around the sweep ----
 * The operators LinearizedTRTOperator::Mult (src/trt_linearized.cpp:230-312)
 * applies between sweeps.  Temperature T is a DG field on the sweep's
 * elements (Ndof entries, same local DOF order as psi); moment vectors are
 * [G][Ndof] (the moment layout with one moment); sigma_abs is the absorption
 * opacity [G][Ne], piecewise constant per cell (sigma_fe_order = 0); ac is the
 * "StefanBoltzmann" constant of src/constants.hpp (a c).  Vectors are device
 * memory; bounds[G + 1] and nu[G] may be host or device.  At most 16 DOFs per
 * cell and no lumping (ALLIUM_ERR_UNSUPPORTED otherwise). */

/* EvalPlanckSpectrum (kind 0) / EvalRosselandSpectrum (kind 1)
 * (src/planck.hpp:157-236): group fractions of the normalised spectrum at
 * temperature T; host arrays, no handle. */
int allium_planck_spectrum(const double* bounds, int num_groups, double T, int kind, double* out);

/* PlanckEmissionNonlinearForm::Mult and ::GetGradient with PlanckEmissionNFI
 * (src/trt_integrators.cpp:56-152, 229-302): emission[g][i] =
 * int sigma_g ac T^4 b_g(T) phi_i, grad[g][e][i][j] = int sigma_g 4 ac T^3
 * r_g(T) phi_i phi_j (row major blocks).  Either output may be NULL. */
int allium_sweep_planck_emission(allium_sweep* s, const double* bounds, const double* sigma_abs, const double* T,
                                 double ac, double* emission, double* grad);

/* The energy-balance form meb_form of exe/scallion.cpp:755-765
 * (GrayPlanckEmissionNFI, src/trt_integrators.cpp:154-208, plus
 * MassIntegrator(c_v/dt)): residual[i] = int sum_g sigma_g b_g ac T^4 phi_i +
 * cv_dt (M T)_i and grad_inv[e] = the inverse of its gradient block
 * (DenseBlockDiagonalSolver over DenseMatrixInverse).  A singular block gives
 * ALLIUM_ERR_SINGULAR. */
int allium_sweep_energy_balance(allium_sweep* s, const double* bounds, const double* sigma_abs, const double* T,
                                double ac, double cv_dt, double* residual, double* grad_inv);

/* Block-diagonal product y_b = alpha B_b x_b (+ y_b when accumulate) for
 * num_sets block sets B[num_sets][Ne][n][n]; x_shared: x is one [Ndof] vector
 * for every set (the gradient of the emission applied to a temperature).
 * blocks == NULL uses the handle's mass matrices: num_sets 1 the unit sigma
 * mass (MGMassIntegrator rule), 2 the MassIntegrator mass (time absorption,
 * heat capacity). */
int allium_sweep_block_apply(allium_sweep* s, const double* blocks, int num_sets, const double* x, int x_shared,
                             double* y, double alpha, int accumulate);

/* y = alpha sum_g M_{sigma_g} phi_g (+ y): Mtot_collapse of
 * exe/scallion.cpp:786-797 (MGMassIntegrator(total) summed over groups). */
int allium_sweep_absorption(allium_sweep* s, const double* sigma_abs, const double* phi, double* y, double alpha,
                            int accumulate);

/* out = q + tau M psi_prev per (group, angle, cell) block: SNTimeMassMatrix::Mult
 * (src/tvector.cpp:76-95) and the backward-Euler source of
 * exe/scallion.cpp:1358-1359 (tau = 1/(c dt)).  q may be NULL; out may alias
 * psi_prev or q. */
int allium_sweep_time_source(allium_sweep* s, const double* psi_prev, const double* q, double tau, double* out);

/* sigma_out[g][e] = C nu_g^a T_c^b, T_c the temperature at the cell centre:
 * an analytic opacity (src/opacity.cpp:47-63) at the group midpoints nu_g,
 * projected onto piecewise constants (OpacityCoefficient::Project with
 * sigma_fe_order = 0). */
int allium_sweep_powerlaw_opacity(allium_sweep* s, const double* T, const double* nu, double C, double a, double b,
                                  double* sigma_out);

/* ---- diffusion synthetic acceleration ----
 * The MIP diffusion operator K of InteriorPenaltyDiscretization::GetOperator
 * (src/moment_discretization.cpp:73-110, "scalar mip" in exe/chive.cpp:663-672):
 * DiffusionIntegrator(1/(3 sigma_t)) + MassIntegrator(sigma_t - sigma_s) +
 * MIPDiffusionIntegrator (src/moment_integrators.cpp:3-200; sigma = -1,
 * penalty max(kappa {D/h}, penalty_min)) on interior faces +
 * BoundaryMassIntegrator(alpha_bdr) on inflow boundaries (+ tau M), one
 * operator per group on the handle's sigma_t.  Negative kappa, penalty_min or
 * alpha_bdr select the reference defaults (p+1)^2, ComputeAlpha(quad, e_x)/2
 * and 0.5.  sigma_s is [G][Ne] (host or device).  At most 16 DOFs per cell,
 * no lumping. */
int allium_sweep_dsa_setup(allium_sweep* s, const double* sigma_s, double kappa, double penalty_min, double alpha_bdr,
                           double tau);

/* y = K x on [G][Ndof] device vectors (the HypreParMatrix product). */
int allium_sweep_dsa_apply(allium_sweep* s, const double* x, double* y);

/* y = (block diagonal of K)^{-1} x: the block-Jacobi preconditioner of the
 * diffusion solve (no reference counterpart: allium uses BoomerAMG). */
int allium_sweep_dsa_jacobi(allium_sweep* s, const double* x, double* y);

/* y = alpha A x + beta y for a CSR matrix on the device (row pointers,
 * column indices, values): the coarse levels of the diffusion
 * preconditioner.  stream is a cudaStream_t (NULL: default stream). */
int allium_csr_spmv(int n, const int* rowptr, const int* col, const double* val, const double* x, double* y,
                    double alpha, double beta, void* stream);

/* Greedy pairwise aggregation of a CSR matrix on the host (coarsening of the
 * diffusion preconditioner): agg[i] = aggregate of row i; returns the number
 * of aggregates (-1 on bad arguments). */
int allium_pair_aggregates(int n, const int* rowptr, const int* col, const double* val, int* agg);

/* Neighbour element across each local face, [Ne][2 dim] host ints, -1 on the
 * boundary (the element-to-face table of src/sweep.cpp:123-135, resolved). */
int allium_sweep_neighbours(allium_sweep* s, int* out);

/* Copy K's blocks [G][Ne][1 + 2 dim][n][n] (self block, then the coupling to
 * the neighbour across each local face) to out (host or device). */
int allium_sweep_dsa_blocks(allium_sweep* s, double* out);

/* ---- learned initial iterate: per-cell MLP kernels (no reference counterpart) ----
 * A small network predicts the next time step's moments from the current
 * state; it only supplies the initial iterate of the outer solve, which still
 * converges to the same tolerance.  Device pointers; stream is a cudaStream_t
 * (NULL: the default stream).  BF16 operands (__nv_bfloat16 / torch.bfloat16),
 * FP32 accumulation and outputs. */

/* C[M][N] = alpha A B (+ beta C) (+ bias[N]) (ReLU if relu): A(m, k) at
 * A[m sam + k sak], B(k, n) at B[k sbk + n sbn] (strides in elements, so
 * transposed operands need no copy); C row stride ldc; C_bf16 receives a BF16
 * copy when not NULL.  mma.sync m16n8k16 tensor-core tiles of 64 x 64. */
int allium_mlp_gemm(int M, int N, int K, const void* A, long long sam, long long sak, const void* B, long long sbk,
                    long long sbn, float* C, long long ldc, void* C_bf16, const float* bias, float alpha, float beta,
                    int relu, void* stream);

/* C[M][N] = alpha A[M][K] B[N][K]^T (+ beta C) (+ bias[N]) (ReLU) on the
 * fifth-generation tensor cores (tcgen05.mma, FP32 accumulator in tensor
 * memory, operands streamed by cp.async.bulk.tensor).  A and B are BF16 with K
 * contiguous; their row strides lda, ldb are multiples of 8 elements and their
 * base addresses 16-byte aligned (ALLIUM_ERR_ARG otherwise).  C row stride
 * ldc, C_bf16 (row stride ldcb) receives a BF16 copy when not NULL.  ksplit > 1
 * splits K over that many tiles' worth of blocks and adds the partial sums into
 * C, which the call zeroes first (C only: no bias, ReLU, beta or BF16 copy). */
int allium_mlp_gemm_tc(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb, float* C,
                       long long ldc, void* C_bf16, long long ldcb, const float* bias, float alpha, float beta, int relu,
                       int ksplit, void* stream);

/* out[c][r] = in[r][c] for a rows x cols BF16 matrix (row strides ldi, ldo). */
int allium_mlp_transpose_bf16(int rows, int cols, const void* in, long long ldi, void* out, long long ldo, void* stream);

/* Synchronizes the stream; ALLIUM_ERR_TIMEOUT (and the word cleared) if a
 * bounded wait inside allium_mlp_gemm_tc gave up since the last call.  The
 * word is one per process and device, shared by every stream and thread. */
int allium_mlp_status(void* stream);

/* dz = dy where y > 0, else 0 (ReLU gradient); dz and/or its BF16 copy. */
int allium_mlp_relu_backward(long long count, const float* dy, const float* y, float* dz, void* dz_bf16, void* stream);

/* db[n] = sum_m dy[m][n]. */
int allium_mlp_bias_grad(int M, int N, const float* dy, float* db, void* stream);

/* dy = 2 (y - target) / count; loss_partials[ceil(count / 256)] receive the
 * blocks' sums of squared errors. */
int allium_mlp_mse_grad(long long count, const float* y, const float* target, float* dy, float* loss_partials,
                        void* stream);

/* One Adam step (step >= 1) on FP32 weights w with moments m, v; refreshes
 * the BF16 copy w_bf16 when not NULL. */
int allium_mlp_adam(long long count, float* w, void* w_bf16, const float* grad, float* m, float* v, float lr,
                    float beta1, float beta2, float eps, int step, void* stream);

/* y = bf16(x). */
int allium_mlp_to_bf16(long long count, const float* x, void* y, void* stream);

/* FP64 multiply-add throughput probe (no reference counterpart): blocks x
 * threads threads each run 8 independent FMA chains for iters steps on the
 * given cudaStream_t (2 * 8 * iters flops per thread); the caller times it.
 * sink is a device buffer of blocks * threads doubles that is written only if
 * the chains reach an impossible value.  The measured rate is the bound of
 * the FP64 sweep, whose work is multiply-adds. */
int allium_fp64_fma_probe(int blocks, int threads, long long iters, double* sink, void* stream);

/* Wait for the handle's stream; report sticky kernel errors and clear them. */
int allium_sweep_synchronize(allium_sweep* s);

const char* allium_sweep_last_error(const allium_sweep* s);
const char* allium_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif /* ALLIUM_SWEEP_H */
