// Internal state of one sweep handle and the kernel launchers shared by the
// translation units of liballium_sweep.so.  Nothing here is part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <mutex>
#include <vector>

#include "../../include/allium_sweep.h"

namespace allium {

struct FusedState;   // fused FP32 sweep and double-float residual (fused.cu)

constexpr int kMaxOrder = 3;
constexpr int kMaxRule = 5;   // largest 1D rule used (p + 2 points, p <= 3)

// Reference-element tables, passed to kernels by value.
struct RefTables {
    int dim, p, n1, n, nf, nface;
    double nodes[kMaxOrder + 1];          // Gauss-Lobatto basis nodes on [0,1]
    // 1D rules: 0 = sigma mass, 1 = convection, 2 = time mass, 3 = face mass,
    //           4 = source domain, 5 = source boundary, 6 = Planck emission
    //           (order 2p + 1), 7 = gray emission (order 2p + 2)
    //           8 = diffusion stiffness (order 2p + dim - 1)
    int rn[9];
    double rx[9][kMaxRule], rw[9][kMaxRule];
};

// Per (cell, local face) topology.  nbr >= 0: interior face; nbr = -1:
// inflow/vacuum boundary; nbr = -2 - c: reflective boundary face number c.
// side = 0 when the cell is the face's element 1 (lower index).
struct Slot {
    int face, nbr, side, attr;
};

// How the neighbour across a face sees it: its local face k2 and the map of
// this cell's face coordinates t in [0,1]^(dim-1) to the neighbour's,
// s_j = b_j + sum_c c[j][c] t_c.
struct FaceOrient {
    int8_t k2, b0, b1, c00, c01, c10, c11, pad;
};

struct Handle {
    // problem description
    int dim = 0, p = 0, n = 0, nf = 0, nface = 0, ne = 0, Nw = 0, G = 0, lump = 0;
    int nfaces = 0;
    long long ndof = 0, psi_size = 0;
    RefTables ref{};
    bool time_dependent = false;
    bool have_mass2 = false;         // d_Mt assembled (time absorption or scattering)
    double tau = 0.0;
    double wsum = 0.0;
    std::vector<double> h_omega, h_weights;
    std::vector<int> h_level_offsets;   // [num_levels + 1]
    int num_levels = 0;

    // device buffers
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    double *d_omega = nullptr, *d_weights = nullptr, *d_corners = nullptr, *d_normals = nullptr;
    // Omega_a . n_f for every face and angle, [nfaces][Nw] (n_f out of element 1);
    // the single source of every upwind decision (graph, levels, sweep, L)
    double* d_dots = nullptr;
    float* f_dots = nullptr;         // FP32 copy with the sign of the FP64 value
    Slot* d_slots = nullptr;
    int* d_face_e1k1 = nullptr;      // [nfaces][2]
    uint8_t* d_nbrmap = nullptr;
    FaceOrient* d_orient = nullptr;   // [ne][2 dim]
    // angle chunks of the host-buffer Mult (copy / sweep / copy pipeline):
    // nodes of chunk c in (level, face pattern, cell, angle) order, their positions in the
    // full level order, offsets [nchunk][num_levels + 1]; copy streams,
    // compute streams (comp[0] unused: h.stream) and events.  pipe_chunks
    // and pipe_streams are the requested chunk count and compute streams.
    static constexpr int kMaxPipeChunks = 32;
    static constexpr int kMaxPipeStreams = 4;
    int pipe_chunks = 8;
    int pipe_streams = 4;
    int pipe_taper = 0;
    int nchunk = 0;
    int chunk_taper = 0;
    std::vector<int> h_chunk_angle;   // [nchunk + 1] first angle of each chunk
    int* d_chunk_nodes = nullptr;
    int* d_chunk_pos = nullptr;
    std::vector<int> h_chunk_offsets;
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaStream_t comp[kMaxPipeStreams] = {};
    std::vector<cudaEvent_t> chunk_events;   // [3 * nchunk + 1]

    // threads per block of the thread-per-node level kernels (FP64, FP32)
    int block64 = 128, block32 = 128;
    int pdl_levels = 1;   // programmatic dependent launch between stored-inverse level launches
    double *d_G = nullptr, *d_M = nullptr, *d_Mt = nullptr, *d_F = nullptr, *d_sigma = nullptr;
    float *f_G = nullptr, *f_M = nullptr, *f_Mt = nullptr, *f_F = nullptr, *f_sigma = nullptr;
    int* d_level = nullptr;          // [ne*Nw]
    int* d_level_nodes = nullptr;    // [ne*Nw] sorted by (level, node)
    int* d_status = nullptr;         // sticky kernel error bits
    double* d_stage = nullptr;       // psi-sized staging buffer for host pointers
    float* f_stage = nullptr;
    double* d_scratch = nullptr;     // reduction partials
    size_t scratch_len = 0;
    double* d_sigma_s = nullptr;     // last scattering cross sections uploaded [G][Ne]
    bool fp32_ready = false;
    // FP64 factor cache: inverse of every local matrix, entry-major over the
    // level-sorted node-group order (allocated on the first FP64 Mult when it fits)
    int factor_cache = 1;            // 0 off, 1 automatic
    double* d_inv = nullptr;
    bool inv_valid = false;
    // FP32 copy of the stored inverses for the node-major FP32 sweep, one
    // contiguous n x n block per (level-order node, group)
    float* f_inv_nodes = nullptr;
    bool f_inv_valid = false;
    bool f_inv_failed = false;        // the copy did not fit: recompute instead
    int f_inv_entry_major = 0;        // 1: entry (i, j) of node-group t at [(i n + j) * total + t]

    // CUDA graphs of the per-level launch sequence, keyed by kind and vectors
    struct GraphEntry {
        int kind = -1;
        const void* src = nullptr;
        void* dst = nullptr;
        cudaGraphExec_t exec = nullptr;
    };
    static constexpr int kGraphSlots = 48;
    GraphEntry graphs[kGraphSlots];
    int graph_next = 0;
    cudaStream_t capture_stream = nullptr;
    bool use_graphs = true;

    // reflective boundaries: reflected angle of each angle at reflective face c
    int nrefl = 0;
    int* d_refl = nullptr;           // [nrefl][Nw] reflected angle feeding each entering angle
    int* d_feed = nullptr;           // [nrefl][Nw] entering angle fed by each angle

    // MIP diffusion (DSA) operator: blocks [G][Ne][1 + 2 dim][n][n] (self,
    // then the neighbour across each local face) and inverted self blocks
    double* d_dsa = nullptr;
    double* d_dsa_inv = nullptr;
    bool dsa_ready = false;

    // thermal radiative transfer inputs (group bounds, group midpoints)
    double* d_bounds = nullptr;      // [G + 1]
    double* d_nu = nullptr;          // [G]

    // negative-flux fixup
    int fix_kind = 0;
    double fix_min = 0.0;
    unsigned long long* d_fix_counts = nullptr;

    // dataflow schedule (one persistent launch per sweep)
    int schedule = 0;                // 0: one launch per wavefront level, 1: dataflow
    unsigned* d_flags = nullptr;     // [ne * Nw * G]
    unsigned* d_flow_words = nullptr;   // [0] epoch, [1] tile counter
    int* d_tile_start = nullptr;
    int* d_tile_count = nullptr;
    int ntiles = 0;

    // fused FP32 inner sweep and double-float residual (fused.cu), built on first use
    FusedState* fused = nullptr;

    std::string last_error;
};

void drop_fused_graphs(Handle& h);

// Launch `body(stream)` through a cached CUDA graph keyed by (kind, src, dst):
// captured once on a private stream, replayed on h.stream afterwards.
template <typename Body>
cudaError_t run_graph_on(Handle& h, int kind, const void* src, void* dst, cudaStream_t stream, Body&& body) {
    if (!h.use_graphs) return body(stream);
    for (auto& g : h.graphs)
        if (g.exec && g.kind == kind && g.src == src && g.dst == dst) return cudaGraphLaunch(g.exec, stream);
    cudaError_t e = cudaSuccess;
    if (!h.capture_stream) {
        e = cudaStreamCreateWithFlags(&h.capture_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
    }
    e = cudaStreamBeginCapture(h.capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cudaError_t be = body(h.capture_stream);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(h.capture_stream, &graph);
    if (be != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return be; }
    if (e != cudaSuccess) return e;
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return e;
    auto& slot = h.graphs[h.graph_next];
    h.graph_next = (h.graph_next + 1) % Handle::kGraphSlots;
    if (slot.exec) cudaGraphExecDestroy(slot.exec);
    slot.kind = kind; slot.src = src; slot.dst = dst; slot.exec = exec;
    return cudaGraphLaunch(exec, stream);
}

template <typename Body>
cudaError_t run_graph(Handle& h, int kind, const void* src, void* dst, Body&& body) {
    return run_graph_on(h, kind, src, dst, h.stream, body);
}

inline void drop_graphs(Handle& h) {
    for (auto& g : h.graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = Handle::GraphEntry{};
    }
    drop_fused_graphs(h);
}

// process-wide lock around the optional caches' "fits in half the free
// memory" decisions (the FP64 factor cache and its FP32 copy)
std::mutex& cache_lock();

// kernel error bits (d_status)
constexpr int kErrSingular = 1;
constexpr int kErrNaN = 2;
constexpr int kErrTimeout = 4;
constexpr int kErrFixup = 8;     // Ryosuke fixup with more than three positive entries
constexpr int kErrSchedule = 16; // a fused-sweep warp holds more cells than its table slots
// node-groups per tile of the dataflow schedule (= threads per block)
constexpr int kTile = 128;

// ---- topology (topology.cpp, host)
struct Topology {
    int nfaces = 0;
    std::vector<int> face_e1k1;       // [nfaces][2]
    std::vector<Slot> slots;          // [ne][2 dim]
    std::vector<uint8_t> nbrmap;      // [ne][2 dim][nf]
    std::vector<double> corners;      // [ne][2^dim][dim], corner order c = c0 + 2 c1 + 4 c2
    std::vector<int> refl_faces;      // face id of reflective boundary face c
    std::vector<FaceOrient> orient;   // [ne][2 dim], interior slots only
};
int build_topology(const allium_mesh_desc& m, int p, Topology& out, std::string& err);
void mark_reflective(Topology& t, int nface, const std::vector<int>& refl_attrs);

// ---- setup kernels (setup.cu)
cudaError_t launch_face_normals(Handle& h);
cudaError_t launch_face_dots(Handle& h);
cudaError_t launch_assemble(Handle& h);
int compute_reflections(Handle& h, const std::vector<int>& refl_faces);   // allium status
cudaError_t launch_relayout(Handle& h, const double* in, double* out, int to_left);
std::vector<int> chunk_bounds(int Nw, int nchunk, int taper);
int build_chunks(Handle& h, int nchunk, int taper);                                     // allium status
cudaError_t launch_sweep_chunk(Handle& h, double* stage, int c, cudaStream_t stream);

// thermal radiative transfer operators (trt.cu)
bool trt_supported(const Handle& h);
cudaError_t launch_trt_emission(Handle& h, const double* bounds, const double* sigma, const double* T, double K,
                                double cv_dt, double* emission, double* dB, double* bt, double* bt_inv);
cudaError_t launch_block_apply(Handle& h, const double* B, int nb, const double* x, long long x_stride, double* y,
                               double alpha, int accumulate);
cudaError_t launch_absorption(Handle& h, const double* sigma, const double* phi, double* y, double alpha, int accumulate);
cudaError_t launch_time_source(Handle& h, const double* psi_prev, const double* q, double tau, double* out);
cudaError_t launch_powerlaw_opacity(Handle& h, const double* T, const double* nu, double C, double a, double b,
                                    double* sigma);

// MIP diffusion operator for DSA (dsa.cu)
bool dsa_supported(const Handle& h);
cudaError_t launch_dsa_assemble(Handle& h, const double* sigma_s, double kappa, double penalty_min, double alpha_bdr,
                                double tau);
cudaError_t launch_dsa_apply(Handle& h, const double* x, double* y);
cudaError_t launch_time_mass(Handle& h);
int compute_levels(Handle& h);   // returns an allium status
cudaError_t launch_form_source(Handle& h, const double* q_cell, const double* q_points, int q_dir, const double* inflow,
                               int nattr, int angular, double* out);
int source_points_per_cell(const Handle& h);
cudaError_t launch_source_points(Handle& h, double* out);
cudaError_t launch_moments(Handle& h, const double* psi, double* phi, int nmom);
cudaError_t launch_moments_transpose(Handle& h, const double* phi, double* psi, int nmom, double alpha, int add);
cudaError_t launch_balance(Handle& h, const double* psi, double* partial, int nblocks_max, int* nblocks);
cudaError_t launch_balance_finish(Handle& h, const double* partial, int nparts, double* out);
cudaError_t launch_scatter_source(Handle& h, const double* sigma_s, const double* phi, const double* qfix, double* out);
cudaError_t launch_moments_f32(Handle& h, const float* psi, double* phi);
cudaError_t launch_scatter_source_f32(Handle& h, const double* sigma_s, const double* phi, const float* qfix, float* out);
cudaError_t make_fp32_copies(Handle& h);
RefTables make_ref_tables(int dim, int p, int lump);

// ---- hot kernels (sweep_fp64.cu, sweep_fp32.cu)
cudaError_t launch_sweep_fp64(Handle& h, const double* src, double* psi);
cudaError_t launch_sweep_fp32(Handle& h, const float* src, float* psi);
cudaError_t launch_apply_L_fp64(Handle& h, const double* x, double* y);
cudaError_t launch_sweep_nodes_f32(Handle& h, const float* src, float* psi);
cudaError_t prepare_flow(Handle& h);
cudaError_t launch_wait_probe(Handle& h, int limit);
cudaError_t launch_layout(Handle& h, int to_nodes, const void* in, void* out);
cudaError_t launch_scatter_nodes(Handle& h, const double* sigma_s, const double* phi, const float* qn, float* out);
cudaError_t launch_moments_nodes(Handle& h, const float* psi, double* phi);
bool factor_cache_supported(const Handle& h);
cudaError_t ensure_factors(Handle& h);

// ---- fused FP32 inner sweep, isotropic source, double-float residual (fused.cu)
// psi-sized vectors in the fused layout v[((g Ne + e) Nw + a) n + i]
bool fused_supported(const Handle& h);
void free_fused(Handle& h);
void set_fused_pdl(Handle& h, int on);
cudaError_t fused_levels(Handle& h, int* num_levels, int* unit_levels);
cudaError_t launch_fused_sweep(Handle& h, const float* iso, const float* src, float* psi, double* phi, int phi_mode,
                               float* acc_hi, float* acc_lo);
cudaError_t launch_iso_source(Handle& h, const double* sigma_s, const double* phi, const double* q_iso, float* out,
                              float* out_hi, float* out_lo);
cudaError_t launch_residual_df(Handle& h, const float* iso_hi, const float* iso_lo, const float* q_hi, const float* q_lo,
                               const float* psi_hi, const float* psi_lo, float* r);
cudaError_t launch_moments_df(Handle& h, const float* hi, const float* lo, double* phi);
cudaError_t launch_residual_update_f32(Handle& h, const float* iso, const float* x, float* r);
cudaError_t launch_fused_layout(Handle& h, int to_fused, const double* right, float* hi, float* lo);

}  // namespace allium

// the opaque handle behind the C ABI
struct allium_sweep {
    allium::Handle h;
};
