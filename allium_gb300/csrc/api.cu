// C ABI of liballium_sweep.so (declared in include/allium_sweep.h).
#include <cmath>
#include <cstdint>
#include <initializer_list>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"
#include "planck.cuh"

using allium::Handle;

namespace {

// cudaErrorNotSupported from the library's own launchers means an unsupported
// option or shape (no kernel was launched), the rest a CUDA failure
#define CUDA_OR_FAIL(h, x)                                   \
    do {                                                     \
        cudaError_t _e = (x);                                \
        if (_e != cudaSuccess) {                             \
            (h).last_error = std::string(#x) + ": " + cudaGetErrorString(_e); \
            if (_e == cudaErrorNotSupported) return ALLIUM_ERR_UNSUPPORTED; \
            return ALLIUM_ERR_CUDA;                          \
        }                                                    \
    } while (0)

bool on_device(const void* p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

template <typename T>
cudaError_t ensure(T** buf, size_t count) {
    if (*buf) return cudaSuccess;
    return cudaMalloc(buf, count * sizeof(T));
}

// device copy of a small input array (host or device pointer)
template <typename T>
int upload(Handle& h, const T* src, size_t count, T** dst) {
    CUDA_OR_FAIL(h, ensure(dst, count));
    CUDA_OR_FAIL(h, cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyDefault, h.stream));
    return ALLIUM_OK;
}

int check_status(Handle& h) {
    int st = 0;
    CUDA_OR_FAIL(h, cudaMemcpyAsync(&st, h.d_status, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    if (st) {
        CUDA_OR_FAIL(h, cudaMemsetAsync(h.d_status, 0, sizeof(int), h.stream));
        if (st & allium::kErrSingular) { h.last_error = "zero pivot in a local solve"; return ALLIUM_ERR_SINGULAR; }
        if (st & allium::kErrTimeout) { h.last_error = "a bounded device wait gave up"; return ALLIUM_ERR_TIMEOUT; }
        if (st & allium::kErrSchedule) {
            h.last_error = "a warp of the fused schedule holds more cells than its table slots";
            return ALLIUM_ERR_UNSUPPORTED;
        }
        if (st & allium::kErrFixup) {
            h.last_error = "Ryosuke fixup with more than three positive entries (src/fixup.cpp:155 aborts)";
            return ALLIUM_ERR_UNSUPPORTED;
        }
        h.last_error = "non-finite value";
        return ALLIUM_ERR_NAN;
    }
    return ALLIUM_OK;
}

void free_all(Handle& h) {
    allium::drop_graphs(h);
    allium::free_fused(h);
    if (h.capture_stream) cudaStreamDestroy(h.capture_stream);
    for (cudaEvent_t ev : h.chunk_events)
        if (ev) cudaEventDestroy(ev);
    for (cudaStream_t st : {h.copy_in, h.copy_out, h.comp[1], h.comp[2], h.comp[3]})
        if (st) cudaStreamDestroy(st);
    void* bufs[] = {h.d_omega, h.d_weights, h.d_corners, h.d_normals, h.d_dots, h.f_dots, h.d_slots, h.d_face_e1k1, h.d_nbrmap,
                    h.d_G, h.d_M, h.d_Mt, h.d_F, h.d_sigma, h.f_G, h.f_M, h.f_Mt, h.f_F, h.f_sigma,
                    h.d_level, h.d_level_nodes, h.d_status, h.d_stage, h.f_stage, h.d_scratch, h.d_inv,
                    h.d_sigma_s, h.d_flags, h.d_flow_words, h.d_tile_start, h.d_tile_count, h.d_fix_counts,
                    h.d_refl, h.d_feed, h.d_bounds, h.d_nu, h.d_orient, h.d_dsa, h.d_dsa_inv,
                    h.d_chunk_nodes, h.d_chunk_pos, h.f_inv_nodes};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (h.own_stream && h.stream) cudaStreamDestroy(h.stream);
}

int refresh_fp32(Handle& h) {
    if (!h.fp32_ready) return ALLIUM_OK;
    CUDA_OR_FAIL(h, allium::make_fp32_copies(h));
    return ALLIUM_OK;
}

}  // namespace

extern "C" {

const char* allium_status_string(int s) {
    switch (s) {
        case ALLIUM_OK: return "ok";
        case ALLIUM_ERR_ARG: return "invalid argument";
        case ALLIUM_ERR_NOT_DAG: return "upwind graph is not a DAG";
        case ALLIUM_ERR_SIZE: return "size mismatch";
        case ALLIUM_ERR_TIMEOUT: return "device wait timed out";
        case ALLIUM_ERR_NAN: return "non-finite value";
        case ALLIUM_ERR_CUDA: return "CUDA error";
        case ALLIUM_ERR_UNSUPPORTED: return "unsupported option";
        case ALLIUM_ERR_MESH: return "malformed mesh";
        case ALLIUM_ERR_SINGULAR: return "singular local system";
        default: return "unknown status";
    }
}

const char* allium_sweep_last_error(const allium_sweep* s) { return s ? s->h.last_error.c_str() : "null handle"; }

int allium_sweep_create(const allium_mesh_desc* mesh, const allium_fe_desc* fe, const allium_quad_desc* quad,
                        int num_groups, const double* sigma_t, const allium_bc_desc* bc, allium_sweep** out) {
    if (!out) return ALLIUM_ERR_ARG;
    *out = nullptr;
    if (!mesh || !fe || !quad || !sigma_t || num_groups < 1) return ALLIUM_ERR_ARG;
    if (mesh->dim < 1 || mesh->dim > 3 || quad->dim != mesh->dim || mesh->num_elements < 1 ||
        !mesh->vertices || !mesh->element_vertices || quad->num_angles < 1 || !quad->omega || !quad->weights)
        return ALLIUM_ERR_ARG;
    if (fe->order < 0 || fe->order > allium::kMaxOrder || fe->basis != ALLIUM_BASIS_GAUSS_LOBATTO ||
        fe->lump < 0 || fe->lump > 7)
        return ALLIUM_ERR_UNSUPPORTED;
    std::vector<int> refl_attrs;
    if (bc)
        for (int i = 0; i < bc->num; ++i) {
            if (bc->kinds[i] == ALLIUM_BC_REFLECTIVE) refl_attrs.push_back(bc->attributes[i]);
            else if (bc->kinds[i] != ALLIUM_BC_INFLOW) return ALLIUM_ERR_ARG;
        }

    allium_sweep* s = new allium_sweep;
    Handle& h = s->h;
    h.dim = mesh->dim; h.p = fe->order; h.lump = fe->lump;
    h.ne = mesh->num_elements; h.Nw = quad->num_angles; h.G = num_groups;
    h.ref = allium::make_ref_tables(h.dim, h.p, h.lump);
    h.n = h.ref.n; h.nf = h.ref.nf; h.nface = h.ref.nface;
    h.ndof = (long long)h.ne * h.n;
    h.psi_size = (long long)h.G * h.Nw * h.ndof;
    h.h_omega.assign(quad->omega, quad->omega + (size_t)h.Nw * h.dim);
    h.h_weights.assign(quad->weights, quad->weights + h.Nw);
    h.wsum = 0.0;
    for (double w : h.h_weights) h.wsum += w;

    auto fail = [&](int st) {
        free_all(h);
        std::fprintf(stderr, "allium_sweep_create: %s (%s)\n", allium_status_string(st), h.last_error.c_str());
        delete s;
        return st;
    };

    allium::Topology topo;
    int st = allium::build_topology(*mesh, h.p, topo, h.last_error);
    if (st != ALLIUM_OK) return fail(st);
    allium::mark_reflective(topo, h.nface, refl_attrs);
    h.nfaces = topo.nfaces;

    if (cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking) != cudaSuccess) {
        h.last_error = "cannot create a CUDA stream (no device?)";
        return fail(ALLIUM_ERR_CUDA);
    }
    h.own_stream = true;
    const long long N = (long long)h.ne * h.Nw;
    const size_t nn = (size_t)h.n * h.n;
#define STEP(x) do { int _s = (x); if (_s != ALLIUM_OK) return fail(_s); } while (0)
#define CSTEP(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { h.last_error = std::string(#x) + ": " + cudaGetErrorString(_e); return fail(ALLIUM_ERR_CUDA); } } while (0)
    STEP(upload(h, h.h_omega.data(), h.h_omega.size(), &h.d_omega));
    STEP(upload(h, h.h_weights.data(), h.h_weights.size(), &h.d_weights));
    STEP(upload(h, topo.corners.data(), topo.corners.size(), &h.d_corners));
    STEP(upload(h, topo.slots.data(), topo.slots.size(), &h.d_slots));
    STEP(upload(h, topo.face_e1k1.data(), topo.face_e1k1.size(), &h.d_face_e1k1));
    STEP(upload(h, topo.nbrmap.data(), topo.nbrmap.size(), &h.d_nbrmap));
    STEP(upload(h, topo.orient.data(), topo.orient.size(), &h.d_orient));
    STEP(upload(h, sigma_t, (size_t)h.G * h.ne, &h.d_sigma));
    CSTEP(cudaMalloc(&h.d_normals, (size_t)h.nfaces * h.dim * sizeof(double)));
    CSTEP(cudaMalloc(&h.d_dots, (size_t)h.nfaces * h.Nw * sizeof(double)));
    CSTEP(cudaMalloc(&h.f_dots, (size_t)h.nfaces * h.Nw * sizeof(float)));
    CSTEP(cudaMalloc(&h.d_G, (size_t)h.ne * h.dim * nn * sizeof(double)));
    CSTEP(cudaMalloc(&h.d_M, (size_t)h.ne * nn * sizeof(double)));
    CSTEP(cudaMalloc(&h.d_F, (size_t)h.ne * h.nface * h.nf * h.nf * sizeof(double)));
    CSTEP(cudaMalloc(&h.d_level, N * sizeof(int)));
    CSTEP(cudaMalloc(&h.d_level_nodes, N * sizeof(int)));
    CSTEP(cudaMalloc(&h.d_status, sizeof(int)));
    CSTEP(cudaMemsetAsync(h.d_status, 0, sizeof(int), h.stream));
    h.scratch_len = 4096;
    CSTEP(cudaMalloc(&h.d_scratch, (h.scratch_len + 1) * sizeof(double)));
    CSTEP(allium::launch_face_normals(h));
    CSTEP(allium::launch_face_dots(h));
    STEP(allium::compute_reflections(h, topo.refl_faces));
    CSTEP(allium::launch_assemble(h));
    STEP(allium::compute_levels(h));
    CSTEP(cudaStreamSynchronize(h.stream));
#undef STEP
#undef CSTEP
    *out = s;
    return ALLIUM_OK;
}

void allium_sweep_destroy(allium_sweep* s) {
    if (!s) return;
    if (s->h.stream) cudaStreamSynchronize(s->h.stream);
    free_all(s->h);
    delete s;
}

int allium_sweep_set_stream(allium_sweep* s, void* stream) {
    if (!s) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (h.own_stream) {
        CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
        cudaStreamDestroy(h.stream);
        h.own_stream = false;
    }
    h.stream = (cudaStream_t)stream;
    return ALLIUM_OK;
}

int allium_sweep_sizes(const allium_sweep* s, long long* psi_size, long long* num_dofs, int* num_levels) {
    if (!s) return ALLIUM_ERR_ARG;
    if (psi_size) *psi_size = s->h.psi_size;
    if (num_dofs) *num_dofs = s->h.ndof;
    if (num_levels) *num_levels = s->h.num_levels;
    return ALLIUM_OK;
}

int allium_sweep_assemble(allium_sweep* s, const double* sigma_t) {
    if (!s || !sigma_t) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    int st = upload(h, sigma_t, (size_t)h.G * h.ne, &h.d_sigma);
    if (st) return st;
    h.inv_valid = false;
    st = refresh_fp32(h);
    if (st) return st;
    CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    return ALLIUM_OK;
}

static int ensure_mass2(Handle& h) {
    if (h.have_mass2) return ALLIUM_OK;
    CUDA_OR_FAIL(h, cudaMalloc(&h.d_Mt, (size_t)h.ne * h.n * h.n * sizeof(double)));
    CUDA_OR_FAIL(h, allium::launch_time_mass(h));
    h.have_mass2 = true;
    return ALLIUM_OK;
}

int allium_sweep_set_time_absorption(allium_sweep* s, double tau) {
    if (!s) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (tau != h.tau || !h.time_dependent) h.inv_valid = false;
    h.tau = tau;
    // captured launches carry tau and the time-mass pointers as arguments
    CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    allium::drop_graphs(h);
    if (!h.time_dependent) {
        int st = ensure_mass2(h);
        if (st) return st;
        h.time_dependent = true;
        st = refresh_fp32(h);
        if (st) return st;
        CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    }
    return ALLIUM_OK;
}

int allium_sweep_scattering_source(allium_sweep* s, const double* sigma_s, const double* phi,
                                   const double* q_fixed, double* out) {
    if (!s || !sigma_s || !phi || !out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    int st = ensure_mass2(h);
    if (st) return st;
    st = upload(h, sigma_s, (size_t)h.G * h.ne, &h.d_sigma_s);
    if (st) return st;
    const size_t pbytes = (size_t)h.psi_size * sizeof(double);
    const size_t mbytes = (size_t)h.G * h.ndof * sizeof(double);
    const bool dph = on_device(phi), dqf = !q_fixed || on_device(q_fixed), dout = on_device(out);
    if (dph && dqf && dout) {
        CUDA_OR_FAIL(h, allium::launch_scatter_source(h, h.d_sigma_s, phi, q_fixed, out));
        return ALLIUM_OK;
    }
    double *dphi = nullptr, *dq = nullptr;
    cudaError_t e = cudaSuccess;
    const double* xp = phi;
    const double* xq = q_fixed;
    double* y = out;
    if (!dph) { e = cudaMalloc(&dphi, mbytes); if (e == cudaSuccess) e = cudaMemcpyAsync(dphi, phi, mbytes, cudaMemcpyHostToDevice, h.stream); xp = dphi; }
    if (e == cudaSuccess && !dqf) { e = cudaMalloc(&dq, pbytes); if (e == cudaSuccess) e = cudaMemcpyAsync(dq, q_fixed, pbytes, cudaMemcpyHostToDevice, h.stream); xq = dq; }
    if (e == cudaSuccess && !dout) { e = ensure(&h.d_stage, (size_t)h.psi_size); y = h.d_stage; }
    if (e == cudaSuccess) e = allium::launch_scatter_source(h, h.d_sigma_s, xp, xq, y);
    if (e == cudaSuccess && !dout) e = cudaMemcpyAsync(out, y, pbytes, cudaMemcpyDeviceToHost, h.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    if (dphi) cudaFree(dphi);
    if (dq) cudaFree(dq);
    CUDA_OR_FAIL(h, e);
    return ALLIUM_OK;
}

static bool misaligned(const void* a, const void* b, bool da, bool db) {
    return (da && ((uintptr_t)a & 15)) || (db && ((uintptr_t)b & 15));
}

// Allocate the FP64 factor cache when enabled, supported and it leaves at
// least half of the free device memory untouched; otherwise sweep without it.
// The check and the allocation hold a process-wide lock (allium::cache_lock),
// so handles used from several threads at once decide one after another.
static void prepare_factor_cache(Handle& h) {
    if (h.d_inv || h.factor_cache == 0 || !allium::factor_cache_supported(h)) return;
    const size_t need = (size_t)h.G * h.ne * h.Nw * h.n * h.n * sizeof(double);
    std::lock_guard<std::mutex> lock(allium::cache_lock());
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) { cudaGetLastError(); return; }
    if (need > free_b / 2) return;
    if (cudaMalloc(&h.d_inv, need) != cudaSuccess) { cudaGetLastError(); h.d_inv = nullptr; return; }
    h.inv_valid = false;
    allium::drop_graphs(h);
}

static bool pinned_host(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// Host buffers, page-locked: the directions are split into chunks that are
// independent sweeps (no reflective coupling), and chunk c's copy in, sweep
// and copy out are pipelined with the other chunks' (copy engines in both
// directions, two compute streams), so the host link and the sweep overlap.
static int mult_host_chunked(Handle& h, const double* source, double* psi) {
    const int C = h.pipe_chunks < h.Nw / 2 ? h.pipe_chunks : h.Nw / 2;
    const int S = h.pipe_streams < C ? h.pipe_streams : C;
    if (int st = allium::build_chunks(h, C, h.pipe_taper)) return st;
    const auto mk = [](cudaStream_t* st) {
        return *st ? cudaSuccess : cudaStreamCreateWithFlags(st, cudaStreamNonBlocking);
    };
    CUDA_OR_FAIL(h, mk(&h.copy_in));
    CUDA_OR_FAIL(h, mk(&h.copy_out));
    for (int k = 1; k < S; ++k) CUDA_OR_FAIL(h, mk(&h.comp[k]));
    if ((int)h.chunk_events.size() < 3 * C + 1) {
        for (cudaEvent_t ev : h.chunk_events) cudaEventDestroy(ev);
        h.chunk_events.assign(3 * C + 1, nullptr);
        for (auto& ev : h.chunk_events) CUDA_OR_FAIL(h, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    CUDA_OR_FAIL(h, ensure(&h.d_stage, (size_t)h.psi_size));
    CUDA_OR_FAIL(h, allium::ensure_factors(h));
    cudaEvent_t* ev = h.chunk_events.data();
    cudaEvent_t start = ev[3 * C];
    CUDA_OR_FAIL(h, cudaEventRecord(start, h.stream));
    CUDA_OR_FAIL(h, cudaStreamWaitEvent(h.copy_in, start, 0));
    CUDA_OR_FAIL(h, cudaStreamWaitEvent(h.copy_out, start, 0));
    for (int k = 1; k < S; ++k) CUDA_OR_FAIL(h, cudaStreamWaitEvent(h.comp[k], start, 0));
    for (int c = 0; c < C; ++c) {
        const int a0 = h.h_chunk_angle[c], a1 = h.h_chunk_angle[c + 1];
        const size_t bytes = (size_t)(a1 - a0) * h.ndof * sizeof(double);
        for (int g = 0; g < h.G; ++g) {
            const size_t off = ((size_t)g * h.Nw + a0) * h.ndof;
            CUDA_OR_FAIL(h, cudaMemcpyAsync(h.d_stage + off, source + off, bytes, cudaMemcpyHostToDevice, h.copy_in));
        }
        CUDA_OR_FAIL(h, cudaEventRecord(ev[3 * c], h.copy_in));
        cudaStream_t cs = (c % S == 0) ? h.stream : h.comp[c % S];
        CUDA_OR_FAIL(h, cudaStreamWaitEvent(cs, ev[3 * c], 0));
        CUDA_OR_FAIL(h, allium::launch_sweep_chunk(h, h.d_stage, c, cs));
        CUDA_OR_FAIL(h, cudaEventRecord(ev[3 * c + 1], cs));
        CUDA_OR_FAIL(h, cudaStreamWaitEvent(h.copy_out, ev[3 * c + 1], 0));
        for (int g = 0; g < h.G; ++g) {
            const size_t off = ((size_t)g * h.Nw + a0) * h.ndof;
            CUDA_OR_FAIL(h, cudaMemcpyAsync(psi + off, h.d_stage + off, bytes, cudaMemcpyDeviceToHost, h.copy_out));
        }
    }
    CUDA_OR_FAIL(h, cudaEventRecord(ev[3 * C - 1], h.copy_out));
    CUDA_OR_FAIL(h, cudaStreamWaitEvent(h.stream, ev[3 * C - 1], 0));
    return check_status(h);
}

int allium_sweep_mult(allium_sweep* s, const double* source, double* psi) {
    if (!s || !source || !psi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    prepare_factor_cache(h);
    const bool ds = on_device(source), dp = on_device(psi);
    if (misaligned(source, psi, ds, dp)) { h.last_error = "device vectors must be 16-byte aligned"; return ALLIUM_ERR_ARG; }
    if (ds && dp) {
        CUDA_OR_FAIL(h, allium::launch_sweep_fp64(h, source, psi));
        return ALLIUM_OK;
    }
    if (!ds && !dp && h.d_inv && h.nrefl == 0 && h.fix_kind == 0 && h.schedule == 0 && h.Nw >= 4 &&
        pinned_host(source) && pinned_host(psi))
        return mult_host_chunked(h, source, psi);
    CUDA_OR_FAIL(h, ensure(&h.d_stage, (size_t)h.psi_size));
    const size_t bytes = (size_t)h.psi_size * sizeof(double);
    const double* src = source;
    if (!ds) {
        CUDA_OR_FAIL(h, cudaMemcpyAsync(h.d_stage, source, bytes, cudaMemcpyHostToDevice, h.stream));
        src = h.d_stage;
    }
    double* out = dp ? psi : h.d_stage;
    CUDA_OR_FAIL(h, allium::launch_sweep_fp64(h, src, out));
    if (!dp) CUDA_OR_FAIL(h, cudaMemcpyAsync(psi, h.d_stage, bytes, cudaMemcpyDeviceToHost, h.stream));
    return check_status(h);
}

int allium_sweep_mult_f32(allium_sweep* s, const float* source, float* psi) {
    if (!s || !source || !psi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (!h.fp32_ready) CUDA_OR_FAIL(h, allium::make_fp32_copies(h));
    const bool ds = on_device(source), dp = on_device(psi);
    if (misaligned(source, psi, ds, dp)) { h.last_error = "device vectors must be 16-byte aligned"; return ALLIUM_ERR_ARG; }
    if (ds && dp) {
        CUDA_OR_FAIL(h, allium::launch_sweep_fp32(h, source, psi));
        return ALLIUM_OK;
    }
    CUDA_OR_FAIL(h, ensure(&h.f_stage, (size_t)h.psi_size));
    const size_t bytes = (size_t)h.psi_size * sizeof(float);
    const float* src = source;
    if (!ds) {
        CUDA_OR_FAIL(h, cudaMemcpyAsync(h.f_stage, source, bytes, cudaMemcpyHostToDevice, h.stream));
        src = h.f_stage;
    }
    float* out = dp ? psi : h.f_stage;
    CUDA_OR_FAIL(h, allium::launch_sweep_fp32(h, src, out));
    if (!dp) CUDA_OR_FAIL(h, cudaMemcpyAsync(psi, h.f_stage, bytes, cudaMemcpyDeviceToHost, h.stream));
    return check_status(h);
}

int allium_sweep_apply_L(allium_sweep* s, const double* x, double* y) {
    if (!s || !x || !y) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if ((const void*)x == (const void*)y) { h.last_error = "apply_L needs distinct x and y"; return ALLIUM_ERR_ARG; }
    const bool dx = on_device(x), dy = on_device(y);
    if (dx && dy) {
        CUDA_OR_FAIL(h, allium::launch_apply_L_fp64(h, x, y));
        return ALLIUM_OK;
    }
    const size_t bytes = (size_t)h.psi_size * sizeof(double);
    double *bx = nullptr, *by = nullptr;
    if (!dx) {
        CUDA_OR_FAIL(h, ensure(&h.d_stage, (size_t)h.psi_size));
        CUDA_OR_FAIL(h, cudaMemcpyAsync(h.d_stage, x, bytes, cudaMemcpyHostToDevice, h.stream));
        bx = h.d_stage;
    }
    if (!dy) CUDA_OR_FAIL(h, cudaMalloc(&by, bytes));
    cudaError_t e = allium::launch_apply_L_fp64(h, dx ? x : bx, dy ? y : by);
    if (e == cudaSuccess && !dy) e = cudaMemcpyAsync(y, by, bytes, cudaMemcpyDeviceToHost, h.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    if (by) cudaFree(by);
    CUDA_OR_FAIL(h, e);
    return ALLIUM_OK;
}

int allium_sweep_balance(allium_sweep* s, const double* psi, double* out) {
    if (!s || !psi || !out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    const double* x = psi;
    if (!on_device(psi)) {
        CUDA_OR_FAIL(h, ensure(&h.d_stage, (size_t)h.psi_size));
        CUDA_OR_FAIL(h, cudaMemcpyAsync(h.d_stage, psi, (size_t)h.psi_size * sizeof(double), cudaMemcpyHostToDevice, h.stream));
        x = h.d_stage;
    }
    int nb = 0;
    CUDA_OR_FAIL(h, allium::launch_balance(h, x, h.d_scratch, (int)h.scratch_len, &nb));
    double* res = h.d_scratch + h.scratch_len;
    CUDA_OR_FAIL(h, allium::launch_balance_finish(h, h.d_scratch, nb, res));
    CUDA_OR_FAIL(h, cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDefault, h.stream));
    if (!on_device(out)) CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    return ALLIUM_OK;
}

int allium_sweep_moments(allium_sweep* s, const double* psi, double* phi, int nmom) {
    if (!s || !psi || !phi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (nmom != 1 && nmom != h.dim + 1) return ALLIUM_ERR_ARG;
    const bool dps = on_device(psi), dph = on_device(phi);
    const size_t pbytes = (size_t)h.psi_size * sizeof(double);
    const size_t mbytes = (size_t)h.G * nmom * h.ndof * sizeof(double);
    const double* x = psi;
    if (!dps) {
        CUDA_OR_FAIL(h, ensure(&h.d_stage, (size_t)h.psi_size));
        CUDA_OR_FAIL(h, cudaMemcpyAsync(h.d_stage, psi, pbytes, cudaMemcpyHostToDevice, h.stream));
        x = h.d_stage;
    }
    double* y = phi;
    if (!dph) CUDA_OR_FAIL(h, cudaMalloc(&y, mbytes));
    cudaError_t e = allium::launch_moments(h, x, y, nmom);
    if (e == cudaSuccess && !dph) e = cudaMemcpyAsync(phi, y, mbytes, cudaMemcpyDeviceToHost, h.stream);
    if (e == cudaSuccess && (!dph || !dps)) e = cudaStreamSynchronize(h.stream);
    if (!dph) cudaFree(y);
    CUDA_OR_FAIL(h, e);
    return ALLIUM_OK;
}

int allium_sweep_relayout(allium_sweep* s, const double* in, int in_layout, double* out, int out_layout) {
    if (!s || !in || !out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    const auto known = [](int l) { return l == ALLIUM_LAYOUT_RIGHT || l == ALLIUM_LAYOUT_LEFT; };
    if (!known(in_layout) || !known(out_layout)) { h.last_error = "unknown layout"; return ALLIUM_ERR_ARG; }
    if (!on_device(in) || !on_device(out)) { h.last_error = "relayout takes device vectors"; return ALLIUM_ERR_ARG; }
    const size_t bytes = (size_t)h.psi_size * sizeof(double);
    const char* a = reinterpret_cast<const char*>(in);
    const char* b = reinterpret_cast<const char*>(out);
    if (a < b + bytes && b < a + bytes) { h.last_error = "relayout vectors overlap"; return ALLIUM_ERR_ARG; }
    if (in_layout == out_layout) CUDA_OR_FAIL(h, cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, h.stream));
    else CUDA_OR_FAIL(h, allium::launch_relayout(h, in, out, out_layout == ALLIUM_LAYOUT_LEFT));
    return ALLIUM_OK;
}

int allium_sweep_moments_transpose(allium_sweep* s, const double* phi, double* psi, int nmom, double alpha, int add) {
    if (!s || !psi || !phi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (nmom != 1 && nmom != h.dim + 1) return ALLIUM_ERR_ARG;
    const bool dps = on_device(psi), dph = on_device(phi);
    const size_t pbytes = (size_t)h.psi_size * sizeof(double);
    const size_t mbytes = (size_t)h.G * nmom * h.ndof * sizeof(double);
    const double* x = phi;
    double* tmp = nullptr;
    if (!dph) {
        CUDA_OR_FAIL(h, cudaMalloc(&tmp, mbytes));
        CUDA_OR_FAIL(h, cudaMemcpyAsync(tmp, phi, mbytes, cudaMemcpyHostToDevice, h.stream));
        x = tmp;
    }
    double* y = psi;
    cudaError_t e = cudaSuccess;
    if (!dps) {
        e = ensure(&h.d_stage, (size_t)h.psi_size);
        if (e == cudaSuccess && add) e = cudaMemcpyAsync(h.d_stage, psi, pbytes, cudaMemcpyHostToDevice, h.stream);
        y = h.d_stage;
    }
    if (e == cudaSuccess) e = allium::launch_moments_transpose(h, x, y, nmom, alpha, add);
    if (e == cudaSuccess && !dps) e = cudaMemcpyAsync(psi, y, pbytes, cudaMemcpyDeviceToHost, h.stream);
    if (e == cudaSuccess && (!dps || !dph)) e = cudaStreamSynchronize(h.stream);
    if (tmp) cudaFree(tmp);
    CUDA_OR_FAIL(h, e);
    return ALLIUM_OK;
}

int allium_sweep_moments_f32(allium_sweep* s, const float* psi, double* phi) {
    if (!s || !psi || !phi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (!on_device(psi) || !on_device(phi)) { h.last_error = "allium_sweep_moments_f32 takes device vectors"; return ALLIUM_ERR_ARG; }
    CUDA_OR_FAIL(h, allium::launch_moments_f32(h, psi, phi));
    return ALLIUM_OK;
}

int allium_sweep_scattering_source_f32(allium_sweep* s, const double* sigma_s, const double* phi,
                                       const float* q_fixed, float* out) {
    if (!s || !sigma_s || !phi || !out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (!on_device(phi) || !on_device(out) || (q_fixed && !on_device(q_fixed))) {
        h.last_error = "allium_sweep_scattering_source_f32 takes device vectors";
        return ALLIUM_ERR_ARG;
    }
    int st = ensure_mass2(h);
    if (st) return st;
    st = upload(h, sigma_s, (size_t)h.G * h.ne, &h.d_sigma_s);
    if (st) return st;
    CUDA_OR_FAIL(h, allium::launch_scatter_source_f32(h, h.d_sigma_s, phi, q_fixed, out));
    return ALLIUM_OK;
}

static int device_only(Handle& h, std::initializer_list<const void*> ptrs, const char* who) {
    for (const void* p : ptrs)
        if (p && !on_device(p)) { h.last_error = std::string(who) + " takes device vectors"; return ALLIUM_ERR_ARG; }
    return ALLIUM_OK;
}

int allium_sweep_to_node_layout_f32(allium_sweep* s, const double* psi, float* out) {
    if (!s || !psi || !out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {psi, out}, "allium_sweep_to_node_layout_f32")) return st;
    CUDA_OR_FAIL(h, allium::launch_layout(h, 1, psi, out));
    return ALLIUM_OK;
}

int allium_sweep_from_node_layout_f32(allium_sweep* s, const float* in, double* psi) {
    if (!s || !in || !psi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {in, psi}, "allium_sweep_from_node_layout_f32")) return st;
    CUDA_OR_FAIL(h, allium::launch_layout(h, 0, in, psi));
    return ALLIUM_OK;
}

int allium_sweep_mult_f32_nodes(allium_sweep* s, const float* source, float* psi) {
    if (!s || !source || !psi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {source, psi}, "allium_sweep_mult_f32_nodes")) return st;
    if (misaligned(source, psi, true, true)) { h.last_error = "device vectors must be 16-byte aligned"; return ALLIUM_ERR_ARG; }
    if (h.nrefl) { h.last_error = "the node layout sweep supports inflow boundaries only"; return ALLIUM_ERR_UNSUPPORTED; }
    if (!h.fp32_ready) CUDA_OR_FAIL(h, allium::make_fp32_copies(h));
    CUDA_OR_FAIL(h, allium::launch_sweep_nodes_f32(h, source, psi));
    return ALLIUM_OK;
}

int allium_sweep_scattering_source_f32_nodes(allium_sweep* s, const double* sigma_s, const double* phi,
                                             const float* q_nodes, float* out) {
    if (!s || !sigma_s || !phi || !out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {phi, q_nodes, out}, "allium_sweep_scattering_source_f32_nodes")) return st;
    int st = ensure_mass2(h);
    if (st) return st;
    st = upload(h, sigma_s, (size_t)h.G * h.ne, &h.d_sigma_s);
    if (st) return st;
    CUDA_OR_FAIL(h, allium::launch_scatter_nodes(h, h.d_sigma_s, phi, q_nodes, out));
    return ALLIUM_OK;
}

int allium_sweep_moments_f32_nodes(allium_sweep* s, const float* psi, double* phi) {
    if (!s || !psi || !phi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {psi, phi}, "allium_sweep_moments_f32_nodes")) return st;
    CUDA_OR_FAIL(h, allium::launch_moments_nodes(h, psi, phi));
    return ALLIUM_OK;
}

static int fused_check(Handle& h, const char* who) {
    if (!allium::fused_supported(h)) {
        h.last_error = std::string(who) + ": orders 0 and 1 with inflow or vacuum boundaries only";
        return ALLIUM_ERR_UNSUPPORTED;
    }
    return ALLIUM_OK;
}

int allium_sweep_isotropic_source(allium_sweep* s, const double* sigma_s, const double* phi, const double* q_iso,
                                  float* out, float* out_hi, float* out_lo) {
    if (!s || (!out && !out_hi) || (!out_hi != !out_lo)) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {phi, q_iso, out, out_hi, out_lo}, "allium_sweep_isotropic_source")) return st;
    if (phi) {
        int st = ensure_mass2(h);
        if (st) return st;
        if (sigma_s) {
            st = upload(h, sigma_s, (size_t)h.G * h.ne, &h.d_sigma_s);
            if (st) return st;
        } else if (!h.d_sigma_s) {
            h.last_error = "allium_sweep_isotropic_source: no scattering cross sections given yet";
            return ALLIUM_ERR_ARG;
        }
    }
    CUDA_OR_FAIL(h, allium::launch_iso_source(h, h.d_sigma_s, phi, q_iso, out, out_hi, out_lo));
    return ALLIUM_OK;
}

int allium_sweep_fused_mult_f32(allium_sweep* s, const float* iso, const float* source, float* psi, double* phi,
                                int phi_mode, float* psi_hi, float* psi_lo) {
    if (!s || !psi || phi_mode < 0 || phi_mode > 3 || (phi_mode && !phi) || (!psi_hi != !psi_lo)) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = fused_check(h, "allium_sweep_fused_mult_f32")) return st;
    if (int st = device_only(h, {iso, source, psi, phi, psi_hi, psi_lo}, "allium_sweep_fused_mult_f32")) return st;
    if (misaligned(source ? source : psi, psi, true, true) || misaligned(iso ? iso : psi, psi_hi ? psi_hi : psi, true, true)) {
        h.last_error = "device vectors must be 16-byte aligned";
        return ALLIUM_ERR_ARG;
    }
    CUDA_OR_FAIL(h, allium::launch_fused_sweep(h, iso, source, psi, phi, phi_mode, psi_hi, psi_lo));
    return ALLIUM_OK;
}

int allium_sweep_fused_levels(allium_sweep* s, int* num_levels, int* unit_levels) {
    if (!s || !num_levels || !unit_levels) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = fused_check(h, "allium_sweep_fused_levels")) return st;
    CUDA_OR_FAIL(h, allium::fused_levels(h, num_levels, unit_levels));
    return ALLIUM_OK;
}

int allium_sweep_set_level_pdl(allium_sweep* s, int on) {
    if (!s) return ALLIUM_ERR_ARG;
    allium::drop_graphs(s->h);
    s->h.pdl_levels = on ? 1 : 0;
    return ALLIUM_OK;
}

int allium_sweep_set_fused_pdl(allium_sweep* s, int on) {
    if (!s) return ALLIUM_ERR_ARG;
    allium::set_fused_pdl(s->h, on);
    return ALLIUM_OK;
}

int allium_sweep_transport_residual_df(allium_sweep* s, const float* iso_hi, const float* iso_lo, const float* q_hi,
                                       const float* q_lo, const float* psi_hi, const float* psi_lo, float* r) {
    if (!s || !iso_hi || !iso_lo || !psi_hi || !psi_lo || !r || (!q_hi != !q_lo)) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = fused_check(h, "allium_sweep_transport_residual_df")) return st;
    if (int st = device_only(h, {iso_hi, iso_lo, q_hi, q_lo, psi_hi, psi_lo, r}, "allium_sweep_transport_residual_df"))
        return st;
    if (misaligned(psi_hi, psi_lo, true, true) || misaligned(r, r, true, true)) {
        h.last_error = "device vectors must be 16-byte aligned";
        return ALLIUM_ERR_ARG;
    }
    CUDA_OR_FAIL(h, allium::launch_residual_df(h, iso_hi, iso_lo, q_hi, q_lo, psi_hi, psi_lo, r));
    return ALLIUM_OK;
}

int allium_sweep_transport_residual_update_f32(allium_sweep* s, const float* iso, const float* dpsi, float* r) {
    if (!s || !iso || !dpsi || !r) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = fused_check(h, "allium_sweep_transport_residual_update_f32")) return st;
    if (int st = device_only(h, {iso, dpsi, r}, "allium_sweep_transport_residual_update_f32")) return st;
    if (misaligned(iso, dpsi, true, true) || misaligned(r, r, true, true)) {
        h.last_error = "device vectors must be 16-byte aligned";
        return ALLIUM_ERR_ARG;
    }
    if (!h.fp32_ready) CUDA_OR_FAIL(h, allium::make_fp32_copies(h));
    CUDA_OR_FAIL(h, allium::launch_residual_update_f32(h, iso, dpsi, r));
    return ALLIUM_OK;
}

int allium_sweep_moments_df(allium_sweep* s, const float* psi_hi, const float* psi_lo, double* phi) {
    if (!s || !psi_hi || !psi_lo || !phi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = fused_check(h, "allium_sweep_moments_df")) return st;
    if (int st = device_only(h, {psi_hi, psi_lo, phi}, "allium_sweep_moments_df")) return st;
    CUDA_OR_FAIL(h, allium::launch_moments_df(h, psi_hi, psi_lo, phi));
    return ALLIUM_OK;
}

int allium_sweep_to_fused_layout(allium_sweep* s, const double* psi_right, float* hi, float* lo) {
    if (!s || !psi_right || !hi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {psi_right, hi, lo}, "allium_sweep_to_fused_layout")) return st;
    CUDA_OR_FAIL(h, allium::launch_fused_layout(h, 1, psi_right, hi, lo));
    return ALLIUM_OK;
}

int allium_sweep_from_fused_layout(allium_sweep* s, const float* hi, const float* lo, double* psi_right) {
    if (!s || !psi_right || !hi) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {psi_right, hi, lo}, "allium_sweep_from_fused_layout")) return st;
    CUDA_OR_FAIL(h, allium::launch_fused_layout(h, 0, psi_right, const_cast<float*>(hi), const_cast<float*>(lo)));
    return ALLIUM_OK;
}

static int form_source(Handle& h, const double* q_cell, const double* q_points, int q_dir, const double* inflow,
                       int num_attr, int angular, double* source) {
    if (!source || (inflow && num_attr < 1)) return ALLIUM_ERR_ARG;
    const long long np = allium::source_points_per_cell(h);
    double *dq = nullptr, *dp = nullptr, *di = nullptr;
    int st = ALLIUM_OK;
    if (q_cell) st = upload(h, q_cell, (size_t)h.G * h.ne, &dq);
    if (!st && q_points) st = upload(h, q_points, (size_t)h.G * (q_dir ? h.Nw : 1) * h.ne * np, &dp);
    if (!st && inflow) st = upload(h, inflow, (size_t)h.G * (angular ? h.Nw : 1) * num_attr, &di);
    if (st) { if (dq) cudaFree(dq); if (dp) cudaFree(dp); if (di) cudaFree(di); return st; }
    const bool dsrc = on_device(source);
    double* out = source;
    cudaError_t e = cudaSuccess;
    if (!dsrc) {
        e = ensure(&h.d_stage, (size_t)h.psi_size);
        out = h.d_stage;
    }
    if (e == cudaSuccess) e = allium::launch_form_source(h, dq, dp, q_dir, di, inflow ? num_attr : 0, angular, out);
    if (e == cudaSuccess && !dsrc)
        e = cudaMemcpyAsync(source, out, (size_t)h.psi_size * sizeof(double), cudaMemcpyDeviceToHost, h.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    if (dq) cudaFree(dq);
    if (dp) cudaFree(dp);
    if (di) cudaFree(di);
    CUDA_OR_FAIL(h, e);
    return ALLIUM_OK;
}

int allium_sweep_form_source(allium_sweep* s, const double* q_cell, const double* inflow, int num_attr, double* source) {
    if (!s) return ALLIUM_ERR_ARG;
    return form_source(s->h, q_cell, nullptr, 0, inflow, num_attr, 0, source);
}

int allium_sweep_form_source_general(allium_sweep* s, const double* q_points, int q_per_direction,
                                     const double* inflow_angular, int num_attr, double* source) {
    if (!s || (q_per_direction != 0 && q_per_direction != 1)) return ALLIUM_ERR_ARG;
    return form_source(s->h, nullptr, q_points, q_per_direction, inflow_angular, num_attr, 1, source);
}

int allium_sweep_source_points(allium_sweep* s, int* points_per_cell, double* coords) {
    if (!s || !points_per_cell) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    const long long np = allium::source_points_per_cell(h);
    *points_per_cell = (int)np;
    if (!coords) return ALLIUM_OK;
    const size_t n = (size_t)h.ne * np * h.dim;
    const bool dc = on_device(coords);
    double* out = coords;
    if (!dc) CUDA_OR_FAIL(h, cudaMalloc(&out, n * sizeof(double)));
    cudaError_t e = allium::launch_source_points(h, out);
    if (e == cudaSuccess && !dc) e = cudaMemcpyAsync(coords, out, n * sizeof(double), cudaMemcpyDeviceToHost, h.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    if (!dc) cudaFree(out);
    CUDA_OR_FAIL(h, e);
    return ALLIUM_OK;
}

int allium_sweep_levels(allium_sweep* s, int* levels) {
    if (!s || !levels) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    CUDA_OR_FAIL(h, cudaMemcpyAsync(levels, h.d_level, (size_t)h.ne * h.Nw * sizeof(int), cudaMemcpyDefault, h.stream));
    CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    return ALLIUM_OK;
}

int allium_sweep_set_factor_cache(allium_sweep* s, int mode) {
    if (!s || mode < 0 || mode > 1) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    h.factor_cache = mode;
    if (mode == 0 && h.d_inv) {
        CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
        allium::drop_graphs(h);
        cudaFree(h.d_inv);
        h.d_inv = nullptr;
        h.inv_valid = false;
        if (h.f_inv_nodes) cudaFree(h.f_inv_nodes);
        h.f_inv_nodes = nullptr;
        h.f_inv_valid = false;
    }
    if (mode == 1) h.f_inv_failed = false;
    return ALLIUM_OK;
}

int allium_sweep_set_schedule(allium_sweep* s, int mode) {
    if (!s || mode < 0 || mode > 1) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (mode != h.schedule) {
        CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
        allium::drop_graphs(h);
        h.schedule = mode;
    }
    return ALLIUM_OK;
}

int allium_sweep_selftest_wait(allium_sweep* s, int poll_limit) {
    if (!s || poll_limit < 1 || poll_limit > (1 << 20)) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    CUDA_OR_FAIL(h, allium::launch_wait_probe(h, poll_limit));
    return check_status(h);
}

int allium_sweep_set_block_size(allium_sweep* s, int precision, int threads) {
    if (!s || (precision != 32 && precision != 64) || (threads != 32 && threads != 64 && threads != 128))
        return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    int& b = precision == 64 ? h.block64 : h.block32;
    if (b != threads) {
        b = threads;
        allium::drop_graphs(h);
    }
    return ALLIUM_OK;
}

int allium_sweep_set_f32_inverse_layout(allium_sweep* s, int entry_major) {
    if (!s || (entry_major != 0 && entry_major != 1)) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (h.f_inv_entry_major != entry_major) {
        CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
        h.f_inv_entry_major = entry_major;
        h.f_inv_valid = false;   // rewritten in the new order on the next node-layout sweep
        allium::drop_graphs(h);
    }
    return ALLIUM_OK;
}

int allium_sweep_set_pipeline(allium_sweep* s, int chunks, int streams, int taper) {
    if (!s || chunks < 2 || chunks > allium::Handle::kMaxPipeChunks || streams < 1 ||
        streams > allium::Handle::kMaxPipeStreams || taper < 0 || taper > 3)
        return ALLIUM_ERR_ARG;
    s->h.pipe_chunks = chunks;
    s->h.pipe_streams = streams;
    s->h.pipe_taper = taper;
    return ALLIUM_OK;
}

int allium_sweep_set_fixup(allium_sweep* s, int kind, double minimum) {
    if (!s || kind < 0) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (kind > 4) { h.last_error = "fixup kinds: 1 zero, 2 zero and scale, 3 Ryosuke, 4 local optimization"; return ALLIUM_ERR_UNSUPPORTED; }
    if (!h.d_fix_counts) {
        CUDA_OR_FAIL(h, cudaMalloc(&h.d_fix_counts, 2 * sizeof(unsigned long long)));
        CUDA_OR_FAIL(h, cudaMemsetAsync(h.d_fix_counts, 0, 2 * sizeof(unsigned long long), h.stream));
    }
    CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    allium::drop_graphs(h);   // captured launches carry the fixup settings
    h.fix_kind = kind;
    h.fix_min = minimum;
    return ALLIUM_OK;
}

int allium_sweep_fixup_counts(allium_sweep* s, long long* applied, long long* failed, int reset) {
    if (!s) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    unsigned long long c[2] = {0, 0};
    if (h.d_fix_counts) {
        CUDA_OR_FAIL(h, cudaMemcpyAsync(c, h.d_fix_counts, sizeof(c), cudaMemcpyDeviceToHost, h.stream));
        if (reset) CUDA_OR_FAIL(h, cudaMemsetAsync(h.d_fix_counts, 0, sizeof(c), h.stream));
        CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    }
    if (applied) *applied = (long long)c[0];
    if (failed) *failed = (long long)c[1];
    return ALLIUM_OK;
}

// ------------------------------------------------------------ thermal radiative transfer
int allium_planck_spectrum(const double* bounds, int num_groups, double T, int kind, double* out) {
    if (!bounds || !out || num_groups < 1 || (kind != 0 && kind != 1) || !(T > 0.0)) return ALLIUM_ERR_ARG;
    double prev = 0.0;
    for (int g = 0; g < num_groups - 1; ++g) {
        const double x = bounds[g + 1] / T;
        double f = allium::planck_fraction(x);
        if (kind == 1) f = allium::rosseland_from_planck(x, f);
        out[g] = f - prev;
        prev = f;
    }
    out[num_groups - 1] = 1.0 - prev;
    return ALLIUM_OK;
}

static int trt_check(Handle& h, const char* who) {
    if (!allium::trt_supported(h)) {
        h.last_error = std::string(who) + ": at most 16 DOFs per cell and no lumping";
        return ALLIUM_ERR_UNSUPPORTED;
    }
    return ALLIUM_OK;
}

int allium_sweep_planck_emission(allium_sweep* s, const double* bounds, const double* sigma_abs, const double* T,
                                 double ac, double* emission, double* grad) {
    if (!s || !bounds || !sigma_abs || !T || (!emission && !grad)) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = trt_check(h, "allium_sweep_planck_emission")) return st;
    if (int st = device_only(h, {sigma_abs, T}, "allium_sweep_planck_emission")) return st;
    if ((emission && !on_device(emission)) || (grad && !on_device(grad))) {
        h.last_error = "allium_sweep_planck_emission: outputs must be device memory";
        return ALLIUM_ERR_ARG;
    }
    if (int st = upload(h, bounds, (size_t)h.G + 1, &h.d_bounds)) return st;
    CUDA_OR_FAIL(h, allium::launch_trt_emission(h, h.d_bounds, sigma_abs, T, ac, 0.0, emission, grad, nullptr, nullptr));
    return ALLIUM_OK;
}

int allium_sweep_energy_balance(allium_sweep* s, const double* bounds, const double* sigma_abs, const double* T,
                                double ac, double cv_dt, double* residual, double* grad_inv) {
    if (!s || !bounds || !sigma_abs || !T || (!residual && !grad_inv)) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = trt_check(h, "allium_sweep_energy_balance")) return st;
    if (int st = device_only(h, {sigma_abs, T}, "allium_sweep_energy_balance")) return st;
    if ((residual && !on_device(residual)) || (grad_inv && !on_device(grad_inv))) {
        h.last_error = "allium_sweep_energy_balance: outputs must be device memory";
        return ALLIUM_ERR_ARG;
    }
    if (int st = upload(h, bounds, (size_t)h.G + 1, &h.d_bounds)) return st;
    if (int st = ensure_mass2(h)) return st;
    CUDA_OR_FAIL(h, allium::launch_trt_emission(h, h.d_bounds, sigma_abs, T, ac, cv_dt, nullptr, nullptr, residual,
                                                grad_inv));
    if (grad_inv) return check_status(h);
    return ALLIUM_OK;
}

int allium_sweep_block_apply(allium_sweep* s, const double* blocks, int num_sets, const double* x, int x_shared,
                             double* y, double alpha, int accumulate) {
    if (!s || !x || !y || num_sets < 1) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    const double* B = blocks;
    if (!blocks) {
        // the handle's own mass matrices: num_sets 1 -> unit sigma mass, 2 -> MassIntegrator mass
        if (num_sets == 2) {
            if (int st = ensure_mass2(h)) return st;
            B = h.d_Mt;
        } else {
            B = h.d_M;
        }
        num_sets = 1;
    }
    if (int st = device_only(h, {B, x, y}, "allium_sweep_block_apply")) return st;
    CUDA_OR_FAIL(h, allium::launch_block_apply(h, B, num_sets, x, x_shared ? 0 : h.ndof, y, alpha, accumulate));
    return ALLIUM_OK;
}

int allium_sweep_absorption(allium_sweep* s, const double* sigma_abs, const double* phi, double* y, double alpha,
                            int accumulate) {
    if (!s || !sigma_abs || !phi || !y) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {sigma_abs, phi, y}, "allium_sweep_absorption")) return st;
    CUDA_OR_FAIL(h, allium::launch_absorption(h, sigma_abs, phi, y, alpha, accumulate));
    return ALLIUM_OK;
}

int allium_sweep_time_source(allium_sweep* s, const double* psi_prev, const double* q, double tau, double* out) {
    if (!s || !psi_prev || !out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {psi_prev, out}, "allium_sweep_time_source")) return st;
    if (q && !on_device(q)) { h.last_error = "allium_sweep_time_source: q must be device memory"; return ALLIUM_ERR_ARG; }
    if (int st = ensure_mass2(h)) return st;
    CUDA_OR_FAIL(h, allium::launch_time_source(h, psi_prev, q, tau, out));
    return ALLIUM_OK;
}

int allium_sweep_powerlaw_opacity(allium_sweep* s, const double* T, const double* nu, double C, double a, double b,
                                  double* sigma_out) {
    if (!s || !T || !nu || !sigma_out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (int st = device_only(h, {T, sigma_out}, "allium_sweep_powerlaw_opacity")) return st;
    if (int st = upload(h, nu, (size_t)h.G, &h.d_nu)) return st;
    CUDA_OR_FAIL(h, allium::launch_powerlaw_opacity(h, T, h.d_nu, C, a, b, sigma_out));
    return ALLIUM_OK;
}

// ------------------------------------------------------------ MIP diffusion (DSA)
int allium_sweep_dsa_setup(allium_sweep* s, const double* sigma_s, double kappa, double penalty_min, double alpha_bdr,
                           double tau) {
    if (!s || !sigma_s) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (!allium::dsa_supported(h)) {
        h.last_error = "allium_sweep_dsa_setup: at most 16 DOFs per cell and no lumping";
        return ALLIUM_ERR_UNSUPPORTED;
    }
    if (kappa < 0.0) kappa = (double)(h.p + 1) * (h.p + 1);
    if (penalty_min < 0.0) {
        // ComputeAlpha(quad, e_x) / 2 (src/angular_quadrature.cpp:266-276, exe/chive.cpp:669)
        double a = 0.0, w = 0.0;
        for (int q = 0; q < h.Nw; ++q) { a += std::fabs(h.h_omega[(size_t)q * h.dim]) * h.h_weights[q]; w += h.h_weights[q]; }
        penalty_min = 0.5 * a / w;
    }
    if (alpha_bdr < 0.0) alpha_bdr = 0.5;
    if (int st = upload(h, sigma_s, (size_t)h.G * h.ne, &h.d_sigma_s)) return st;
    if (int st = ensure_mass2(h)) return st;
    CUDA_OR_FAIL(h, allium::launch_dsa_assemble(h, h.d_sigma_s, kappa, penalty_min, alpha_bdr, tau));
    h.dsa_ready = true;
    return check_status(h);
}

int allium_sweep_dsa_apply(allium_sweep* s, const double* x, double* y) {
    if (!s || !x || !y) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (!h.dsa_ready) { h.last_error = "allium_sweep_dsa_setup has not been called"; return ALLIUM_ERR_ARG; }
    if (int st = device_only(h, {x, y}, "allium_sweep_dsa_apply")) return st;
    CUDA_OR_FAIL(h, allium::launch_dsa_apply(h, x, y));
    return ALLIUM_OK;
}

int allium_sweep_dsa_jacobi(allium_sweep* s, const double* x, double* y) {
    if (!s || !x || !y) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (!h.dsa_ready) { h.last_error = "allium_sweep_dsa_setup has not been called"; return ALLIUM_ERR_ARG; }
    if (int st = device_only(h, {x, y}, "allium_sweep_dsa_jacobi")) return st;
    CUDA_OR_FAIL(h, allium::launch_block_apply(h, h.d_dsa_inv, h.G, x, h.ndof, y, 1.0, 0));
    return ALLIUM_OK;
}

int allium_sweep_neighbours(allium_sweep* s, int* out) {
    if (!s || !out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    std::vector<allium::Slot> slots((size_t)h.ne * h.nface);
    CUDA_OR_FAIL(h, cudaMemcpyAsync(slots.data(), h.d_slots, slots.size() * sizeof(allium::Slot), cudaMemcpyDeviceToHost,
                                    h.stream));
    CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    for (size_t i = 0; i < slots.size(); ++i) out[i] = slots[i].nbr >= 0 ? slots[i].nbr : -1;
    return ALLIUM_OK;
}

int allium_sweep_dsa_blocks(allium_sweep* s, double* out) {
    if (!s || !out) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    if (!h.dsa_ready) { h.last_error = "allium_sweep_dsa_setup has not been called"; return ALLIUM_ERR_ARG; }
    const size_t count = (size_t)h.G * h.ne * (1 + h.nface) * h.n * h.n;
    CUDA_OR_FAIL(h, cudaMemcpyAsync(out, h.d_dsa, count * sizeof(double), cudaMemcpyDefault, h.stream));
    CUDA_OR_FAIL(h, cudaStreamSynchronize(h.stream));
    return ALLIUM_OK;
}

int allium_sweep_synchronize(allium_sweep* s) {
    if (!s) return ALLIUM_ERR_ARG;
    Handle& h = s->h;
    CUDA_OR_FAIL(h, cudaGetLastError());
    return check_status(h);
}

}  // extern "C"
