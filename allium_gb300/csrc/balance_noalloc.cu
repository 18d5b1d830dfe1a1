// allium_sweep_balance_noalloc: the balance reduction for callers that cannot
// allocate GPU memory at the point of the call.
//
// Who needs it: code that runs under a caller-owned memory pool or in a
// real-time time-step loop where allocating is forbidden (an allocation would
// synchronise the device or exceed the caller's budget), and embedded uses
// where the host runtime hands the library only the vectors it works on.  allium_sweep_balance itself needs no
// allocation on a device pointer either, but it relies on a partial-sum buffer
// that the handle allocated; this variant keeps its partial sums in a
// file-scope device array instead.
//
// The array (kNoAllocMaxPartials + 1 doubles, 32 KB) lives in the library's
// device image, so every GPU that loads the library holds it until the
// process exits.  Its device address is looked up with cudaGetSymbolAddress
// the first time the entry point runs on a device (with that device current);
// make that first call before any stream capture begins.  The address is kept
// per device index for the process, which assumes one CUDA context per device
// for the library's lifetime.  All calls share the
// array: each call writes every partial it later reads and the result slot,
// so nothing has to be cleared between calls, but two calls whose kernels
// overlap on the GPU (different streams, or different handles on one device)
// race on it.
#include <mutex>
#include <string>

#include "internal.h"

namespace {

constexpr int kNoAllocMaxPartials = 4096;                 // partial sums held in the array
constexpr long long kItemsPerPartial = 256LL * 128;       // (group, angle, cell) items per block
constexpr long long kNoAllocMaxItems = kNoAllocMaxPartials * kItemsPerPartial;  // 134,217,728
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_balance_scratch[kNoAllocMaxPartials + 1];

std::mutex g_mutex;
double* g_scratch_address[kMaxDevices] = {};

// device address of g_balance_scratch on the current device (set up once per device)
int scratch_address(allium::Handle& h, double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        h.last_error = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
        return ALLIUM_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        h.last_error = "device index above the supported range";
        return ALLIUM_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_address[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_balance_scratch);
        if (e != cudaSuccess || !p) {
            h.last_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return ALLIUM_ERR_CUDA;
        }
        g_scratch_address[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_address[dev];
    return ALLIUM_OK;
}

bool is_device_memory(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" int allium_sweep_balance_noalloc(allium_sweep* s, const double* psi, double* out) {
    if (!s || !psi || !out) return ALLIUM_ERR_ARG;
    allium::Handle& h = s->h;
    const long long items = (long long)h.G * h.Nw * h.ne;
    if (items > kNoAllocMaxItems) {
        h.last_error = "allium_sweep_balance_noalloc handles at most 134217728 (group, angle, cell) items; "
                       "this problem has " + std::to_string(items) + " (use allium_sweep_balance)";
        return ALLIUM_ERR_SIZE;
    }
    if (!is_device_memory(psi)) {
        h.last_error = "allium_sweep_balance_noalloc needs psi in device memory";
        return ALLIUM_ERR_ARG;
    }
    double* scratch = nullptr;
    int st = scratch_address(h, &scratch);
    if (st != ALLIUM_OK) return st;
    const int parts = (int)((items + kItemsPerPartial - 1) / kItemsPerPartial);
    int nb = 0;
    cudaError_t e = allium::launch_balance(h, psi, scratch, parts, &nb);
    if (e == cudaSuccess) e = allium::launch_balance_finish(h, scratch, nb, scratch + kNoAllocMaxPartials);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, scratch + kNoAllocMaxPartials, sizeof(double), cudaMemcpyDefault, h.stream);
    if (e == cudaSuccess && !is_device_memory(out)) e = cudaStreamSynchronize(h.stream);
    if (e != cudaSuccess) {
        h.last_error = std::string("allium_sweep_balance_noalloc: ") + cudaGetErrorString(e);
        return ALLIUM_ERR_CUDA;
    }
    return ALLIUM_OK;
}
