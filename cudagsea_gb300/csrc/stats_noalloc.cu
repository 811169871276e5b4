// stats_noalloc.cu -- final statistics without any device allocation.
//
// Who needs this: a host that cannot let a library allocate device memory.
// Examples are an application that hands all of the GPU's memory to its own
// pool allocator at start-up, or a tight loop that must not call cudaMalloc /
// cudaFree because those calls can synchronise the whole device.  Such a
// caller already holds the ES matrix and an output buffer on the device and
// only wants the statistics (ES, NES, NP, FWER, FDR) written into it.
//
// The statistics kernels need a little working memory (per-set factors,
// per-permutation extrema and FDR counters).  Here it lives in one
// file-scope __device__ array of kNoAllocScratchBytes (4 MiB) that every GPU
// loading this library holds until the process exits.  Host code cannot use
// the array's name as a device address, so the address is looked up with
// cudaGetSymbolAddress, with the device current, the first time the entry
// point runs on a device's context: the look-up is cached per device under
// the context's process-unique id (cuCtxGetId), so that a context that was
// reset (cudaDeviceReset) and re-created -- whose module, and with it the
// array, is loaded anew -- gets a fresh look-up instead of a stale address.
// Make the first call on a context before any stream capture.  All calls
// share the array and it keeps the previous call's
// contents: the counters that must start at zero are cleared on the stream
// by every call, and calls whose work overlaps on the GPU race on the array.
#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/gsea103.h"
#include "kernels.h"

namespace gsea {
void set_last_error(const char* msg);  // capi.cu
}

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_stats_scratch[kNoAllocScratchBytes];

std::mutex g_lock;
void* g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};  // context id of each cached address (0: none)

// the driver's cuCtxGetCurrent / cuCtxGetId, fetched through the runtime (no
// link against the driver library); null where the driver lacks them
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);
struct CtxFns {
    CtxGetCurrentFn current = nullptr;
    CtxGetIdFn id = nullptr;
};
const CtxFns& ctx_fns() {
    static const CtxFns fns = [] {
        CtxFns f;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.current = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.id = reinterpret_cast<CtxGetIdFn>(p);
        return f;
    }();
    return fns;
}

// process-unique id of the current context, 0 if unknown (no context yet, or
// a driver without cuCtxGetId: every call then looks the address up again)
unsigned long long current_context_id() {
    const CtxFns& f = ctx_fns();
    if (!f.current || !f.id) return 0;
    void* ctx = nullptr;
    if (f.current(&ctx) != 0 || !ctx) return 0;
    unsigned long long id = 0;
    return f.id(ctx, &id) == 0 ? id : 0;
}

int scratch_for_current_device(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        gsea::set_last_error(cudaGetErrorString(e));
        return GSEA_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        gsea::set_last_error("device ordinal beyond the fixed-scratch table");
        return GSEA_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> guard(g_lock);
    const unsigned long long ctx = current_context_id();
    if (!g_scratch_addr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_stats_scratch);  // creates the context if there is none yet
        if (e != cudaSuccess || !p) {
            gsea::set_last_error((std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
            return GSEA_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
        g_scratch_ctx[dev] = ctx != 0 ? ctx : current_context_id();
    }
    *out = g_scratch_addr[dev];
    return GSEA_OK;
}

}  // namespace

extern "C" int gsea_stats_device_noalloc(const void* es, int64_t num_sets, int64_t num_perms, int precision,
                                         void* stats, void* stream) {
    if (!es || !stats) {
        gsea::set_last_error("null device pointer");
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    if (num_sets < 1 || num_perms < 1 || num_sets > INT32_MAX || (precision != 32 && precision != 64)) {
        gsea::set_last_error("need num_sets >= 1, num_perms >= 1 and precision 32 or 64");
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    const size_t need = precision == 64 ? gsea::stats_scratch_bytes<double>((int)num_sets, num_perms)
                                        : gsea::stats_scratch_bytes<float>((int)num_sets, num_perms);
    if (need > kNoAllocScratchBytes) {
        gsea::set_last_error(("statistics of " + std::to_string(num_sets) + " sets x " + std::to_string(num_perms) +
                              " permutations need " + std::to_string(need) +
                              " bytes of scratch, more than the fixed 4 MiB of the allocation-free entry point")
                                 .c_str());
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    void* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = precision == 64
                        ? gsea::launch_stats<double>(static_cast<const double*>(es), (int)num_sets, num_perms,
                                                     static_cast<double*>(stats), scratch, st)
                        : gsea::launch_stats<float>(static_cast<const float*>(es), (int)num_sets, num_perms,
                                                    static_cast<float*>(stats), scratch, st);
    if (e != cudaSuccess) {
        gsea::set_last_error((std::string("statistics kernels: ") + cudaGetErrorString(e)).c_str());
        return GSEA_ERR_CUDA;
    }
    return GSEA_OK;
}
