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
// cudaGetSymbolAddress once per device, with that device current, the first
// time the entry point runs on it; make that first call before any stream
// capture.  All calls share the array and it keeps the previous call's
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
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_stats_scratch);
        if (e != cudaSuccess || !p) {
            gsea::set_last_error((std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
            return GSEA_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
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
