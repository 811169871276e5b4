// stats_device.cu -- final statistics of a device ES matrix with the caller's
// own scratch memory.
//
// The reference computes final_statistics on the host over the whole [K][P]
// matrix (src/include/statistics.cuh:46-117).  Here a caller that already
// holds the matrix on the device (a sharded run that gathered every rank's
// columns, a consumer of another pipeline) gets the same kernels as a plan's
// statistics stage.  The caller sizes the working memory with
// gsea_stats_scratch_bytes and passes it in, so there is no size limit beyond
// the device's memory and the library allocates nothing.
#include <cstdint>
#include <string>

#include "../../include/gsea103.h"
#include "kernels.h"

namespace gsea {
void set_last_error(const char* msg);  // capi.cu
}

namespace {

bool valid(int64_t K, int64_t P, int precision) {
    return K >= 1 && P >= 1 && K <= INT32_MAX && (precision == 32 || precision == 64);
}

size_t need_bytes(int64_t K, int64_t P, int precision) {
    return precision == 64 ? gsea::stats_scratch_bytes<double>((int)K, P)
                           : gsea::stats_scratch_bytes<float>((int)K, P);
}

}  // namespace

extern "C" int gsea_stats_scratch_bytes(int64_t num_sets, int64_t num_perms, int precision, size_t* bytes) {
    if (!bytes || !valid(num_sets, num_perms, precision)) {
        gsea::set_last_error("need num_sets >= 1, num_perms >= 1, precision 32 or 64 and an output pointer");
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    *bytes = need_bytes(num_sets, num_perms, precision);
    return GSEA_OK;
}

extern "C" int gsea_stats_device(const void* es, int64_t num_sets, int64_t num_perms, int precision, void* stats,
                                 void* scratch, size_t scratch_bytes, void* stream) {
    if (!es || !stats || !scratch) {
        gsea::set_last_error("null device pointer");
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    if (!valid(num_sets, num_perms, precision)) {
        gsea::set_last_error("need num_sets >= 1, num_perms >= 1 and precision 32 or 64");
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    if (reinterpret_cast<uintptr_t>(scratch) % 256 != 0) {
        gsea::set_last_error("scratch must be 256-byte aligned");
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    const size_t need = need_bytes(num_sets, num_perms, precision);
    if (scratch_bytes < need) {
        gsea::set_last_error(("statistics of " + std::to_string(num_sets) + " sets x " + std::to_string(num_perms) +
                              " permutations need " + std::to_string(need) + " bytes of scratch, " +
                              std::to_string(scratch_bytes) + " given")
                                 .c_str());
        return GSEA_ERR_INVALID_ARGUMENT;
    }
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
