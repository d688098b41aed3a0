// errors.cpp -- error texts (the meanings of MatlabInterface.cu:24-272, getErrorMsg).
#include <mutex>
#include <string>

#include "sstmc_internal.h"

namespace sstmc {

namespace {
std::mutex g_mu;
std::string g_last;
}  // namespace

void set_last_error_text(const std::string& s)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_last = s;
}

}  // namespace sstmc

extern "C" const char* sstmc_error_string(int32_t code)
{
    switch (code) {
    case SSTMC_NO_ERROR: return "No error.";
    case SSTMC_DEVICE_ERROR: return "Bad device number or device failure.";
    case SSTMC_ALLOCATION_ERROR: return "Allocation error: CPU / GPU exceed maximal memory. Try to decrease batchSize.";
    case SSTMC_KERNEL_ERROR: return "Error occurred during a kernel operation.";
    case SSTMC_CUBLAS_ERROR: return "Error occurred during the illumination x view contraction.";
    case SSTMC_NOT_SUPPORTED: return "Illumination and view combination is not supported.";
    case SSTMC_MISC_ERROR: return "Unknown error.";
    case SSTMC_KERNEL_ERROR_HetroMedium_heterogeneousAttenuationKernel:
        return "Error occurred during a kernel operation. HetroMedium_heterogeneousAttenuationKernel.";
    case SSTMC_KERNEL_ERROR_HetroMedium_heterogeneousSampleKernel:
        return "Error occurred during a kernel operation. HetroMedium_heterogeneousSampleKernel.";
    case SSTMC_INVALID_CONFIG: return "Invalid configuration.";
    case SSTMC_TIMEOUT: return "A bounded wait ran out.";
    case SSTMC_CANCELLED: return "The request was cancelled.";
    case SSTMC_INVALID_HANDLE: return "Invalid handle.";
    case SSTMC_PATH_LIMIT: return "A path exceeded the vertex or first-vertex retry limit.";
    case SSTMC_SCRATCH_LIMIT: return "The request does not fit the 64 MiB static scratch of sstmc_render_static; use sstmc_render.";
    default: return "Unknown error code.";
    }
}

extern "C" const char* sstmc_last_error_text(void)
{
    std::lock_guard<std::mutex> lk(sstmc::g_mu);
    return sstmc::g_last.c_str();
}
