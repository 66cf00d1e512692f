// genie/utility/cuda_macros.h -- CUDA status checks of the legacy interface
// (reference src/genie/utility/cuda_macros.h:23-33): a failed call throws
// genie::exception::gpu_runtime_error naming the file and line.
#ifndef GENIE_UTILITY_CUDAMACROS_H_
#define GENIE_UTILITY_CUDAMACROS_H_

#include <cuda_runtime.h>

#include <string>

#include <genie/exception/exception.h>

namespace genie {
namespace utility {
inline void cuda_check(cudaError_t err, const char *file, int line) {
    if (err != cudaSuccess)
        throw genie::exception::gpu_runtime_error(std::string(cudaGetErrorString(err)) + " at " + file + ":" +
                                                  std::to_string(line));
}
}  // namespace utility
}  // namespace genie

#define cudaCheckErrors(err) genie::utility::cuda_check((err), __FILE__, __LINE__)
#define CUDA_CHECK_ERROR(err) genie::utility::cuda_check((err), __FILE__, __LINE__)
#define CUDA_LAST_ERROR() genie::utility::cuda_check(cudaGetLastError(), __FILE__, __LINE__)

#endif
