// ref_gpu_prelude.h -- TEST INFRASTRUCTURE ONLY (forced include).
//
// The reference's matching sources (src/genie/matching/{match,knn,
// heap_count}.cu) say `using namespace thrust;` at file scope.  With the
// CCCL of CUDA 13 that makes `cub` ambiguous in the code nvcc generates, so
// they do not compile as shipped.  This header, force-included before them,
// includes the thrust headers they use and then makes `thrust` name a
// namespace that re-exports only the names they take from it; the sources
// themselves stay as they lie in the reference tree.
#pragma once
#include <thrust/copy.h>
#include <thrust/count.h>
#include <thrust/device_vector.h>
#include <thrust/fill.h>
#include <thrust/host_vector.h>
#include <thrust/system_error.h>
namespace genie_ref_thrust {
using ::thrust::copy;
using ::thrust::count;
using ::thrust::device_vector;
using ::thrust::fill;
using ::thrust::host_vector;
using ::thrust::raw_pointer_cast;
namespace system = ::thrust::system;
}  // namespace genie_ref_thrust
#define thrust genie_ref_thrust
