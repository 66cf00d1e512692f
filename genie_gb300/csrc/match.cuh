// match.cuh -- host-side entry points of the match path (match.cu).
#pragma once
#include "device.cuh"

#include <cstddef>

namespace gg {

Tuning default_tuning();
// First out-of-bounds report of a build with -DGG_CHECKED: site, index,
// bound, block<<32|thread (zeros when nothing was reported or unchecked).
void read_oob(unsigned long long out[4]);
size_t sparse_smem_bytes(const Tuning &t, bool packed);
size_t dense_smem_bytes(const Tuning &t, bool small);
cudaError_t prepare_kernels(const Tuning &t);
// Allow the largest dynamic shared memory on every match kernel (once per device).
cudaError_t prepare_kernels_max();

// Enqueue plan + bitmap + sparse + dense kernels for one batch on stream s.
// All pointers in Q and W are device pointers; W arrays are sized for Q.
// Returns the number of kernel launches issued.  With `ev` (5 events), event
// i+1 is recorded after stage i: plan, bitmap, sparse (both slot widths),
// dense (both counter widths); event 0 before the plan.
constexpr int kStages = 4;
// Whether the bitmap kernel's shared memory fits an id space of n objects.
bool bitmap_fits(const Tuning &t, int64_t n_objects);
int launch_match(const DevIndex &ix, const DevQueries &Q, const Work &W, const Tuning &t,
                 int num_sms, cudaStream_t s, cudaEvent_t *ev = nullptr);

}  // namespace gg
