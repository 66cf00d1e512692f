// ref_gpu_compile.cu -- TEST INFRASTRUCTURE ONLY.
//
// One translation unit of the reference's own CUDA search path (index build,
// query compile, match_AT, heap_count_topk, knn) compiled for sm_103a from
// the reference tree where it lies (`make -C oracle ref_gpu`), to show that
// it builds offline with CUDA 13.  It is compiled only: it cannot run in the
// build container (no GPU) nor on the GPU machine (built objects are x86, and the
// reference tree is not there).
#include <cstdint>
#include <cstdarg>
#include <vector>
#include "genie/utility/Timing.cc"
#include "genie/table/inv_list.cc"
#include "genie/table/inv_table.cu"
#include "genie/query/query.cc"
#include "genie/matching/match_common.cu"
#include "genie/matching/heap_count.cu"
#include "genie/matching/match.cu"
#include "genie/matching/knn.cu"
