// capi_internal.h -- host-side state behind the C ABI handles.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/genie_gb300.h"
#include "host_index.h"
#include "match.cuh"

namespace gg {

int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

// One growable device allocation.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t want);
    void release();
};

struct DeviceContext {
    bool ready = false;
    int num_sms = 0;
    cudaError_t prepare_error = cudaSuccess;
    Tuning tuning;
};
DeviceContext &device_context(int dev);

// Device buffers of one in-flight search (query inputs, plan, work lists,
// part scratch, results), grown on demand.
struct Workspace {
    DevBuf item_off, dim, low, up, weight, weighted, k, out_off;
    DevBuf item_k0, item_nk, item_inc;
    DevBuf span_start, span_len, inc, qinfo, work, ctr, qstate, done, lb, part_cnt, scratch;
    DevBuf out_ids, out_counts, out_scores;
    DevBuf counters;                 // per-object counters of a subsequence search
    DevBuf unit_key;
    bool done_zeroed = false;
    int64_t done_q = 0;
    cudaError_t reserve(int64_t Q, int64_t items, int64_t units, int64_t sumk);
    void release();
    Work view(int64_t Q, bool scores) const;
};

int validate_queries(const genie_queries *q, std::vector<int64_t> &out_off, int64_t &n_items);

// The device view of an index for a tuning: ix->dev plus the tile
// directories of the tuning's two tile sizes (built on first use).
DevIndex index_view(genie_index *ix, const Tuning &t);

// Asynchronous steps of one batch for the serving loop (batch.cu): stage,
// launch and download on the batch's own stream; poll; copy the results out.
int batch_submit_async(genie_batch *b, const genie_queries *q, bool scores);
int batch_ready(genie_batch *b);      // 1 done, 0 still running, < 0 a CUDA error
int batch_collect(genie_batch *b, uint32_t *ids, uint32_t *counts, float *scores);
int check_device_error(uint32_t err);
// Drop the fixed workspace's cached device address of a device (after a reset).
void noalloc_forget(int dev);
// Search of a subsequence index (subseq.cu), on ix->stream; waits when sync.
int subseq_search(genie_index *ix, const genie_queries *q, const std::vector<int64_t> &out_off, int64_t n_items,
                  uint32_t *out_ids, uint32_t *out_counts, float *out_scores, bool sync);
int64_t count_units(const HostIndex &h, const genie_queries *q);

}  // namespace gg

namespace gg {
// Device arrays and view of an index from its host mirror; with device_ids
// >= 0 the ids and key offsets are on the device already (device build).
int upload_index(genie_index *ix, int64_t device_ids = -1);
int finish_index_create(genie_index *ix, genie_index **out, int64_t device_ids = -1);
// Device build of a one-value-per-object index (build_index.cu); *used is
// false when a dim's value range needs the host builder.
int build_device_index(const int32_t *values, int64_t n, int32_t d, genie_index *ix, bool *used);
}  // namespace gg

struct genie_index {
    int device = 0;
    bool is_bag = false;
    int32_t sub_shift = -1;          // subsequence index: ids are rowID << sub_shift | offset (-1: not one)
    gg::HostIndex host;              // host mirror: bounds and key offsets (ids live on the device)
    int64_t n_ids = 0;
    int32_t codec = 0;
    int32_t max_seg = 0;
    int64_t n_words = 0;
    int64_t n_segs = 0;
    gg::DevBuf d_ids, d_key_off, d_key_base, d_dim_min, d_dim_max;
    gg::DevBuf d_words, d_key_seg, d_seg_word_off, d_seg_first, d_seg_len;
    gg::DevIndex dev{};
    gg::Tuning tuning{};
    // tile directories (tile_dir.cu), built on first use per tile size and
    // kept while the index lives
    std::mutex dir_mu;
    bool dir_rows_ready = false;
    int64_t dir_rows = -1;
    gg::DevBuf d_dir_slot, d_dir_row_key;
    bool bm_ready = false;
    int64_t bm_words = 0;
    gg::DevBuf d_bm_slot, d_bm_rows;
    std::vector<std::pair<int32_t, gg::DevBuf *>> dirs;
    cudaStream_t stream = nullptr;
    std::mutex mu;                   // serialises searches on this handle's workspace
    gg::Workspace ws;
    uint32_t *host_err = nullptr;    // pinned error word of the last search
    int last_launches = 0;
    ~genie_index();
};
