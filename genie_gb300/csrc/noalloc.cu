// noalloc.cu -- a search entry point that allocates no memory at all.
//
// Who needs it: a caller whose device memory is owned by someone else -- a
// host framework or serving process that hands every allocation out of its
// own pool, or that runs with a hard memory budget -- may not call
// cudaMalloc, and cudaMalloc/cudaFree also synchronise the whole device,
// which a latency-critical caller cannot afford in the middle of its work.
// genie_search (capi.cu) grows its workspace with cudaMalloc on demand;
// genie_search_noalloc instead takes the workspace from one fixed array in
// this file that exists from the moment the library is loaded.
//
// The array is shared by every call in the process: it keeps the previous
// call's contents (everything a call reads is written earlier in the same
// call; the counters that must start at zero are cleared by the call), and
// two calls whose device work overlaps -- on two streams, or from two host
// threads -- would race on it.  Host calls are serialised here, and each call
// waits for its own device work before it returns.
#include "capi_internal.h"

#include <mutex>

namespace gg {
namespace {

// Largest batch one call accepts.
constexpr int64_t kNaMaxQueries = 1024;
constexpr int64_t kNaMaxItems = 262144;
constexpr int64_t kNaMaxUnits = 262144;     // the items, plus lists of queries with multi-list items
constexpr int64_t kNaMaxResults = 32768;    // sum of k over the batch

constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// Byte layout of the workspace inside the array.
struct NaLayout {
    size_t item_k0, item_nk, item_inc, span_start, span_len, inc, qinfo, work, ctr, qstate, done, lb,
        part_cnt, scratch, total;
};

constexpr NaLayout na_layout() {
    NaLayout L{};
    size_t o = 0;
    L.item_k0 = o;    o += align256(kNaMaxItems * 8);
    L.item_nk = o;    o += align256(kNaMaxItems * 4);
    L.item_inc = o;   o += align256(kNaMaxItems * 4);
    L.span_start = o; o += align256(kNaMaxUnits * 8);
    L.span_len = o;   o += align256(kNaMaxUnits * 8);
    L.inc = o;        o += align256(kNaMaxUnits * 4);
    L.qinfo = o;      o += align256(kNaMaxQueries * sizeof(QInfo));
    L.work = o;       o += align256((size_t)kNumLists * kNaMaxQueries * kMaxParts * sizeof(uint2));
    L.ctr = o;        o += align256(kCtrWords * 4);
    L.qstate = o;     o += align256(kNaMaxQueries * 4);
    L.done = o;       o += align256(kNaMaxQueries * 4);
    L.lb = o;         o += align256(kNaMaxQueries * 4);
    L.part_cnt = o;   o += align256(kNaMaxQueries * kMaxParts * 4);
    L.scratch = o;    o += align256(kNaMaxResults * kMaxParts * 8);
    L.total = o;
    return L;
}

constexpr NaLayout kNa = na_layout();
constexpr size_t kNaScratchBytes = 16u << 20;
static_assert(kNa.total <= kNaScratchBytes, "workspace layout exceeds the fixed scratch array");

// The fixed workspace: every GPU that loads this library holds these 16 MiB
// until the process exits.
static __device__ __align__(256) unsigned char g_search_scratch[kNaScratchBytes];

std::mutex g_na_mu;
void *g_na_ptr[64] = {};      // device address of g_search_scratch, per device

}  // namespace

void noalloc_forget(int dev) {
    std::lock_guard<std::mutex> g(g_na_mu);
    g_na_ptr[dev & 63] = nullptr;
}

}  // namespace gg

using namespace gg;

extern "C" int genie_search_noalloc(genie_index *ix, const genie_queries *q, const int64_t *out_off,
                                    int64_t n_items, int64_t total_k, uint32_t *out_ids, uint32_t *out_counts,
                                    float *out_scores, void *stream) {
    if (!ix || !q || !out_off || !out_ids || !out_counts)
        return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    if (q->n_queries < 0 || n_items < 0 || total_k < 0) return fail(GENIE_ERR_INVALID_ARG, "negative size");
    if (q->n_queries > kNaMaxQueries || n_items > kNaMaxItems || total_k > kNaMaxResults)
        return fail(GENIE_ERR_INVALID_ARG,
                    "genie_search_noalloc takes at most %lld queries, %lld items and %lld results per call "
                    "(got %d, %lld, %lld): its workspace is a fixed %zu-byte array",
                    (long long)kNaMaxQueries, (long long)kNaMaxItems, (long long)kNaMaxResults, q->n_queries,
                    (long long)n_items, (long long)total_k, (size_t)kNaScratchBytes);
    if (q->n_queries == 0) return GENIE_OK;
    if (ix->sub_shift >= 0)
        return fail(GENIE_ERR_NOT_IMPLEMENTED, "a subsequence index is searched through genie_search");
    if (!q->item_off || !q->dim || !q->low || !q->up) return fail(GENIE_ERR_INVALID_ARG, "NULL query arrays");
    if (!q->k && (q->uniform_k == 0 || q->uniform_k > (uint32_t)kMaxK))
        return fail(GENIE_ERR_INVALID_ARG, "uniform k must be in [1, %d]", kMaxK);
    std::lock_guard<std::mutex> g(g_na_mu);
    cudaError_t e = cudaSetDevice(ix->device);
    if (e) return cuda_fail(e, "cudaSetDevice");
    DeviceContext &ctx = device_context(ix->device);
    if (ctx.prepare_error) return cuda_fail(ctx.prepare_error, "kernel setup");
    // first call on this device: look up the array's device address (the
    // symbol name is only a host-side stand-in for it)
    void *&base_ptr = g_na_ptr[ix->device & 63];
    if (!base_ptr) {
        e = cudaGetSymbolAddress(&base_ptr, g_search_scratch);
        if (e) {
            base_ptr = nullptr;
            return cuda_fail(e, "cudaGetSymbolAddress of the search scratch");
        }
    }
    unsigned char *base = (unsigned char *)base_ptr;
    Work w;
    w.item_k0 = (int64_t *)(base + kNa.item_k0);
    w.item_nk = (uint32_t *)(base + kNa.item_nk);
    w.item_inc = (uint32_t *)(base + kNa.item_inc);
    w.span_start = (int64_t *)(base + kNa.span_start);
    w.span_len = (int64_t *)(base + kNa.span_len);
    w.inc = (uint32_t *)(base + kNa.inc);
    w.unit_key = nullptr;         // no tile directories: lists are searched per tile
    w.qinfo = (QInfo *)(base + kNa.qinfo);
    w.work = (uint2 *)(base + kNa.work);
    w.work_stride = kNaMaxQueries * kMaxParts;
    w.ctr = (uint32_t *)(base + kNa.ctr);
    w.qstate = (uint32_t *)(base + kNa.qstate);
    w.done = (uint32_t *)(base + kNa.done);
    w.lb = (uint32_t *)(base + kNa.lb);
    w.part_cnt = (uint32_t *)(base + kNa.part_cnt);
    w.scratch = (uint64_t *)(base + kNa.scratch);
    w.max_parts = kMaxParts;      // the fixed array holds 16 part results per result slot
    w.out_ids = out_ids;
    w.out_counts = out_counts;
    w.out_scores = out_scores;
    w.units_cap = kNaMaxUnits;
    // the plan kernel holds every query to these (item_off[n_queries] <=
    // n_items, out_off[q] + k[q] <= total_k) before anything is written, so a
    // device array that disagrees with the host sizes is an error, not a fault
    w.items_cap = n_items;
    w.q_cap = kNaMaxQueries;
    w.out_cap = total_k;
    DevQueries dq;
    dq.n_queries = q->n_queries;
    dq.item_off = q->item_off;
    dq.dim = q->dim;
    dq.low = q->low;
    dq.up = q->up;
    dq.weight = q->weighted ? q->weight : nullptr;
    dq.weighted = q->weight ? q->weighted : nullptr;
    dq.k = q->k;
    dq.uniform_k = q->uniform_k;
    dq.out_off = out_off;
    dq.dyn = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    // the work counters must start at zero (launch_match clears them); the
    // per-query completion counters are reset by the plan kernel
    launch_match(ix->dev, dq, w, ix->tuning, ctx.num_sms, s);
    if ((e = cudaGetLastError())) return cuda_fail(e, "search launch");
    uint32_t err = 0;
    if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "search");
    if ((e = cudaMemcpy(&err, w.ctr + kCtrError, 4, cudaMemcpyDeviceToHost))) return cuda_fail(e, "error word");
    return check_device_error(err);
}
