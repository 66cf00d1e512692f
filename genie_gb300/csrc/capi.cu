// capi.cu -- the C ABI (include/genie_gb300.h): resident indexes, the plain
// per-batch search, index persistence.  Every entry point returns a
// genie_status; the message of the last failure is kept per thread.
#include "../../include/genie_gb300.h"
#include "capi_internal.h"

#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace gg {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? GENIE_ERR_GPU_ALLOC : GENIE_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

cudaError_t DevBuf::reserve(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    size_t b = want + want / 4 + 256;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    return e;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

namespace {
DeviceContext g_ctx[64];
std::mutex g_ctx_mu;
}  // namespace

DeviceContext &device_context(int dev) {
    std::lock_guard<std::mutex> g(g_ctx_mu);
    DeviceContext &c = g_ctx[dev & 63];
    if (!c.ready) {
        cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, dev);
        c.tuning = default_tuning();
        c.prepare_error = prepare_kernels_max();
        c.ready = true;
    }
    return c;
}

cudaError_t Workspace::reserve(int64_t Q, int64_t items, int64_t units, int64_t sumk) {
    cudaError_t e;
#define RES(buf, n) if ((e = buf.reserve((size_t)(n))) != cudaSuccess) return e
    RES(item_off, (Q + 1) * 8);
    RES(dim, items * 4 + 16);
    RES(low, items * 4 + 16);
    RES(up, items * 4 + 16);
    RES(weight, items * 4 + 16);
    RES(weighted, Q + 16);
    RES(k, Q * 4 + 16);
    RES(out_off, (Q + 1) * 8);
    RES(item_k0, items * 8 + 16);
    RES(item_nk, items * 4 + 16);
    RES(item_inc, items * 4 + 16);
    RES(span_start, units * 8 + 16);
    RES(span_len, units * 8 + 16);
    RES(inc, units * 4 + 16);
    RES(unit_key, units * 4 + 16);
    RES(qinfo, Q * sizeof(QInfo) + 16);
    RES(work, (size_t)kNumLists * Q * kMaxParts * sizeof(uint2) + 16);
    RES(ctr, kCtrWords * 4);
    RES(qstate, Q * 4 + 16);
    RES(done, Q * 4 + 16);
    RES(lb, Q * 4 + 16);
    RES(part_cnt, Q * kMaxDenseParts * 4 + 16);
    RES(scratch, sumk * kMaxDenseParts * 8 + 16);
    RES(out_ids, sumk * 4 + 16);
    RES(out_counts, sumk * 4 + 16);
    RES(out_scores, sumk * 4 + 16);
#undef RES
    if (!done_zeroed || done_q < Q) {
        cudaMemset(done.p, 0, done.bytes);
        done_zeroed = true;
        done_q = Q;
    }
    return cudaSuccess;
}

void Workspace::release() {
    DevBuf *all[] = {&item_off, &dim, &low, &up, &weight, &weighted, &k, &out_off, &item_k0, &item_nk,
                     &item_inc, &span_start,
                     &span_len, &inc, &qinfo, &work, &ctr, &qstate, &done, &lb, &part_cnt, &scratch,
                     &out_ids, &out_counts, &out_scores, &counters, &unit_key};
    for (DevBuf *b : all) b->release();
}

Work Workspace::view(int64_t Q, bool scores) const {
    Work w;
    w.item_k0 = (int64_t *)item_k0.p;
    w.item_nk = (uint32_t *)item_nk.p;
    w.item_inc = (uint32_t *)item_inc.p;
    w.span_start = (int64_t *)span_start.p;
    w.span_len = (int64_t *)span_len.p;
    w.inc = (uint32_t *)inc.p;
    w.unit_key = (uint32_t *)unit_key.p;
    w.qinfo = (QInfo *)qinfo.p;
    w.work = (uint2 *)work.p;
    w.work_stride = Q * kMaxParts;
    w.ctr = (uint32_t *)ctr.p;
    w.qstate = (uint32_t *)qstate.p;
    w.done = (uint32_t *)done.p;
    w.lb = (uint32_t *)lb.p;
    w.part_cnt = (uint32_t *)part_cnt.p;
    w.scratch = (uint64_t *)scratch.p;
    w.max_parts = kMaxDenseParts;
    w.out_ids = (uint32_t *)out_ids.p;
    w.out_counts = (uint32_t *)out_counts.p;
    w.out_scores = scores ? (float *)out_scores.p : nullptr;
    w.units_cap = (int64_t)(span_len.bytes / 8);
    w.items_cap = (int64_t)(item_nk.bytes / 4);
    w.q_cap = Q;
    w.out_cap = (int64_t)(out_ids.bytes / 4);
    return w;
}

// Host-side validation shared by every search entry point.
int validate_queries(const genie_queries *q, std::vector<int64_t> &out_off, int64_t &n_items) {
    if (!q) return fail(GENIE_ERR_INVALID_ARG, "queries is NULL");
    if (q->n_queries < 0) return fail(GENIE_ERR_INVALID_ARG, "n_queries < 0");
    const int64_t Q = q->n_queries;
    out_off.assign(Q + 1, 0);
    n_items = 0;
    if (Q == 0) return GENIE_OK;
    if (!q->item_off || !q->dim || !q->low || !q->up)
        return fail(GENIE_ERR_INVALID_ARG, "item_off/dim/low/up must not be NULL");
    if (q->item_off[0] != 0) return fail(GENIE_ERR_INVALID_ARG, "item_off[0] must be 0");
    for (int64_t i = 0; i < Q; ++i) {
        if (q->item_off[i + 1] < q->item_off[i]) return fail(GENIE_ERR_INVALID_ARG, "item_off not monotone at %lld", (long long)i);
        const uint32_t k = q->k ? q->k[i] : q->uniform_k;
        if (k == 0) return fail(GENIE_ERR_INVALID_ARG, "K should be larger than 0 (query %lld)", (long long)i);
        if (k > (uint32_t)kMaxK) return fail(GENIE_ERR_INVALID_ARG, "k=%u exceeds the supported maximum %d", k, kMaxK);
        out_off[i + 1] = out_off[i] + k;
    }
    n_items = q->item_off[Q];
    if (q->weighted) {
        if (!q->weight) return fail(GENIE_ERR_INVALID_ARG, "weighted queries need weights");
        for (int64_t i = 0; i < Q; ++i) {
            if (!q->weighted[i]) continue;
            for (int64_t t = q->item_off[i]; t < q->item_off[i + 1]; ++t) {
                const float w = q->weight[t];
                if (!(w > 0.0f) || !std::isfinite(w))
                    return fail(GENIE_ERR_INVALID_ARG, "weight of item %lld is not finite and > 0", (long long)t);
            }
        }
    }
    return GENIE_OK;
}

// Units a batch may need: a query whose items each cover at most one
// (dim,value) list uses its items as units; any other takes one unit per
// covered list past the batch's items.  So the item count, plus for a batch
// with range items the lists they cover (a bound).  Exact-match items (up is
// the low array) cover one list at most.
int64_t count_units(const HostIndex &h, const genie_queries *q) {
    int64_t units = 0;
    const int64_t n = q->n_queries > 0 ? q->item_off[q->n_queries] : 0;
    if (q->up == q->low) return n;
    for (int64_t i = 0; i < n; ++i) {
        const int32_t d = q->dim[i];
        if (d < 0 || d >= h.n_dims) continue;
        const int64_t lo = std::max<int64_t>(q->low[i], h.dim_min[d]);
        const int64_t hi = std::min<int64_t>(q->up[i], h.dim_max[d]);
        if (hi >= lo) units += hi - lo + 1;
    }
    return n + units;
}

int check_device_error(uint32_t err) {
    unsigned long long oob[4];
    read_oob(oob);
    if (oob[0])
        return fail(GENIE_ERR_CUDA, "checked build: index out of bounds at site %llu: %llu >= %llu (block %llu thread %llu)",
                    oob[0], oob[1], oob[2], oob[3] >> 32, oob[3] & 0xffffffffull);
    if (err & kErrWeight) return fail(GENIE_ERR_INVALID_ARG, "a weighted query holds a weight that is not finite and > 0");
    if (err & kErrCapacity) return fail(GENIE_ERR_INVALID_ARG, "k outside [1, %d]", kMaxK);
    if (err & kErrTimeout)
        return fail(GENIE_ERR_DEVICE_TIMEOUT, "a bounded device wait ran out of time");
    if (err & kErrBounds)
        return fail(GENIE_ERR_INVALID_ARG, "a query's items or result slots lie outside the batch's arrays "
                                           "(item_off or out_off and k disagree with the sizes passed)");
    if (err & kErrUnits)
        return fail(GENIE_ERR_INVALID_ARG, "the batch's items cover more (dim,value) lists than its unit capacity");
    if (err) return fail(GENIE_ERR_CUDA, "device reported error flags 0x%x", err);
    return GENIE_OK;
}

// Upload a host CSR and fill the device view.
int upload_index(genie_index *ix, int64_t device_ids) {
    const HostIndex &h = ix->host;
    cudaError_t e;
    if (device_ids < 0) {       // ids and key offsets come from the host mirror
        // padded: a warp reads 32 ids from any list position, and the padding
        // (zeros) holds valid ids
        const size_t ids_bytes = h.ids.size() * 4 + kIdsPadBytes;
        if ((e = ix->d_ids.reserve(ids_bytes))) return cuda_fail(e, "index ids");
        if ((e = cudaMemset(ix->d_ids.p, 0, ids_bytes))) return cuda_fail(e, "index ids");
        if (!h.ids.empty() && (e = cudaMemcpy(ix->d_ids.p, h.ids.data(), h.ids.size() * 4, cudaMemcpyHostToDevice)))
            return cuda_fail(e, "index ids upload");
        if ((e = ix->d_key_off.reserve(h.key_off.size() * 8))) return cuda_fail(e, "key offsets");
        if ((e = cudaMemcpy(ix->d_key_off.p, h.key_off.data(), h.key_off.size() * 8, cudaMemcpyHostToDevice)))
            return cuda_fail(e, "key offsets upload");
    }
    if ((e = ix->d_key_base.reserve(h.key_base.size() * 8))) return cuda_fail(e, "key base");
    if ((e = cudaMemcpy(ix->d_key_base.p, h.key_base.data(), h.key_base.size() * 8, cudaMemcpyHostToDevice)))
        return cuda_fail(e, "key base upload");
    if ((e = ix->d_dim_min.reserve(h.dim_min.size() * 4))) return cuda_fail(e, "dim min");
    if ((e = cudaMemcpy(ix->d_dim_min.p, h.dim_min.data(), h.dim_min.size() * 4, cudaMemcpyHostToDevice)))
        return cuda_fail(e, "dim min upload");
    if ((e = ix->d_dim_max.reserve(h.dim_max.size() * 4))) return cuda_fail(e, "dim max");
    if ((e = cudaMemcpy(ix->d_dim_max.p, h.dim_max.data(), h.dim_max.size() * 4, cudaMemcpyHostToDevice)))
        return cuda_fail(e, "dim max upload");
    ix->n_ids = device_ids < 0 ? (int64_t)h.ids.size() : device_ids;
    DevIndex &d = ix->dev;
    memset(&d, 0, sizeof(d));
    d.ids = (const uint32_t *)ix->d_ids.p;
    d.key_off = (const int64_t *)ix->d_key_off.p;
    d.key_base = (const int64_t *)ix->d_key_base.p;
    d.dim_min = (const int32_t *)ix->d_dim_min.p;
    d.dim_max = (const int32_t *)ix->d_dim_max.p;
    d.n_objects = h.n_objects;
    d.n_ids = ix->n_ids;
    d.n_dims = h.n_dims;
    d.mult_max = h.mult_max;
    d.is_bag = ix->is_bag ? 1 : 0;
    return GENIE_OK;
}

int finish_index_create(genie_index *ix, genie_index **out, int64_t device_ids) {
    int rc = upload_index(ix, device_ids);
    if (rc) {
        delete ix;
        return rc;
    }
    std::vector<uint32_t>().swap(ix->host.ids);   // the device copy is authoritative
    cudaError_t e = cudaStreamCreateWithFlags(&ix->stream, cudaStreamNonBlocking);
    if (e) {
        delete ix;
        return cuda_fail(e, "stream");
    }
    *out = ix;
    return GENIE_OK;
}

int finish_loaded_index(genie_index *ix, genie_index **out) {
    std::vector<uint32_t>().swap(ix->host.ids);
    cudaError_t e = cudaStreamCreateWithFlags(&ix->stream, cudaStreamNonBlocking);
    if (e) {
        delete ix;
        return cuda_fail(e, "stream");
    }
    *out = ix;
    return GENIE_OK;
}

int run_search(genie_index *ix, const genie_queries *q, const std::vector<int64_t> &out_off, int64_t n_items,
               uint32_t *out_ids, uint32_t *out_counts, float *out_scores, bool sync) {
    if (ix->sub_shift >= 0) return subseq_search(ix, q, out_off, n_items, out_ids, out_counts, out_scores, sync);
    const int64_t Q = q->n_queries;
    const int64_t sumk = out_off[Q];
    Workspace &ws = ix->ws;
    cudaError_t e = ws.reserve(Q, n_items, count_units(ix->host, q), sumk);
    if (e) return cuda_fail(e, "search workspace");
    cudaStream_t s = ix->stream;
#define H2D(dst, src, n) if ((n) > 0 && (e = cudaMemcpyAsync(dst, src, (size_t)(n), cudaMemcpyHostToDevice, s))) return cuda_fail(e, "query upload")
    H2D(ws.item_off.p, q->item_off, (Q + 1) * 8);
    H2D(ws.dim.p, q->dim, n_items * 4);
    H2D(ws.low.p, q->low, n_items * 4);
    H2D(ws.up.p, q->up, n_items * 4);
    const bool has_w = q->weighted && q->weight;
    if (has_w) {
        H2D(ws.weight.p, q->weight, n_items * 4);
        H2D(ws.weighted.p, q->weighted, Q);
    }
    if (q->k) H2D(ws.k.p, q->k, Q * 4);
    H2D(ws.out_off.p, out_off.data(), (Q + 1) * 8);
#undef H2D
    DevQueries dq;
    dq.n_queries = (int32_t)Q;
    dq.item_off = (const int64_t *)ws.item_off.p;
    dq.dim = (const int32_t *)ws.dim.p;
    dq.low = (const int32_t *)ws.low.p;
    dq.up = (const int32_t *)ws.up.p;
    dq.weight = has_w ? (const float *)ws.weight.p : nullptr;
    dq.weighted = has_w ? (const uint8_t *)ws.weighted.p : nullptr;
    dq.k = q->k ? (const uint32_t *)ws.k.p : nullptr;
    dq.uniform_k = q->uniform_k;
    dq.out_off = (const int64_t *)ws.out_off.p;
    dq.dyn = nullptr;
    Work w = ws.view(Q, out_scores != nullptr);
    DeviceContext &ctx = device_context(ix->device);
    ix->last_launches = launch_match(index_view(ix, ix->tuning), dq, w, ix->tuning, ctx.num_sms, s);
    if ((e = cudaGetLastError())) return cuda_fail(e, "match launch");
    if ((e = cudaMemcpyAsync(ix->host_err, w.ctr + kCtrError, 4, cudaMemcpyDeviceToHost, s))) return cuda_fail(e, "error word");
    if ((e = cudaMemcpyAsync(out_ids, w.out_ids, sumk * 4, cudaMemcpyDeviceToHost, s))) return cuda_fail(e, "result ids");
    if ((e = cudaMemcpyAsync(out_counts, w.out_counts, sumk * 4, cudaMemcpyDeviceToHost, s))) return cuda_fail(e, "result counts");
    if (out_scores && (e = cudaMemcpyAsync(out_scores, w.out_scores, sumk * 4, cudaMemcpyDeviceToHost, s)))
        return cuda_fail(e, "result scores");
    if (!sync) return GENIE_OK;
    if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "search");
    return check_device_error(*ix->host_err);
}

}  // namespace gg

using namespace gg;

genie_index::~genie_index() {
    cudaSetDevice(device);
    if (stream) cudaStreamDestroy(stream);
    d_ids.release(); d_key_off.release(); d_key_base.release(); d_dim_min.release(); d_dim_max.release();
    d_words.release(); d_key_seg.release(); d_seg_word_off.release(); d_seg_first.release(); d_seg_len.release();
    ws.release();
    d_dir_slot.release();
    d_dir_row_key.release();
    d_bm_slot.release();
    d_bm_rows.release();
    for (auto &d : dirs) {
        d.second->release();
        delete d.second;
    }
    if (host_err) cudaFreeHost(host_err);
}

extern "C" {

const char *genie_last_error(void) { return g_last_error.c_str(); }

int genie_version(void) { return 1 * 10000 + 0 * 100 + 0; }

int genie_device_reset(void) {
    int dev = 0;
    cudaGetDevice(&dev);
    const cudaError_t e = cudaDeviceReset();
    {   // the kernels' shared-memory settings went with the context: prepare them again on next use
        std::lock_guard<std::mutex> g(g_ctx_mu);
        g_ctx[dev & 63] = DeviceContext();
    }
    noalloc_forget(dev);
    return e ? cuda_fail(e, "cudaDeviceReset") : GENIE_OK;
}

int genie_init(int device) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= n) return fail(GENIE_ERR_INVALID_ARG, "device %d not present (%d devices)", device, n);
    if ((e = cudaSetDevice(device))) return cuda_fail(e, "cudaSetDevice");
    device_context(device);
    return GENIE_OK;
}

static genie_index *new_index() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (device_context(dev).prepare_error != cudaSuccess) return nullptr;
    genie_index *ix = new genie_index();
    ix->device = dev;
    ix->tuning = device_context(dev).tuning;
    cudaMallocHost((void **)&ix->host_err, 16);
    return ix;
}

int genie_index_create(const int32_t *values, int64_t n_objects, int32_t n_dims, genie_index **out) {
    return genie_index_create_with(values, n_objects, n_dims, GENIE_BUILD_AUTO, out);
}

int genie_index_create_with(const int32_t *values, int64_t n_objects, int32_t n_dims, int32_t where,
                            genie_index **out) {
    if (!out) return fail(GENIE_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!values || n_objects <= 0 || n_dims <= 0) return fail(GENIE_ERR_INVALID_ARG, "no data input");
    if (where < GENIE_BUILD_AUTO || where > GENIE_BUILD_DEVICE) return fail(GENIE_ERR_INVALID_ARG, "unknown builder");
    if (n_objects > (int64_t)UINT32_MAX) return fail(GENIE_ERR_INVALID_ARG, "index build failed (N must be < 2^32)");
    genie_index *ix = new_index();
    if (!ix) return cuda_fail(device_context(0).prepare_error, "kernel setup");
    if (where != GENIE_BUILD_HOST) {
        bool used = false;
        const int rc = build_device_index(values, n_objects, n_dims, ix, &used);
        if (rc) {
            delete ix;
            return rc;
        }
        if (used) return finish_index_create(ix, out, n_objects * (int64_t)n_dims);
        if (where == GENIE_BUILD_DEVICE) {
            delete ix;
            return fail(GENIE_ERR_NOT_IMPLEMENTED, "device build: a dim spans more than 16384 values");
        }
    }
    if (!build_host_index(values, n_objects, n_dims, ix->host)) {
        delete ix;
        return fail(GENIE_ERR_INVALID_ARG, "index build failed (N must be < 2^32)");
    }
    return finish_index_create(ix, out);
}

int genie_index_create_bag(const int32_t *values, const int64_t *row_off, int64_t n_objects, genie_index **out) {
    if (!out) return fail(GENIE_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!values || !row_off || n_objects <= 0) return fail(GENIE_ERR_INVALID_ARG, "no data input");
    genie_index *ix = new_index();
    if (!ix) return cuda_fail(device_context(0).prepare_error, "kernel setup");
    if (!build_host_index_bag(values, row_off, n_objects, ix->host)) {
        delete ix;
        return fail(GENIE_ERR_INVALID_ARG, "bag index build failed");
    }
    ix->is_bag = true;
    return finish_index_create(ix, out);
}

int genie_index_device_ids(const genie_index *ix, const uint32_t **ids) {
    if (!ix || !ids) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    *ids = ix->dev.ids;
    return GENIE_OK;
}

int genie_index_destroy(genie_index *ix) {
    delete ix;
    return GENIE_OK;
}

int genie_index_get_info(const genie_index *ix, genie_index_info *out) {
    if (!ix || !out) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    out->n_objects = ix->host.n_objects;
    out->n_dims = ix->host.n_dims;
    out->codec = ix->codec;
    out->n_ids = ix->n_ids;
    out->n_keys = ix->host.n_keys();
    out->n_words = ix->n_words;
    out->n_segments = ix->n_segs;
    out->max_multiplicity = ix->host.mult_max;
    out->max_segment = ix->max_seg;
    out->device_bytes = (int64_t)(ix->d_ids.bytes + ix->d_key_off.bytes + ix->d_key_base.bytes + ix->d_dim_min.bytes +
                                  ix->d_dim_max.bytes + ix->d_words.bytes + ix->d_key_seg.bytes +
                                  ix->d_seg_word_off.bytes + ix->d_seg_first.bytes + ix->d_seg_len.bytes);
    return GENIE_OK;
}

int genie_index_copy_out(const genie_index *ix, uint32_t *ids, int64_t *key_offsets, int64_t *key_base,
                         int32_t *dim_min, int32_t *dim_max) {
    if (!ix) return fail(GENIE_ERR_INVALID_ARG, "index is NULL");
    cudaSetDevice(ix->device);
    const HostIndex &h = ix->host;
    if (ids && ix->n_ids) {
        if (ix->codec) return fail(GENIE_ERR_INVALID_ARG, "a compressed index keeps no plain posting array on the device");
        cudaError_t e = cudaMemcpy(ids, ix->d_ids.p, ix->n_ids * 4, cudaMemcpyDeviceToHost);
        if (e) return cuda_fail(e, "ids download");
    }
    if (key_offsets) memcpy(key_offsets, h.key_off.data(), h.key_off.size() * 8);
    if (key_base) memcpy(key_base, h.key_base.data(), h.key_base.size() * 8);
    if (dim_min) memcpy(dim_min, h.dim_min.data(), h.dim_min.size() * 4);
    if (dim_max) memcpy(dim_max, h.dim_max.data(), h.dim_max.size() * 4);
    return GENIE_OK;
}

int genie_index_item_span(const genie_index *ix, int32_t dim, int32_t low, int32_t up, int64_t *start, int64_t *end) {
    if (!ix || !start || !end) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    item_span(ix->host, dim, low, up, *start, *end);
    return GENIE_OK;
}

int genie_index_adaptive_range(const genie_index *ix, int32_t dim, float selectivity, int32_t *low, int32_t *up) {
    if (!ix || !low || !up) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    adaptive_range(ix->host, dim, selectivity, *low, *up);
    return GENIE_OK;
}

// ---------------------------------------------------------------- match registry
//
// The match function of each codec id, as the reference keeps a
// COMPRESSION_TYPE -> MatchIntegratedFunPtr map (compression/
// DeviceCodecFactory.h:23-30, DeviceCodecFactory.cu:48-70) that knn() looks up
// for a table's codec (matching/knn.cu:130-140).  An empty entry means the
// built-in path (plain kernels, or the fused warp decoders of the codec).

namespace {
struct MatchEntry {
    genie_match_fn fn = nullptr;
    void *user = nullptr;
};
MatchEntry g_match[GENIE_N_CODECS];
std::mutex g_match_mu;

bool registered_match(int32_t codec, MatchEntry &out) {
    if (codec < 0 || codec >= GENIE_N_CODECS) return false;
    std::lock_guard<std::mutex> g(g_match_mu);
    out = g_match[codec];
    return out.fn != nullptr;
}
}  // namespace

int genie_codec_set_match(int32_t codec, genie_match_fn fn, void *user) {
    if (codec < 0 || codec >= GENIE_N_CODECS) return fail(GENIE_ERR_INVALID_ARG, "unknown codec %d", codec);
    std::lock_guard<std::mutex> g(g_match_mu);
    g_match[codec].fn = fn;
    g_match[codec].user = fn ? user : nullptr;
    return GENIE_OK;
}

int genie_codec_get_match(int32_t codec, genie_match_fn *fn, void **user) {
    if (codec < 0 || codec >= GENIE_N_CODECS) return fail(GENIE_ERR_INVALID_ARG, "unknown codec %d", codec);
    std::lock_guard<std::mutex> g(g_match_mu);
    if (fn) *fn = g_match[codec].fn;
    if (user) *user = g_match[codec].user;
    return GENIE_OK;
}

int genie_match_builtin(genie_index *ix, const genie_queries *q, uint32_t *out_ids, uint32_t *out_counts,
                        float *out_scores) {
    if (!ix) return fail(GENIE_ERR_INVALID_ARG, "index is NULL");
    std::vector<int64_t> out_off;
    int64_t n_items = 0;
    int rc = validate_queries(q, out_off, n_items);
    if (rc) return rc;
    if (q->n_queries == 0) return GENIE_OK;
    if (!out_ids || !out_counts) return fail(GENIE_ERR_INVALID_ARG, "output buffers are NULL");
    std::lock_guard<std::mutex> g(ix->mu);
    cudaSetDevice(ix->device);
    return run_search(ix, q, out_off, n_items, out_ids, out_counts, out_scores, true);
}

int genie_search(genie_index *ix, const genie_queries *q, uint32_t *out_ids, uint32_t *out_counts, float *out_scores) {
    if (!ix) return fail(GENIE_ERR_INVALID_ARG, "index is NULL");
    MatchEntry m;
    if (registered_match(ix->codec, m)) return m.fn(ix, q, out_ids, out_counts, out_scores, m.user);
    std::vector<int64_t> out_off;
    int64_t n_items = 0;
    int rc = validate_queries(q, out_off, n_items);
    if (rc) return rc;
    if (q->n_queries == 0) return GENIE_OK;
    if (!out_ids || !out_counts) return fail(GENIE_ERR_INVALID_ARG, "output buffers are NULL");
    std::lock_guard<std::mutex> g(ix->mu);
    cudaSetDevice(ix->device);
    return run_search(ix, q, out_off, n_items, out_ids, out_counts, out_scores, true);
}

int genie_search_multi(genie_index *const *ixs, const genie_queries *qs, int32_t n_index, uint32_t *out_ids,
                       uint32_t *out_counts, float *out_scores) {
    if (!ixs || !qs || n_index < 0) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    std::vector<std::vector<int64_t>> offs(n_index);
    std::vector<int64_t> items(n_index), base(n_index + 1, 0);
    for (int32_t i = 0; i < n_index; ++i) {
        if (!ixs[i]) return fail(GENIE_ERR_INVALID_ARG, "index %d is NULL", i);
        int rc = validate_queries(&qs[i], offs[i], items[i]);
        if (rc) return rc;
        base[i + 1] = base[i] + offs[i].back();
    }
    // indexes whose codec has a registered match function run it first
    std::vector<char> custom(n_index, 0);
    for (int32_t i = 0; i < n_index; ++i) {
        MatchEntry m;
        if (qs[i].n_queries == 0 || !registered_match(ixs[i]->codec, m)) continue;
        custom[i] = 1;
        int rc = m.fn(ixs[i], &qs[i], out_ids + base[i], out_counts + base[i], out_scores ? out_scores + base[i] : nullptr,
                      m.user);
        if (rc) return rc;
    }
    // every other index runs on its own stream; all batches are in flight together
    for (int32_t i = 0; i < n_index; ++i) {
        if (qs[i].n_queries == 0 || custom[i]) continue;
        ixs[i]->mu.lock();
        cudaSetDevice(ixs[i]->device);
        int rc = run_search(ixs[i], &qs[i], offs[i], items[i], out_ids + base[i], out_counts + base[i],
                            out_scores ? out_scores + base[i] : nullptr, false);
        if (rc) {
            for (int32_t j = 0; j <= i; ++j) if (qs[j].n_queries && !custom[j]) ixs[j]->mu.unlock();
            return rc;
        }
    }
    int rc = GENIE_OK;
    for (int32_t i = 0; i < n_index; ++i) {
        if (qs[i].n_queries == 0 || custom[i]) continue;
        cudaError_t e = cudaStreamSynchronize(ixs[i]->stream);
        if (e && !rc) rc = cuda_fail(e, "multi-index search");
        if (!rc) rc = check_device_error(*ixs[i]->host_err);
        ixs[i]->mu.unlock();
    }
    return rc;
}

}  // extern "C"
