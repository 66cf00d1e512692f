// subseq.cu -- subsequence search: rows are sequences, and a query counts,
// for every (row, start offset), the query items that match the row at
// start offset + the item's position in the query.
//
// Reference counterparts: inv_list::invert_subsequence (table/inv_list.cc:
// 193-235) lists rowID << bits | offset under each value, bits the least with
// 2^bits >= the longest row; the match kernel maps a listed id with offset o
// to id - order for an item of order <= o and skips it otherwise
// (matching/match.cu:84-94); get_rowID_offset splits a result id
// (original/interface.cc:914-926).
//
// The index is a bag index over the virtual objects rowID << bits | offset
// (an object per row position, one value each), so building, persistence of
// the lists and span lookup are the bag index's.  Counting runs in two
// kernels per chunk of queries: one CTA per (query, slice of each item's
// span) adds into global per-query counters over the virtual id space, and
// one CTA per query selects the exact top-k (count desc, id asc) with the
// block selection of the other paths.  Queries are taken in chunks whose
// counters fit kSubseqCounterBytes.
#include "capi_internal.h"
#include "select.cuh"

#include <algorithm>

namespace gg {
namespace {

constexpr size_t kSubseqCounterBytes = size_t(1) << 30;
constexpr int kSubseqThreads = 256;
constexpr int kSubseqSlices = 8;          // CTAs per query in the counting kernel

struct CounterSet {                       // the per-object counters of one query
    const uint32_t *cnt;
    int64_t n;
    template <class F>
    __device__ void for_each(F f) const {
        for (int64_t b = 0; b < n; b += blockDim.x) {
            const int64_t i = b + threadIdx.x;
            const bool act = i < n;
            const uint32_t c = act ? __ldg(cnt + i) : 0u;
            f(act && c > 0, c, (uint32_t)i);
        }
    }
};

// Item it of query q (chunk-local) adds 1 to object id - order for every id of
// its span whose row offset is at least its order.
__global__ void __launch_bounds__(kSubseqThreads) k_subseq_count(const uint32_t *__restrict__ ids,
                                                                 const int64_t *__restrict__ start,
                                                                 const int64_t *__restrict__ len,
                                                                 const uint32_t *__restrict__ order,
                                                                 const int64_t *__restrict__ item_off, int64_t q0,
                                                                 uint32_t *cnt, int64_t nv, uint32_t mask) {
    const int64_t q = blockIdx.y;
    const int64_t i0 = item_off[q0 + q], i1 = item_off[q0 + q + 1];
    uint32_t *c = cnt + q * nv;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t it = i0; it < i1; ++it) {
        const int64_t s = start[it], n = len[it];
        const uint32_t o = order[it];
        for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
            const uint32_t id = __ldg(ids + s + p);
            if ((id & mask) >= o && (int64_t)(id - o) < nv) atomicAdd(&c[id - o], 1u);
        }
    }
}

__global__ void __launch_bounds__(1024, 1) k_subseq_topk(const uint32_t *cnt, int64_t nv, const uint32_t *k,
                                                         uint32_t uniform_k, const int64_t *out_off, int64_t q0,
                                                         uint32_t *out_ids, uint32_t *out_counts, float *out_scores) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *cand = (uint64_t *)smem;
    SelectScratch &ss = *(SelectScratch *)(smem + kCandCap * 8);
    const int64_t q = blockIdx.x;
    const uint32_t kq = k ? k[q0 + q] : uniform_k;
    const uint32_t n = select_topk(CounterSet{cnt + q * nv, nv}, kq, 32, cand, kCandCap, ss);
    const int64_t o = out_off[q0 + q];
    for (uint32_t j = threadIdx.x; j < kq; j += blockDim.x) {
        const uint64_t key = j < n ? cand[j] : 0ull;
        const uint32_t c = j < n ? key_prim(key) : 0u;
        out_ids[o + j] = j < n ? key_id(key) : 0u;
        out_counts[o + j] = c;
        if (out_scores) out_scores[o + j] = (float)c;
    }
}

}  // namespace

// Search of a subsequence index: spans and item orders on the host, counting
// and selection on the device (stream ix->stream; waits when sync).
int subseq_search(genie_index *ix, const genie_queries *q, const std::vector<int64_t> &out_off, int64_t n_items,
                  uint32_t *out_ids, uint32_t *out_counts, float *out_scores, bool sync) {
    const int64_t Q = q->n_queries;
    const int64_t sumk = out_off[Q];
    const int64_t nv = ix->host.n_objects;
    const uint32_t mask = ix->sub_shift >= 32 ? 0xFFFFFFFFu : ((1u << ix->sub_shift) - 1u);
    std::vector<int64_t> start((size_t)std::max<int64_t>(1, n_items)), len(start.size());
    std::vector<uint32_t> order(start.size());
    for (int64_t i = 0; i < Q; ++i)
        for (int64_t it = q->item_off[i]; it < q->item_off[i + 1]; ++it) {
            int64_t a = 0, b = 0;
            item_span(ix->host, q->dim[it], q->low[it], q->up[it], a, b);
            start[it] = a;
            len[it] = b - a;
            order[it] = (uint32_t)(it - q->item_off[i]);
        }
    const int64_t per_chunk = std::max<int64_t>(1, (int64_t)(kSubseqCounterBytes / ((size_t)nv * 4)));
    const int64_t chunk = std::min<int64_t>(std::min<int64_t>(Q, per_chunk), 65535);   // grid y
    Workspace &ws = ix->ws;
    cudaError_t e;
    if ((e = ws.reserve(Q, n_items, n_items, sumk))) return cuda_fail(e, "search workspace");
    if ((e = ws.counters.reserve((size_t)chunk * nv * 4 + 16))) return cuda_fail(e, "subsequence counters");
    cudaStream_t s = ix->stream;
#define H2D(dst, src, n) if ((n) > 0 && (e = cudaMemcpyAsync(dst, src, (size_t)(n), cudaMemcpyHostToDevice, s))) return cuda_fail(e, "query upload")
    H2D(ws.item_off.p, q->item_off, (Q + 1) * 8);
    H2D(ws.span_start.p, start.data(), n_items * 8);
    H2D(ws.span_len.p, len.data(), n_items * 8);
    H2D(ws.inc.p, order.data(), n_items * 4);
    if (q->k) H2D(ws.k.p, q->k, Q * 4);
    H2D(ws.out_off.p, out_off.data(), (Q + 1) * 8);
#undef H2D
    const size_t smem = (size_t)kCandCap * 8 + sizeof(SelectScratch) + 64;
    static bool smem_set = false;
    if (!smem_set) {
        if ((e = cudaFuncSetAttribute(k_subseq_topk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
            return cuda_fail(e, "subsequence kernel setup");
        smem_set = true;
    }
    uint32_t *cnt = (uint32_t *)ws.counters.p;
    for (int64_t q0 = 0; q0 < Q; q0 += chunk) {
        const int64_t nq = std::min<int64_t>(chunk, Q - q0);
        if ((e = cudaMemsetAsync(cnt, 0, (size_t)nq * nv * 4, s))) return cuda_fail(e, "subsequence counters");
        k_subseq_count<<<dim3(kSubseqSlices, (unsigned)nq), kSubseqThreads, 0, s>>>(
            ix->dev.ids, (const int64_t *)ws.span_start.p, (const int64_t *)ws.span_len.p,
            (const uint32_t *)ws.inc.p, (const int64_t *)ws.item_off.p, q0, cnt, nv, mask);
        k_subseq_topk<<<(unsigned)nq, 1024, smem, s>>>(cnt, nv, q->k ? (const uint32_t *)ws.k.p : nullptr,
                                                      q->uniform_k, (const int64_t *)ws.out_off.p, q0,
                                                      (uint32_t *)ws.out_ids.p, (uint32_t *)ws.out_counts.p,
                                                      out_scores ? (float *)ws.out_scores.p : nullptr);
    }
    if ((e = cudaGetLastError())) return cuda_fail(e, "subsequence launch");
    *ix->host_err = 0;
    if ((e = cudaMemcpyAsync(out_ids, ws.out_ids.p, sumk * 4, cudaMemcpyDeviceToHost, s))) return cuda_fail(e, "result ids");
    if ((e = cudaMemcpyAsync(out_counts, ws.out_counts.p, sumk * 4, cudaMemcpyDeviceToHost, s)))
        return cuda_fail(e, "result counts");
    if (out_scores && (e = cudaMemcpyAsync(out_scores, ws.out_scores.p, sumk * 4, cudaMemcpyDeviceToHost, s)))
        return cuda_fail(e, "result scores");
    ix->last_launches = (int)(2 * ((Q + chunk - 1) / chunk));
    if (!sync) return GENIE_OK;
    if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "subsequence search");
    return GENIE_OK;
}

}  // namespace gg

using namespace gg;

extern "C" int genie_index_create_subsequence(const int32_t *values, const int64_t *row_off, int64_t n_rows,
                                              genie_index **out) {
    if (!out) return fail(GENIE_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!values || !row_off || n_rows <= 0) return fail(GENIE_ERR_INVALID_ARG, "no data input");
    int64_t longest = 0;
    for (int64_t r = 0; r < n_rows; ++r) {
        if (row_off[r + 1] < row_off[r]) return fail(GENIE_ERR_INVALID_ARG, "row offsets decrease at row %lld", (long long)r);
        longest = std::max<int64_t>(longest, row_off[r + 1] - row_off[r]);
    }
    int bits = 0;                         // the least with 2^bits >= the longest row
    while (((int64_t)1 << bits) < longest) ++bits;
    if (bits > 31 || (n_rows << bits) > ((int64_t)1 << 32))
        return fail(GENIE_ERR_INVALID_ARG, "%lld rows of up to %lld values exceed 32-bit row<<offset ids",
                    (long long)n_rows, (long long)longest);
    // virtual object rowID << bits | offset holds the one value at that offset
    const int64_t nv = n_rows << bits;
    std::vector<int64_t> voff((size_t)nv + 1, 0);
    for (int64_t r = 0; r < n_rows; ++r) {
        const int64_t l = row_off[r + 1] - row_off[r];
        for (int64_t p = 0; p < l; ++p) voff[(size_t)((r << bits) + p) + 1] = 1;
    }
    for (int64_t v = 0; v < nv; ++v) voff[v + 1] += voff[v];
    std::vector<int32_t> vals((size_t)row_off[n_rows] - (size_t)row_off[0]);
    std::copy(values + row_off[0], values + row_off[n_rows], vals.begin());
    genie_index *ix = nullptr;
    int rc = genie_index_create_bag(vals.data(), voff.data(), nv, &ix);
    if (rc) return rc;
    ix->sub_shift = bits;
    *out = ix;
    return GENIE_OK;
}

extern "C" int genie_index_subsequence_bits(const genie_index *ix, int32_t *bits) {
    if (!ix || !bits) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    *bits = ix->sub_shift;
    return GENIE_OK;
}
