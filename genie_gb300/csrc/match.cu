// match.cu -- the match-count hot path: query plan, presence-bitmap, sparse
// (hash) and dense (id-tiled) counting kernels, exact top-k and the cross-part
// merge.
//
// Reference counterpart: matching::match / match_AT (matching/match.cu:43-464),
// the c-PQ and bitmap counters (matching/match_device_utils.h:160-473),
// convert_to_data + heap_count_topk (match_common.cu:9-20, heap_count.cu:24-282)
// and extract_index_and_count (knn.cu:47-55).  The reference counts every
// posting id with a global-memory atomicCAS on a packed per-query bitmap and
// probes a per-query global hash; here every count lives in shared memory.
#include "codecs.cuh"
#include "match.cuh"
#include "select.cuh"

#include <algorithm>
#include <cstdio>

namespace gg {

// First out-of-bounds report of a checked build (all zero otherwise).
void read_oob(unsigned long long out[4]) {
    out[0] = out[1] = out[2] = out[3] = 0;
#ifdef GG_CHECKED
    cudaMemcpyFromSymbol(out, gg_oob, sizeof(unsigned long long) * 4);
#endif
}

// ------------------------------------------------------------------ plan
//
// Query compile on the device, one CTA per query in one launch: clamp every
// item (Query::attr / Query::build, query/query.cc:87-113, 273-333), count the
// (dim,value) lists it covers and the posting ids it touches, the fixed-point
// scale of a weighted query; the query's units (one per covered list: a
// sorted posting list, or the segment range of a compressed one) are its items
// when each covers at most one list, else a contiguous range taken from a
// device counter past the batch's items (ranges of different queries need no
// order between them); then the bitmap/sparse/dense decision and the work
// lists.
// A range item covers several lists whose concatenation is not sorted, so
// every later search inside a span happens per unit.

constexpr int kPlanThreads = 256;

// Id-range parts of a dense query: each sweeps T.dense_part_work objects in
// whole counter tiles (at least one), at most W.max_parts parts.  Fewer,
// longer parts pay a part's setup and merge less often and let its later
// tiles merge against a full running top-k.  Every dense query of one
// counter width has the same number, so that the dense kernel can take its
// work part-major (take_dense).
__device__ __forceinline__ int64_t dense_parts(const DevIndex &ix, const Work &W, const Tuning &T, bool small) {
    const int64_t tile = small ? T.dense_tile_u8 : T.dense_tile_u32;
    const int64_t ntiles = (ix.n_objects + tile - 1) / tile;
    int64_t per = T.dense_part_work / tile;
    if (per < 1) per = 1;
    const int64_t np = (ntiles + per - 1) / per;
    const int64_t pd = np < W.max_parts ? np : W.max_parts;
    return pd < 1 ? 1 : pd;
}

__global__ void __launch_bounds__(kPlanThreads, 8) k_plan(DevIndex ix, DevQueries Q, Work W, Tuning T) {
    __shared__ unsigned long long s_total, s_units, s_unit0;
    __shared__ unsigned int s_maxw, s_bad, s_multi, s_oob;
    __shared__ uint32_t s_tmp[48];
    const int64_t q = blockIdx.x;
    const int64_t nq = Q.dyn ? (int64_t)Q.dyn[0] : (int64_t)Q.n_queries;
    if (q >= nq) return;
    const uint32_t tid = threadIdx.x, nt = blockDim.x, lane = lane_id();
    const int64_t i0 = Q.item_off[q], i1 = Q.item_off[q + 1];
    const int32_t m = (int32_t)(i1 - i0);
    const uint32_t k = Q.k ? Q.k[q] : (Q.dyn ? Q.dyn[1] : Q.uniform_k);
    // The query's items and result slots must lie inside the workspace, also
    // when the caller's device arrays (item_off, out_off, k) disagree with the
    // sizes it passed: a query outside them is reported and gets no work, so
    // nothing downstream indexes past the item, unit, scratch or result arrays.
    if (tid == 0) {
        const int64_t last = Q.item_off[nq], o = Q.out_off[q];
        s_oob = !(i0 >= 0 && i0 <= i1 && i1 <= last && last <= W.items_cap && o >= 0 && o <= W.out_cap &&
                  (int64_t)k <= W.out_cap - o);
        if (s_oob) {
            atomicOr(&W.ctr[kCtrError], kErrBounds);
            QInfo none{};
            none.cls = kClsNone;
            W.qinfo[q] = none;
            W.done[q] = 0;
            W.qstate[q] = 0;
        }
    }
    __syncthreads();
    if (s_oob) return;
    const bool weighted = Q.weighted && Q.weight && Q.weighted[q];
    const bool exact = Q.dyn && Q.dyn[2];      // a batch of exact items sends no upper bounds
    if (tid == 0) {
        s_total = 0;
        s_units = 0;
        s_maxw = 0;
        s_bad = 0;
        s_multi = 0;
    }
    __syncthreads();
    int32_t scale = 0;
    if (weighted) {
        // the scale depends on m * max(w) only, so it is independent of any
        // summation order: every sum of the item weights stays below 2^31
        float mx = 0.0f;
        unsigned bad = 0;
        for (int64_t i = i0 + tid; i < i1; i += nt) {
            const float w = Q.weight[i];
            if (!(w > 0.0f) || isinf(w)) bad = 1;
            else mx = fmaxf(mx, w);
        }
        atomicMax(&s_maxw, __float_as_uint(mx));     // positive floats order as their bits
        if (bad) atomicOr(&s_bad, 1u);
        __syncthreads();
        int e = 0;
        (void)frexp((double)m * (double)__uint_as_float(s_maxw), &e);
        scale = 31 - e;
        if (s_bad && tid == 0) atomicOr(&W.ctr[kCtrError], kErrWeight);
    }
    // items: key range, touched ids; this thread's first item stays in
    // registers, later ones (queries of more than nt items) go through W
    uint64_t total = 0, units = 0;
    int64_t k0_first = 0, a_first = 0, e_first = 0;     // a, e: list offsets around the keys
    uint32_t nk_first = 0, inc_first = 1;
    for (int64_t i = i0 + tid; i < i1; i += nt) {
        if (!GG_OK(i, W.items_cap, 7)) break;
        int32_t d = Q.dim[i], lo = Q.low[i], hi = exact ? lo : Q.up[i];
        int64_t k0 = 0, nk = 0, a = 0, e = 0;
        if (d >= 0 && d < ix.n_dims) {
            int32_t mn = ix.dim_min[d], mx = ix.dim_max[d];
            if (!(lo > hi || lo > mx || hi < mn)) {
                if (lo < mn) lo = mn;
                if (hi > mx) hi = mx;
                k0 = ix.key_base[d] + ((int64_t)lo - mn);
                nk = (int64_t)hi - lo + 1;
                a = ix.key_off[k0];
                e = ix.key_off[k0 + nk];
                total += (uint64_t)(e - a);
            }
        }
        uint32_t inc = 1;
        if (weighted) inc = (uint32_t)__double2ll_rn(ldexp((double)Q.weight[i], scale));
        // An item covering at most one list is also unit i: when every item
        // of the query is, the query's units are its items and nothing more
        // is written.  Otherwise the query takes a unit range past the
        // batch's items and these slots, in its own item range, stay unread.
        if (nk <= 1 && i < W.units_cap) {
            if (ix.codec) {
                a = nk ? ix.key_seg[k0] : 0;
                e = nk ? ix.key_seg[k0 + 1] : 0;
            }
            W.span_start[i] = a;
            W.span_len[i] = e - a;
            W.inc[i] = inc;
            if (W.unit_key) W.unit_key[i] = (uint32_t)k0;
        }
        if (nk > 1) s_multi = 1;
        if (i == i0 + tid) {
            k0_first = k0;
            nk_first = (uint32_t)nk;
            inc_first = inc;
            a_first = a;
            e_first = e;
        } else {
            W.item_k0[i] = k0;
            W.item_nk[i] = (uint32_t)nk;
            W.item_inc[i] = inc;
        }
        units += (uint64_t)nk;
    }
    total = warp_sum_u64(total);
    units = warp_sum_u64(units);
    if (lane == 0) {
        atomicAdd(&s_total, (unsigned long long)total);
        atomicAdd(&s_units, (unsigned long long)units);
    }
    __syncthreads();
    const bool single = s_multi == 0;      // block-uniform
    if (tid == 0)
        s_unit0 = single ? (unsigned long long)i0
                         : (unsigned long long)Q.item_off[nq] +
                               atomicAdd((unsigned long long *)&W.ctr[kCtrUnits], s_units);
    __syncthreads();
    const int64_t unit0 = (int64_t)s_unit0, n_units = single ? (int64_t)m : (int64_t)s_units;
    total = s_total;
    const bool fits = unit0 + n_units <= W.units_cap;
    if (tid == 0 && !fits) atomicOr(&W.ctr[kCtrError], kErrUnits);
    // one unit per covered list (a query with several lists in one item)
    if (fits && !single) {
        int64_t base = unit0;
        for (int64_t c = i0; c < i1; c += nt) {
            const int64_t i = c + tid;
            uint32_t nk = 0, inc = 1;
            int64_t k0 = 0;
            if (i < i1) {
                if (c == i0) {
                    k0 = k0_first;
                    nk = nk_first;
                    inc = inc_first;
                } else {
                    k0 = W.item_k0[i];
                    nk = W.item_nk[i];
                    inc = W.item_inc[i];
                }
            }
            uint32_t tot = 0;
            const uint32_t ex = block_excl_scan(nk, s_tmp, &tot);
            if (c == i0 && nk == 1 && !ix.codec) {      // a single list: its offsets are at hand
                if (GG_OK(base + ex, W.units_cap, 14)) {
                    W.span_start[base + ex] = a_first;
                    W.span_len[base + ex] = e_first - a_first;
                    W.inc[base + ex] = inc;
                    if (W.unit_key) W.unit_key[base + ex] = (uint32_t)k0;
                }
                nk = 0;
            }
            for (uint32_t j = 0; j < nk; ++j) {
                const int64_t u = base + ex + j, key = k0 + j;
                if (!GG_OK(u, W.units_cap, 14)) break;
                const int64_t a = ix.codec ? ix.key_seg[key] : ix.key_off[key];
                const int64_t e = ix.codec ? ix.key_seg[key + 1] : ix.key_off[key + 1];
                W.span_start[u] = a;
                W.span_len[u] = e - a;
                W.inc[u] = inc;
                if (W.unit_key) W.unit_key[u] = (uint32_t)key;
            }
            base += tot;
        }
    }
    QInfo qi;
    qi.total = (int64_t)total;
    qi.unit0 = unit0;
    qi.n_units = (int32_t)n_units;
    qi.item0 = i0;
    qi.n_items = m;
    qi.k = k;
    qi.scale = scale;
    qi.flags = weighted ? kFlagWeighted : 0;
    // bound on any object's count: one match per item on a one-value-per-dim
    // table; on a bag table, every covered list may repeat the object
    const int64_t bound = ix.is_bag ? n_units * ix.mult_max : (int64_t)m;
    if (!weighted && bound <= 255) qi.flags |= kFlagSmallCount;
    qi.parts = 1;
    qi.cls = kClsNone;
    if (tid == 0) {
        W.done[q] = 0;
        W.qstate[q] = 0;
        W.lb[q] = 0;
        if (k == 0 || k > (uint32_t)kMaxK) atomicOr(&W.ctr[kCtrError], kErrCapacity);
        const bool small = (qi.flags & kFlagSmallCount) != 0;
        const int64_t total = qi.total;
        int list = -1;
        if (fits && k >= 1 && k <= (uint32_t)kMaxK && total > 0) {
            const bool packed = small && ix.n_objects <= (int64_t)(1u << 24);
            const int64_t slots = packed ? T.sparse_slots_packed : T.sparse_slots_wide;
            const int64_t cap = slots * T.sparse_load_pct / 100;     // table load factor bound
            const int64_t ps = (total + cap - 1) / cap;
            if (total <= T.sparse_max_total && total * 4 <= ix.n_objects * 3 && packed && !ix.codec &&
                T.bitmap_bits > 0 && T.bitmap_ready && ix.n_objects <= T.bitmap_bits &&
                qi.n_units <= (int32_t)kBmSpanCap && total <= (int64_t)kBmMaxIds &&
                ix.n_ids <= (int64_t)0xFFFFFFFFll - 64) {       // posting positions in 32 bits
                // presence bitmap over the whole id space + a table of repeated ids
                qi.cls = kClsSparse;
                qi.parts = 1;
                qi.flags |= kFlagPacked;
                list = kListBitmap;
            } else if (total <= T.sparse_max_total && ps <= kMaxParts && total * 4 <= ix.n_objects * 3) {
                qi.cls = kClsSparse;
                qi.parts = (uint16_t)ps;
                if (packed) qi.flags |= kFlagPacked;
                list = packed ? kListSparsePacked : kListSparseWide;
            } else {
                qi.cls = kClsDense;
                qi.parts = (uint16_t)dense_parts(ix, W, T, small);
                list = small ? kListDenseSmall : kListDenseWide;
            }
        }
        W.qinfo[q] = qi;
        if (list >= 0) {
            // a dense list holds the query once: its parts are taken part-major
            const uint32_t entries = (list == kListDenseSmall || list == kListDenseWide) ? 1u : qi.parts;
            uint2 *wl = W.work + (size_t)list * W.work_stride;
            uint32_t b = atomicAdd(&W.ctr[2 * list], entries);
            for (uint32_t p = 0; p < entries; ++p)
                if (GG_OK(b + p, W.work_stride, 8)) wl[b + p] = make_uint2((uint32_t)q, p);
        }
    }
    // queries without any matching posting: padded results right away
    if (qi.k >= 1 && qi.k <= (uint32_t)kMaxK && qi.total == 0) {
        const int64_t o = Q.out_off[q];
        for (uint32_t j = tid; j < qi.k; j += nt) {
            if (!GG_OK(o + j, W.out_cap, 4)) break;
            W.out_ids[o + j] = 0;
            W.out_counts[o + j] = 0;
            if (W.out_scores) W.out_scores[o + j] = 0.0f;
        }
    }
}

// ------------------------------------------------------------------ shared

// Sparse kernel: promoted-slot list placed behind the staged units.
constexpr int kPromOff = ((kItemChunk * 20 + 4) + 15) / 16 * 16;
constexpr int kPromCap = 1024;
static_assert(kPromOff + kPromCap * 4 <= kCandCap * 8, "promoted list must fit the union region");
static_assert(kPromCap * 8 <= kPromOff, "candidate keys of the promoted list must end below it");

// Items of one query part staged in shared memory.
struct ItemStage {
    int64_t *start;   // [kItemChunk] global position of the sub-span
    uint32_t *len;    // [kItemChunk]
    uint32_t *inc;    // [kItemChunk]
    uint32_t *flat;   // [kItemChunk+1] exclusive prefix of len
};

// Stream every posting id of the staged sub-spans through `visit(id, inc)`.
// Warps take 256-position chunks of the flattened span list; each lane loads
// 8 ids (coalesced within a span) before visiting them.
template <class V>
__device__ __forceinline__ void stream_ids(const uint32_t *__restrict__ ids, int64_t n_ids, const ItemStage &st,
                                           uint32_t n_items, uint32_t F, V &&visit) {
    (void)n_ids;
    const uint32_t lane = lane_id();
    const uint32_t nw = blockDim.x >> 5;
    for (uint32_t base = warp_id() * 256u; base < F; base += nw * 256u) {
        uint32_t it = 0;
        if (lane == 0) {
            uint32_t lo = 0, hi = n_items;       // last item with flat <= base
            while (lo < hi) {
                uint32_t mid = (lo + hi + 1) >> 1;
                if (st.flat[mid] <= base) lo = mid; else hi = mid - 1;
            }
            it = lo;
        }
        it = __shfl_sync(0xffffffffu, it, 0);
        uint32_t v[8], inc[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            uint32_t f = base + j * 32 + lane;
            inc[j] = 0;
            v[j] = 0;
            if (f < F) {
                while (GG_OK(it + 1, n_items + 1, 11) && st.flat[it + 1] <= f) ++it;
                int64_t pos = st.start[it] + (int64_t)(f - st.flat[it]);
                if (GG_OK(pos, n_ids, 1)) {
                    v[j] = __ldg(ids + pos);
                    inc[j] = st.inc[it];
                }
            }
        }
        visit(v, inc);
    }
}

// Per-id form of stream_ids.
template <class V>
__device__ __forceinline__ void stream_ids1(const uint32_t *__restrict__ ids, int64_t n_ids, const ItemStage &st,
                                            uint32_t n_items, uint32_t F, V &&visit) {
    stream_ids(ids, n_ids, st, n_items, F, [&](uint32_t(&v)[8], uint32_t(&inc)[8]) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (inc[j]) visit(v[j], inc[j]);
    });
}

// Home slot of an id in a table of `cap` slots (multiplicative hash, then a
// multiply-high range reduction, so cap need not be a power of two).
__device__ __forceinline__ uint32_t slot_of(uint32_t id, uint32_t cap) {
    return (uint32_t)(((uint64_t)(id * 0x9E3779B1u) * cap) >> 32);
}

// Lane-queue hash insert.  Each lane holds up to 8 ids (inc == 0: no id) and
// moves on to its next id as soon as the current one is placed, so a warp
// step costs the longest per-lane sum of probes instead of the sum of the
// per-id longest probes.  Linear probing, at most `cap` probes per id.
// PACKED slots are id<<8 | count (ids < 2^24, counts <= 255); the one
// increment taking a slot from 1 to 2 appends the slot to `prom`.
// Wide slots are (id+1)<<32 | sum.
template <bool PACKED>
__device__ __forceinline__ void hash_insert8(void *tab_raw, uint32_t cap, uint32_t (&v)[8], uint32_t (&inc)[8],
                                             uint32_t *prom, uint32_t *s_prom) {
    auto pop = [&]() {
#pragma unroll
        for (int t = 0; t < 7; ++t) {
            v[t] = v[t + 1];
            inc[t] = inc[t + 1];
        }
        v[7] = 0;
        inc[7] = 0;
    };
    int left = 8;
    while (left > 0 && inc[0] == 0) {
        pop();
        --left;
    }
    uint32_t h = left ? slot_of(v[0], cap) : 0u, probes = 0;
    while (__any_sync(0xffffffffu, left > 0)) {
        if (left <= 0) continue;
        bool done = false;
        const uint32_t id = v[0];
        if (!GG_OK(h, cap, 2)) {
            done = true;
        } else if (PACKED) {
            uint32_t *tab = (uint32_t *)tab_raw;
            uint32_t cur = tab[h];
            if (cur == 0u) {
                const uint32_t old = atomicCAS(&tab[h], 0u, (id << 8) | 1u);
                if (old == 0u) done = true;
                else cur = old;
            }
            if (!done && (cur >> 8) == id) {
                if ((atomicAdd(&tab[h], 1u) & 255u) == 1u) {
                    const uint32_t at = atomicAdd(s_prom, 1u);
                    if (at < (uint32_t)kPromCap) prom[at] = h;
                }
                done = true;
            }
        } else {
            unsigned long long *tab = (unsigned long long *)tab_raw;
            const unsigned long long tag = (unsigned long long)(id + 1u) << 32;
            unsigned long long cur = tab[h];
            if (cur == 0ull) {
                const unsigned long long old = atomicCAS(&tab[h], 0ull, tag | inc[0]);
                if (old == 0ull) done = true;
                else cur = old;
            }
            if (!done && (cur & 0xFFFFFFFF00000000ull) == tag) {
                atomicAdd(&tab[h], (unsigned long long)inc[0]);
                done = true;
            }
        }
        if (!done) {
            h = (h + 1 == cap) ? 0u : h + 1;
            if (++probes >= cap) done = true;
        }
        if (done) {
            pop();
            --left;
            while (left > 0 && inc[0] == 0) {
                pop();
                --left;
            }
            if (left > 0) {
                h = slot_of(v[0], cap);
                probes = 0;
            }
        }
    }
}

// Compressed index: every warp decodes whole segments (<= 1024 ids) and
// visits the ids inside [lo, hi).  Decoding is fused into counting: ids go
// from the unpacked words straight to the shared-memory counters.
template <class V>
__device__ __forceinline__ void stream_segments(const DevIndex &ix, const ItemStage &st, uint32_t n_items,
                                                uint32_t F, uint32_t lo, uint32_t hi, V &&visit) {
    const uint32_t nw = blockDim.x >> 5;
    for (uint32_t f = warp_id(); f < F; f += nw) {
        uint32_t a = 0, b = n_items;       // last item with flat <= f
        while (a < b) {
            uint32_t mid = (a + b + 1) >> 1;
            if (st.flat[mid] <= f) a = mid; else b = mid - 1;
        }
        const int64_t seg = st.start[a] + (int64_t)(f - st.flat[a]);
        const uint32_t inc = st.inc[a];
        auto v = [&](uint32_t id, uint32_t) {
            if (id >= lo && id < hi && inc) visit(id, inc);
        };
        decode_segment_values(ix.codec, ix.words, ix.seg_word_off[seg], ix.seg_word_off[seg + 1], v);
    }
}

template <class V>
__device__ __forceinline__ void stream_units(const DevIndex &ix, const ItemStage &st, uint32_t n_items, uint32_t F,
                                             uint32_t lo, uint32_t hi, V &&visit) {
    if (ix.codec) stream_segments(ix, st, n_items, F, lo, hi, visit);
    else stream_ids1(ix.ids, ix.n_ids, st, n_items, F, visit);
}

// Plain lists in long runs (the dense kernel): warp tasks of kRun consecutive
// posting positions of one staged sub-span.  st.flat holds the exclusive
// prefix of the sub-spans' task counts, st.len their lengths.  The item
// lookup happens once per task instead of once per id, and a lane's loads
// are immediate offsets from one pointer, so the per-id work is the load and
// visit(id, inc).
constexpr uint32_t kRun = 1024;
template <class V>
__device__ __forceinline__ void stream_runs(const uint32_t *__restrict__ ids, const ItemStage &st, uint32_t n_items,
                                            uint32_t n_tasks, V &&visit) {
    constexpr int R = 32;                 // loads in flight per lane: a full task in one round
    const uint32_t lane = lane_id(), nw = blockDim.x >> 5;
    for (uint32_t f = warp_id(); f < n_tasks; f += nw) {
        uint32_t a = 0, b = n_items;      // last sub-span with flat <= f
        while (a < b) {
            const uint32_t mid = (a + b + 1) >> 1;
            if (st.flat[mid] <= f) a = mid; else b = mid - 1;
        }
        const uint32_t r0 = (f - st.flat[a]) * kRun;
        const uint32_t n = min(kRun, st.len[a] - r0);
        const uint32_t inc = st.inc[a];
        const uint32_t *p = ids + st.start[a] + r0 + lane;
        if (n == kRun) {
            for (uint32_t g = 0; g < kRun / 32; g += R) {
                uint32_t v[R];
#pragma unroll
                for (int r = 0; r < R; ++r) v[r] = __ldg(p + 32 * (g + r));
#pragma unroll
                for (int r = 0; r < R; ++r) visit(v[r], inc);
            }
        } else {
            for (uint32_t g = 0; 32 * g < n; g += R) {
                uint32_t v[R];
#pragma unroll
                for (int r = 0; r < R; ++r) v[r] = 32 * (g + r) + lane < n ? __ldg(p + 32 * (g + r)) : 0u;
#pragma unroll
                for (int r = 0; r < R; ++r)
                    if (32 * (g + r) + lane < n) visit(v[r], inc);
            }
        }
    }
}

// Compressed lists in runs (the dense kernel): warp tasks of up to kSegRun
// consecutive segments of one staged unit.  The item lookup and the
// segments' word offsets and lengths are loaded once per task (one lane per
// segment).  A full 128-id segment of a BP32-based codec (BP32,
// SERIAL_DELTA_BP32, SERIAL_DELTA_COMP_BP32_COPY/VARINT: one 128-value BP32
// block, no tail) is unpacked straight from the words: lane l reads the one
// or two words holding its four values of miniblock l/8 (L1 hits after the
// first lane), extracts them with shifts, and the delta stage is one warp
// prefix sum.  Other segments (list tails, other codecs) take the generic
// warp decoder.  Ids outside [lo, hi) are skipped.  Runs are one segment
// long: a tile holds few segments of most lists, so a long run keeps one
// warp busy while the others wait at the tile's barrier, and the run's
// per-lane state raises the register pressure of the whole dense kernel
// (config2 batch: 67.9 ms with runs of 8 segments, 62.4 with 4, 61.3 with 2,
// 58.3 with 1; spill stores of k_dense 3,740 / 612 / 104 bytes for 8 / 2 / 1).
constexpr uint32_t kSegRun = 1;
constexpr uint32_t kBlockIds = 128;

// Whether a codec's full segments are one bare BP32 block (after an optional
// composite length word), and its delta stages.
__host__ __device__ __forceinline__ bool bp32_block_codec(int codec, int &deltas, bool &len_word) {
    int inner = 0;
    codec_parts(codec, deltas, inner);
    len_word = inner == kInnerCompCopy || inner == kInnerCompVarint;
    return (inner == kInnerBP32 || len_word) && (deltas == 0 || deltas == 1);
}

template <class V>
__device__ __forceinline__ void stream_segment_runs(const DevIndex &ix, const ItemStage &st, uint32_t n_items,
                                                    uint32_t n_tasks, uint32_t lo, uint32_t hi, V &&visit) {
    int deltas = 0;
    bool len_word = false;
    const bool fast_codec = bp32_block_codec(ix.codec, deltas, len_word);
    const uint32_t lane = lane_id(), nw = blockDim.x >> 5;
    for (uint32_t f = warp_id(); f < n_tasks; f += nw) {
        uint32_t a = 0, b = n_items;      // last unit with flat <= f
        while (a < b) {
            const uint32_t mid = (a + b + 1) >> 1;
            if (st.flat[mid] <= f) a = mid; else b = mid - 1;
        }
        const uint32_t r0 = (f - st.flat[a]) * kSegRun;
        const uint32_t ns = min(kSegRun, st.len[a] - r0);
        const uint32_t inc = st.inc[a];
        const int64_t s0 = st.start[a] + r0;
        // word offset and posting position of segments s0 .. s0+ns (one per lane)
        int64_t wo = 0, sp = 0;
        if (lane <= ns) {
            wo = __ldg(ix.seg_word_off + s0 + lane);
            sp = __ldg(ix.seg_pos + s0 + lane);
        }
        for (uint32_t j = 0; j < ns; ++j) {
            const int64_t w0 = __shfl_sync(0xffffffffu, wo, j), w1 = __shfl_sync(0xffffffffu, wo, j + 1);
            const int64_t n = __shfl_sync(0xffffffffu, sp, j + 1) - __shfl_sync(0xffffffffu, sp, j);
            if (!(fast_codec && n == (int64_t)kBlockIds)) {
                auto v = [&](uint32_t id, uint32_t) {
                    if (id >= lo && id < hi) visit(id, inc);
                };
                decode_segment_values(ix.codec, ix.words, w0, w1, v);
                continue;
            }
            // [len1] [n = 128] [widths] [miniblock 0] .. [miniblock 3]
            const uint32_t *w = ix.words + w0 + (len_word ? 1 : 0);
            const uint32_t hdr = __ldg(w + 1);
            const uint32_t m = lane >> 3;
            const uint32_t b = (hdr >> (24 - 8 * m)) & 255u;
            const uint32_t before = (m > 0 ? (hdr >> 24) : 0u) + (m > 1 ? (hdr >> 16) & 255u : 0u) +
                                    (m > 2 ? (hdr >> 8) & 255u : 0u);
            const uint32_t *mb = w + 2 + before;
            const uint32_t j0 = (lane & 7u) * 4u;
            const uint32_t mask = b >= 32 ? 0xFFFFFFFFu : (1u << b) - 1u;
            uint32_t v[4];
            if (b <= 8) {       // the four values lie in one 64-bit window
                const uint32_t bit0 = j0 * b, wi = bit0 >> 5, sh = bit0 & 31u;
                const uint32_t lo_w = b ? __ldg(mb + wi) : 0u;
                const uint32_t hi_w = (b && sh + 4 * b > 32) ? __ldg(mb + wi + 1) : 0u;
                const uint64_t win = (((uint64_t)hi_w << 32) | lo_w) >> sh;
#pragma unroll
                for (int k = 0; k < 4; ++k) v[k] = (uint32_t)(win >> (k * b)) & mask;
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t bit = (j0 + k) * b, wi = bit >> 5, sh = bit & 31u;
                    const uint32_t lo_w = __ldg(mb + wi);
                    const uint32_t hi_w = sh + b > 32 ? __ldg(mb + wi + 1) : 0u;
                    v[k] = (uint32_t)((((uint64_t)hi_w << 32) | lo_w) >> sh) & mask;
                }
            }
            if (deltas) {       // ids = prefix sums of the gaps, from 0 in every segment
                v[1] += v[0];
                v[2] += v[1];
                v[3] += v[2];
                const uint32_t incl = warp_incl_scan(v[3]);
                const uint32_t pre = incl - v[3];
#pragma unroll
                for (int k = 0; k < 4; ++k) v[k] += pre;
            }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (v[k] >= lo && v[k] < hi) visit(v[k], inc);
        }
    }
}

// Searches in a sorted list [s0, e0) over ids [0, N) (or its segments' first
// ids) that start at the position the list's density predicts: ids of a list
// are spread over the id space, so the error is about the square root of the
// count, and an 8-way probe search (probe8_first_ge) needs a few steps.
__device__ __forceinline__ int64_t near_win(int64_t expect) {
    int64_t w = 4;
    while (w * w < expect) w <<= 1;
    return w;
}
// First unit of [s0, e0) that can hold an id >= x.
__device__ __forceinline__ int64_t first_unit_near(const DevIndex &ix, int64_t s0, int64_t e0, uint32_t x, uint64_t N) {
    const int64_t len = e0 - s0, expect = (int64_t)((double)len * x / (double)N);
    const int64_t w = near_win(expect) / 2;
    if (!ix.codec) return probe8_first_ge(ix.ids, s0, e0, x, s0 + expect, w);
    const int64_t a = probe8_first_ge(ix.seg_first, s0, e0, x, s0 + expect, w);
    return a > s0 ? a - 1 : a;
}
// From a (the tile's first unit), the first unit holding ids >= hi (for a
// compressed index: the first segment starting at >= hi).
__device__ __forceinline__ int64_t next_unit_near(const DevIndex &ix, int64_t a, int64_t s0, int64_t e0, uint32_t lo,
                                                  uint32_t hi, uint64_t N) {
    const int64_t expect = (int64_t)((double)(e0 - s0) * (hi - lo) / (double)N);
    return probe8_first_ge(ix.codec ? ix.seg_first : ix.ids, a, e0, hi, a + expect, near_win(expect) / 2);
}

// First unit (posting position, or segment of a compressed index) of the
// range [s0, e0) that can hold an id >= x.
__device__ __forceinline__ int64_t first_unit(const DevIndex &ix, int64_t s0, int64_t e0, uint32_t x) {
    if (!ix.codec) return lower_bound_u32(ix.ids, s0, e0, x);
    int64_t a = lower_bound_u32(ix.seg_first, s0, e0, x);
    return a > s0 ? a - 1 : a;
}

// Stage items [c0, c0+mc) of a query restricted to the ids [lo, hi): posting
// positions (or, for a compressed index, segment indices) in st.start/len,
// increments in st.inc, the exclusive prefix of len in st.flat.  cut_lo /
// cut_hi request the binary searches for lo / hi.  Returns an upper bound on
// the posting ids staged (block-uniform).
__device__ uint64_t stage_range(const DevIndex &ix, const Work &W, const QInfo &qi, int32_t c0, int32_t mc,
                                bool cut_lo, bool cut_hi, uint32_t lo, uint32_t hi, ItemStage &st,
                                SelectScratch &ss) {
    const uint32_t tid = threadIdx.x;
    uint32_t len = 0;
    uint64_t ids = 0;
    if (tid == 0) ss.tot64 = 0;
    if ((int32_t)tid < mc && GG_OK(qi.unit0 + c0 + tid, W.units_cap, 9)) {
        const int64_t it = qi.unit0 + c0 + tid;
        const int64_t s0 = W.span_start[it], e0 = s0 + W.span_len[it];
        int64_t a = s0, b = e0;
        if (e0 > s0) {
            if (!ix.codec) {
                if (cut_lo) a = lower_bound_u32(ix.ids, s0, e0, lo);
                if (cut_hi) b = lower_bound_u32(ix.ids, a, e0, hi);
                ids = (uint64_t)(b - a);
            } else {
                if (cut_lo) {       // the segment before the first one starting at >= lo may reach lo
                    a = lower_bound_u32(ix.seg_first, s0, e0, lo);
                    if (a > s0) --a;
                }
                if (cut_hi) b = lower_bound_u32(ix.seg_first, a, e0, hi);
                ids = (uint64_t)(ix.seg_pos[b] - ix.seg_pos[a]);
            }
        }
        st.start[tid] = a;
        st.inc[tid] = W.inc[it];
        len = (uint32_t)(b - a);
        st.len[tid] = len;
    }
    uint32_t tot = 0;
    const uint32_t off = block_excl_scan(len, ss.tmp, &tot);
    if ((int32_t)tid < mc) st.flat[tid] = off;
    if (tid == 0) st.flat[mc] = tot;
    if (!ix.codec) return tot;
    ids = warp_sum_u64(ids);
    if (lane_id() == 0 && ids) atomicAdd((unsigned long long *)&ss.tot64, (unsigned long long)ids);
    __syncthreads();
    const uint64_t r = ss.tot64;
    __syncthreads();
    return r;
}

// Next item of a work list for this CTA, or ~0 when the list is done.  The
// list's count is fixed while its kernel runs (re-queued work goes to a list
// of a later kernel).  The count is read first, so a CTA that finds the list
// empty or drained takes no atomic: an empty list costs every CTA one read
// instead of an atomic on the counter all CTAs share.
__device__ __forceinline__ uint32_t take_work(const Work &W, int list) {
    const uint32_t n = *(volatile uint32_t *)&W.ctr[2 * list];
    if (*(volatile uint32_t *)&W.ctr[2 * list + 1] >= n) return 0xFFFFFFFFu;
    const uint32_t w = atomicAdd(&W.ctr[2 * list + 1], 1u);
    return w < n ? w : 0xFFFFFFFFu;
}

// Next (query, part) of a dense work list (P parts per query), part-major:
// every query's part 0, then every query's part 1, ...  The CTAs running at
// one time then count the same id range of different queries, and the slice
// of the posting lists in that range (a fraction of the index that fits L2)
// is read from HBM about once and from L2 by the other queries covering it.
__device__ __forceinline__ bool take_dense(const Work &W, int list, uint32_t P, uint2 &out) {
    const uint32_t nq = *(volatile uint32_t *)&W.ctr[2 * list];
    const uint32_t n = nq * P;
    if (*(volatile uint32_t *)&W.ctr[2 * list + 1] >= n) return false;
    const uint32_t w = atomicAdd(&W.ctr[2 * list + 1], 1u);
    if (w >= n) return false;
    const uint32_t p = w / nq, i = w - p * nq;
    out = make_uint2(W.work[(size_t)list * W.work_stride + i].x, p);
    return true;
}

// Scratch / merge of a query's parts.  Part p of query q keeps its sorted
// top-k keys in scratch[out_off*max_parts + p*k ..].
struct MergeSet {
    const uint64_t *keys;
    const uint32_t *cnt;
    uint32_t parts, k, max_parts;
    template <class F>
    __device__ void for_each(F f) const {
        for (uint32_t p = 0; p < parts; ++p) {
            const uint32_t n = __ldcg(cnt + p);
            for (uint32_t b = 0; b < n; b += blockDim.x) {
                uint32_t i = b + threadIdx.x;
                bool act = i < n;
                act = act && GG_OK((size_t)p * k + i, (size_t)max_parts * k, 6);
                uint64_t key = act ? __ldcg(keys + (size_t)p * k + i) : 0ull;
                f(act, key_prim(key), key_id(key));
            }
        }
    }
};

__device__ void convert_to_dense(const DevIndex &ix, const Work &W, const Tuning &T, uint32_t q) {
    QInfo qi = W.qinfo[q];
    const bool small = (qi.flags & kFlagSmallCount) != 0;
    qi.parts = (uint16_t)dense_parts(ix, W, T, small);
    qi.cls = kClsDense;
    W.qinfo[q] = qi;
    W.done[q] = 0;
    W.qstate[q] = 0;         // the dense parts' merge must not see the sparse overflow again
    W.lb[q] = 0;
    const int list = small ? kListDenseSmall : kListDenseWide;
    uint2 *wl = W.work + (size_t)list * W.work_stride;
    const uint32_t at = atomicAdd(&W.ctr[2 * list], 1u);
    if (GG_OK(at, W.work_stride, 13)) wl[at] = make_uint2(q, 0u);
}

// Finish one part: publish its keys, and let the last part merge them.
__device__ void finish_part(const DevIndex &ix, const Work &W, const Tuning &T, const DevQueries &Q,
                            uint32_t q, uint32_t p, const QInfo &qi, uint64_t *cand, uint32_t n,
                            SelectScratch &ss, bool failed) {
    const int64_t out_off = Q.out_off[q];
    const bool weighted = (qi.flags & kFlagWeighted) != 0;
    if (qi.parts == 1 && !failed) {
        write_results(W, out_off, qi.k, cand, n, weighted, qi.scale);
        return;
    }
    const size_t mp = (size_t)W.max_parts;
    uint64_t *dst = W.scratch + (size_t)out_off * mp + (size_t)p * qi.k;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        if (GG_OK((size_t)out_off * mp + (size_t)p * qi.k + i, (size_t)W.out_cap * mp, 5))
            __stcg(dst + i, cand[i]);
    if (threadIdx.x == 0) {
        __stcg(W.part_cnt + (size_t)q * mp + p, failed ? 0u : n);
        if (failed) atomicOr(&W.qstate[q], 1u);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t prev = atomicAdd(&W.done[q], 1u);
        ss.sc[12] = (prev == (uint32_t)qi.parts - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (!ss.sc[12]) return;
    __threadfence();
    if (atomicAdd(&W.qstate[q], 0u) & 1u) {       // a sparse part overflowed: redo densely
        if (threadIdx.x == 0) convert_to_dense(ix, W, T, q);
        __syncthreads();
        return;
    }
    MergeSet ms{W.scratch + (size_t)out_off * mp, W.part_cnt + (size_t)q * mp, qi.parts, qi.k,
                (uint32_t)mp};
    const int bits = (qi.flags & kFlagSmallCount) ? 8 : 32;
    uint32_t nn = select_topk(ms, qi.k, bits, cand, kCandCap, ss);
    write_results(W, out_off, qi.k, cand, nn, weighted, qi.scale);
    __syncthreads();
    if (threadIdx.x == 0) W.done[q] = 0;
}

// ------------------------------------------------------------------ sparse


template <bool PACKED>
struct HashSet {
    const void *tab;
    uint32_t cap;
    template <class F>
    __device__ void for_each(F f) const {
        for (uint32_t b = 0; b < cap; b += blockDim.x) {
            uint32_t i = b + threadIdx.x;
            bool act = i < cap;
            uint32_t prim = 0, id = 0;
            if (PACKED) {
                uint32_t v = act ? ((const uint32_t *)tab)[i] : 0u;
                act = act && v != 0;
                prim = v & 255u;
                id = v >> 8;
            } else {
                uint64_t v = act ? ((const uint64_t *)tab)[i] : 0ull;
                act = act && v != 0;
                prim = (uint32_t)v;
                id = (uint32_t)(v >> 32) - 1u;
            }
            f(act, prim, id);
        }
    }
};

// Per-part hash of object id -> count (or fixed-point weight sum) in shared
// memory; replaces the per-query bitmap + c-PQ (match_device_utils.h:160-446).
// NT = 512: two CTAs per SM with mid-size tables; NT = 1024: one CTA per SM
// with the largest table, so a query needs fewer id-range parts.
template <bool PACKED, int NT>
__device__ __forceinline__ void sparse_list(const DevIndex &ix, const DevQueries &Q, const Work &W, const Tuning &T) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t tid = threadIdx.x;
    const uint32_t slots_max = PACKED ? (uint32_t)T.sparse_slots_packed : (uint32_t)T.sparse_slots_wide;
    const size_t tab_bytes = (size_t)slots_max * (PACKED ? 4 : 8);
    unsigned char *tab_raw = smem;
    unsigned char *uni = smem + tab_bytes;                      // items | candidates
    ItemStage st;
    st.start = (int64_t *)uni;
    st.len = (uint32_t *)(uni + kItemChunk * 8);
    st.inc = (uint32_t *)(uni + kItemChunk * 12);
    st.flat = (uint32_t *)(uni + kItemChunk * 16);
    uint64_t *cand = (uint64_t *)uni;
    SelectScratch &ss = *(SelectScratch *)(uni + kCandCap * 8);
    // slots whose count reached 2, behind the staged units (candidates later
    // overwrite the units, never this list: kPromCap keys end below it)
    uint32_t *prom = (uint32_t *)(uni + kPromOff);
    __shared__ uint32_t s_work, s_prom;

    const int list = PACKED ? kListSparsePacked : kListSparseWide;
    for (;;) {
        if (tid == 0) s_work = take_work(W, list);
        __syncthreads();
        const uint32_t w = s_work;
        __syncthreads();
        if (w == 0xFFFFFFFFu) break;
        const uint2 wk = W.work[(size_t)list * W.work_stride + w];
        const uint32_t q = wk.x, p = wk.y;
        if (!GG_OK(q, W.q_cap, 12)) continue;
        const QInfo qi = W.qinfo[q];
        const uint32_t P = qi.parts;
        const uint32_t id_lo = (uint32_t)(((uint64_t)ix.n_objects * p) / P);
        const uint32_t id_hi = (uint32_t)(((uint64_t)ix.n_objects * (p + 1)) / P);

        // pass 1: part size (posting ids in the part's sub-spans) bounds the distinct ids
        uint64_t part_total = 0;
        for (int32_t c0 = 0; c0 < qi.n_units; c0 += kItemChunk) {
            const int32_t mc = min(kItemChunk, qi.n_units - c0);
            part_total += stage_range(ix, W, qi, c0, mc, P > 1 && p > 0, P > 1 && p < P - 1, id_lo, id_hi, st, ss);
            if (qi.n_units > kItemChunk) __syncthreads();
        }
        const bool single = qi.n_units <= kItemChunk;
        const bool overflow = part_total * 100 > (uint64_t)slots_max * T.sparse_load_pct;
        uint64_t *cand_out = cand;
        uint32_t nres = 0;
        if (!overflow) {
            uint32_t cap = (uint32_t)umin64((uint64_t)slots_max, part_total * 100 / T.sparse_load_pct + 64);
            cap = (cap + 31) & ~31u;
            if (cap > slots_max) cap = slots_max;
            // zero the table
            uint4 *t4 = (uint4 *)tab_raw;
            const uint32_t n4 = (cap * (PACKED ? 4 : 8) + 15) / 16;
            for (uint32_t i = tid; i < n4; i += blockDim.x) t4[i] = make_uint4(0, 0, 0, 0);
            if (tid == 0) s_prom = 0;
            __syncthreads();
            for (int32_t c0 = 0; c0 < qi.n_units; c0 += kItemChunk) {
                const int32_t mc = min(kItemChunk, qi.n_units - c0);
                if (!single)          // restage this chunk (pass 1 kept only the last)
                    stage_range(ix, W, qi, c0, mc, P > 1 && p > 0, P > 1 && p < P - 1, id_lo, id_hi, st, ss);
                __syncthreads();
                const uint32_t F = st.flat[mc];
                if (!ix.codec) {
                    // plain lists: 8 ids per lane, lane-queue insert
                    stream_ids(ix.ids, ix.n_ids, st, (uint32_t)mc, F, [&](uint32_t(&v)[8], uint32_t(&inc)[8]) {
                        hash_insert8<PACKED>(tab_raw, cap, v, inc, prom, &s_prom);
                    });
                } else if (PACKED) {
                    // compressed lists: ids arrive one by one from the warp decoders
                    // (divergent lanes), so every lane probes on its own
                    uint32_t *tab = (uint32_t *)tab_raw;
                    stream_units(ix, st, (uint32_t)mc, F, id_lo, id_hi, [&](uint32_t id, uint32_t) {
                        uint32_t h = slot_of(id, cap);
                        const uint32_t want = (id << 8) | 1u;
                        for (uint32_t probe = 0; probe < cap; ++probe) {
                            if (!GG_OK(h, cap, 2)) return;
                            uint32_t cur = tab[h];
                            if (cur == 0u) {
                                uint32_t old = atomicCAS(&tab[h], 0u, want);
                                if (old == 0u) return;
                                cur = old;
                            }
                            if ((cur >> 8) == id) {
                                // the one increment that takes a slot from 1 to 2 promotes it
                                if ((atomicAdd(&tab[h], 1u) & 255u) == 1u) {
                                    const uint32_t at = atomicAdd(&s_prom, 1u);
                                    if (at < (uint32_t)kPromCap) prom[at] = h;
                                }
                                return;
                            }
                            h = (h + 1 == cap) ? 0 : h + 1;
                        }
                    });
                } else {
                    unsigned long long *tab = (unsigned long long *)tab_raw;
                    stream_units(ix, st, (uint32_t)mc, F, id_lo, id_hi, [&](uint32_t id, uint32_t inc) {
                        uint32_t h = slot_of(id, cap);
                        const unsigned long long tag = (unsigned long long)(id + 1u) << 32;
                        for (uint32_t probe = 0; probe < cap; ++probe) {
                            if (!GG_OK(h, cap, 2)) return;
                            unsigned long long cur = tab[h];
                            if (cur == 0ull) {
                                unsigned long long old = atomicCAS(&tab[h], 0ull, tag | inc);
                                if (old == 0ull) return;
                                cur = old;
                            }
                            if ((cur & 0xFFFFFFFF00000000ull) == tag) {
                                atomicAdd(&tab[h], (unsigned long long)inc);
                                return;
                            }
                            h = (h + 1 == cap) ? 0 : h + 1;
                        }
                    });
                }
                __syncthreads();
            }
            const uint32_t n_prom = PACKED ? s_prom : 0u;
            if (PACKED && n_prom >= qi.k && n_prom <= (uint32_t)kPromCap) {
                // every slot outside the promoted list holds a count of 1, below
                // every promoted count: the exact top-k lies inside the list
                const uint32_t *tab = (const uint32_t *)tab_raw;
                const uint32_t np2 = next_pow2(n_prom);
                for (uint32_t i = tid; i < np2; i += blockDim.x) {
                    uint64_t key = 0;
                    if (i < n_prom) {
                        const uint32_t v = tab[prom[i]];
                        key = make_key(v & 255u, v >> 8);
                    }
                    cand_out[i] = key;
                }
                bitonic_sort_desc(cand_out, np2);
                nres = qi.k;
            } else {
                HashSet<PACKED> hs{tab_raw, cap};
                const int bits = PACKED ? 8 : 32;
                nres = select_topk(hs, qi.k, bits, cand_out, kCandCap, ss);
            }
        }
        finish_part(ix, W, T, Q, q, p, qi, cand_out, nres, ss, overflow);
        __syncthreads();
    }
}

// Both sparse work lists in one launch (their tables take the same shared
// memory): the 4-byte-slot list, then the 8-byte-slot list.  Each list is
// drained before the next; a launch whose lists are empty costs one check.
template <int NT>
__global__ void __launch_bounds__(NT, NT == 512 ? 2 : 1) k_sparse(DevIndex ix, DevQueries Q, Work W, Tuning T) {
    sparse_list<true, NT>(ix, Q, W, T);
    sparse_list<false, NT>(ix, Q, W, T);
}

// ------------------------------------------------------------------ bitmap

}  // namespace gg

#include "bitmap.cuh"

namespace gg {

// ------------------------------------------------------------------ dense

template <bool SMALL>
struct TileSet {
    const uint32_t *cnt;     // counters (bytes packed 4 per word when SMALL)
    uint32_t n_ids;          // ids in this tile (multiple of 16 when SMALL)
    uint32_t tile_lo;
    uint32_t thr;            // admit primaries > thr
    const uint64_t *S;
    uint32_t nS;
    template <class F>
    __device__ void for_each(F f) const {
        for (uint32_t b = 0; b < nS; b += blockDim.x) {
            uint32_t i = b + threadIdx.x;
            bool act = i < nS;
            uint64_t key = act ? S[i] : 0ull;
            f(act, key_prim(key), key_id(key));
        }
        const uint32_t per = SMALL ? 16u : 4u;
        const uint32_t nvec = (n_ids + per - 1) / per;
        const uint32_t thr4 = SMALL ? thr * 0x01010101u : thr;
        for (uint32_t b = 0; b < nvec; b += blockDim.x) {
            uint32_t v = b + threadIdx.x;
            bool act = v < nvec;
            uint4 w = act ? ((const uint4 *)cnt)[v] : make_uint4(0, 0, 0, 0);
            bool any;
            if (SMALL)
                any = (__vcmpgtu4(w.x, thr4) | __vcmpgtu4(w.y, thr4) | __vcmpgtu4(w.z, thr4) |
                       __vcmpgtu4(w.w, thr4)) != 0u;
            else
                any = w.x > thr || w.y > thr || w.z > thr || w.w > thr;
            if (__ballot_sync(0xffffffffu, act && any) == 0u) continue;
            const uint32_t words[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (uint32_t e = 0; e < per; ++e) {
                uint32_t prim = SMALL ? ((words[e >> 2] >> ((e & 3) * 8)) & 255u) : words[e];
                uint32_t local = v * per + e;
                f(act && prim > thr && local < n_ids, prim, tile_lo + local);
            }
        }
    }
};

// Id-tiled dense counters in shared memory; one CTA sweeps the tiles of one
// query part, keeping its running top-k.  Replaces the per-query global bitmap
// (match.cu:276-294, match_device_utils.h:422-446), which wraps above
// 2^bits - 1; these counters are sized from the item count and never wrap.
template <bool SMALL>
__device__ __forceinline__ void dense_list(const DevIndex &ix, const DevQueries &Q, const Work &W, const Tuning &T) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t tid = threadIdx.x;
    const uint32_t tile_cap = SMALL ? (uint32_t)T.dense_tile_u8 : (uint32_t)T.dense_tile_u32;
    const size_t cnt_bytes = (size_t)tile_cap * (SMALL ? 1 : 4);
    uint32_t *cnt = (uint32_t *)smem;
    uint64_t *S = (uint64_t *)(smem + cnt_bytes);
    uint64_t *cand = S + kMaxK;
    unsigned char *it_raw = (unsigned char *)(cand + kCandCap);
    int64_t *cur = (int64_t *)it_raw;
    ItemStage st;
    st.start = (int64_t *)(it_raw + kItemChunk * 8);
    st.len = (uint32_t *)(it_raw + kItemChunk * 16);
    st.inc = (uint32_t *)(it_raw + kItemChunk * 20);
    st.flat = (uint32_t *)(it_raw + kItemChunk * 24);
    SelectScratch &ss = *(SelectScratch *)(it_raw + kItemChunk * 28 + 16);
    // units counted from a dense-list bitmap: their bitmap row and increment,
    // and per unit of a single-chunk query its bitmap row (~0u: none)
    uint32_t *bm_row = (uint32_t *)(it_raw + kItemChunk * 28 + 16 + sizeof(SelectScratch));
    uint32_t *bm_inc = bm_row + kItemChunk;
    uint32_t *unit_bm = bm_inc + kItemChunk;
    __shared__ uint32_t s_q, s_p, s_nS, s_nc, s_L, s_nbm;

    const int list = SMALL ? kListDenseSmall : kListDenseWide;
    const uint32_t P_list = (uint32_t)dense_parts(ix, W, T, SMALL);
    // the tile directory of this counter width, when built for this tile size
    const uint32_t *dir = SMALL ? ix.dir8 : ix.dir32;
    const bool use_dir = dir != nullptr && ix.dir_slot != nullptr && W.unit_key != nullptr &&
                         (SMALL ? ix.dir8_tile : ix.dir32_tile) == (int32_t)tile_cap;
    // dense lists counted from their bitmaps (tiles start at a word boundary)
    const bool use_bm = ix.bm_slot != nullptr && W.unit_key != nullptr && tile_cap % 32u == 0 &&
                        (T.dense_bitmaps & (SMALL ? 1 : 2)) != 0;
    for (;;) {
        if (tid == 0) {
            uint2 wk;
            if (!take_dense(W, list, P_list, wk)) wk.x = 0xFFFFFFFFu;
            s_q = wk.x;
            s_p = wk.y;
        }
        __syncthreads();
        const uint32_t q = s_q, p = s_p;
        __syncthreads();
        if (q == 0xFFFFFFFFu) break;
        if (!GG_OK(q, W.q_cap, 12)) continue;
        const QInfo qi = W.qinfo[q];
        const uint32_t P = qi.parts;
        const uint64_t N = (uint64_t)ix.n_objects;
        const uint64_t ntiles = (N + tile_cap - 1) / tile_cap;
        const uint64_t t0 = ntiles * p / P, t1 = ntiles * (p + 1) / P;
        const bool single = qi.n_units <= kItemChunk;
        if (tid == 0) {
            s_nS = 0;
            s_nbm = 0;
        }
        // per unit of a single-chunk query: its tile-directory row, kept in
        // cur as -1 - row, or else a cursor at the part's first id; and its
        // dense-list bitmap row
        if (single && (int32_t)tid < qi.n_units) {
            const int64_t it = qi.unit0 + tid;
            const int64_t s0 = W.span_start[it], e0 = s0 + W.span_len[it];
            unit_bm[tid] = (use_bm && e0 > s0) ? ix.bm_slot[W.unit_key[it]] : 0xFFFFFFFFu;
            const uint32_t row = (use_dir && e0 > s0) ? ix.dir_slot[W.unit_key[it]] : 0xFFFFFFFFu;
            cur[tid] = row != 0xFFFFFFFFu ? -1 - (int64_t)row
                                          : ((t0 == 0 || e0 == s0) ? s0
                                                                   : first_unit_near(ix, s0, e0, (uint32_t)(t0 * tile_cap), N));
        }
        __syncthreads();
        for (uint64_t t = t0; t < t1; ++t) {
            // the query's lower bound, read now so that its latency passes
            // during the tile's stream (a bound read earlier is still a bound)
            uint32_t L_early = 0;
            if (tid == 0) L_early = *(volatile uint32_t *)&W.lb[q];
            const uint32_t tile_lo = (uint32_t)(t * tile_cap);
            const uint32_t tile_hi = (uint32_t)umin64(N, (t + 1) * tile_cap);
            const uint32_t n_ids = tile_hi - tile_lo;
            const uint32_t n_pad = (n_ids + 15) & ~15u;
            // zero the counters of this tile
            uint4 *c4 = (uint4 *)cnt;
            const uint32_t n4 = (n_pad * (SMALL ? 1 : 4)) / 16;
            for (uint32_t i = tid; i < n4; i += blockDim.x) c4[i] = make_uint4(0, 0, 0, 0);
            bool any_ids = false;
            for (int32_t c0 = 0; c0 < qi.n_units; c0 += kItemChunk) {
                const int32_t mc = min(kItemChunk, qi.n_units - c0);
                uint32_t len = 0;
                if ((int32_t)tid < mc) {
                    const int64_t it = qi.unit0 + c0 + tid;
                    const int64_t s0 = W.span_start[it], e0 = s0 + W.span_len[it];
                    uint32_t row = 0xFFFFFFFFu;
                    if (single) {
                        if (cur[tid] < 0) row = (uint32_t)(-1 - cur[tid]);
                    } else if (use_dir && e0 > s0) {
                        row = ix.dir_slot[W.unit_key[it]];
                    }
                    int64_t a, b;
                    const uint32_t brow = single ? unit_bm[tid]
                                                 : ((use_bm && e0 > s0) ? ix.bm_slot[W.unit_key[it]] : 0xFFFFFFFFu);
                    if (brow != 0xFFFFFFFFu) {          // counted from its bitmap, not streamed
                        const uint32_t at = atomicAdd(&s_nbm, 1u);
                        bm_row[at] = brow;
                        bm_inc[at] = W.inc[it];
                        a = b = s0;
                    } else if (row != 0xFFFFFFFFu) {
                        // the tile's cut from the directory: the first id (segment) at or past
                        // each bound; a compressed segment straddling tile_lo starts the cut
                        const uint32_t *r = dir + (size_t)row * (size_t)(ntiles + 1);
                        const uint32_t fa = __ldg(r + t), fb = __ldg(r + t + 1);
                        a = s0 + (ix.codec ? (fa ? fa - 1 : 0) : fa);
                        b = s0 + fb;
                    } else {
                        a = single ? cur[tid] : (t == 0 ? s0 : first_unit(ix, s0, e0, tile_lo));
                        b = (tile_hi >= N) ? e0 : next_unit_near(ix, a, s0, e0, tile_lo, tile_hi, N);
                        // a compressed segment may straddle tile_hi: the next tile starts at it again
                        if (single) cur[tid] = (ix.codec && b > a) ? b - 1 : b;
                    }
                    st.start[tid] = a;
                    st.inc[tid] = W.inc[it];
                    len = (uint32_t)(b - a);
                    st.len[tid] = len;
                }
                // plain lists go by warp tasks of kRun positions, segments in runs of kSegRun
                const uint32_t units = ix.codec ? (len + kSegRun - 1) / kSegRun : (len + kRun - 1) / kRun;
                uint32_t tot = 0;
                uint32_t off = block_excl_scan(units, ss.tmp, &tot);
                if ((int32_t)tid < mc) st.flat[tid] = off;
                if (tid == 0) st.flat[mc] = tot;
                __syncthreads();
                if (tot) any_ids = true;
                // dense lists from their bitmaps: thread j owns the tile's objects
                // 32j .. 32j+31 (counter words 8j .. 8j+7, or 32j .. 32j+31), so the
                // adds need no atomics; the id stream below waits for them
                const uint32_t nbm = s_nbm;
                if (nbm) {
                    any_ids = true;
                    const uint32_t *rows = ix.bm_rows + (tile_lo >> 5);
                    const uint32_t nwords = (n_ids + 31) >> 5;
                    constexpr uint32_t kBmLoads = 8;      // bitmap words in flight per thread
                    static_assert(kBmLoads == 8, "the adder tree takes eight rows a group");
                    for (uint32_t j = tid; j < nwords; j += blockDim.x) {
                        // byte counters: the lists' bits are summed bit-sliced (plane t holds
                        // bit t of each object's count so far, at most 24 lists a pass), then
                        // each nibble of the planes is spread into its four counter bytes
                        uint32_t p0 = 0, p1 = 0, p2 = 0, p3 = 0, p4 = 0, in_pass = 0;
                        // the next group's words load while this group is summed
                        uint32_t wn[kBmLoads];
#pragma unroll
                        for (uint32_t i = 0; i < kBmLoads; ++i)
                            wn[i] = i < nbm ? __ldg(rows + (size_t)bm_row[i] * (size_t)ix.bm_words + j) : 0u;
                        for (uint32_t u0 = 0; u0 < nbm; u0 += kBmLoads) {
                            uint32_t w[kBmLoads];
#pragma unroll
                            for (uint32_t i = 0; i < kBmLoads; ++i) w[i] = wn[i];
#pragma unroll
                            for (uint32_t i = 0; i < kBmLoads; ++i)
                                wn[i] = u0 + kBmLoads + i < nbm
                                            ? __ldg(rows + (size_t)bm_row[u0 + kBmLoads + i] * (size_t)ix.bm_words + j)
                                            : 0u;
                            if (SMALL) {
                                // the eight rows' bits into the planes by a carry-save adder
                                // tree (full adders: sum a^b^c, carry majority(a,b,c)); a group
                                // adds at most 8, so one weight-8 carry ripples into p3, p4
                                auto csa = [](uint32_t &s, uint32_t &c, uint32_t a, uint32_t b, uint32_t d) {
                                    const uint32_t u = a ^ b;
                                    s = u ^ d;
                                    c = (a & b) | (u & d);
                                };
                                uint32_t t2a, t2b, t2c, t2d, t4a, t4b, t8;
                                csa(p0, t2a, p0, w[0], w[1]);
                                csa(p0, t2b, p0, w[2], w[3]);
                                csa(p1, t4a, p1, t2a, t2b);
                                csa(p0, t2c, p0, w[4], w[5]);
                                csa(p0, t2d, p0, w[6], w[7]);
                                csa(p1, t4b, p1, t2c, t2d);
                                csa(p2, t8, p2, t4a, t4b);
                                const uint32_t c3 = p3 & t8;
                                p3 ^= t8;
                                p4 ^= c3;
                                in_pass += kBmLoads;
                                if (in_pass + kBmLoads > 31 || u0 + kBmLoads >= nbm) {
#pragma unroll
                                    for (int k = 0; k < 8; ++k) {
                                        auto spread = [](uint32_t x) { return (x * 0x00204081u) & 0x01010101u; };
                                        const int sh = 4 * k;
                                        cnt[8 * j + k] += spread((p0 >> sh) & 15u) + (spread((p1 >> sh) & 15u) << 1) +
                                                          (spread((p2 >> sh) & 15u) << 2) + (spread((p3 >> sh) & 15u) << 3) +
                                                          (spread((p4 >> sh) & 15u) << 4);
                                    }
                                    p0 = p1 = p2 = p3 = p4 = 0;
                                    in_pass = 0;
                                }
                            } else {
#pragma unroll
                                for (uint32_t i = 0; i < kBmLoads; ++i) {
                                    const uint32_t inc = u0 + i < nbm ? bm_inc[u0 + i] : 0u;
                                    uint32_t x = w[i];
                                    while (x) {
                                        const uint32_t bit = (uint32_t)__ffs((int)x) - 1u;
                                        cnt[32 * j + bit] += inc;
                                        x &= x - 1u;
                                    }
                                }
                            }
                        }
                    }
                    __syncthreads();
                    if (tid == 0) s_nbm = 0;
                }
                if (SMALL) {
                    // byte counters, four to a word: the word at loc & ~3, the byte (loc & 3)
                    auto add = [&](uint32_t id, uint32_t) {
                        const uint32_t loc = id - tile_lo;
                        if (GG_OK(loc, n_ids, 3))
                            atomicAdd((uint32_t *)((unsigned char *)cnt + (loc & ~3u)), __funnelshift_l(0u, 1u, loc << 3));
                    };
                    if (ix.codec) stream_segment_runs(ix, st, (uint32_t)mc, tot, tile_lo, tile_hi, add);
                    else stream_runs(ix.ids, st, (uint32_t)mc, tot, add);
                } else {
                    auto add = [&](uint32_t id, uint32_t inc) {
                        if (GG_OK(id - tile_lo, n_ids, 3)) atomicAdd(&cnt[id - tile_lo], inc);
                    };
                    if (ix.codec) stream_segment_runs(ix, st, (uint32_t)mc, tot, tile_lo, tile_hi, add);
                    else stream_runs(ix.ids, st, (uint32_t)mc, tot, add);
                }
                __syncthreads();
            }
            if (!any_ids) continue;
            // Merge this tile into the running top-k S.  A tile id enters
            // with a primary above S's k-th once S is full (on a tie S's id,
            // from an earlier tile of this part, is smaller), and never below
            // L, the largest k-th primary a finished tile of another part of
            // the query has found: the query's final k-th primary is at least
            // L, so nothing below it can place.
            if (tid == 0) s_L = L_early;
            __syncthreads();
            const uint32_t nS = s_nS, L = s_L;
            uint32_t thr = nS == qi.k ? key_prim(S[qi.k - 1]) : 0u;
            if (L > 0 && L - 1 > thr) thr = L - 1;
            // A query's first tile (nothing known yet), byte counters: T, the
            // k-th largest of the 16-counter vectors' maxima, bounds the
            // tile's k-th count from below (k vectors hold a counter >= T),
            // so the counters >= T hold the tile's top-k.
            bool bounded = false;
            if (SMALL && nS == 0 && L == 0) {
                const uint32_t nvec = (n_ids + 15) / 16;
                for (uint32_t i = tid; i < 256; i += blockDim.x) ss.hist[i] = 0;
                __syncthreads();
                for (uint32_t b = 0; b < nvec; b += blockDim.x) {
                    const uint32_t v = b + tid;
                    const bool act = v < nvec;
                    const uint4 w = act ? ((const uint4 *)cnt)[v] : make_uint4(0, 0, 0, 0);
                    uint32_t mx = __vmaxu4(__vmaxu4(w.x, w.y), __vmaxu4(w.z, w.w));
                    mx = __vmaxu4(mx, mx >> 16);
                    const uint32_t m8 = max(mx & 255u, (mx >> 8) & 255u);
                    hist_add(ss.hist, m8, act && m8 > 0);
                }
                __syncthreads();
                if (warp_id() == 0) find_digit(ss, qi.k, true);
                __syncthreads();
                if (!ss.sc[3]) {
                    thr = ss.sc[0] - 1;
                    bounded = true;
                }
                __syncthreads();
            }
            if (nS == qi.k || L > 0 || bounded) {
                // Few counters usually pass: collect them behind a copy of S
                // and sort the union.
                if (tid == 0) s_nc = 0;
                for (uint32_t i = tid; i < nS; i += blockDim.x) cand[i] = S[i];
                __syncthreads();
                const uint32_t room = (uint32_t)kCandCap - nS;
                const uint32_t per = SMALL ? 16u : 4u;
                const uint32_t nvec = (n_ids + per - 1) / per;
                const uint32_t thr4 = SMALL ? thr * 0x01010101u : thr;
                // bytes above thr < 127: bit 7 of (low seven bits + 127 - thr),
                // which carries into no other byte, or the byte's own bit 7
                const bool narrow = SMALL && thr < 127u;
                const uint32_t bias4 = narrow ? (127u - thr) * 0x01010101u : 0u;
                // each thread walks its own passing counters (a handful per
                // tile), so a vector without one costs a load and compares
                for (uint32_t v = tid; v < nvec; v += blockDim.x) {
                    const uint4 w = ((const uint4 *)cnt)[v];
                    const uint32_t words[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                    for (uint32_t h = 0; h < 4; ++h) {
                        // a nonzero bit in each byte of a passing counter
                        uint32_t hit = !SMALL  ? (words[h] > thr ? 0xFFu : 0u)
                                       : narrow ? ((((words[h] & 0x7F7F7F7Fu) + bias4) | words[h]) & 0x80808080u)
                                                : __vcmpgtu4(words[h], thr4);
                        while (hit) {
                            const uint32_t byte = (uint32_t)(__ffs((int)hit) - 1) >> 3;
                            hit &= ~(0xFFu << (8 * byte));
                            const uint32_t prim = SMALL ? (words[h] >> (8 * byte)) & 255u : words[h];
                            const uint32_t local = SMALL ? v * 16 + h * 4 + byte : v * 4 + h;
                            if (local < n_ids) {
                                const uint32_t at = atomicAdd(&s_nc, 1u);
                                if (at < room) cand[nS + at] = make_key(prim, tile_lo + local);
                            }
                        }
                    }
                }
                __syncthreads();
                const uint32_t m = s_nc;
                if (m <= room) {
                    const uint32_t np2 = next_pow2(nS + m);
                    for (uint32_t i = nS + m + tid; i < np2; i += blockDim.x) cand[i] = 0ull;
                    bitonic_sort_desc(cand, np2);
                    const uint32_t nk = min(nS + m, qi.k);
                    for (uint32_t i = tid; i < nk; i += blockDim.x) S[i] = cand[i];
                    if (tid == 0) s_nS = nk;
                    __syncthreads();
                    // a full S raises the query's lower bound for its other parts
                    if (tid == 0 && nk == qi.k && key_prim(S[qi.k - 1]) > L)
                        atomicMax(&W.lb[q], key_prim(S[qi.k - 1]));
                    continue;
                }
            }
            TileSet<SMALL> ts{cnt, n_ids, tile_lo, thr, S, nS};
            const uint32_t nn = select_topk(ts, qi.k, SMALL ? 8 : 32, cand, kCandCap, ss);
            for (uint32_t i = tid; i < nn; i += blockDim.x)
                if (GG_OK(i, kMaxK, 10)) S[i] = cand[i];
            if (tid == 0) s_nS = nn;
            __syncthreads();
            if (tid == 0 && nn == qi.k && key_prim(S[qi.k - 1]) > L) atomicMax(&W.lb[q], key_prim(S[qi.k - 1]));
        }
        const uint32_t nS = s_nS;
        for (uint32_t i = tid; i < nS; i += blockDim.x) cand[i] = S[i];
        __syncthreads();
        finish_part(ix, W, T, Q, q, p, qi, cand, nS, ss, false);
        __syncthreads();
    }
}

// Both dense work lists in one launch (1-byte and 4-byte counter tiles take
// the same shared memory), one after the other.
__global__ void __launch_bounds__(1024, 1) k_dense(DevIndex ix, DevQueries Q, Work W, Tuning T) {
    dense_list<true>(ix, Q, W, T);
    dense_list<false>(ix, Q, W, T);
}

// ------------------------------------------------------------------ host side

size_t sparse_smem_bytes(const Tuning &t, bool packed) {
    size_t tab = (size_t)(packed ? t.sparse_slots_packed * 4 : t.sparse_slots_wide * 8);
    size_t uni = std::max<size_t>(kItemChunk * 20 + 16, kCandCap * 8);
    return tab + uni + sizeof(SelectScratch) + 64;
}

size_t dense_smem_bytes(const Tuning &t, bool small) {
    size_t c = (size_t)(small ? t.dense_tile_u8 : t.dense_tile_u32 * 4);
    return c + (size_t)kMaxK * 8 + (size_t)kCandCap * 8 + kItemChunk * 28 + 16 + sizeof(SelectScratch) + kItemChunk * 12 +
           64;
}

Tuning default_tuning() {
    Tuning t;
    t.sparse_slots_packed = 22528;   // 88 KiB of 4-byte slots: two CTAs per SM
    t.sparse_slots_wide = 11264;     // 88 KiB of 8-byte slots
    t.sparse_threads = 512;
    t.dense_tile_u8 = 147456;        // 144 KiB of 1-byte counters
    t.dense_tile_u32 = 36864;        // 144 KiB of 4-byte counters
    t.dense_threads = 1024;
    t.sparse_max_total = 16 * 16896;
    t.dense_part_work = 147456;      // one 1-byte tile (four 4-byte tiles) per dense part
    t.sparse_ctas_per_sm = 2;
    t.dense_ctas_per_sm = 1;
    t.sparse_load_pct = 50;
    t.bitmap_bits = 1179648;         // id spaces up to 144 KiB of presence bits
    t.bitmap_multi_slots = 2048;     // 8 KiB table of repeated ids
    t.bitmap_ready = 0;              // set per launch
    t.dense_bitmaps = 1;             // dense lists from their bitmaps for byte counters (unweighted)
    return t;
}

static cudaError_t set_smem(const void *fn, size_t bytes) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

size_t sparse_smem_both(const Tuning &t) { return std::max(sparse_smem_bytes(t, true), sparse_smem_bytes(t, false)); }
size_t dense_smem_both(const Tuning &t) { return std::max(dense_smem_bytes(t, true), dense_smem_bytes(t, false)); }

cudaError_t prepare_kernels(const Tuning &t) {
    cudaError_t e;
    if ((e = set_smem((const void *)k_sparse<512>, sparse_smem_both(t)))) return e;
    if ((e = set_smem((const void *)k_sparse<1024>, sparse_smem_both(t)))) return e;
    if ((e = set_smem((const void *)k_dense, dense_smem_both(t)))) return e;
    return cudaSuccess;
}

cudaError_t prepare_kernels_max() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (optin <= 0) optin = 227 * 1024;
    const void *fns[] = {(const void *)k_sparse<512>, (const void *)k_sparse<1024>, (const void *)k_dense,
                         (const void *)k_bitmap};
    for (const void *fn : fns) {
        cudaFuncAttributes a;
        cudaError_t e = cudaFuncGetAttributes(&a, fn);
        if (e) return e;
        // static and dynamic shared memory together may not exceed the opt-in limit
        if ((e = set_smem(fn, (size_t)optin - a.sharedSizeBytes))) return e;
    }
    return cudaSuccess;
}

// Whether the bitmap kernel's shared memory (bitmap, table, chunk entries)
// fits for an id space of n objects under this tuning.
bool bitmap_fits(const Tuning &t, int64_t n_objects) {
    static size_t limit = 0;
    if (!limit) {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (optin <= 0) optin = 227 * 1024;
        cudaFuncAttributes a;
        size_t st = 1024;
        if (cudaFuncGetAttributes(&a, (const void *)k_bitmap) == cudaSuccess) st = a.sharedSizeBytes;
        limit = (size_t)optin - st;
    }
    // the table's entries (half its slots) fit the tie and candidate buffers
    if (t.bitmap_bits <= 0 || n_objects > t.bitmap_bits || t.bitmap_multi_slots <= 0 ||
        t.bitmap_multi_slots > 2 * kCandCap)
        return false;
    return bm_layout(n_objects, (uint32_t)t.bitmap_multi_slots).bytes <= limit;
}

// Per-launch tuning: SM count, and whether the bitmap kernel fits this index.
Tuning launch_tuning(const DevIndex &ix, const Tuning &tun, int num_sms) {
    Tuning t = tun;
    t.num_sms = num_sms;
    t.bitmap_ready = bitmap_fits(t, ix.n_objects) ? 1 : 0;
    if (!t.bitmap_ready) t.bitmap_bits = 0;
    return t;
}

int launch_plan(const DevIndex &ix, const DevQueries &Q, const Work &W, const Tuning &t, cudaStream_t s) {
    cudaMemsetAsync(W.ctr, 0, kCtrWords * sizeof(uint32_t), s);
    k_plan<<<Q.n_queries, kPlanThreads, 0, s>>>(ix, Q, W, t);
    return 1;
}

// The match kernels as persistent grids: the bitmap kernel, the sparse
// kernel (both slot widths), the dense kernel (both counter widths).
enum : int { kKernBitmap = 0, kKernSparse = 1, kKernDense = 2, kNumKern = 3 };
int launch_kernel(int kern, const DevIndex &ix, const DevQueries &Q, const Work &W, const Tuning &t, int num_sms,
                  cudaStream_t s) {
    // persistent grids: as many CTAs as fit on every SM at once
    auto grid = [&](const void *fn, int threads, size_t smem) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
        return num_sms * std::max(1, per_sm);
    };
    switch (kern) {
    case kKernBitmap: {
        if (t.bitmap_bits <= 0) return 0;
        const size_t bp = bm_layout(ix.n_objects, (uint32_t)t.bitmap_multi_slots).bytes;
        k_bitmap<<<num_sms, kBmThreads, bp, s>>>(ix, Q, W, t);
        return 1;
    }
    case kKernSparse: {
        const size_t sp = sparse_smem_both(t);
        if (t.sparse_threads == 1024) k_sparse<1024><<<grid((const void *)k_sparse<1024>, 1024, sp), 1024, sp, s>>>(ix, Q, W, t);
        else k_sparse<512><<<grid((const void *)k_sparse<512>, 512, sp), 512, sp, s>>>(ix, Q, W, t);
        return 1;
    }
    default: {
        const size_t dp = dense_smem_both(t);
        k_dense<<<grid((const void *)k_dense, t.dense_threads, dp), t.dense_threads, dp, s>>>(ix, Q, W, t);
        return 1;
    }
    }
}

int launch_match(const DevIndex &ix, const DevQueries &Q, const Work &W, const Tuning &tun,
                 int num_sms, cudaStream_t s, cudaEvent_t *ev) {
    if (Q.n_queries <= 0) return 0;
    const Tuning t = launch_tuning(ix, tun, num_sms);
    int launches = 0;
    if (ev) cudaEventRecord(ev[0], s);
    launches += launch_plan(ix, Q, W, t, s);
    if (ev) cudaEventRecord(ev[1], s);
    // dense last: sparse parts that overflow are re-queued to the dense lists
    for (int k = 0; k < kNumKern; ++k) {
        launches += launch_kernel(k, ix, Q, W, t, num_sms, s);
        if (ev) cudaEventRecord(ev[2 + k], s);
    }
    return launches;
}

}  // namespace gg
