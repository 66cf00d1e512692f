// device.cuh -- shared device-side types and primitives of the match path.
//
// Layout in HBM (one resident index):
//   ids       u32[n_ids (+pad)]   posting ids, ordered by (dim, value, id)
//                                 -- identical to the reference's inv_table::_inv
//                                 (table/inv_table.cu:281-337)
//   key_off   i64[n_keys+1]       start of each (dim,value) list in ids
//   key_base  i64[D+1]            first key of each dim (no 16-bit value limit,
//                                 unlike the reference's (dim<<16)+value keys,
//                                 table/inv_table.h:212)
//   dim_min / dim_max i32[D]      value bounds of each dim
// A compressed index adds the reference codec segments (see codecs.cuh).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gg {

constexpr int kMaxParts = 16;        // id-range parts of one sparse query
constexpr int kMaxDenseParts = 64;   // id-range parts of one dense query (Work::max_parts bounds a search)
constexpr int kMaxK = 2048;          // largest k per query
constexpr int kItemChunk = 512;      // query items staged in shared memory at once
constexpr int kCandCap = 2048;       // candidate buffer of the top-k selection

enum : uint8_t { kClsNone = 0, kClsSparse = 1, kClsDense = 2 };
enum : uint8_t { kFlagWeighted = 1, kFlagSmallCount = 2, kFlagRetry = 4, kFlagPacked = 8 };
// posting lists a query may cover on the bitmap path (one per thread)
constexpr uint32_t kBmSpanCap = 1024;
// posting ids of a query on the bitmap path (its 32-id chunk entries)
constexpr uint32_t kBmMaxIds = 40 * 1024;
// zero bytes behind the posting ids of a plain index: 32 ids read from the
// last position stay inside the allocation
constexpr size_t kIdsPadBytes = 128;

enum : uint32_t { kErrWeight = 1, kErrOverflow = 2, kErrCapacity = 4, kErrUnits = 8, kErrTimeout = 16,
                  kErrBounds = 32 };

struct DevIndex {
    const uint32_t *ids;
    const int64_t *key_off;
    const int64_t *key_base;
    const int32_t *dim_min;
    const int32_t *dim_max;
    int64_t n_objects;
    int64_t n_ids;
    int32_t n_dims;
    int32_t mult_max;
    int32_t is_bag;
    // compressed layout (codec != 0)
    int32_t codec;
    int32_t max_seg;
    const uint32_t *words;         // encoded segments
    const int64_t *key_seg;        // [n_keys+1] first segment of each key
    const int64_t *seg_word_off;   // [n_segs+1] first word of each segment
    const uint32_t *seg_first;     // [n_segs] first id of each segment (skip pointer)
    const int64_t *seg_pos;        // [n_segs+1] posting position of each segment
    // tile directories (tile_dir.cu): dir_slot[key] = row of a long list (~0u:
    // none); row r of dir8 / dir32 holds, for the tiles of dir8_tile /
    // dir32_tile ids, the offset in the list of its first id (segment) at or
    // past each tile boundary, ntiles + 1 entries.  Null / 0 when absent.
    const uint32_t *dir_slot;
    const uint32_t *dir8;
    const uint32_t *dir32;
    int32_t dir8_tile;
    int32_t dir32_tile;
    // presence bitmaps of the dense lists (tile_dir.cu): bm_slot[key] = row of
    // a list holding >= 1/16 of the objects (~0u: none); a row is bm_words
    // words, bit o set when object o is listed.  Null when absent.
    const uint32_t *bm_slot;
    const uint32_t *bm_rows;
    int64_t bm_words;
};

struct DevQueries {
    int32_t n_queries;
    const int64_t *item_off;
    const int32_t *dim;
    const int32_t *low;
    const int32_t *up;
    const float *weight;
    const uint8_t *weighted;
    const uint32_t *k;
    uint32_t uniform_k;
    const int64_t *out_off;
    // optional device-side size of a captured batch: dyn[0] = queries in this
    // run (<= n_queries, the capacity), dyn[1] = uniform k, dyn[2] = 1 when
    // every item is exact (up = low; the up array is not sent)
    const uint32_t *dyn;
};

// Per-query plan written by k_plan.
struct QInfo {
    int64_t total;      // posting ids touched (sum of span lengths)
    int64_t unit0;      // first unit (one sorted posting list of one item)
    int64_t item0;      // first item
    int32_t n_units;
    int32_t n_items;
    uint32_t k;
    int32_t scale;      // fixed-point exponent of a weighted query
    uint16_t parts;     // id-range parts
    uint8_t cls;        // kClsSparse / kClsDense / kClsNone
    uint8_t flags;
};

struct Tuning {
    int32_t sparse_slots_packed;   // hash slots per CTA, 4-byte entries
    int32_t sparse_slots_wide;     // hash slots per CTA, 8-byte entries
    int32_t sparse_threads;
    int32_t dense_tile_u8;         // ids per tile, 1-byte counters
    int32_t dense_tile_u32;        // ids per tile, 4-byte counters
    int32_t dense_threads;
    int64_t sparse_max_total;      // more touched ids than this -> dense
    int64_t dense_part_work;       // objects per dense id-range part (whole tiles, at least one)
    int32_t sparse_ctas_per_sm;
    int32_t dense_ctas_per_sm;
    int32_t sparse_load_pct;       // posting ids per part <= this % of the hash slots
    int32_t bitmap_bits;           // largest id space of the bitmap kernel (0: off)
    int32_t bitmap_multi_slots;    // slots of its table of ids seen twice or more
    int32_t bitmap_ready;          // 1 when its shared memory fits the id space (set per launch)
    int32_t num_sms;               // SMs of the device (set per launch)
    int32_t dense_bitmaps;         // counter widths whose dense lists use their bitmaps: 1 bytes, 2 words
};

// Work lists, one per kernel variant.
enum : int { kListSparsePacked = 0, kListSparseWide = 1, kListDenseSmall = 2, kListDenseWide = 3,
             kListBitmap = 4, kNumLists = 5 };
constexpr int kCtrError = 2 * kNumLists;     // ctr[2c] = items in list c, ctr[2c+1] = next
constexpr int kCtrUnits = 2 * kNumLists + 2;  // 64-bit: units handed out to queries so far
constexpr int kCtrWords = 2 * kNumLists + 4;

// Device work state of one search (all arrays sized for the batch).
struct Work {
    int64_t *item_k0;      // [items] first key an item covers
    uint32_t *item_nk;     // [items] keys it covers (0: matches nothing)
    uint32_t *item_inc;    // [items] increment per match (1, or fixed-point weight)
    int64_t *span_start;   // [units] start of the unit's sorted list (or first segment)
    int64_t *span_len;     // [units] its length (or segment count)
    uint32_t *inc;         // [units] increment per match
    uint32_t *unit_key;    // [units] (dim,value) key of the unit's list (null: not written)
    QInfo *qinfo;          // [Q]
    uint2 *work;           // [kNumLists][Q*kMaxParts] (query, part); a dense list holds (query, 0) once
    int64_t work_stride;   // Q*kMaxParts
    uint32_t *ctr;         // [kCtrWords]
    uint32_t *qstate;      // [Q] bit0: a sparse part overflowed
    uint32_t *done;        // [Q] finished parts
    uint32_t *lb;          // [Q] lower bound on the k-th primary of a dense query (from its finished tiles)
    uint32_t *part_cnt;    // [Q*max_parts]
    uint64_t *scratch;     // [sum(k)*max_parts] part results (keys)
    int32_t max_parts;     // parts of a dense query (<= kMaxDenseParts); scratch stride per result slot
    uint32_t *out_ids;
    uint32_t *out_counts;
    float *out_scores;     // may be null
    // capacities: units_cap, items_cap and out_cap are enforced by the plan
    // kernel in every build (a query outside them gets no work); q_cap
    // bounds the checked build
    int64_t units_cap;
    int64_t items_cap;
    int64_t q_cap;
    int64_t out_cap;
};

// ---------------------------------------------------------------- checked builds
//
// Built with -DGG_CHECKED, every index below is bounds-checked; the first
// violation is recorded (site, index, bound) in gg_oob and the access is
// skipped, so a faulty index shows up as a report instead of a memory fault.
#ifdef GG_CHECKED
// one copy per translation unit: only match.cu's kernels report into theirs
static __device__ unsigned long long gg_oob[4];
__device__ __forceinline__ bool gg_report(uint32_t site, uint64_t idx, uint64_t n) {
    if (atomicCAS(&gg_oob[0], 0ull, (unsigned long long)site) == 0ull) {
        gg_oob[1] = idx;
        gg_oob[2] = n;
        gg_oob[3] = ((unsigned long long)blockIdx.x << 32) | threadIdx.x;
    }
    return false;
}
#define GG_OK(idx, n, site) (((uint64_t)(idx) < (uint64_t)(n)) || gg::gg_report((site), (uint64_t)(idx), (uint64_t)(n)))
#else
#define GG_OK(idx, n, site) true
#endif

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t warp_id() { return threadIdx.x >> 5; }

// First position p in [lo, hi) with ids[p] >= x.
__device__ __forceinline__ int64_t lower_bound_u32(const uint32_t *__restrict__ a, int64_t lo,
                                                   int64_t hi, uint32_t x) {
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Galloping search from lo: first position in [lo, hi) with a[p] >= x.
__device__ __forceinline__ int64_t gallop_u32(const uint32_t *__restrict__ a, int64_t lo,
                                              int64_t hi, uint32_t x) {
    if (lo >= hi || __ldg(a + lo) >= x) return lo;
    int64_t step = 1, prev = lo;
    while (true) {
        int64_t probe = prev + step;
        if (probe >= hi) return lower_bound_u32(a, prev + 1, hi, x);
        if (__ldg(a + probe) >= x) return lower_bound_u32(a, prev + 1, probe, x);
        prev = probe;
        step <<= 1;
    }
}

// First position p in [lo, hi) with a[p] >= x (hi if none), a sorted, by
// 8-way probes: every step issues 8 independent loads and keeps the
// sub-range between the last probe below x and the first at or above it.
// The first step centres its probes on `guess` at a spacing of `win` (an
// estimate of the answer and of its error), later steps split the range
// evenly, so a good guess needs ~3 dependent steps instead of the ~2 log2(n)
// of a galloping search.
__device__ __forceinline__ int64_t probe8_first_ge(const uint32_t *__restrict__ a, int64_t lo, int64_t hi,
                                                   uint32_t x, int64_t guess, int64_t win) {
    int64_t L = lo, H = hi;          // the answer lies in [L, H]
    bool first = true;
    while (H - L > 8) {
        // probe offsets from L (a list holds < 2^32 ids)
        const uint32_t n = (uint32_t)(H - L);
        const int64_t c = guess - L;
        uint32_t off[8], v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            int64_t q = first ? c + (int64_t)(j - 4) * win : (int64_t)(((uint64_t)n * (j + 1)) / 9);
            off[j] = (uint32_t)(q < 0 ? 0 : (q > (int64_t)n - 1 ? (int64_t)n - 1 : q));
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = __ldg(a + L + off[j]);
        uint32_t nl = 0, nh = n;      // new range [L + nl, L + nh]
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (v[j] < x) nl = max(nl, off[j] + 1);
            else nh = min(nh, off[j]);
        }
        H = L + nh;
        L = L + min(nl, nh);
        first = false;
    }
    uint32_t below = 0;      // the last <= 8 positions, loaded together
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (L + j < H && __ldg(a + L + j) < x) ++below;
    return L + below;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane_id() >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide exclusive scan of one u32 per thread; s_tmp holds >= 33 words.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *s_tmp, uint32_t *total) {
    const uint32_t nw = (blockDim.x + 31) >> 5;
    uint32_t incl = warp_incl_scan(v);
    __syncthreads();
    if (lane_id() == 31) s_tmp[warp_id()] = incl;
    __syncthreads();
    if (warp_id() == 0) {
        uint32_t x = lane_id() < nw ? s_tmp[lane_id()] : 0u;
        uint32_t xi = warp_incl_scan(x);
        if (lane_id() < nw) s_tmp[lane_id()] = xi - x;
        if (lane_id() == nw - 1) s_tmp[32] = xi;
    }
    __syncthreads();
    uint32_t r = s_tmp[warp_id()] + incl - v;
    if (total) *total = s_tmp[32];
    __syncthreads();
    return r;
}

// Exclusive scan over a group of whole warps (G::rank() order); tmp holds 33
// words.  Starts with a barrier, so back-to-back calls may share tmp.
template <class G>
__device__ uint32_t group_excl_scan(uint32_t v, uint32_t *tmp, uint32_t *total) {
    const uint32_t r = G::rank(), w = r >> 5, nw = G::size() >> 5, l = lane_id();
    const uint32_t incl = warp_incl_scan(v);
    G::sync();
    if (l == 31) tmp[w] = incl;
    G::sync();
    if (w == 0) {
        const uint32_t x = l < nw ? tmp[l] : 0u;
        const uint32_t xi = warp_incl_scan(x);
        if (l < nw) tmp[l] = xi - x;
        if (l == 31) tmp[32] = xi;
    }
    G::sync();
    if (total) *total = tmp[32];
    return tmp[w] + incl - v;
}

// block_excl_scan without its first and last barriers, for callers that
// order the earlier readers of s_tmp before the call and its later writers
// after it (a barrier on each side within the caller's own flow).
__device__ __forceinline__ uint32_t block_excl_scan_lean(uint32_t v, uint32_t *s_tmp, uint32_t *total) {
    const uint32_t nw = (blockDim.x + 31) >> 5;
    const uint32_t incl = warp_incl_scan(v);
    if (lane_id() == 31) s_tmp[warp_id()] = incl;
    __syncthreads();
    if (warp_id() == 0) {
        const uint32_t x = lane_id() < nw ? s_tmp[lane_id()] : 0u;
        const uint32_t xi = warp_incl_scan(x);
        if (lane_id() < nw) s_tmp[lane_id()] = xi - x;
        if (lane_id() == nw - 1) s_tmp[32] = xi;
    }
    __syncthreads();
    if (total) *total = s_tmp[32];
    return s_tmp[warp_id()] + incl - v;
}

// Warp-aggregated shared-memory histogram increment: lanes holding the same
// bin combine into one atomic (__match_any_sync).  All 32 lanes must call.
__device__ __forceinline__ void hist_add(uint32_t *hist, uint32_t bin, bool active) {
    uint32_t act = __ballot_sync(0xffffffffu, active);
    if (!active) return;
    uint32_t peers = __match_any_sync(act, bin);
    if (lane_id() == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&hist[bin], (uint32_t)__popc(peers));
}

// Result key: primary (count or fixed-point weight sum) high, inverted id low,
// so that a larger key ranks first and equal primaries rank by ascending id.
__device__ __forceinline__ uint64_t make_key(uint32_t prim, uint32_t id) {
    return ((uint64_t)prim << 32) | (uint64_t)(0xFFFFFFFFu - id);
}
__device__ __forceinline__ uint32_t key_prim(uint64_t k) { return (uint32_t)(k >> 32); }
__device__ __forceinline__ uint32_t key_id(uint64_t k) { return 0xFFFFFFFFu - (uint32_t)k; }

// A group of threads that cooperates like a block (rank, size, barrier); the
// helpers below take one, here always the whole block.
struct BlockGroup {
    __device__ static uint32_t rank() { return threadIdx.x; }
    __device__ static uint32_t size() { return blockDim.x; }
    __device__ static void sync() { __syncthreads(); }
};

// Compare-exchange: the larger key when keep_max, else the smaller.
__device__ __forceinline__ uint64_t cmpx(uint64_t x, uint64_t y, bool keep_max) {
    return (keep_max == (x > y)) ? x : y;
}

// Bitonic stages of one merge size with strides <= 32 on two keys per thread
// (x0 = key 2t, x1 = key 2t+1): the partner of a stride >= 2 lives in lane
// t ^ (stride/2) of the same warp, so no shared memory or barrier is needed.
// Every lane of the warp must take part.
__device__ __forceinline__ void bitonic_reg_stages(uint64_t &x0, uint64_t &x1, uint32_t t, uint32_t size,
                                                   uint32_t stride) {
    const bool desc = ((2u * t) & size) == 0;
    for (; stride >= 2; stride >>= 1) {
        const uint32_t d = stride >> 1;
        const bool lower = ((2u * t) & stride) == 0;
        const uint64_t y0 = __shfl_xor_sync(0xffffffffu, x0, d);
        const uint64_t y1 = __shfl_xor_sync(0xffffffffu, x1, d);
        x0 = cmpx(x0, y0, lower == desc);
        x1 = cmpx(x1, y1, lower == desc);
    }
    const uint64_t hi = x0 > x1 ? x0 : x1, lo = x0 > x1 ? x1 : x0;
    x0 = desc ? hi : lo;
    x1 = desc ? lo : hi;
}

// Descending bitonic sort of n (power of two) keys in shared memory.  Strides
// up to 32 run in registers (shuffles); only the longer strides of the merges
// of 128 keys and more go through shared memory, one barrier each.
template <class G = BlockGroup>
__device__ __forceinline__ void bitonic_sort_desc(uint64_t *a, uint32_t n) {
    const uint32_t t = G::rank(), nt = G::size();
    G::sync();
    if (n <= 1) return;
    if (n <= 64) {          // one warp, keys past n read as 0 (the smallest key)
        if (t < 32) {
            uint64_t x0 = 2 * t < n ? a[2 * t] : 0ull, x1 = 2 * t + 1 < n ? a[2 * t + 1] : 0ull;
            for (uint32_t size = 2; size <= 64; size <<= 1) bitonic_reg_stages(x0, x1, t, size, size >> 1);
            if (2 * t < n) a[2 * t] = x0;
            if (2 * t + 1 < n) a[2 * t + 1] = x1;
        }
        G::sync();
        return;
    }
    if (n <= 2 * nt) {
        const bool act = t < n / 2;      // whole warps: n/2 is a multiple of 32
        uint64_t x0 = 0, x1 = 0;
        if (act) {
            x0 = a[2 * t];
            x1 = a[2 * t + 1];
            for (uint32_t size = 2; size <= 64; size <<= 1) bitonic_reg_stages(x0, x1, t, size, size >> 1);
        }
        for (uint32_t size = 128; size <= n; size <<= 1) {
            if (act) {
                a[2 * t] = x0;
                a[2 * t + 1] = x1;
            }
            for (uint32_t stride = size >> 1; stride >= 64; stride >>= 1) {
                G::sync();
                if (act) {
                    const uint32_t i = 2 * t - (t & (stride - 1)), j = i + stride;
                    const bool desc = (i & size) == 0;
                    const uint64_t x = a[i], y = a[j];
                    if ((x < y) == desc) { a[i] = y; a[j] = x; }
                }
            }
            G::sync();
            if (act) {
                x0 = a[2 * t];
                x1 = a[2 * t + 1];
                bitonic_reg_stages(x0, x1, t, size, 32);
            }
        }
        if (act) {
            a[2 * t] = x0;
            a[2 * t + 1] = x1;
        }
        G::sync();
        return;
    }
    for (uint32_t size = 2; size <= n; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            G::sync();
            for (uint32_t u = t; u < n / 2; u += nt) {
                uint32_t i = 2 * u - (u & (stride - 1));
                uint32_t j = i + stride;
                bool desc = ((i & size) == 0);
                uint64_t x = a[i], y = a[j];
                if ((x < y) == desc) { a[i] = y; a[j] = x; }
            }
        }
    }
    G::sync();
}

__device__ __forceinline__ uint32_t next_pow2(uint32_t v) {
    return v <= 1 ? 1u : 1u << (32 - __clz(v - 1));
}

// Write the final k results of query q from sorted keys.
__device__ __forceinline__ void write_results(const Work &W, int64_t out_off, uint32_t k,
                                              const uint64_t *sorted, uint32_t n, bool weighted,
                                              int32_t scale) {
    for (uint32_t j = threadIdx.x; j < k; j += blockDim.x) {
        if (!GG_OK(out_off + j, W.out_cap, 4)) continue;
        uint32_t id = 0, cnt = 0;
        float sc = 0.0f;
        if (j < n) {
            uint64_t key = sorted[j];
            uint32_t prim = key_prim(key);
            id = key_id(key);
            if (weighted) {
                sc = __double2float_rn(ldexp((double)prim, -scale));
                cnt = (uint32_t)sc;              // (int) aggregation, knn.cu:54
            } else {
                cnt = prim;
                sc = (float)prim;
            }
        }
        W.out_ids[out_off + j] = id;
        W.out_counts[out_off + j] = cnt;
        if (W.out_scores) W.out_scores[out_off + j] = sc;
    }
}

}  // namespace gg

namespace gg {
__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }
}  // namespace gg
