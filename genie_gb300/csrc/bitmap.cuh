// bitmap.cuh -- k_bitmap: match counting of unweighted sparse queries with a
// presence bitmap over the whole id space.
//
// Reference counterpart: the per-query bitmap counter plus c-PQ of match_AT
// (matching/match_device_utils.h:160-446, match.cu:43-464).  The reference
// keeps a packed counter per object in global memory and updates it with a
// global atomicCAS per posting id; here one CTA per SM owns an n-bit bitmap in
// shared memory and a small table of the ids seen twice or more.
//
// One CTA per SM, queries assigned round-robin, per query:
//   stage   one 32-id chunk entry per 32 posting ids of every covered list
//           (the lists' spans were loaded into registers during the previous
//           query);
//   stream  warp w takes chunks w, w+32, ...: 16 coalesced chunk loads in
//           flight per lane, then 16 independent atomicOr on the bitmap; a
//           first occurrence sets the id's bit, a repeat goes to the table
//           (id<<8 | count, count >= 2), which also keeps a histogram of its
//           counts;
//   select  with >= k table ids, the histogram gives the k-th count c*; the
//           (few) ids above c* are placed by rank, and the ids at c* go
//           through a counting sort by id range (1024 buckets, each then
//           sorted in place; a crowded bucket falls back to a bitonic sort of
//           all ties); these buffers lie over the bitmap, which nothing reads
//           any more; the result is the first k.  With fewer, the result is the whole
//           table, then the smallest ids whose bit is set and that are not in
//           the table (count 1).  A full table hands the query to the dense
//           kernel.  New table entries are listed as they are made, so these
//           passes and the clear touch the entries, not every slot;
//   clear   bitmap, table entries and histogram.
// Posting lists are ~100-500 byte runs at random places of the id array:
// plain loads with many in flight per lane keep more bytes in flight per SM
// than per-list asynchronous copies.
#pragma once

namespace gg {

constexpr uint32_t kBmThreads = 1024;
constexpr uint32_t kBmChunks = 2048;      // 32-id chunks per query on this path
// selection buffers of a query with >= k table entries, over the bitmap (which
// nothing reads then): candidate keys, tie ids, tie keys, bucket counters,
// the ranked candidates
constexpr uint32_t kBmScrTieIds = kCandCap * 8;
constexpr uint32_t kBmScrTieKeys = kBmScrTieIds + kCandCap * 4;
constexpr uint32_t kBmScrBuckets = kBmScrTieKeys + kCandCap / 2 * 8;
constexpr uint32_t kBmScrRanked = kBmScrBuckets + 1024 * 4;
constexpr uint32_t kBmRankMax = 256;      // entries above c* ordered by rank (more: a bitonic sort)
constexpr uint32_t kBmScratch = kBmScrRanked + kBmRankMax * 8;
static_assert(kBmChunks >= (uint32_t)kMaxK, "the chunk region holds the keys of a query with < k table entries");
constexpr uint32_t kBmProbe = 128;        // longest probe run of the repeated-id table
constexpr int kBmRound = 16;              // chunk loads in flight per lane
static_assert(kBmRound == 16, "the repeat loop selects v[r] by four bits of r");
constexpr uint32_t kBmDescRing = 128;     // query descriptors kept in shared memory
constexpr uint32_t kBmDescFill = 64;      // descriptors loaded at a time

// Byte offsets of the shared-memory regions (host and device agree).
struct BmLayout {
    uint32_t bm, mt, mlist, chunk, ss, bytes, bm_words;
};
__host__ __device__ inline uint32_t bm_align(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }
__host__ __device__ inline BmLayout bm_layout(int64_t n_objects, uint32_t mslots) {
    BmLayout L;
    uint32_t o = 0;
    L.bm_words = (uint32_t)((n_objects + 127) / 128) * 4;
    L.bm = o;     o += bm_align(L.bm_words * 4 > kBmScratch ? L.bm_words * 4 : kBmScratch, 128);
    L.mt = o;     o += bm_align(mslots * 4, 128);
    L.mlist = o;  o += bm_align(mslots / 2 * 4, 128);     // slots of the table's entries
    L.chunk = o;  o += kBmChunks * 8;      // also the result keys of a query with < k table entries
    L.ss = o;     o += bm_align((uint32_t)sizeof(SelectScratch), 16);
    L.bytes = bm_align(o, 128);
    return L;
}

// ------------------------------------------------------------ selection helpers

// The `need` smallest ids whose bit is set in bm[0, words), ascending, as keys
// (prim, id) into out[].  Warp w of the group scans a contiguous range of
// 16-byte groups; only warps whose range starts below `need` set bits emit.
// Returns the number of set bits.
template <class G>
__device__ uint32_t bitmap_take_smallest(const uint32_t *bm, uint32_t words, uint32_t need, uint32_t prim,
                                         uint64_t *out, SelectScratch &ss) {
    const uint32_t lane = lane_id(), w = G::rank() >> 5, nw = G::size() >> 5;
    const uint4 *g4 = (const uint4 *)bm;
    const uint32_t groups = (words + 3) / 4;
    const uint32_t per = (groups + nw - 1) / nw;
    const uint32_t g0 = min(groups, w * per), g1 = min(groups, g0 + per);
    uint32_t c = 0;
    for (uint32_t g = g0 + lane; g < g1; g += 32) {
        const uint4 x = g4[g];
        c += __popc(x.x) + __popc(x.y) + __popc(x.z) + __popc(x.w);
    }
    const uint32_t wsum = __shfl_sync(0xffffffffu, warp_incl_scan(c), 31);
    G::sync();
    if (lane == 0) ss.tmp[w] = wsum;
    G::sync();
    if (w == 0) {
        const uint32_t x = lane < nw ? ss.tmp[lane] : 0u;
        const uint32_t xi = warp_incl_scan(x);
        if (lane < nw) ss.tmp[lane] = xi - x;
        if (lane == 31) ss.tmp[32] = xi;
    }
    G::sync();
    uint32_t base = ss.tmp[w];
    const uint32_t total = ss.tmp[32];
    for (uint32_t g = g0; g < g1 && base < need; g += 32) {     // warp-uniform
        const uint32_t gi = g + lane;
        const uint4 x = gi < g1 ? g4[gi] : make_uint4(0u, 0u, 0u, 0u);
        const uint32_t cnt = __popc(x.x) + __popc(x.y) + __popc(x.z) + __popc(x.w);
        const uint32_t incl = warp_incl_scan(cnt);
        uint32_t r = base + incl - cnt;
        if (r < need && cnt) {
            const uint32_t wv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint32_t bits = wv[q];
                while (bits && r < need) {
                    const uint32_t b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    out[r++] = make_key(prim, (gi * 4 + q) * 32 + b);
                }
            }
        }
        base += __shfl_sync(0xffffffffu, incl, 31);
    }
    G::sync();
    return total;
}

// Append `keep` entries of a warp to dst (warp-aggregated); all lanes call.
__device__ __forceinline__ void warp_append(bool keep, uint64_t key, uint64_t *dst, uint32_t *counter) {
    const uint32_t mk = __ballot_sync(0xffffffffu, keep);
    uint32_t at = 0;
    if (lane_id() == 0 && mk) at = atomicAdd(counter, (uint32_t)__popc(mk));
    at = __shfl_sync(0xffffffffu, at, 0);
    if (keep) dst[at + __popc(mk & ((1u << lane_id()) - 1u))] = key;
}

// ------------------------------------------------------------ kernel

struct BmQuery {
    uint32_t q, k, n_units, pad;
    int64_t unit0, out_off;
};

__global__ void __launch_bounds__(kBmThreads, 1) k_bitmap(DevIndex ix, DevQueries Q, Work W, Tuning T) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t mslots = (uint32_t)T.bitmap_multi_slots;
    const BmLayout L = bm_layout(ix.n_objects, mslots);
    uint32_t *bm = (uint32_t *)(smem + L.bm);
    uint32_t *mt = (uint32_t *)(smem + L.mt);
    // chunk entry: posting position of its first id, ids in it (1..32); an
    // empty entry (0, 0) reads ids [0, 32) and counts none of them
    uint2 *chunk = (uint2 *)(smem + L.chunk);
    uint32_t *mlist = (uint32_t *)(smem + L.mlist);
    uint64_t *cand_few = (uint64_t *)(smem + L.chunk);                    // [0, kMaxK)
    uint64_t *cand_s = (uint64_t *)(smem + L.bm);                         // [0, kCandCap)
    uint32_t *tie_ids = (uint32_t *)(smem + L.bm + kBmScrTieIds);         // [0, kCandCap)
    uint64_t *tie_keys = (uint64_t *)(smem + L.bm + kBmScrTieKeys);       // [0, kCandCap / 2)
    uint64_t *ranked = (uint64_t *)(smem + L.bm + kBmScrRanked);          // [0, kBmRankMax)
    SelectScratch &ss = *(SelectScratch *)(smem + L.ss);
    uint32_t *hist = ss.hist;
    __shared__ uint32_t s_multi, s_ovf, s_n, s_big;
    __shared__ BmQuery s_desc[kBmDescRing];     // item i of this CTA in slot i % kBmDescRing

    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = warp_id();
    const uint32_t G = gridDim.x, n_work = W.ctr[2 * kListBitmap];
    if (blockIdx.x >= n_work) return;
    const uint2 *work = W.work + (size_t)kListBitmap * W.work_stride;
    const uint32_t mcap = mslots / 2;
    const uint32_t words = L.bm_words;

    // descriptors of this CTA's items [i0, i0 + kBmDescFill) into their slots
    // (block-uniform call; a later barrier publishes them).  Loaded in bulk so
    // that no load of a later query waits in a register through a query.
    auto fill_desc = [&](uint32_t i0) {
        if (tid < kBmDescFill) {
            const uint32_t i = i0 + tid;
            BmQuery d{};
            d.q = 0xFFFFFFFFu;
            const uint64_t w = (uint64_t)blockIdx.x + (uint64_t)i * G;
            if (w < n_work && GG_OK(w, W.work_stride, 16)) {
                const uint32_t q = work[w].x;
                if (GG_OK(q, W.q_cap, 16)) {
                    const QInfo qi = W.qinfo[q];
                    d.q = q;
                    d.k = qi.k;
                    d.n_units = (uint32_t)qi.n_units;
                    d.unit0 = qi.unit0;
                    d.out_off = Q.out_off[q];
                }
            }
            s_desc[i % kBmDescRing] = d;
        }
    };

    for (uint32_t i = tid; i < words / 4; i += kBmThreads) ((uint4 *)bm)[i] = make_uint4(0u, 0u, 0u, 0u);
    for (uint32_t i = tid; i < mslots; i += kBmThreads) mt[i] = 0u;
    for (uint32_t i = tid; i < 256; i += kBmThreads) hist[i] = 0u;
    if (tid == 0) {
        s_multi = 0;
        s_ovf = 0;
    }
    fill_desc(0);
    __syncthreads();
    // spans of this thread's list in the current query (prefetched one query ahead)
    int64_t sp_start = 0, sp_len = 0;
    if (tid < s_desc[0].n_units && GG_OK(s_desc[0].unit0 + tid, W.units_cap, 9)) {
        sp_start = W.span_start[s_desc[0].unit0 + tid];
        sp_len = W.span_len[s_desc[0].unit0 + tid];
    }

    for (uint32_t it = 0; blockIdx.x + it * G < n_work; ++it) {
        const bool more = blockIdx.x + (it + 1) * G < n_work;
        // the next descriptors, before the span loads of item it + 1 read them;
        // the slots they take held items finished long ago
        if (more && (it + 1) % kBmDescFill == 0) fill_desc(it + 1);
        // ---- stage: chunk entries of every list
        const uint32_t nch = (uint32_t)((sp_len + 31) / 32);
        uint32_t n_chunks = 0;
        // (the previous query ended with a barrier; the stream starts after one)
        const uint32_t c0 = block_excl_scan_lean(nch, ss.tmp, &n_chunks);
        for (uint32_t c = 0; c < nch && c0 + c < kBmChunks; ++c)
            chunk[c0 + c] = make_uint2((uint32_t)(sp_start + 32 * (int64_t)c),
                                       (uint32_t)min((int64_t)32, sp_len - 32 * (int64_t)c));
        // empty entries up to whole rounds of every warp, so rounds need no bounds
        const uint32_t round_ids = 32u * kBmRound;
        const uint32_t padded = min(kBmChunks, (n_chunks + round_ids - 1) / round_ids * round_ids);
        for (uint32_t c = n_chunks + tid; c < padded; c += kBmThreads) chunk[c] = make_uint2(0u, 0u);
        // spans of the next query, in flight during this one
        sp_start = 0;
        sp_len = 0;
        if (more) {
            const BmQuery dn = s_desc[(it + 1) % kBmDescRing];
            if (tid < dn.n_units && GG_OK(dn.unit0 + tid, W.units_cap, 9)) {
                sp_start = W.span_start[dn.unit0 + tid];
                sp_len = W.span_len[dn.unit0 + tid];
            }
        }
        __syncthreads();

        // ---- stream
        auto repeat = [&](uint32_t id) -> uint32_t {     // 1 for a new table entry
            uint32_t h = slot_of(id, mslots);
            for (uint32_t probe = 0; probe < kBmProbe; ++probe) {
                uint32_t cur = mt[h];
                if (cur == 0u) {
                    const uint32_t old = atomicCAS(&mt[h], 0u, (id << 8) | 2u);
                    if (old == 0u) {
                        atomicAdd(&hist[2], 1u);
                        const uint32_t at = atomicAdd(&s_multi, 1u);
                        if (at < mcap) mlist[at] = h;
                        else s_ovf = 1;
                        return 1u;
                    }
                    cur = old;
                }
                if ((cur >> 8) == id) {
                    const uint32_t c = atomicAdd(&mt[h], 1u) & 255u;     // c + 1 <= 255: small-count query
                    atomicSub(&hist[c], 1u);
                    atomicAdd(&hist[c + 1], 1u);
                    return 0u;
                }
                h = (h + 1 == mslots) ? 0u : h + 1;
            }
            s_ovf = 1;
            return 0u;
        };
        // Integer work per id is what bounds this loop, so it is kept small:
        // every lane loads 32 ids past its entry's position (the id array is
        // padded for that, and every value there is a valid id), and a lane
        // past the entry's count ORs an empty mask into the word of whatever
        // id it read.  Ids are below n_objects (checked when an index is
        // built or loaded), so every word index is inside the bitmap.
        const uint32_t nc = min(n_chunks, kBmChunks);
        const uint32_t *lane_ids = ix.ids + lane;
        for (uint32_t j0 = warp; j0 < nc; j0 += 32 * kBmRound) {
            uint32_t v[kBmRound], ok = 0;
#pragma unroll
            for (int r = 0; r < kBmRound; ++r) {
                const uint2 e = chunk[j0 + r * 32];
                v[r] = __ldg(lane_ids + e.x);
                ok |= lane < e.y ? 1u << r : 0u;
            }
            uint32_t old[kBmRound];
#pragma unroll
            for (int r = 0; r < kBmRound; ++r) {      // independent atomics, all in flight
                if (!GG_OK(v[r] >> 5, words, 15)) v[r] = 0;
                const uint32_t m = __funnelshift_l(0u, (ok >> r) & 1u, v[r]);     // (ok bit r) << (id % 32)
                old[r] = atomicOr(&bm[v[r] >> 5], m) & m;
            }
            uint32_t rep = 0;
#pragma unroll
            for (int r = 0; r < kBmRound; ++r) rep |= (old[r] != 0u ? 1u : 0u) << r;
            while (__any_sync(0xffffffffu, rep != 0u)) {
                if (rep) {
                    const uint32_t r = __ffs(rep) - 1;
                    rep &= rep - 1;
                    // v[r] by a tree of selects on the bits of r (kBmRound = 16)
                    uint32_t t8[8], t4[4], t2[2];
#pragma unroll
                    for (int j = 0; j < 8; ++j) t8[j] = (r & 1u) ? v[2 * j + 1] : v[2 * j];
#pragma unroll
                    for (int j = 0; j < 4; ++j) t4[j] = (r & 2u) ? t8[2 * j + 1] : t8[2 * j];
#pragma unroll
                    for (int j = 0; j < 2; ++j) t2[j] = (r & 4u) ? t4[2 * j + 1] : t4[2 * j];
                    repeat((r & 8u) ? t2[1] : t2[0]);
                }
            }
        }
        __syncthreads();

        // ---- exact top-k of this query
        const BmQuery d = s_desc[it % kBmDescRing];
        const uint32_t k = d.k, q = d.q;
        const int64_t out_off = d.out_off;
        const uint32_t n_multi = min(s_multi, mcap);
        const bool ovf = s_ovf != 0;
        bool failed = ovf || n_chunks > kBmChunks;
        uint32_t nres = 0, n_hi = 0, cstar = 0;     // keys cand[0, n_hi), then tie ids at c*
        uint64_t *cand = cand_few;
        if (!failed && n_multi >= k) {
            cand = cand_s;
            // tie ids go to id-range buckets (counting sort): bucket b holds ids
            // [b << sh, (b+1) << sh); the counters, cleared while warp 0 finds
            // c*, and these buffers lie over the bitmap
            const uint32_t nb = min(1024u, words);
            uint32_t sh = 0;
            while (((uint32_t)(ix.n_objects - 1) >> sh) >= nb) ++sh;
            uint32_t *bcnt = (uint32_t *)((unsigned char *)bm + kBmScrBuckets);
            for (uint32_t x = tid; x < nb; x += kBmThreads) bcnt[x] = 0u;
            if (warp == 0) find_digit(ss, k, true);     // k-th largest count
            if (tid == 0) {
                s_n = 0;
                s_big = 0;
            }
            __syncthreads();
            cstar = ss.sc[0];
            const uint32_t above = ss.sc[1], n_eq = ss.sc[2];
            // entries above c* to cand (warp-aggregated); count the ties per bucket
            for (uint32_t b = 0; b < n_multi; b += kBmThreads) {
                const uint32_t x = b + tid;
                const uint32_t e = x < n_multi ? mt[mlist[x]] : 0u;
                const uint32_t c = e & 255u;
                warp_append(e != 0u && c > cstar, make_key(c, e >> 8), cand, &s_n);
                if (e != 0u && c == cstar) atomicAdd(&bcnt[(e >> 8) >> sh], 1u);
            }
            __syncthreads();
            const uint32_t bc = tid < nb ? bcnt[tid] : 0u;
            if (bc > 32) s_big = 1;      // a crowded id range: sort all ties instead
            uint32_t tot = 0;
            const uint32_t boff = block_excl_scan_lean(bc, ss.tmp, &tot);     // barriers before and after
            if (tid < nb) bcnt[tid] = boff;                              // cursor
            __syncthreads();
            for (uint32_t b = 0; b < n_multi; b += kBmThreads) {
                const uint32_t x = b + tid;
                const uint32_t e = x < n_multi ? mt[mlist[x]] : 0u;
                if (e != 0u && (e & 255u) == cstar) {
                    const uint32_t at = atomicAdd(&bcnt[(e >> 8) >> sh], 1u);
                    if (at < (uint32_t)kCandCap) tie_ids[at] = e >> 8;
                }
            }
            // the entries above c*: few and distinct, each placed at its rank
            if (above <= kBmRankMax && tid < above) {
                const uint64_t key = cand[tid];
                uint32_t rank = 0;
                for (uint32_t j = 0; j < above; ++j) rank += cand[j] > key ? 1u : 0u;
                ranked[rank] = key;
            }
            __syncthreads();
            if (above > kBmRankMax) {
                const uint32_t hp2 = next_pow2(above);
                for (uint32_t x = above + tid; x < hp2; x += kBmThreads) cand[x] = 0ull;
                bitonic_sort_desc(cand, hp2);
            } else {
                cand = ranked;
            }
            const bool big = s_big != 0;
            if (big && next_pow2(n_eq) <= kCandCap / 2) {
                const uint32_t tp2 = next_pow2(n_eq);
                for (uint32_t x = tid; x < tp2; x += kBmThreads)
                    tie_keys[x] = x < n_eq ? make_key(cstar, tie_ids[x]) : 0ull;
                bitonic_sort_desc(tie_keys, tp2);     // one count: ascending ids
                for (uint32_t x = tid; x < n_eq; x += kBmThreads) tie_ids[x] = key_id(tie_keys[x]);
            } else if (big) {
                failed = true;
            } else if (tid < nb && bc > 1) {      // each bucket in id order (a few ids each)
                uint32_t *bk = tie_ids + boff;
                for (uint32_t i = 1; i < bc; ++i) {
                    const uint32_t x = bk[i];
                    uint32_t j = i;
                    while (j > 0 && bk[j - 1] > x) {
                        bk[j] = bk[j - 1];
                        --j;
                    }
                    bk[j] = x;
                }
            }
            __syncthreads();
            n_hi = above;
            nres = k;
            if (n_eq != tot || n_eq > kCandCap) failed = true;
        } else if (!failed) {
            // the whole table, then the smallest ids seen once
            if (tid == 0) s_n = 0;
            __syncthreads();
            for (uint32_t b = 0; b < n_multi; b += kBmThreads) {
                const uint32_t x = b + tid;
                const uint32_t e = x < n_multi ? mt[mlist[x]] : 0u;
                if (e) atomicAnd(&bm[(e >> 8) >> 5], ~(1u << ((e >> 8) & 31)));
                warp_append(e != 0u, make_key(e & 255u, e >> 8), cand, &s_n);
            }
            const uint32_t np2 = next_pow2(n_multi);
            __syncthreads();
            for (uint32_t x = n_multi + tid; x < np2; x += kBmThreads) cand[x] = 0ull;
            bitonic_sort_desc(cand, np2);
            const uint32_t r = k - n_multi;
            const uint32_t singles = bitmap_take_smallest<BlockGroup>(bm, words, r, 1u, cand + n_multi, ss);
            n_hi = n_multi + min(r, singles);
            nres = n_hi;
        }
        if (failed) {
            if (tid == 0) convert_to_dense(ix, W, T, q);
        } else {
            for (uint32_t j = tid; j < k; j += kBmThreads) {
                if (!GG_OK(out_off + j, W.out_cap, 4)) continue;
                uint32_t id = 0, cnt = 0;
                if (j < nres) {
                    if (j < n_hi) {
                        const uint64_t key = cand[j];
                        id = key_id(key);
                        cnt = key_prim(key);
                    } else {
                        id = tie_ids[j - n_hi];
                        cnt = cstar;
                    }
                }
                W.out_ids[out_off + j] = id;
                W.out_counts[out_off + j] = cnt;
                if (W.out_scores) W.out_scores[out_off + j] = (float)cnt;
            }
        }
        // ---- clear the state for the next query
        __syncthreads();
        for (uint32_t x = tid; x < words / 4; x += kBmThreads) ((uint4 *)bm)[x] = make_uint4(0u, 0u, 0u, 0u);
        if (ovf) {
            for (uint32_t x = tid; x < mslots; x += kBmThreads) mt[x] = 0u;
        } else {
            for (uint32_t x = tid; x < n_multi; x += kBmThreads) mt[mlist[x]] = 0u;
        }
        for (uint32_t x = tid; x < 256; x += kBmThreads) hist[x] = 0u;
        if (tid == 0) {      // every thread read both right after the stream, barriers ago
            s_multi = 0;
            s_ovf = 0;
        }
        __syncthreads();
    }
}

}  // namespace gg
