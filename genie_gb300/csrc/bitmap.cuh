// bitmap.cuh -- k_bitmap: match counting of unweighted sparse queries with a
// presence bitmap over the whole id space, fed by bulk asynchronous copies.
//
// Reference counterpart: the per-query bitmap counter plus c-PQ of match_AT
// (matching/match_device_utils.h:160-446, match.cu:43-464).  The reference
// keeps a packed counter per object in global memory and updates it with a
// global atomicCAS per posting id; here one CTA per SM owns an n-bit bitmap in
// shared memory and a small table of the ids seen twice or more.
//
// Warp specialization, one CTA per SM, queries assigned round-robin:
//   warp 0 (producer)   streams each query's posting lists into a ring of
//                       shared-memory pages with cp.async.bulk (16-byte
//                       aligned pieces; the alignment padding is masked out),
//                       one page per mbarrier phase, running ahead across
//                       queries so the next query's ids load while the
//                       consumers select;
//   warps 1..31         take each page: a first occurrence of an id is one
//   (consumers)         atomicOr on its bit; a repeat goes to the table
//                       (id<<8 | count, count >= 2), which also keeps a
//                       histogram of its counts.  After the last page of a
//                       query they select its exact top-k and clear the state.
// Selection: with >= k table ids, the histogram gives the k-th count c*; the
// ids above c* and the ids at c* are sorted apart (ties by ascending id) and
// the result is the first k.  With fewer, the result is the whole table, then
// the smallest ids whose bit is set and that are not in the table (count 1).
// A full table (overflow) hands the query to the dense kernel.
#pragma once

namespace gg {

constexpr uint32_t kBmThreads = 1024;
constexpr uint32_t kBmConsumers = kBmThreads - 32;
using BmConsumers = TailGroup<kBmConsumers>;
constexpr uint32_t kBmPageIds = 2048;     // ids per ring page (8 KiB)
constexpr uint32_t kBmMaxPages = 8;
constexpr uint32_t kBmProbe = 128;        // longest probe run of the repeated-id table
constexpr uint32_t kBmSpanSlot = ((kBmSpanCap + 4) * 16 + (kBmSpanCap + 4) * 4 + 127) / 128 * 128;
constexpr unsigned long long kBmWaitNs = 2000000000ull;   // bound of every wait

struct BmPageHdr {
    uint32_t q, k, fill, last;
    int64_t out_off;
    uint32_t pad[2];
};

// Byte offsets of the shared-memory regions (host and device agree).
struct BmLayout {
    uint32_t bm, mt, ring, hdr, mask, span, cand, ss, bar, bytes, bm_words;
};
__host__ __device__ inline uint32_t bm_align(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }
__host__ __device__ inline BmLayout bm_layout(int64_t n_objects, uint32_t mslots, uint32_t pages) {
    BmLayout L;
    uint32_t o = 0;
    L.bm_words = (uint32_t)((n_objects + 127) / 128) * 4;
    L.bm = o;   o += bm_align(L.bm_words * 4, 128);
    L.mt = o;   o += bm_align(mslots * 4, 128);
    L.ring = o; o += pages * kBmPageIds * 4;
    L.hdr = o;  o += pages * (uint32_t)sizeof(BmPageHdr);
    L.mask = o; o += pages * (kBmPageIds / 32) * 4;
    L.span = o; o += 2 * kBmSpanSlot;
    L.cand = o; o += kCandCap * 8;
    L.ss = o;   o += bm_align((uint32_t)sizeof(SelectScratch), 16);
    L.bar = o;  o += (2 * pages + 2) * 8;
    L.bytes = bm_align(o, 128);
    return L;
}

// ------------------------------------------------------------ async copies

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.release.cta.shared::cta.b64 st, [%0];\n\t}" ::"r"(
                     smem_addr(b))
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n\t}" ::
                     "r"(smem_addr(b)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait for the phase of parity `parity` to complete; false after limit_ns.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, unsigned long long limit_ns = kBmWaitNs) {
    if (mbar_try_wait(b, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(b, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}
// Global -> shared bulk copy (16-byte aligned ends) completing on mbarrier b.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(b))
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

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

__global__ void __launch_bounds__(kBmThreads, 1) k_bitmap(DevIndex ix, DevQueries Q, Work W, Tuning T) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t P = (uint32_t)T.bitmap_pages;
    const uint32_t mslots = (uint32_t)T.bitmap_multi_slots;
    const BmLayout L = bm_layout(ix.n_objects, mslots, P);
    uint32_t *bm = (uint32_t *)(smem + L.bm);
    uint32_t *mt = (uint32_t *)(smem + L.mt);
    uint32_t *ring = (uint32_t *)(smem + L.ring);
    BmPageHdr *hdr = (BmPageHdr *)(smem + L.hdr);
    uint32_t *mask = (uint32_t *)(smem + L.mask);
    unsigned char *span = smem + L.span;
    uint64_t *cand = (uint64_t *)(smem + L.cand);
    SelectScratch &ss = *(SelectScratch *)(smem + L.ss);
    uint64_t *full = (uint64_t *)(smem + L.bar), *empty = full + P, *span_full = empty + P;
    __shared__ uint32_t s_multi, s_ovf, s_n, s_t, s_abort;
    __shared__ uint32_t s_spare[32];

    const uint32_t tid = threadIdx.x, lane = lane_id();
    const uint32_t G = gridDim.x, n_work = W.ctr[2 * kListBitmap];
    if (blockIdx.x >= n_work) return;
    const uint2 *work = W.work + (size_t)kListBitmap * W.work_stride;
    if (tid == 0) {
        for (uint32_t i = 0; i < P; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], kBmConsumers / 32);
        }
        mbar_init(&span_full[0], 1);
        mbar_init(&span_full[1], 1);
        fence_mbar_init();
        s_abort = 0;
        s_multi = 0;
        s_ovf = 0;
    }
    __syncthreads();

    if (tid < 32) {
        // ---------------------------------------------------------- producer
        struct QD {
            uint32_t q, k, n_units;
            int64_t unit0, out_off;
        };
        auto load_qd = [&](uint32_t i) {
            QD d{};
            const uint32_t w = blockIdx.x + i * G;
            if (w < n_work && GG_OK(w, W.work_stride, 16)) {
                d.q = work[w].x;
                if (GG_OK(d.q, W.q_cap, 16)) {
                    const QInfo qi = W.qinfo[d.q];
                    d.k = qi.k;
                    d.n_units = (uint32_t)qi.n_units;
                    d.unit0 = qi.unit0;
                    d.out_off = Q.out_off[d.q];
                }
            }
            return d;
        };
        auto issue_span = [&](uint32_t slot, const QD &d) {     // lane 0
            fence_proxy_async();
            unsigned char *sp = span + slot * kBmSpanSlot;
            const int64_t a0 = d.unit0 & ~(int64_t)1, a1 = (d.unit0 + d.n_units + 1) & ~(int64_t)1;
            const uint32_t bytes = (uint32_t)(a1 - a0) * 8;
            mbar_arrive_expect_tx(&span_full[slot], 2 * bytes);
            bulk_load(sp, W.span_start + a0, bytes, &span_full[slot]);
            bulk_load(sp + (kBmSpanCap + 4) * 8, W.span_len + a0, bytes, &span_full[slot]);
        };
        QD cur{}, nxt{};
        if (lane == 0) {
            cur = load_qd(0);
            issue_span(0, cur);
            nxt = load_qd(1);
        }
        uint32_t pg = 0;
        bool abort = false;
        for (uint32_t i = 0; blockIdx.x + i * G < n_work && !abort; ++i) {
            const uint32_t slot = i & 1;
            QD after{};
            if (lane == 0) {
                if (blockIdx.x + (i + 1) * G < n_work) issue_span(slot ^ 1, nxt);
                after = load_qd(i + 2);
                if (!mbar_wait(&span_full[slot], (i >> 1) & 1)) abort = true;
            }
            abort = __shfl_sync(0xffffffffu, abort ? 1u : 0u, 0) != 0;
            if (abort) break;
            const uint32_t n_units = __shfl_sync(0xffffffffu, cur.n_units, 0);
            const uint32_t sh = __shfl_sync(0xffffffffu, (uint32_t)(cur.unit0 & 1), 0);
            const int64_t *sstart = (const int64_t *)(span + slot * kBmSpanSlot) + sh;
            const int64_t *slen = (const int64_t *)(span + slot * kBmSpanSlot + (kBmSpanCap + 4) * 8) + sh;
            uint32_t *F = (uint32_t *)(span + slot * kBmSpanSlot + (kBmSpanCap + 4) * 16);
            // flat offsets of the 16-byte aligned copies of every list
            uint32_t ftot = 0;
            for (uint32_t j0 = 0; j0 < n_units; j0 += 32) {
                const uint32_t j = j0 + lane;
                uint32_t m = 0;
                if (j < n_units) {
                    const int64_t s = sstart[j], e = s + slen[j];
                    m = (uint32_t)(((e + 3) & ~(int64_t)3) - (s & ~(int64_t)3));
                }
                const uint32_t incl = warp_incl_scan(m);
                if (j < n_units) F[j] = ftot + incl - m;
                ftot += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (lane == 0) F[n_units] = ftot;
            __syncwarp();
            uint32_t jc = 0;     // first list not wholly issued
            for (uint32_t p0 = 0; p0 < ftot; p0 += kBmPageIds, ++pg) {
                const uint32_t p1 = min(p0 + kBmPageIds, ftot);
                const uint32_t ps = pg % P;
                if (lane == 0 && !mbar_wait(&empty[ps], ((pg / P) & 1u) ^ 1u)) abort = true;
                abort = __shfl_sync(0xffffffffu, abort ? 1u : 0u, 0) != 0;
                if (abort) break;
                uint32_t *page = ring + ps * kBmPageIds;
                uint32_t *pm = mask + ps * (kBmPageIds / 32);
                const uint32_t cnt = p1 - p0;
                for (uint32_t x = lane; x < kBmPageIds / 32; x += 32) {
                    const uint32_t b0 = x * 32;
                    pm[x] = b0 >= cnt ? 0u : (cnt - b0 >= 32 ? ~0u : (1u << (cnt - b0)) - 1u);
                }
                __syncwarp();
                for (uint32_t j0 = jc; j0 < n_units && F[j0] < p1; j0 += 32) {
                    const uint32_t j = j0 + lane;
                    if (j < n_units) {
                        const uint32_t fj = F[j], fe = F[j + 1];
                        const uint32_t lo = max(fj, p0), hi = min(fe, p1);
                        if (lo < hi) {
                            const int64_t s = sstart[j], e = s + slen[j];
                            const int64_t a = s & ~(int64_t)3;
                            const uint32_t bytes = (hi - lo) * 4;
                            if (GG_OK(a + (lo - fj) + (hi - lo) - 1, ix.n_ids + 4, 17)) {
                                mbar_expect_tx(&full[ps], bytes);
                                bulk_load(page + (lo - p0), ix.ids + a + (lo - fj), bytes, &full[ps]);
                            }
                            // the alignment padding before and after the list is not an id
                            const uint32_t v0 = fj + (uint32_t)(s - a), v1 = v0 + (uint32_t)(e - s);
                            for (uint32_t x = max(lo, fj); x < min(hi, v0); ++x)
                                atomicAnd(&pm[(x - p0) >> 5], ~(1u << ((x - p0) & 31)));
                            for (uint32_t x = max(lo, v1); x < min(hi, fe); ++x)
                                atomicAnd(&pm[(x - p0) >> 5], ~(1u << ((x - p0) & 31)));
                        }
                    }
                }
                while (jc < n_units && F[jc + 1] <= p1) ++jc;
                if (lane == 0) {
                    BmPageHdr h;
                    h.q = cur.q;
                    h.k = cur.k;
                    h.fill = cnt;
                    h.last = p1 >= ftot ? 1u : 0u;
                    h.out_off = cur.out_off;
                    h.pad[0] = h.pad[1] = 0;
                    hdr[ps] = h;
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[ps]);
            }
            if (lane == 0) {
                cur = nxt;
                nxt = after;
            }
        }
        if (abort && lane == 0) {
            atomicOr(&W.ctr[kCtrError], kErrTimeout);
            s_abort = 1;
            // let the copies already issued land before the block can exit
            for (uint32_t b = pg > P ? pg - P : 0; b < pg; ++b) mbar_wait(&full[b % P], (b / P) & 1u, 10000000ull);
        }
        return;
    }

    // -------------------------------------------------------------- consumers
    const uint32_t ct = tid - 32;
    const uint32_t mcap = mslots / 2;
    const uint32_t words = L.bm_words;
    uint32_t *hist = ss.hist;
    for (uint32_t i = ct; i < words / 4; i += kBmConsumers) ((uint4 *)bm)[i] = make_uint4(0u, 0u, 0u, 0u);
    for (uint32_t i = ct; i < mslots; i += kBmConsumers) mt[i] = 0u;
    for (uint32_t i = ct; i < 256; i += kBmConsumers) hist[i] = 0u;
    BmConsumers::sync();

    // a repeated id: count it in the table and the histogram; 1 for a new entry
    auto repeat = [&](uint32_t id) -> uint32_t {
        uint32_t h = slot_of(id, mslots);
        for (uint32_t probe = 0; probe < kBmProbe; ++probe) {
            uint32_t cur = mt[h];
            if (cur == 0u) {
                const uint32_t old = atomicCAS(&mt[h], 0u, (id << 8) | 2u);
                if (old == 0u) {
                    atomicAdd(&hist[2], 1u);
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

    uint32_t pg = 0;
    constexpr int R = (kBmPageIds + kBmConsumers - 1) / kBmConsumers;
    for (uint32_t i = 0; blockIdx.x + i * G < n_work; ++i) {
        uint32_t q = 0, k = 0;
        int64_t out_off = 0;
        bool first = true, aborted = false;
        for (;;) {
            const uint32_t ps = pg % P;
            if (!mbar_wait(&full[ps], (pg / P) & 1u)) {
                aborted = true;
                break;
            }
            const BmPageHdr h = hdr[ps];
            if (first) {
                q = h.q;
                k = h.k;
                out_off = h.out_off;
                first = false;
            }
            const uint32_t *page = ring + ps * kBmPageIds;
            const uint32_t *pm = mask + ps * (kBmPageIds / 32);
            uint32_t v[R], old[R];
            uint32_t ok = 0;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const uint32_t p = ct + r * kBmConsumers;
                const bool in = p < h.fill;
                const uint32_t mw = in ? pm[p >> 5] : 0u;
                v[r] = in ? page[p] : 0u;
                ok |= ((mw >> (p & 31)) & 1u) << r;
            }
#pragma unroll
            for (int r = 0; r < R; ++r) {      // independent atomics, all in flight
                bool g = (ok >> r & 1u) != 0;
                g = g && GG_OK(v[r] >> 5, words, 15);
                const uint32_t m = g ? 1u << (v[r] & 31) : 0u;
                old[r] = atomicOr(g ? &bm[v[r] >> 5] : &s_spare[lane], m) & m;
            }
            uint32_t rep = 0;
#pragma unroll
            for (int r = 0; r < R; ++r) rep |= (old[r] != 0u ? 1u : 0u) << r;
            uint32_t added = 0;
            while (__any_sync(0xffffffffu, rep != 0u)) {
                if (rep) {
                    const uint32_t r = __ffs(rep) - 1;
                    rep &= rep - 1;
                    uint32_t id = v[0];
#pragma unroll
                    for (int j = 1; j < R; ++j) id = (r == (uint32_t)j) ? v[j] : id;
                    added += repeat(id);
                }
            }
            added = __reduce_add_sync(0xffffffffu, added);
            if (lane == 0 && added && atomicAdd(&s_multi, added) + added > mcap) s_ovf = 1;
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[ps]);
            ++pg;
            if (h.last) break;
        }
        if (aborted && lane == 0) {
            atomicOr(&W.ctr[kCtrError], kErrTimeout);
            s_abort = 1;
        }
        BmConsumers::sync();
        if (*(volatile uint32_t *)&s_abort) break;

        // ---- exact top-k of this query
        const uint32_t n_multi = s_multi;
        bool failed = s_ovf != 0;
        uint32_t nres = 0;
        uint32_t n_hi = 0;             // keys at cand[0, n_hi) first, then ties
        const uint64_t *ties = cand;
        if (!failed && n_multi >= k) {
            if (ct < 32) find_digit(ss, k, true);     // k-th largest count
            if (ct == 0) {
                s_n = 0;
                s_t = 0;
            }
            BmConsumers::sync();
            const uint32_t cstar = ss.sc[0], above = ss.sc[1], n_eq = ss.sc[2];
            const uint32_t hp2 = next_pow2(above), tp2 = next_pow2(n_eq);
            if (hp2 + tp2 <= kCandCap) {
                uint64_t *tie_buf = cand + hp2;
                for (uint32_t b = 0; b < mslots; b += kBmConsumers) {
                    const uint32_t x = b + ct;
                    const uint32_t e = x < mslots ? mt[x] : 0u;
                    const uint32_t c = e & 255u;
                    warp_append(e != 0u && c > cstar, make_key(c, e >> 8), cand, &s_n);
                    warp_append(e != 0u && c == cstar, make_key(c, e >> 8), tie_buf, &s_t);
                }
                for (uint32_t x = above + ct; x < hp2; x += kBmConsumers) cand[x] = 0ull;
                for (uint32_t x = n_eq + ct; x < tp2; x += kBmConsumers) tie_buf[x] = 0ull;
                bitonic_sort_desc<BmConsumers>(cand, hp2);
                bitonic_sort_desc<BmConsumers>(tie_buf, tp2);
                n_hi = above;
                ties = tie_buf;
                nres = k;
            } else {
                failed = true;
            }
        } else if (!failed) {
            // the whole table, then the smallest ids seen once
            if (ct == 0) s_n = 0;
            BmConsumers::sync();
            for (uint32_t b = 0; b < mslots; b += kBmConsumers) {
                const uint32_t x = b + ct;
                const uint32_t e = x < mslots ? mt[x] : 0u;
                if (e) atomicAnd(&bm[(e >> 8) >> 5], ~(1u << ((e >> 8) & 31)));
                warp_append(e != 0u, make_key(e & 255u, e >> 8), cand, &s_n);
            }
            const uint32_t np2 = next_pow2(n_multi);
            BmConsumers::sync();
            for (uint32_t x = n_multi + ct; x < np2; x += kBmConsumers) cand[x] = 0ull;
            bitonic_sort_desc<BmConsumers>(cand, np2);
            const uint32_t r = k - n_multi;
            const uint32_t singles = bitmap_take_smallest<BmConsumers>(bm, words, r, 1u, cand + n_multi, ss);
            n_hi = n_multi + min(r, singles);
            nres = n_hi;
        }
        if (failed) {
            if (ct == 0) convert_to_dense(ix, W, T, q);
        } else {
            for (uint32_t j = ct; j < k; j += kBmConsumers) {
                if (!GG_OK(out_off + j, W.out_cap, 4)) continue;
                uint32_t id = 0, cnt = 0;
                if (j < nres) {
                    const uint64_t key = j < n_hi ? cand[j] : ties[j - n_hi];
                    id = key_id(key);
                    cnt = key_prim(key);
                }
                W.out_ids[out_off + j] = id;
                W.out_counts[out_off + j] = cnt;
                if (W.out_scores) W.out_scores[out_off + j] = (float)cnt;
            }
        }
        // ---- clear the state for the next query
        BmConsumers::sync();
        for (uint32_t x = ct; x < words / 4; x += kBmConsumers) ((uint4 *)bm)[x] = make_uint4(0u, 0u, 0u, 0u);
        for (uint32_t x = ct; x < mslots; x += kBmConsumers) mt[x] = 0u;
        for (uint32_t x = ct; x < 256; x += kBmConsumers) hist[x] = 0u;
        if (ct == 0) {
            s_multi = 0;
            s_ovf = 0;
        }
        BmConsumers::sync();
    }
}

}  // namespace gg
