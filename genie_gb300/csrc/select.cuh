// select.cuh -- exact block-wide top-k over a virtual set of (primary, id)
// entries, ranked by primary descending then id ascending.
//
// This replaces the reference's c-PQ threshold bookkeeping plus
// heap_count_topk (matching/heap_count.cu:161-282), whose output is unordered
// and whose ties are nondeterministic.  Here the k-th entry is found by an
// MSD radix select on the primary (8-bit digits, warp-aggregated shared
// histograms), ties at the boundary are resolved by a second radix select on
// the id, and the admitted entries are sorted.
//
// A Set provides  template<class F> void for_each(F f) const  that makes every
// thread call f(bool active, uint32_t primary, uint32_t id) the same number of
// times (warp-uniform), so f may use warp votes.  Ids in a set are unique.
#pragma once
#include "device.cuh"

namespace gg {

struct SelectScratch {
    uint32_t hist[256];
    uint32_t sc[16];
    uint32_t tmp[48];
    unsigned long long tot64;
    unsigned long long pad;
};

// Find, in a warp, the digit d (scanning bins from `from_top` order) at which
// the cumulative count reaches `need`.  Lane l owns 8 consecutive bins.
// Writes sc[0]=digit, sc[1]=count strictly before d, sc[2]=hist[d],
// sc[3]=1 if the whole histogram holds fewer than need entries, sc[4]=total.
__device__ __forceinline__ void find_digit(SelectScratch &s, uint32_t need, bool descending) {
    uint32_t l = lane_id();
    uint32_t bins[8];
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        uint32_t b = descending ? (255u - (8u * l + j)) : (8u * l + j);
        bins[j] = s.hist[b];
        sum += bins[j];
    }
    uint32_t incl = warp_incl_scan(sum);
    uint32_t before = incl - sum;
    uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (l == 0) { s.sc[3] = total < need ? 1u : 0u; s.sc[4] = total; }
    if (total >= need && before < need && incl >= need) {
        uint32_t cum = before;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (cum + bins[j] >= need) {
                uint32_t b = descending ? (255u - (8u * l + j)) : (8u * l + j);
                s.sc[0] = b;
                s.sc[1] = cum;
                s.sc[2] = bins[j];
                break;
            }
            cum += bins[j];
        }
    }
}

// Top-k of `set` into cand[0..ret) sorted descending by key.  prim_bits is an
// upper bound on the bit width of any primary.  cand_cap is a power of two
// >= k.  Returns the number of entries written (min(k, set size)).
template <class Set>
__device__ uint32_t select_topk(const Set &set, uint32_t k, int prim_bits, uint64_t *cand,
                                uint32_t cand_cap, SelectScratch &s) {
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    uint32_t need = k;
    uint32_t prefix = 0;
    int top = ((prim_bits + 7) / 8) * 8 - 8;
    if (top < 0) top = 0;
    int shift = top;
    int mode = 0;           // 0: tie resolution needed, 1: take all, 2: exact bin
    uint32_t count_eq = 0;
    for (; shift >= 0; shift -= 8) {
        for (uint32_t i = tid; i < 256; i += nt) s.hist[i] = 0;
        __syncthreads();
        const int hs = shift + 8;
        const uint32_t pre_hi = hs >= 32 ? 0u : (prefix >> hs);
        set.for_each([&](bool act, uint32_t prim, uint32_t id) {
            bool ok = act && (hs >= 32 || (prim >> hs) == pre_hi);
            hist_add(s.hist, (prim >> shift) & 255u, ok);
        });
        __syncthreads();
        if (warp_id() == 0) find_digit(s, need, true);
        __syncthreads();
        if (s.sc[3]) {      // fewer than `need` entries under this prefix
            mode = 1;       // only possible on the first pass: take everything
            __syncthreads();
            break;
        }
        uint32_t d = s.sc[0];
        need -= s.sc[1];
        count_eq = s.sc[2];
        prefix |= d << shift;
        __syncthreads();
        if (count_eq == need) { mode = 2; break; }
    }
    // id threshold for the tie case: the need-th smallest id with primary == prefix
    uint32_t id_cut = 0xFFFFFFFFu;
    bool ties_fit = false;
    if (mode == 0) {
        // all entries with primary >= prefix fit in the candidate buffer?
        ties_fit = (k - need) + count_eq <= cand_cap;
        if (!ties_fit) {
            uint32_t r = need, idp = 0;
            for (int sh = 24; sh >= 0; sh -= 8) {
                for (uint32_t i = tid; i < 256; i += nt) s.hist[i] = 0;
                __syncthreads();
                const int hs = sh + 8;
                const uint32_t idp_hi = hs >= 32 ? 0u : (idp >> hs);
                set.for_each([&](bool act, uint32_t prim, uint32_t id) {
                    bool ok = act && prim == prefix && (hs >= 32 || (id >> hs) == idp_hi);
                    hist_add(s.hist, (id >> sh) & 255u, ok);
                });
                __syncthreads();
                if (warp_id() == 0) find_digit(s, r, false);
                __syncthreads();
                r -= s.sc[1];
                idp |= s.sc[0] << sh;
                __syncthreads();
            }
            id_cut = idp;
        }
    }
    // compaction of admitted entries
    if (tid == 0) s.sc[8] = 0;
    __syncthreads();
    const uint32_t lo = prefix;
    set.for_each([&](bool act, uint32_t prim, uint32_t id) {
        bool ok;
        if (mode == 1) ok = act;
        else if (mode == 2) ok = act && prim >= lo;
        else if (ties_fit) ok = act && prim >= lo;
        else ok = act && (prim > lo || (prim == lo && id <= id_cut));
        uint32_t m = __ballot_sync(0xffffffffu, ok);
        uint32_t base = 0;
        if (lane_id() == 0 && m) base = atomicAdd(&s.sc[8], (uint32_t)__popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (ok) {
            uint32_t pos = base + __popc(m & ((1u << lane_id()) - 1u));
            if (pos < cand_cap) cand[pos] = make_key(prim, id);
        }
    });
    __syncthreads();
    uint32_t n = s.sc[8];
    if (n > cand_cap) n = cand_cap;
    uint32_t np2 = next_pow2(n);
    for (uint32_t i = n + tid; i < np2; i += nt) cand[i] = 0;
    bitonic_sort_desc(cand, np2);
    return n < k ? n : k;
}

}  // namespace gg
