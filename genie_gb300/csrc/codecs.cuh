// codecs.cuh -- warp-level decoders of the reference posting-list codecs,
// emitting values in sequence order straight into the counting loop.
//
// Formats (byte-compatible with the reference's host encoders):
//   COPY     words are the values                       (DeviceCodecs.h:113-154)
//   DELTA    words are differences, first from 0        (DeviceCodecs.cu:89-139)
//   BP32     [n][w0<<24|w1<<16|w2<<8|w3][w0 words]..[w3 words] per 128 values;
//            value j of a 32-value miniblock sits at bits [j*w, j*w+w), LSB
//            first; a short tail packs ceil(rem/32) zero-padded miniblocks
//                                                      (DeviceBitPackingCodec.cu:15-58)
//   VARINT   7-bit groups, low first, the LAST byte of a value has bit 7 set,
//            zero-padded to whole words                 (DeviceVarintCodec.cu:14-78)
//   COMP(BP32,C2)  [len1][BP32 over floor(n/8)*8 values][C2 over the rest]
//                                                      (DeviceCompositeCodec.cu:28-58)
//   SERIAL(C1,C2)  C2 decoded first, then C1            (DeviceSerialCodec.cu:67-137)
//
// The reference decodes one segment per 256-thread block through shared
// memory with a sequential header parse on thread 0
// (DeviceBitPackingCodec.cu:160-200) and block-wide scans (utility/scan.cu).
// Here one warp decodes one segment: miniblock offsets come from the header
// bytes, varint boundaries from the terminal bits of each lane's word, and
// delta runs as a warp prefix sum with a carry.
#pragma once
#include "codecs_host.h"
#include "device.cuh"

namespace gg {

// Emits a group of values: lane l holds `cnt` values val[0..cnt) whose
// sequence positions are base + before(l) + 0..cnt-1 (before = exclusive
// prefix of cnt over lanes).  The emitter applies the delta stages in
// sequence order and hands each value to `visit`.
template <class V, bool POS = true>
struct Emitter {
    int deltas;
    uint32_t carry1 = 0, carry2 = 0;
    uint32_t emitted = 0;      // values emitted so far (sequence position of the next)
    V &visit;
    __device__ Emitter(int d, V &v) : deltas(d), visit(v) {}
    __device__ __forceinline__ void emit(const uint32_t *val, int cnt) {
        // sequence position of this lane's first value (skipped when the
        // visitor does not use positions)
        uint32_t pos0 = 0;
        if (POS) {
            const uint32_t cincl = warp_incl_scan((uint32_t)cnt);
            pos0 = emitted + cincl - (uint32_t)cnt;
            emitted += __shfl_sync(0xffffffffu, cincl, 31);
        }
        // stage 1: inclusive running sum within the lane, then across lanes
        uint32_t loc[4];
        uint32_t s = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j < cnt) s += val[j];
            loc[j] = s;
        }
        if (deltas == 0) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (j < cnt) visit(val[j], pos0 + j);
            return;
        }
        uint32_t incl = warp_incl_scan(s);
        uint32_t pre = carry1 + incl - s;
        carry1 += __shfl_sync(0xffffffffu, incl, 31);
        uint32_t v1[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v1[j] = pre + loc[j];
        if (deltas == 1) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (j < cnt) visit(v1[j], pos0 + j);
            return;
        }
        // stage 2 (SERIAL_DELTA_DELTA)
        uint32_t s2 = 0, loc2[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j < cnt) s2 += v1[j];
            loc2[j] = s2;
        }
        uint32_t incl2 = warp_incl_scan(s2);
        uint32_t pre2 = carry2 + incl2 - s2;
        carry2 += __shfl_sync(0xffffffffu, incl2, 31);
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j < cnt) visit(pre2 + loc2[j], pos0 + j);
    }
};

// Word sources of the decoders.  Every lane of the warp calls word() the
// same number of times (the register source shuffles).
struct GlobalWords {      // words read from global memory
    const uint32_t *__restrict__ w;
    __device__ __forceinline__ uint32_t word(int64_t i) const { return __ldg(w + i); }
    // word i where cond holds, else 0 (read only where cond holds)
    __device__ __forceinline__ uint32_t word_if(int64_t i, bool cond) const { return cond ? __ldg(w + i) : 0u; }
};
struct RegWords {         // a segment of <= 64 words held two per lane
    int64_t base;
    uint32_t r0, r1;
    __device__ __forceinline__ uint32_t word(int64_t i) const {
        const uint32_t rel = (uint32_t)(i - base);
        const uint32_t a = __shfl_sync(0xffffffffu, r0, rel & 31u);
        const uint32_t b = __shfl_sync(0xffffffffu, r1, rel & 31u);
        return rel < 32u ? a : (rel < 64u ? b : 0u);
    }
    __device__ __forceinline__ uint32_t word_if(int64_t i, bool cond) const {
        const uint32_t x = word(i);      // every lane shuffles
        return cond ? x : 0u;
    }
};

// Words [w0, w1) as values, 32 per step.
template <class S, class E>
__device__ __forceinline__ void dec_copy(const S &src, int64_t w0, int64_t w1, E &em) {
    for (int64_t b = w0; b < w1; b += 32) {
        int64_t i = b + lane_id();
        const uint32_t x = src.word(i < w1 ? i : w0);
        uint32_t v[1] = {i < w1 ? x : 0u};
        em.emit(v, i < w1 ? 1 : 0);
    }
}

// One BP32 stream starting at word w0 ([n][blocks...]); returns the word
// after it.  Lane l decodes values 4l..4l+3 of each 128-value block (all in
// miniblock l/8), so one emit (one prefix scan) covers the whole block.
template <class S, class E>
__device__ __forceinline__ int64_t dec_bp32(const S &src, int64_t w0, E &em) {
    const uint32_t lane = lane_id();
    const uint32_t n = src.word(w0);
    int64_t p = w0 + 1;
    for (uint32_t done = 0; done < n; done += 128) {
        const uint32_t hdr = src.word(p);
        const uint32_t rem = n - done;
        const uint32_t howmany = rem >= 128 ? 4u : (rem + 31) / 32;
        // widths of the miniblocks present (a short tail packs fewer)
        uint32_t bw[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) bw[m] = (uint32_t)m < howmany ? (hdr >> (24 - 8 * m)) & 255u : 0u;
        const uint32_t mb = lane >> 3;
        uint32_t b = bw[0], before = 0;
#pragma unroll
        for (int m = 1; m < 4; ++m)
            if ((uint32_t)m <= mb) {
                before += bw[m - 1];
                b = bw[m];
            }
        const int64_t off = p + 1 + before;
        const uint32_t j0 = (lane & 7u) * 4u;
        const uint32_t mask = b >= 32 ? 0xFFFFFFFFu : (1u << b) - 1u;
        uint32_t v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t bit = (j0 + k) * b, wi = bit >> 5, sh = bit & 31;
            const uint32_t lo = src.word_if(off + wi, b > 0);
            const uint32_t hi = src.word_if(off + wi + 1, b > 0 && sh + b > 32);
            v[k] = (uint32_t)((((uint64_t)hi << 32) | lo) >> sh) & mask;
        }
        const int have = (int)min(4u, rem > 4 * lane ? rem - 4 * lane : 0u);
        em.emit(v, have);
        p += 1 + bw[0] + bw[1] + bw[2] + bw[3];
    }
    return p;
}

// Varint bytes of words [w0, w1): a lane owns one word; each byte with bit 7
// set ends a value of at most five bytes, so a value spans at most this word
// and the previous one.
template <class S, class E>
__device__ __forceinline__ void dec_varint(const S &src, int64_t w0, int64_t w1, E &em) {
    const uint32_t lane = lane_id();
    uint32_t prev_last = 0;            // previous chunk's last word
    bool have_prev = false;
    for (int64_t b = w0; b < w1; b += 32) {
        const int64_t i = b + lane;
        const uint32_t raw = src.word(i < w1 ? i : w0);
        const uint32_t cur = i < w1 ? raw : 0u;
        uint32_t prv = __shfl_up_sync(0xffffffffu, cur, 1);
        if (lane == 0) prv = have_prev ? prev_last : 0u;
        const bool prv_valid = lane > 0 || have_prev;
        // terminal flags of the 8-byte window [prv | cur]
        const uint64_t win = ((uint64_t)cur << 32) | prv;
        uint32_t vals[4];
        int cnt = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int pos = 4 + j;                       // byte index in the window
            const uint32_t byte = (uint32_t)(win >> (8 * pos)) & 255u;
            if (!(byte & 0x80u)) continue;
            // walk back to the byte after the previous terminal (<= 4 bytes)
            int start = pos;
            while (start > 0 && (pos - start) < 4) {
                const uint32_t pb = (uint32_t)(win >> (8 * (start - 1))) & 255u;
                if (pb & 0x80u) break;
                if (start - 1 < 4 && !prv_valid) break;
                --start;
            }
            uint32_t v = 0;
            for (int t = pos; t >= start; --t) v = (v << 7) | ((uint32_t)(win >> (8 * t)) & 0x7Fu);
            vals[cnt++] = v;
        }
        em.emit(vals, cnt);
        prev_last = __shfl_sync(0xffffffffu, cur, 31);
        have_prev = true;
    }
}

// Decode one encoded segment (words [w0, w1)) from a word source and visit
// its values in order.
template <bool POS, class S, class V>
__device__ __forceinline__ void decode_words(int codec, const S &src, int64_t w0, int64_t w1, V &visit) {
    int deltas, inner;
    codec_parts(codec, deltas, inner);
    Emitter<V, POS> em(deltas, visit);
    switch (inner) {
    case kInnerCopy:
        dec_copy(src, w0, w1, em);
        break;
    case kInnerBP32:
        dec_bp32(src, w0, em);
        break;
    case kInnerVarint:
        dec_varint(src, w0, w1, em);
        break;
    default: {     // composite: [len1][BP32 (len1 words)][tail]
        const uint32_t len1 = src.word(w0);
        int64_t p = w0 + 1;
        if (len1) dec_bp32(src, p, em);
        p += len1;
        if (p < w1) {
            if (inner == kInnerCompCopy) dec_copy(src, p, w1, em);
            else dec_varint(src, p, w1, em);
        }
    }
    }
}

// Decode one encoded segment and visit (value, sequence position) in order.
// A segment of at most 64 words is read in one coalesced step and decoded
// from registers; a longer one is read word by word.
template <class V>
__device__ __forceinline__ void decode_segment(int codec, const uint32_t *__restrict__ w, int64_t w0, int64_t w1,
                                               V &visit) {
    if (w1 - w0 <= 64) {
        const uint32_t lane = lane_id();
        RegWords src{w0, w0 + lane < w1 ? __ldg(w + w0 + lane) : 0u,
                     w0 + 32 + lane < w1 ? __ldg(w + w0 + 32 + lane) : 0u};
        decode_words<true>(codec, src, w0, w1, visit);
    } else {
        decode_words<true>(codec, GlobalWords{w}, w0, w1, visit);
    }
}

// The same for a visitor of values only (no sequence positions).
template <class V>
__device__ __forceinline__ void decode_segment_values(int codec, const uint32_t *__restrict__ w, int64_t w0,
                                                      int64_t w1, V &visit) {
    if (w1 - w0 <= 64) {
        const uint32_t lane = lane_id();
        RegWords src{w0, w0 + lane < w1 ? __ldg(w + w0 + lane) : 0u,
                     w0 + 32 + lane < w1 ? __ldg(w + w0 + 32 + lane) : 0u};
        decode_words<false>(codec, src, w0, w1, visit);
    } else {
        decode_words<false>(codec, GlobalWords{w}, w0, w1, visit);
    }
}

}  // namespace gg
