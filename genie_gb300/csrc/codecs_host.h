// codecs_host.h -- host encoders and the compressed index layout.
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

#include "host_index.h"

#ifndef __host__
#define __host__
#define __device__
#define GG_UNDEF_HD
#endif
namespace gg {
// Codec ids and their (delta stages, inner format) split, shared with the
// device decoders.
enum : int {
    kCodecNone = 0, kCodecCopy, kCodecDelta, kCodecBP32, kCodecVarint, kCodecCompBP32Copy,
    kCodecCompBP32Varint, kCodecSerialCopyCopy, kCodecSerialDeltaCopy, kCodecSerialDeltaDelta,
    kCodecSerialDeltaVarint, kCodecSerialDeltaBP32, kCodecSerialDeltaCompBP32Copy,
    kCodecSerialDeltaCompBP32Varint, kNumCodecs
};
enum : int { kInnerCopy = 0, kInnerBP32 = 1, kInnerVarint = 2, kInnerCompCopy = 3, kInnerCompVarint = 4 };

__host__ __device__ inline void codec_parts(int codec, int &deltas, int &inner) {
    deltas = 0;
    inner = kInnerCopy;
    switch (codec) {
    case kCodecCopy: case kCodecSerialCopyCopy: break;
    case kCodecDelta: case kCodecSerialDeltaCopy: deltas = 1; break;
    case kCodecBP32: inner = kInnerBP32; break;
    case kCodecVarint: inner = kInnerVarint; break;
    case kCodecCompBP32Copy: inner = kInnerCompCopy; break;
    case kCodecCompBP32Varint: inner = kInnerCompVarint; break;
    case kCodecSerialDeltaDelta: deltas = 2; break;
    case kCodecSerialDeltaVarint: deltas = 1; inner = kInnerVarint; break;
    case kCodecSerialDeltaBP32: deltas = 1; inner = kInnerBP32; break;
    case kCodecSerialDeltaCompBP32Copy: deltas = 1; inner = kInnerCompCopy; break;
    case kCodecSerialDeltaCompBP32Varint: deltas = 1; inner = kInnerCompVarint; break;
    default: deltas = -1;
    }
}

struct ComprLayout {
    std::vector<uint32_t> words;
    std::vector<int64_t> key_seg;       // [n_keys+1]
    std::vector<int64_t> seg_word_off;  // [n_segs+1]
    std::vector<uint32_t> seg_first;    // [n_segs]
    std::vector<uint32_t> seg_len;      // [n_segs]
};

int64_t encode_bound(int64_t n);
// Append the encoding of in[0..n) to out; false for an unknown codec or n == 0.
bool encode(int codec, const uint32_t *in, size_t n, std::vector<uint32_t> &out);
// Cut every (dim,value) list into max_seg-id segments and encode each.
bool build_compressed(const HostIndex &ix, int codec, int32_t max_seg, ComprLayout &out);
}  // namespace gg
#ifdef GG_UNDEF_HD
#undef __host__
#undef __device__
#undef GG_UNDEF_HD
#endif
