// codecs_host.cc -- host encoders of the reference posting-list codecs and
// the compressed index layout.
//
// The byte formats are the reference's (so a table compressed here decodes
// like one compressed by inv_compr_table::build, inv_compr_table.cu:30-119);
// see codecs.cuh for the format summary.  Encoders are composed from three
// primitives (bit packing, varint, delta) instead of one class per codec.
#include "codecs_host.h"

#include <algorithm>
#include <cstring>

namespace gg {

namespace {

inline uint32_t width_of(uint32_t v) { return v ? 32u - (uint32_t)__builtin_clz(v) : 0u; }

// Pack 32 values at `bits` bits each into `bits` words, value j at bit j*bits.
void pack_miniblock(const uint32_t *in, uint32_t bits, std::vector<uint32_t> &out) {
    if (!bits) return;
    const size_t base = out.size();
    out.resize(base + bits, 0u);
    uint32_t *o = out.data() + base;
    for (uint32_t j = 0; j < 32; ++j) {
        const uint64_t bit = (uint64_t)j * bits;
        const uint64_t shifted = (uint64_t)in[j] << (bit & 31);
        o[bit >> 5] |= (uint32_t)shifted;
        if ((bit & 31) + bits > 32) o[(bit >> 5) + 1] |= (uint32_t)(shifted >> 32);
    }
}

void bp32(const uint32_t *in, size_t n, std::vector<uint32_t> &out) {
    out.push_back((uint32_t)n);
    uint32_t block[128];
    for (size_t at = 0; at < n; at += 128) {
        const size_t take = std::min<size_t>(128, n - at);
        const size_t minis = take == 128 ? 4 : (take + 31) / 32;
        memset(block, 0, sizeof(block));
        memcpy(block, in + at, take * sizeof(uint32_t));
        uint32_t w[4] = {0, 0, 0, 0};
        for (size_t m = 0; m < minis; ++m) {
            uint32_t acc = 0;
            for (int j = 0; j < 32; ++j) acc |= block[m * 32 + j];
            w[m] = width_of(acc);
        }
        out.push_back(w[0] << 24 | w[1] << 16 | w[2] << 8 | w[3]);
        for (size_t m = 0; m < minis; ++m) pack_miniblock(block + m * 32, w[m], out);
    }
}

void varint(const uint32_t *in, size_t n, std::vector<uint32_t> &out) {
    std::vector<uint8_t> bytes;
    bytes.reserve(n * 2 + 4);
    for (size_t i = 0; i < n; ++i) {
        uint32_t v = in[i];
        while (v >= 128u) {
            bytes.push_back((uint8_t)(v & 127u));
            v >>= 7;
        }
        bytes.push_back((uint8_t)(v | 128u));        // bit 7 marks the last byte
    }
    while (bytes.size() % 4) bytes.push_back(0);
    const size_t base = out.size();
    out.resize(base + bytes.size() / 4);
    memcpy(out.data() + base, bytes.data(), bytes.size());
}

void copy_words(const uint32_t *in, size_t n, std::vector<uint32_t> &out) { out.insert(out.end(), in, in + n); }

// [len1][BP32 over floor(n/8)*8 values][tail codec over the remainder]
void composite(const uint32_t *in, size_t n, bool tail_varint, std::vector<uint32_t> &out) {
    const size_t head = n / 8 * 8;
    const size_t at = out.size();
    out.push_back(0);
    if (head) bp32(in, head, out);
    out[at] = (uint32_t)(out.size() - at - 1);
    if (n > head) {
        if (tail_varint) varint(in + head, n - head, out);
        else copy_words(in + head, n - head, out);
    }
}

}  // namespace

int64_t encode_bound(int64_t n) { return (5 * n) / 4 + 96; }

bool encode(int codec, const uint32_t *in, size_t n, std::vector<uint32_t> &out) {
    int deltas, inner;
    codec_parts(codec, deltas, inner);
    if (deltas < 0 || codec == kCodecNone || n == 0) return false;
    std::vector<uint32_t> tmp;
    const uint32_t *src = in;
    for (int d = 0; d < deltas; ++d) {          // SERIAL(DELTA, ..) applies delta first
        std::vector<uint32_t> nxt(n);
        uint32_t prev = 0;
        for (size_t i = 0; i < n; ++i) {
            nxt[i] = src[i] - prev;
            prev = src[i];
        }
        tmp.swap(nxt);
        src = tmp.data();
    }
    switch (inner) {
    case kInnerCopy: copy_words(src, n, out); break;
    case kInnerBP32: bp32(src, n, out); break;
    case kInnerVarint: varint(src, n, out); break;
    case kInnerCompCopy: composite(src, n, false, out); break;
    case kInnerCompVarint: composite(src, n, true, out); break;
    default: return false;
    }
    return true;
}

bool build_compressed(const HostIndex &ix, int codec, int32_t max_seg, ComprLayout &out) {
    if (max_seg <= 0 || max_seg > 1024) return false;
    out = ComprLayout();
    const int64_t nk = ix.n_keys();
    out.key_seg.assign((size_t)nk + 1, 0);
    for (int64_t k = 0; k < nk; ++k) {
        out.key_seg[k] = (int64_t)out.seg_len.size();
        for (int64_t p = ix.key_off[k]; p < ix.key_off[k + 1]; p += max_seg) {
            const int64_t len = std::min<int64_t>(max_seg, ix.key_off[k + 1] - p);
            out.seg_word_off.push_back((int64_t)out.words.size());
            out.seg_first.push_back(ix.ids[p]);
            out.seg_len.push_back((uint32_t)len);
            if (!encode(codec, ix.ids.data() + p, (size_t)len, out.words)) return false;
        }
    }
    out.key_seg[nk] = (int64_t)out.seg_len.size();
    out.seg_word_off.push_back((int64_t)out.words.size());
    return true;
}

}  // namespace gg
