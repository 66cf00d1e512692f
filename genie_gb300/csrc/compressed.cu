// compressed.cu -- compressed resident indexes and the codec entry points.
//
// A compressed index keeps the reference's layout (inv_compr_table,
// table/inv_compr_table.h:27-41): every (dim,value) list cut into segments of
// at most max_segment ids, each encoded independently.  On top of it this
// library stores, per segment, its first id (a skip pointer: the match kernels
// find the segments of an id range by binary search instead of decoding) and
// its posting position.  Decoding runs inside the match kernels (codecs.cuh).
#include "capi_internal.h"
#include "codecs.cuh"
#include "codecs_host.h"

#include <cstring>
#include <vector>

namespace gg {

int upload_compressed(genie_index *ix, const std::vector<uint32_t> &words, const std::vector<int64_t> &key_seg,
                      const std::vector<int64_t> &seg_word_off, const std::vector<uint32_t> &seg_first,
                      const std::vector<uint32_t> &seg_len) {
    // bounds and key offsets as for a plain index, without the posting ids
    std::vector<uint32_t> keep;
    keep.swap(ix->host.ids);
    int rc = upload_index(ix);
    keep.swap(ix->host.ids);
    if (rc) return rc;
    const int64_t n_segs = (int64_t)seg_len.size();
    std::vector<int64_t> seg_pos((size_t)n_segs + 1, 0);
    for (int64_t s = 0; s < n_segs; ++s) seg_pos[s + 1] = seg_pos[s] + seg_len[s];
    cudaError_t e;
    auto put = [&](DevBuf &b, const void *src, size_t bytes) -> bool {
        if ((e = b.reserve(bytes + 64))) return false;
        if ((e = cudaMemset(b.p, 0, bytes + 64))) return false;
        if (bytes && (e = cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice))) return false;
        return true;
    };
    if (!put(ix->d_words, words.data(), words.size() * 4) || !put(ix->d_key_seg, key_seg.data(), key_seg.size() * 8) ||
        !put(ix->d_seg_word_off, seg_word_off.data(), seg_word_off.size() * 8) ||
        !put(ix->d_seg_first, seg_first.data(), seg_first.size() * 4) ||
        !put(ix->d_seg_len, seg_pos.data(), seg_pos.size() * 8))
        return cuda_fail(e, "compressed index upload");
    ix->n_words = (int64_t)words.size();
    ix->n_segs = n_segs;
    ix->n_ids = seg_pos[n_segs];
    DevIndex &d = ix->dev;
    d.n_ids = ix->n_ids;
    d.codec = ix->codec;
    d.max_seg = ix->max_seg;
    d.words = (const uint32_t *)ix->d_words.p;
    d.key_seg = (const int64_t *)ix->d_key_seg.p;
    d.seg_word_off = (const int64_t *)ix->d_seg_word_off.p;
    d.seg_first = (const uint32_t *)ix->d_seg_first.p;
    d.seg_pos = (const int64_t *)ix->d_seg_len.p;
    return GENIE_OK;
}

// One warp per segment: decode into out[out_off[s] ..] and report the length.
__global__ void k_decode_segments(int codec, const uint32_t *words, const int64_t *word_off, int64_t n_segments,
                                  const int64_t *out_off, uint32_t *out, uint32_t *out_len) {
    const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (s >= n_segments) return;
    uint32_t *dst = out + out_off[s];
    uint32_t n = 0;
    auto v = [&](uint32_t value, uint32_t pos) {
        dst[pos] = value;
        n = pos + 1 > n ? pos + 1 : n;
    };
    decode_segment(codec, words, word_off[s], word_off[s + 1], v);
    n = __reduce_max_sync(0xffffffffu, n);
    if (lane_id() == 0) out_len[s] = n;
}

}  // namespace gg

using namespace gg;

namespace gg {
int finish_loaded_index(genie_index *ix, genie_index **out);
}

extern "C" {

int genie_index_create_compressed(const int32_t *values, int64_t n_objects, int32_t n_dims, int32_t codec,
                                  int32_t max_segment, genie_index **out) {
    if (!out) return fail(GENIE_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!values || n_objects <= 0 || n_dims <= 0) return fail(GENIE_ERR_INVALID_ARG, "no data input");
    int deltas, inner;
    codec_parts(codec, deltas, inner);
    if (codec <= 0 || codec >= kNumCodecs || deltas < 0)
        return fail(GENIE_ERR_INVALID_ARG, "unknown codec %d", codec);
    // inv_compr_table.cu:58: a segment must fit one decode (<= 1024 ids)
    if (max_segment <= 0 || max_segment > 1024)
        return fail(GENIE_ERR_INVALID_ARG, "max_segment must be in [1, 1024]");
    int dev = 0;
    cudaGetDevice(&dev);
    if (device_context(dev).prepare_error) return cuda_fail(device_context(dev).prepare_error, "kernel setup");
    genie_index *ix = new genie_index();
    ix->device = dev;
    ix->tuning = device_context(dev).tuning;
    cudaMallocHost((void **)&ix->host_err, 16);
    if (!build_host_index(values, n_objects, n_dims, ix->host)) {
        delete ix;
        return fail(GENIE_ERR_INVALID_ARG, "index build failed (N must be < 2^32)");
    }
    ComprLayout L;
    if (!build_compressed(ix->host, codec, max_segment, L)) {
        delete ix;
        return fail(GENIE_ERR_INVALID_ARG, "compression failed");
    }
    ix->codec = codec;
    ix->max_seg = max_segment;
    int rc = upload_compressed(ix, L.words, L.key_seg, L.seg_word_off, L.seg_first, L.seg_len);
    if (rc) {
        delete ix;
        return rc;
    }
    return finish_loaded_index(ix, out);
}

int genie_index_copy_compressed(const genie_index *ix, uint32_t *words, int64_t *key_seg, int64_t *seg_word_off,
                                uint32_t *seg_first, uint32_t *seg_len) {
    if (!ix) return fail(GENIE_ERR_INVALID_ARG, "index is NULL");
    if (!ix->codec) return fail(GENIE_ERR_INVALID_ARG, "index is not compressed");
    cudaSetDevice(ix->device);
    cudaError_t e = cudaSuccess;
    const int64_t nk = ix->host.n_keys();
    if (words && !e) e = cudaMemcpy(words, ix->d_words.p, ix->n_words * 4, cudaMemcpyDeviceToHost);
    if (key_seg && !e) e = cudaMemcpy(key_seg, ix->d_key_seg.p, (nk + 1) * 8, cudaMemcpyDeviceToHost);
    if (seg_word_off && !e) e = cudaMemcpy(seg_word_off, ix->d_seg_word_off.p, (ix->n_segs + 1) * 8, cudaMemcpyDeviceToHost);
    if (seg_first && !e) e = cudaMemcpy(seg_first, ix->d_seg_first.p, ix->n_segs * 4, cudaMemcpyDeviceToHost);
    if (seg_len && !e && ix->n_segs) {
        std::vector<int64_t> pos((size_t)ix->n_segs + 1);
        e = cudaMemcpy(pos.data(), ix->d_seg_len.p, pos.size() * 8, cudaMemcpyDeviceToHost);
        for (int64_t s = 0; s < ix->n_segs && !e; ++s) seg_len[s] = (uint32_t)(pos[s + 1] - pos[s]);
    }
    return e ? cuda_fail(e, "compressed index download") : GENIE_OK;
}

int64_t genie_codec_encode_bound(int64_t n) { return encode_bound(n); }

int64_t genie_codec_encode(int32_t codec, const uint32_t *in, int64_t n, uint32_t *out, int64_t cap) {
    if (!in || !out || n <= 0) return -fail(GENIE_ERR_INVALID_ARG, "NULL or empty input");
    std::vector<uint32_t> w;
    w.reserve((size_t)encode_bound(n));
    if (!encode(codec, in, (size_t)n, w)) return -fail(GENIE_ERR_INVALID_ARG, "unknown codec %d", codec);
    if ((int64_t)w.size() > cap) return -fail(GENIE_ERR_INVALID_ARG, "output capacity %lld < %lld words", (long long)cap, (long long)w.size());
    memcpy(out, w.data(), w.size() * 4);
    return (int64_t)w.size();
}

int genie_codec_decode_device(int32_t codec, const uint32_t *words, const int64_t *word_off, int64_t n_segments,
                              const int64_t *out_off, uint32_t *out, uint32_t *out_len, void *stream) {
    int deltas, inner;
    codec_parts(codec, deltas, inner);
    if (codec <= 0 || codec >= kNumCodecs || deltas < 0) return fail(GENIE_ERR_INVALID_ARG, "unknown codec %d", codec);
    if (n_segments < 0 || (n_segments && (!words || !word_off || !out_off || !out || !out_len)))
        return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    if (!n_segments) return GENIE_OK;
    const int threads = 256;
    const int64_t blocks = (n_segments * 32 + threads - 1) / threads;
    k_decode_segments<<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(codec, words, word_off, n_segments,
                                                                            out_off, out, out_len);
    cudaError_t e = cudaGetLastError();
    return e ? cuda_fail(e, "decode launch") : GENIE_OK;
}

}  // extern "C"
