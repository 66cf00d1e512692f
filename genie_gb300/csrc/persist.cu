// persist.cu -- this library's own versioned index file format.
//
// Replaces the reference's Boost binary archive (utility/serialization.cc:23-146),
// which stores the whole inv_table object graph.  Layout (little endian):
//   "GENIEGB3"  u32 version  u32 flags(bit0 bag, bit1 compressed)
//   i64 n_objects  i32 n_dims  i32 mult_max  i32 codec  i32 max_seg
//   i64 n_keys  i64 n_ids  i64 n_words  i64 n_segs
//   i32 dim_min[D]  i32 dim_max[D]  i64 key_base[D+1]  i64 key_off[n_keys+1]
//   u32 ids[n_ids]                                  (uncompressed)
//   or u32 words[n_words] i64 key_seg[n_keys+1] i64 seg_word_off[n_segs+1]
//      u32 seg_first[n_segs] u32 seg_len[n_segs]    (compressed)
//   u64 FNV-1a checksum of every byte above
#include "capi_internal.h"

#include <cstdio>
#include <cstring>
#include <fstream>

namespace gg {

namespace {

const char kMagic[8] = {'G', 'E', 'N', 'I', 'E', 'G', 'B', '3'};
const uint32_t kVersion = 1;

struct Hasher {
    uint64_t h = 1469598103934665603ull;
    void add(const void *p, size_t n) {
        const unsigned char *b = (const unsigned char *)p;
        for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    }
};

struct Writer {
    std::ofstream f;
    Hasher h;
    bool put(const void *p, size_t n) {
        h.add(p, n);
        f.write((const char *)p, (std::streamsize)n);
        return (bool)f;
    }
};

struct Reader {
    std::ifstream f;
    Hasher h;
    bool get(void *p, size_t n) {
        f.read((char *)p, (std::streamsize)n);
        if (!f) return false;
        h.add(p, n);
        return true;
    }
};

template <class T>
bool get_vec(Reader &r, std::vector<T> &v, int64_t n) {
    if (n < 0 || n > (int64_t)1 << 40) return false;
    v.resize((size_t)n);
    return n == 0 || r.get(v.data(), (size_t)n * sizeof(T));
}

}  // namespace

int save_index(const genie_index *ix, const char *path) {
    const HostIndex &h = ix->host;
    Writer w;
    w.f.open(path, std::ios::binary | std::ios::trunc);
    if (!w.f) return fail(GENIE_ERR_IO, "cannot open %s for writing", path);
    uint32_t flags = (ix->is_bag ? 1u : 0u) | (ix->codec ? 2u : 0u);
    int64_t n_keys = h.n_keys();
    bool ok = w.put(kMagic, 8) && w.put(&kVersion, 4) && w.put(&flags, 4) && w.put(&h.n_objects, 8) &&
              w.put(&h.n_dims, 4) && w.put(&h.mult_max, 4) && w.put(&ix->codec, 4) && w.put(&ix->max_seg, 4) &&
              w.put(&n_keys, 8) && w.put(&ix->n_ids, 8) && w.put(&ix->n_words, 8) && w.put(&ix->n_segs, 8) &&
              w.put(h.dim_min.data(), h.dim_min.size() * 4) && w.put(h.dim_max.data(), h.dim_max.size() * 4) &&
              w.put(h.key_base.data(), h.key_base.size() * 8) && w.put(h.key_off.data(), h.key_off.size() * 8);
    if (!ok) return fail(GENIE_ERR_IO, "write failed: %s", path);
    cudaSetDevice(ix->device);
    auto dump = [&](const DevBuf &b, size_t bytes) -> bool {
        if (!bytes) return true;
        std::vector<unsigned char> tmp(bytes);
        if (cudaMemcpy(tmp.data(), b.p, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
        return w.put(tmp.data(), bytes);
    };
    if (!ix->codec) {
        ok = dump(ix->d_ids, (size_t)ix->n_ids * 4);
    } else {
        ok = dump(ix->d_words, (size_t)ix->n_words * 4) && dump(ix->d_key_seg, (size_t)(n_keys + 1) * 8) &&
             dump(ix->d_seg_word_off, (size_t)(ix->n_segs + 1) * 8) && dump(ix->d_seg_first, (size_t)ix->n_segs * 4);
        if (ok) {   // the device keeps segment positions; the file keeps lengths
            std::vector<int64_t> pos((size_t)ix->n_segs + 1);
            std::vector<uint32_t> len((size_t)ix->n_segs);
            ok = cudaMemcpy(pos.data(), ix->d_seg_len.p, pos.size() * 8, cudaMemcpyDeviceToHost) == cudaSuccess;
            for (size_t s = 0; ok && s < len.size(); ++s) len[s] = (uint32_t)(pos[s + 1] - pos[s]);
            ok = ok && (len.empty() || w.put(len.data(), len.size() * 4));
        }
    }
    if (!ok) return fail(GENIE_ERR_IO, "write failed: %s", path);
    uint64_t sum = w.h.h;
    w.f.write((const char *)&sum, 8);
    if (!w.f) return fail(GENIE_ERR_IO, "write failed: %s", path);
    return GENIE_OK;
}

int upload_compressed(genie_index *ix, const std::vector<uint32_t> &words, const std::vector<int64_t> &key_seg,
                      const std::vector<int64_t> &seg_word_off, const std::vector<uint32_t> &seg_first,
                      const std::vector<uint32_t> &seg_len);

int load_index(const char *path, genie_index *ix) {
    Reader r;
    r.f.open(path, std::ios::binary);
    if (!r.f) return fail(GENIE_ERR_IO, "cannot open %s", path);
    char magic[8];
    uint32_t version = 0, flags = 0;
    int64_t n_keys = 0;
    HostIndex &h = ix->host;
    bool ok = r.get(magic, 8) && memcmp(magic, kMagic, 8) == 0 && r.get(&version, 4) && version == kVersion &&
              r.get(&flags, 4) && r.get(&h.n_objects, 8) && r.get(&h.n_dims, 4) && r.get(&h.mult_max, 4) &&
              r.get(&ix->codec, 4) && r.get(&ix->max_seg, 4) && r.get(&n_keys, 8) && r.get(&ix->n_ids, 8) &&
              r.get(&ix->n_words, 8) && r.get(&ix->n_segs, 8);
    if (!ok || h.n_dims <= 0 || h.n_objects <= 0) return fail(GENIE_ERR_IO, "%s is not a genie index file", path);
    ok = get_vec(r, h.dim_min, h.n_dims) && get_vec(r, h.dim_max, h.n_dims) && get_vec(r, h.key_base, h.n_dims + 1) &&
         get_vec(r, h.key_off, n_keys + 1);
    std::vector<uint32_t> words, seg_first, seg_len;
    std::vector<int64_t> key_seg, seg_word_off;
    if (ok && !ix->codec) ok = get_vec(r, h.ids, ix->n_ids);
    if (ok && ix->codec)
        ok = get_vec(r, words, ix->n_words) && get_vec(r, key_seg, n_keys + 1) &&
             get_vec(r, seg_word_off, ix->n_segs + 1) && get_vec(r, seg_first, ix->n_segs) &&
             get_vec(r, seg_len, ix->n_segs);
    uint64_t want = r.h.h, sum = 0;
    if (ok) {
        r.f.read((char *)&sum, 8);
        ok = (bool)r.f;
    }
    if (!ok) return fail(GENIE_ERR_IO, "%s is truncated", path);
    if (sum != want) return fail(GENIE_ERR_IO, "%s fails its checksum", path);
    if (h.key_base.back() != n_keys || h.key_off.back() < 0) return fail(GENIE_ERR_IO, "%s is inconsistent", path);
    // the kernels index shared memory by object id and search lists by
    // bisection: a file whose checksum holds must still describe a valid index
    for (int32_t d = 0; d < h.n_dims; ++d) {
        const int64_t width = (int64_t)h.dim_max[d] - h.dim_min[d] + 1;
        if (h.key_base[d] < 0 || h.key_base[d + 1] < h.key_base[d] ||
            (width > 0 && h.key_base[d] + width > h.key_base[d + 1]))
            return fail(GENIE_ERR_IO, "%s is inconsistent (dimension %d)", path, d);
    }
    if (!ix->codec) {
        if (h.key_off[0] != 0 || h.key_off.back() != ix->n_ids)
            return fail(GENIE_ERR_IO, "%s is inconsistent (list offsets)", path);
        for (int64_t k = 0; k < n_keys; ++k) {
            const int64_t a = h.key_off[k], b = h.key_off[k + 1];
            if (b < a) return fail(GENIE_ERR_IO, "%s is inconsistent (list %lld)", path, (long long)k);
            for (int64_t p = a; p < b; ++p)
                if ((int64_t)h.ids[p] >= h.n_objects || (p > a && h.ids[p] < h.ids[p - 1]))
                    return fail(GENIE_ERR_IO, "%s is inconsistent (list %lld)", path, (long long)k);
        }
    }
    ix->is_bag = (flags & 1u) != 0;
    if (!ix->codec) return upload_index(ix);
    return upload_compressed(ix, words, key_seg, seg_word_off, seg_first, seg_len);
}

}  // namespace gg

using namespace gg;

extern "C" int genie_index_save(const genie_index *ix, const char *path) {
    if (!ix || !path) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    if (ix->sub_shift >= 0)
        return fail(GENIE_ERR_NOT_IMPLEMENTED, "the file format holds no subsequence index");
    return save_index(ix, path);
}

namespace gg {
int finish_loaded_index(genie_index *ix, genie_index **out);
}

extern "C" int genie_index_load(const char *path, genie_index **out) {
    if (!path || !out) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    int dev = 0;
    cudaGetDevice(&dev);
    genie_index *ix = new genie_index();
    ix->device = dev;
    ix->tuning = device_context(dev).tuning;
    cudaMallocHost((void **)&ix->host_err, 16);
    int rc = load_index(path, ix);
    if (rc) {
        delete ix;
        return rc;
    }
    return finish_loaded_index(ix, out);
}
