// tile_dir.cu -- tile directories and dense-list bitmaps of a resident index.
//
// The dense kernel counts a query one id tile at a time, so for every tile it
// needs, in each posting list the query covers, the positions where the tile
// begins and ends.  Searching for them (chains of dependent global loads per
// list per tile, while the rest of the block waits) took a quarter of the
// dense kernel's time on the uneven-range batch.  A tile directory holds, for
// every long list and every tile boundary t * tile, the offset in the list of
// the first id >= t * tile (for a compressed list: of the first segment
// starting at >= t * tile); a tile's cut of a list is then two independent
// loads.
//
// Layout: dir_slot[key] is the row of a key (~0u: no row, the list is
// shorter than the budget allows rows for, and is searched), row r holds
// ntiles + 1 u32 offsets relative to the list
// start.  Rows are shared by the directories of the two counter widths (one
// per tile size).  A directory is built once per (index, tile size) by one
// thread per (row, boundary) and kept while the index lives: batches capture
// its address in their CUDA graphs.
//
// Dense-list bitmaps: a posting list holding at least 1/16 of the objects
// (the lists of a dimension's most common value) is also kept as a presence
// bitmap of n_objects bits, a tenth or less of its ids' bytes at such
// densities.  The dense kernel counts such a list from its bitmap words
// (each thread owns 32 objects of the tile, so plain adds replace the
// shared-memory atomics) and streams (or decodes) only the other lists.
// Built once per index with one value per object and dim (no list repeats an
// id; a compressed index decodes its dense lists' segments to build them), on
// first use, within a budget; kept while the index lives.
#include "capi_internal.h"
#include "codecs.cuh"

#include <algorithm>

namespace gg {
namespace {

constexpr size_t kDirBudget = size_t(1) << 30;   // bytes of one directory at most
// A list shorter than a tile's cut search is worth nothing but still makes
// the whole block wait for the search: every list gets a row when the
// directories fit their budget, else lists of at least the smallest of these
// lengths (ids, or segments of a compressed index) that fits.
constexpr int64_t kDirMinLens[] = {1, 16, 64, 256, 1024, 4096};
// the smallest tile a directory is sized for (the 4-byte counter tile of the
// smallest autotuner tile)
constexpr int64_t kDirSmallestTile = 98304 / 4;
constexpr int64_t kBmMinObjects = 65536;         // id spaces too small for bitmaps to pay
constexpr int64_t kBmDensity = 16;               // a list with len * 16 >= n_objects gets a bitmap
constexpr size_t kBmBudget = size_t(2) << 30;    // bytes of all bitmap rows at most

// Bit o of row r for every id o of row r's list; one CTA row per blockIdx.y.
__global__ void k_bm_build(const uint32_t *__restrict__ ids, const int64_t *__restrict__ key_off,
                           const uint32_t *__restrict__ row_key, int64_t words, uint32_t *__restrict__ rows) {
    const uint32_t r = blockIdx.y;
    const uint32_t key = row_key[r];
    const int64_t a = key_off[key], e = key_off[key + 1];
    uint32_t *row = rows + (size_t)r * (size_t)words;
    for (int64_t p = a + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < e; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t id = ids[p];
        atomicOr(&row[id >> 5], 1u << (id & 31u));
    }
}

__global__ void k_tile_dir(const uint32_t *__restrict__ keys_first, const int64_t *__restrict__ list_off,
                           const uint32_t *__restrict__ row_key, int64_t n_rows, int64_t ntiles, int64_t tile,
                           uint32_t *__restrict__ dir) {
    const int64_t n = n_rows * (ntiles + 1);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / (ntiles + 1), t = i - r * (ntiles + 1);
        const uint32_t key = row_key[r];
        const int64_t a = list_off[key], e = list_off[key + 1];
        const uint64_t x = (uint64_t)t * (uint64_t)tile;
        const int64_t pos = (t == ntiles || x > 0xFFFFFFFFull) ? e : lower_bound_u32(keys_first, a, e, (uint32_t)x);
        dir[i] = (uint32_t)(pos - a);
    }
}

// Rows of the index's long lists (once per index); false when it has none.
bool ensure_dir_rows(genie_index *ix) {
    if (ix->dir_rows_ready) return ix->dir_rows > 0;
    ix->dir_rows_ready = true;
    ix->dir_rows = -1;
    const int64_t nk = ix->host.n_keys();
    if (nk <= 0 || nk >= (int64_t)0xFFFFFFFFll) return false;
    std::vector<int64_t> off;
    if (ix->codec) {            // segment offsets of the keys
        off.resize((size_t)nk + 1);
        if (cudaMemcpy(off.data(), ix->d_key_seg.p, (size_t)(nk + 1) * 8, cudaMemcpyDeviceToHost)) {
            cudaGetLastError();
            return false;
        }
    } else {
        off = ix->host.key_off;
    }
    const int64_t max_tiles = (ix->host.n_objects + kDirSmallestTile - 1) / kDirSmallestTile + 1;
    int64_t min_len = kDirMinLens[sizeof(kDirMinLens) / sizeof(kDirMinLens[0]) - 1];
    for (int64_t len : kDirMinLens) {
        int64_t rows = 0;
        for (int64_t k = 0; k < nk; ++k) rows += off[k + 1] - off[k] >= len ? 1 : 0;
        if ((size_t)rows * (size_t)max_tiles * 4 <= kDirBudget) {
            min_len = len;
            break;
        }
    }
    std::vector<uint32_t> slot((size_t)nk, 0xFFFFFFFFu), row_key;
    for (int64_t k = 0; k < nk; ++k)
        if (off[k + 1] - off[k] >= min_len) {
            slot[(size_t)k] = (uint32_t)row_key.size();
            row_key.push_back((uint32_t)k);
        }
    if (row_key.empty()) return false;
    cudaError_t e;
    if ((e = ix->d_dir_slot.reserve(slot.size() * 4)) ||
        (e = cudaMemcpy(ix->d_dir_slot.p, slot.data(), slot.size() * 4, cudaMemcpyHostToDevice)) ||
        (e = ix->d_dir_row_key.reserve(row_key.size() * 4)) ||
        (e = cudaMemcpy(ix->d_dir_row_key.p, row_key.data(), row_key.size() * 4, cudaMemcpyHostToDevice))) {
        cudaGetLastError();
        return false;
    }
    ix->dir_rows = (int64_t)row_key.size();
    return true;
}

// The directory of one tile size (built on first use); nullptr when the index
// has no long lists or the directory would exceed its budget.
const uint32_t *tile_dir(genie_index *ix, int32_t tile) {
    if (tile <= 0) return nullptr;
    for (const auto &d : ix->dirs)
        if (d.first == tile) return (const uint32_t *)d.second->p;
    if (!ensure_dir_rows(ix)) return nullptr;
    const int64_t ntiles = (ix->host.n_objects + tile - 1) / tile;
    const size_t bytes = (size_t)ix->dir_rows * (size_t)(ntiles + 1) * 4;
    if (bytes > kDirBudget) return nullptr;
    DevBuf *b = new DevBuf();
    if (b->reserve(bytes)) {
        cudaGetLastError();
        delete b;
        return nullptr;
    }
    const uint32_t *first = ix->codec ? ix->dev.seg_first : ix->dev.ids;
    const int64_t *off = ix->codec ? ix->dev.key_seg : ix->dev.key_off;
    const int64_t n = ix->dir_rows * (ntiles + 1);
    const int grid = (int)std::min<int64_t>((n + 255) / 256, 152 * 32);
    k_tile_dir<<<grid, 256, 0, ix->stream>>>(first, off, (const uint32_t *)ix->d_dir_row_key.p, ix->dir_rows,
                                             ntiles, tile, (uint32_t *)b->p);
    if (cudaGetLastError() || cudaStreamSynchronize(ix->stream)) {
        cudaGetLastError();
        b->release();
        delete b;
        return nullptr;
    }
    ix->dirs.emplace_back(tile, b);
    return (const uint32_t *)b->p;
}

// The same for a compressed index: warp w of the block decodes segments
// w, w + warps, ... of row r's list and sets their ids' bits.
__global__ void k_bm_build_compressed(int codec, const uint32_t *__restrict__ words,
                                      const int64_t *__restrict__ seg_word_off, const int64_t *__restrict__ key_seg,
                                      const uint32_t *__restrict__ row_key, int64_t n_words_row,
                                      uint32_t *__restrict__ rows) {
    const uint32_t r = blockIdx.y;
    const uint32_t key = row_key[r];
    uint32_t *row = rows + (size_t)r * (size_t)n_words_row;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t w0 = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (int64_t sg = key_seg[key] + w0; sg < key_seg[key + 1]; sg += warps) {
        auto set = [&](uint32_t id, uint32_t) { atomicOr(&row[id >> 5], 1u << (id & 31u)); };
        decode_segment_values(codec, words, seg_word_off[sg], seg_word_off[sg + 1], set);
    }
}

// The dense-list bitmaps (built on first use); false when the index has none.
bool dense_bitmaps(genie_index *ix) {
    if (ix->bm_ready) return ix->bm_words > 0;
    ix->bm_ready = true;
    ix->bm_words = 0;
    const int64_t n = ix->host.n_objects, nk = ix->host.n_keys();
    if (ix->is_bag || ix->sub_shift >= 0 || n < kBmMinObjects || nk <= 0 ||
        nk >= (int64_t)0xFFFFFFFFll)
        return false;
    const int64_t words = (n + 31) / 32;
    std::vector<uint32_t> slot((size_t)nk, 0xFFFFFFFFu), row_key;
    for (int64_t k = 0; k < nk; ++k)
        if ((ix->host.key_off[k + 1] - ix->host.key_off[k]) * kBmDensity >= n &&
            (row_key.size() + 1) * (size_t)words * 4 <= kBmBudget && row_key.size() < 65535) {
            slot[(size_t)k] = (uint32_t)row_key.size();
            row_key.push_back((uint32_t)k);
        }
    if (row_key.empty()) return false;
    DevBuf rk;
    cudaError_t e;
    if ((e = ix->d_bm_slot.reserve(slot.size() * 4)) ||
        (e = cudaMemcpy(ix->d_bm_slot.p, slot.data(), slot.size() * 4, cudaMemcpyHostToDevice)) ||
        (e = rk.reserve(row_key.size() * 4)) ||
        (e = cudaMemcpy(rk.p, row_key.data(), row_key.size() * 4, cudaMemcpyHostToDevice)) ||
        (e = ix->d_bm_rows.reserve(row_key.size() * (size_t)words * 4)) ||
        (e = cudaMemsetAsync(ix->d_bm_rows.p, 0, row_key.size() * (size_t)words * 4, ix->stream))) {
        cudaGetLastError();
        rk.release();
        ix->d_bm_slot.release();
        ix->d_bm_rows.release();
        return false;
    }
    if (ix->codec)
        k_bm_build_compressed<<<dim3(64, (unsigned)row_key.size()), 256, 0, ix->stream>>>(
            ix->codec, ix->dev.words, ix->dev.seg_word_off, ix->dev.key_seg, (const uint32_t *)rk.p, words,
            (uint32_t *)ix->d_bm_rows.p);
    else
        k_bm_build<<<dim3(64, (unsigned)row_key.size()), 256, 0, ix->stream>>>(
            ix->dev.ids, ix->dev.key_off, (const uint32_t *)rk.p, words, (uint32_t *)ix->d_bm_rows.p);
    e = cudaGetLastError();
    if (!e) e = cudaStreamSynchronize(ix->stream);
    rk.release();
    if (e) {
        cudaGetLastError();
        ix->d_bm_slot.release();
        ix->d_bm_rows.release();
        return false;
    }
    ix->bm_words = words;
    return true;
}

}  // namespace

DevIndex index_view(genie_index *ix, const Tuning &t) {
    std::lock_guard<std::mutex> g(ix->dir_mu);
    DevIndex d = ix->dev;
    d.dir8 = tile_dir(ix, t.dense_tile_u8);
    d.dir32 = tile_dir(ix, t.dense_tile_u32);
    d.dir8_tile = d.dir8 ? t.dense_tile_u8 : 0;
    d.dir32_tile = d.dir32 ? t.dense_tile_u32 : 0;
    d.dir_slot = (d.dir8 || d.dir32) ? (const uint32_t *)ix->d_dir_slot.p : nullptr;
    const bool bm = dense_bitmaps(ix);
    d.bm_slot = bm ? (const uint32_t *)ix->d_bm_slot.p : nullptr;
    d.bm_rows = bm ? (const uint32_t *)ix->d_bm_rows.p : nullptr;
    d.bm_words = bm ? ix->bm_words : 0;
    return d;
}

}  // namespace gg
