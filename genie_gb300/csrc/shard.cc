// shard.cc -- the one exchange of an id-range sharded search: merge the
// per-shard top-k lists of every query into the global top-k.
//
// A shard holds the objects [id_offset, id_offset + n) of the table under
// local ids 0..n-1 and answers each query with its own sorted top-k.  Counts
// (and weighted sums) are per object, so the global top-k is the top-k of the
// union of the shards' lists once local ids are offset: exact for unweighted
// queries.  The reference merges the same way on the host: multiload merge
// (original/interface.cc:114-149, 301-312) and the MPI gather + sort of
// dist_genie (sorting.cc:20-64, id offsets online.cu:83-105).
#include "../../include/genie_gb300.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace gg {
int fail(int code, const char *fmt, ...);
}

namespace {

struct Cand {
    float score;
    uint32_t count;
    uint32_t id;
};

}  // namespace

extern "C" int genie_merge_shards(int32_t n_shards, const uint32_t *const *ids, const uint32_t *const *counts,
                                  const float *const *scores, const int64_t *id_offset, int32_t n_queries,
                                  const uint32_t *k, uint32_t uniform_k, uint32_t *out_ids, uint32_t *out_counts,
                                  float *out_scores) {
    using gg::fail;
    if (n_shards < 1 || !ids || !counts || !id_offset || n_queries < 0 || !out_ids || !out_counts)
        return fail(GENIE_ERR_INVALID_ARG, "merge: NULL or negative argument");
    for (int32_t s = 0; s < n_shards; ++s)
        if (!ids[s] || !counts[s] || id_offset[s] < 0 || id_offset[s] > (int64_t)0xFFFFFFFFll)
            return fail(GENIE_ERR_INVALID_ARG, "merge: shard %d has no results or an id offset out of range", s);
    const bool weighted = scores != nullptr;
    if (weighted)
        for (int32_t s = 0; s < n_shards; ++s)
            if (!scores[s]) return fail(GENIE_ERR_INVALID_ARG, "merge: shard %d has no scores", s);
    std::vector<Cand> c;
    int64_t off = 0;
    for (int32_t q = 0; q < n_queries; ++q) {
        const uint32_t kq = k ? k[q] : uniform_k;
        c.clear();
        for (int32_t s = 0; s < n_shards; ++s) {
            for (uint32_t j = 0; j < kq; ++j) {
                const int64_t i = off + j;
                const float sc = weighted ? scores[s][i] : (float)counts[s][i];
                if (counts[s][i] == 0 && sc == 0.0f) continue;       // (0, 0) padding
                const int64_t gid = id_offset[s] + (int64_t)ids[s][i];
                if (gid > (int64_t)0xFFFFFFFFll) return fail(GENIE_ERR_INVALID_ARG, "merge: id beyond 32 bits");
                c.push_back(Cand{sc, counts[s][i], (uint32_t)gid});
            }
        }
        const size_t keep = std::min<size_t>(kq, c.size());
        auto better = [weighted](const Cand &a, const Cand &b) {
            if (weighted && a.score != b.score) return a.score > b.score;
            if (a.count != b.count) return a.count > b.count;
            return a.id < b.id;
        };
        std::partial_sort(c.begin(), c.begin() + keep, c.end(), better);
        for (uint32_t j = 0; j < kq; ++j) {
            const bool have = j < keep;
            out_ids[off + j] = have ? c[j].id : 0u;
            out_counts[off + j] = have ? c[j].count : 0u;
            if (out_scores) out_scores[off + j] = have ? c[j].score : 0.0f;
        }
        off += kq;
    }
    return GENIE_OK;
}
