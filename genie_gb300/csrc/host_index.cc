// host_index.cc -- host CSR builder and query-compile helpers.
#include "host_index.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>

namespace gg {

namespace {

template <class F>
void parallel_for(int64_t n, F f) {
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int64_t nt = std::min<int64_t>(n, (int64_t)hw);
    if (nt <= 1) {
        for (int64_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> pool;
    std::atomic_int64_t next{0};
    for (int64_t t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            for (int64_t i = next++; i < n; i = next++) f(i);
        });
    for (auto &th : pool) th.join();
}

}  // namespace

bool build_host_index(const int32_t *values, int64_t n, int32_t d, HostIndex &ix) {
    if (!values || n <= 0 || d <= 0 || n > (int64_t)UINT32_MAX) return false;
    ix = HostIndex();
    ix.n_objects = n;
    ix.n_dims = d;
    ix.mult_max = 1;
    ix.dim_min.assign(d, 0);
    ix.dim_max.assign(d, 0);
    parallel_for(d, [&](int64_t j) {
        int32_t mn = values[j], mx = values[j];
        for (int64_t i = 1; i < n; ++i) {
            int32_t v = values[i * d + j];
            mn = v < mn ? v : mn;
            mx = v > mx ? v : mx;
        }
        ix.dim_min[j] = mn;
        ix.dim_max[j] = mx;
    });
    ix.key_base.assign(d + 1, 0);
    for (int32_t j = 0; j < d; ++j)
        ix.key_base[j + 1] = ix.key_base[j] + ((int64_t)ix.dim_max[j] - ix.dim_min[j] + 1);
    ix.key_off.assign(ix.n_keys() + 1, 0);
    ix.ids.resize((size_t)(n * d));
    // Every dim holds exactly n postings, so dim j owns ids[j*n, (j+1)*n).
    parallel_for(d, [&](int64_t j) {
        const int64_t kb = ix.key_base[j], nk = ix.key_base[j + 1] - kb;
        const int32_t mn = ix.dim_min[j];
        std::vector<int64_t> pos((size_t)nk + 1, 0);
        for (int64_t i = 0; i < n; ++i) pos[(size_t)(values[i * d + j] - mn) + 1]++;
        for (int64_t v = 0; v < nk; ++v) pos[v + 1] += pos[v];
        for (int64_t v = 0; v < nk; ++v) ix.key_off[kb + v] = j * n + pos[v];
        uint32_t *dst = ix.ids.data() + j * n;
        for (int64_t i = 0; i < n; ++i) dst[pos[(size_t)(values[i * d + j] - mn)]++] = (uint32_t)i;
    });
    ix.key_off[ix.n_keys()] = n * d;
    return true;
}

bool build_host_index_bag(const int32_t *values, const int64_t *row_off, int64_t n, HostIndex &ix) {
    if (!values || !row_off || n <= 0 || n > (int64_t)UINT32_MAX) return false;
    const int64_t total = row_off[n];
    if (total <= 0) return false;
    ix = HostIndex();
    ix.n_objects = n;
    ix.n_dims = 1;
    int32_t mn = values[0], mx = values[0];
    for (int64_t t = 1; t < total; ++t) {
        mn = std::min(mn, values[t]);
        mx = std::max(mx, values[t]);
    }
    ix.dim_min = {mn};
    ix.dim_max = {mx};
    ix.key_base = {0, (int64_t)mx - mn + 1};
    const int64_t nk = ix.key_base[1];
    ix.key_off.assign((size_t)nk + 1, 0);
    for (int64_t t = 0; t < total; ++t) ix.key_off[(size_t)(values[t] - mn) + 1]++;
    for (int64_t v = 0; v < nk; ++v) ix.key_off[v + 1] += ix.key_off[v];
    std::vector<int64_t> pos(ix.key_off.begin(), ix.key_off.end() - 1);
    ix.ids.resize((size_t)total);
    for (int64_t r = 0; r < n; ++r)
        for (int64_t t = row_off[r]; t < row_off[r + 1]; ++t) ix.ids[pos[(size_t)(values[t] - mn)]++] = (uint32_t)r;
    // a row repeating a value repeats its id in that list (adjacent entries)
    int32_t best = 1;
    for (int64_t v = 0; v < nk; ++v) {
        int32_t run = 1;
        for (int64_t p = ix.key_off[v] + 1; p < ix.key_off[v + 1]; ++p) {
            run = ix.ids[p] == ix.ids[p - 1] ? run + 1 : 1;
            best = std::max(best, run);
        }
    }
    ix.mult_max = best;
    return true;
}

bool item_span(const HostIndex &ix, int32_t dim, int32_t low, int32_t up, int64_t &start, int64_t &end) {
    start = end = 0;
    if (dim < 0 || dim >= ix.n_dims) return false;
    const int32_t mn = ix.dim_min[dim], mx = ix.dim_max[dim];
    if (low > up || low > mx || up < mn) return false;
    low = std::max(low, mn);
    up = std::min(up, mx);
    start = ix.key_off[ix.key_base[dim] + ((int64_t)low - mn)];
    end = ix.key_off[ix.key_base[dim] + ((int64_t)up - mn) + 1];
    return true;
}

void adaptive_range(const HostIndex &ix, int32_t dim, float sel, int32_t &low, int32_t &up) {
    if (dim < 0 || dim >= ix.n_dims || !(sel > 0.0f)) return;
    auto contains = [&](int64_t v) { return v >= ix.dim_min[dim] && v <= ix.dim_max[dim]; };
    auto size = [&](int64_t v) -> uint64_t {
        if (!contains(v)) return 0;
        const int64_t key = ix.key_base[dim] + (v - ix.dim_min[dim]);
        return (uint64_t)(ix.key_off[key + 1] - ix.key_off[key]);
    };
    // threshold in float arithmetic, as the reference computes it
    const float want = sel * (float)ix.n_objects;
    const uint32_t threshold = (uint32_t)std::ceil(want);
    int64_t lo = low, hi = up;
    uint64_t count = 0;
    for (int64_t v = lo; v <= hi; ++v) count += size(v);
    while (count < threshold) {
        if (lo > 0) {
            --lo;
            if (!contains(lo)) continue;
            count += size(lo);
        }
        if (contains(hi + 1)) {
            ++hi;
            count += size(hi);
        } else if (lo == 0) {
            break;
        }
    }
    low = (int32_t)lo;
    up = (int32_t)hi;
}

}  // namespace gg
