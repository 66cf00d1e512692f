// host_index.h -- host-side CSR builder and query-compile helpers.
#pragma once
#include <cstdint>
#include <vector>

namespace gg {

// CSR inverted index keyed by (dim, value): the host mirror of a resident index.
struct HostIndex {
    int64_t n_objects = 0;
    int32_t n_dims = 0;
    int32_t mult_max = 1;
    std::vector<int32_t> dim_min, dim_max;
    std::vector<int64_t> key_base;     // [D+1]
    std::vector<int64_t> key_off;      // [n_keys+1]
    std::vector<uint32_t> ids;         // ordered by (dim, value, id)
    int64_t n_keys() const { return key_base.empty() ? 0 : key_base.back(); }
};

// One value per object per dim (row-major n x d).  Dims are inverted in
// parallel; each is a stable counting sort, so ids ascend within a list as
// inv_list::invert + inv_table::build produce them (inv_list.cc:295-320,
// inv_table.cu:267-350).
bool build_host_index(const int32_t *values, int64_t n, int32_t d, HostIndex &out);
// Single dim, row r lists r under each of its values (inv_list.cc:51-84).
bool build_host_index_bag(const int32_t *values, const int64_t *row_off, int64_t n, HostIndex &out);

// Query::build span of one item (query/query.cc:273-333); false if empty.
bool item_span(const HostIndex &ix, int32_t dim, int32_t low, int32_t up, int64_t &start, int64_t &end);
// Query::apply_adaptive_query_range for one item (query/query.cc:196-261).
void adaptive_range(const HostIndex &ix, int32_t dim, float sel, int32_t &low, int32_t &up);

}  // namespace gg
