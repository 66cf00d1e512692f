// ref_shim_index.cu -- TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's own index builder and query compiler
// (src/genie/table/inv_list.cc, src/genie/table/inv_table.cu,
// src/genie/query/query.cc) from the read-only reference tree, with no-op
// Boost serialization headers from oracle/ref_stubs/, into oracle/_ref/.  A
// plain C ABI lets tests/golden/make_golden.py pin the oracle's posting order,
// item spans and adaptive ranges against the reference itself.
#include <cstdint>
#include <cstdarg>
#include <vector>

#include "genie/utility/Timing.cc"
#include "genie/table/inv_list.cc"
#include "genie/table/inv_table.cu"
#include "genie/query/query.cc"

const char *const genie::utility::Logger::LEVEL_NAMES[] = {"NONE", "ALERT", "INFO", "VERBOSE", "DEBUG"};
int genie::utility::Logger::log(int, const char *, ...) { return 0; }

using genie::query::Query;
using genie::table::inv_list;
using genie::table::inv_table;

// Builds the reference inv_table (load_table / load_table_bijectMap order,
// original/interface.cc:316-353, 621-646), copies its _inv, then compiles one
// Query per item (attr + optional adaptive range + build) and reports the span.
extern "C" int ref_index_spans(const int32_t *values, int32_t n, int32_t d, int32_t bag,
                               const int64_t *row_off, int32_t n_items, const int32_t *qdim,
                               const int32_t *qlow, const int32_t *qup, const float *qsel,
                               uint32_t *out_ids, int64_t *out_n_ids, int64_t *out_start,
                               int64_t *out_end) {
    inv_table table;
    inv_list list;
    if (!bag) {
        for (int32_t j = 0; j < d; ++j) {
            std::vector<int> col(n);
            for (int32_t i = 0; i < n; ++i) col[i] = values[(int64_t)i * d + j];
            list.invert(col);
            table.append(list);
        }
    } else {
        std::vector<std::vector<int>> rows(n);
        for (int32_t r = 0; r < n; ++r)
            rows[r].assign(values + row_off[r], values + row_off[r + 1]);
        list.invert_bijectMap(rows);
        table.append(list);
    }
    table.build((size_t)-1, false);
    std::vector<int> &inv = *table.inv();
    for (size_t t = 0; t < inv.size(); ++t) out_ids[t] = (uint32_t)inv[t];
    *out_n_ids = (int64_t)inv.size();
    for (int32_t it = 0; it < n_items; ++it) {
        Query q(table, 0);
        float sel = qsel ? qsel[it] : 0.0f;
        q.attr(qdim[it], qlow[it], qup[it], 1.0f, sel, 0);
        if (sel > 0.0f) q.apply_adaptive_query_range();
        std::vector<Query::dim> dims;
        q.build(dims);
        out_start[it] = dims.empty() ? 0 : dims[0].start_pos;
        out_end[it] = dims.empty() ? 0 : dims[0].end_pos;
    }
    return 0;
}
