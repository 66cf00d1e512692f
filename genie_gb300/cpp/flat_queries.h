// flat_queries.h -- a list of genie::query::Query flattened into the
// arrays of a genie_queries (item ranges, weights, per-query k), shared by
// the first/second-level interface (genie.cc) and the legacy one
// (original.cc).
#pragma once
#include <genie/exception/exception.h>
#include <genie/query/query.h>

#include <cstdint>
#include <vector>

#include "../../include/genie_gb300.h"

namespace genie {

// Flattened genie_queries of a query list (arrays owned here).
struct FlatQueries {
    std::vector<int64_t> item_off{0};
    std::vector<int32_t> dim, low, up;
    std::vector<float> weight;
    std::vector<uint8_t> weighted;
    std::vector<uint32_t> k;
    bool any_weighted = false;
    int64_t total_k = 0;

    explicit FlatQueries(const std::vector<query::Query> &qs) {
        for (const query::Query &cq : qs) {
            query::Query &q = const_cast<query::Query &>(cq);
            std::vector<query::Query::range> rs;
            q.dump(rs);
            for (const auto &r : rs) {
                dim.push_back(r.dim);
                low.push_back(r.low);
                up.push_back(r.up);
                weight.push_back(r.weight);
            }
            item_off.push_back((int64_t)dim.size());
            weighted.push_back(q.weighted() ? 1 : 0);
            any_weighted = any_weighted || q.weighted();
            if (q.topk() <= 0) throw exception::InvalidConfigurationException("a query has no top-k");
            k.push_back((uint32_t)q.topk());
            total_k += q.topk();
        }
    }
    genie_queries view() const {
        genie_queries g{};
        g.n_queries = (int32_t)k.size();
        g.item_off = item_off.data();
        g.dim = dim.data();
        g.low = low.data();
        g.up = up.data();
        g.weight = any_weighted ? weight.data() : nullptr;
        g.weighted = any_weighted ? weighted.data() : nullptr;
        g.k = k.data();
        g.uniform_k = 0;
        return g;
    }
};

}  // namespace genie
