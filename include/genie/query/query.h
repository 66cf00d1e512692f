// genie/query/query.h -- one query: items (dim, low..up, weight) over a table
// (reference src/genie/query/query.h:36-200).  Spans are computed by the
// library on the device at search time; build() computes them on the host
// for inspection (Query::build, query.cc:273-333).
#ifndef GENIE_QUERY_QUERY_H_
#define GENIE_QUERY_QUERY_H_

#include <vector>

#include <genie/table/inv_table.h>

typedef unsigned int u32;
typedef unsigned long long u64;

namespace genie {
namespace query {

class Query {
  public:
    struct range {
        int query;
        int order;
        int dim;
        int low;
        int up;
        float weight;
        int low_offset;
        int up_offset;
        float selectivity;
    };
    struct dim {
        int query;
        int order;
        int start_pos;
        int end_pos;
        float weight;
        dim(int query_, int order_, int start, int end, float weight_)
            : query(query_), order(order_), start_pos(start), end_pos(end), weight(weight_) {}
    };

    Query(genie::table::inv_table *ref, int index);
    Query(genie::table::inv_table &ref, int index);
    Query();

    genie::table::inv_table *ref_table();
    // Items on dims outside [0, m_size) are dropped (query.cc:87-113).
    void attr(int index, int low, int up, float weight, int order);
    void attr(int index, int value, float weight, float selectivity, int order);
    void attr(int index, int low, int up, float weight, float selectivity, int order);
    void clear_dim(int index);
    void selectivity(float s);
    float selectivity();
    // Widen every item until it covers ceil(selectivity * N) posting ids.
    void apply_adaptive_query_range();
    void topk(int k);
    int topk();
    // Spans [start, end) of the items (empty items are skipped).
    void build();
    int dump(std::vector<dim> &vout);
    int dump(std::vector<range> &ranges);
    int index();
    int count_ranges();
    // Weighted: the item weights count (an extension; the reference counts matches only).
    void weighted(bool w) { weighted_ = w; }
    bool weighted() const { return weighted_; }

  private:
    genie::table::inv_table *ref_ = nullptr;
    int index_ = 0;
    int topk_ = 0;
    float selectivity_ = -1.0f;
    bool weighted_ = false;
    std::vector<range> ranges_;
    std::vector<dim> dims_;
};

}  // namespace query
}  // namespace genie

#endif
