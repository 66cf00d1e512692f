// genie/interface/execution_policy.h -- how tables and queries are built and
// matched (reference src/genie/interface/execution_policy.h:21-71).
#ifndef GENIE_INTERFACE_EXECUTION_POLICY_H_
#define GENIE_INTERFACE_EXECUTION_POLICY_H_

#include <cstdint>
#include <memory>
#include <vector>

#include <genie/interface/config.h>
#include <genie/interface/types.h>
#include <genie/query/query.h>
#include <genie/table/inv_table.h>

namespace genie {

class ExecutionPolicy {
  public:
    virtual ~ExecutionPolicy() = default;
    virtual std::shared_ptr<genie::table::inv_table> BuildTable(const genie::TableData &table_data) = 0;
    virtual std::vector<genie::query::Query> BuildQuery(const std::shared_ptr<const genie::table::inv_table> &table,
                                                        const genie::QueryData &query_data) = 0;
    virtual genie::SearchResult Match(const std::shared_ptr<const genie::table::inv_table> &table,
                                      const std::vector<genie::query::Query> &queries) = 0;
    // Several tables at once: results of table t follow those of table t-1.
    virtual genie::SearchResult Match(const std::vector<std::shared_ptr<const genie::table::inv_table> > &tables,
                                      const std::vector<std::vector<genie::query::Query> > &queries) = 0;
    virtual void Validate();
    void SetK(const uint32_t k);
    void SetNumOfQueries(const uint32_t num_of_queries);
    uint32_t GetNumOfQueries() const;

  protected:
    uint32_t k_ = 0;
    uint32_t dim_ = 0;
    uint32_t num_of_queries_ = 0;
};

// Exact-value matching (query_range unset) or matching within +- query_range.
std::shared_ptr<ExecutionPolicy> MakePolicy(const Config &config);

}  // namespace genie

#endif
