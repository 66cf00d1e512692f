// genie/interface/search.h -- first- and second-level entry points
// (reference src/genie/interface/search.h:16-38).
#ifndef GENIE_INTERFACE_SEARCH_H_
#define GENIE_INTERFACE_SEARCH_H_

#include <memory>
#include <string>
#include <vector>

#include <genie/interface/execution_policy.h>
#include <genie/interface/types.h>

namespace genie {

// Load both CSV files, build, match.
SearchResult Search(std::shared_ptr<genie::ExecutionPolicy> &policy, const std::string &table_filename,
                    const std::string &query_filename);
std::shared_ptr<genie::table::inv_table> BuildTable(std::shared_ptr<genie::ExecutionPolicy> &policy,
                                                    const TableData &table_data);
std::vector<genie::query::Query> BuildQuery(std::shared_ptr<genie::ExecutionPolicy> &policy,
                                            const std::shared_ptr<genie::table::inv_table> &table,
                                            const QueryData &query_data);
SearchResult Match(std::shared_ptr<genie::ExecutionPolicy> &policy,
                   const std::shared_ptr<genie::table::inv_table> &table,
                   const std::vector<genie::query::Query> &queries);

}  // namespace genie

#endif
