// genie/interface/io.h -- CSV and binary table I/O
// (reference src/genie/interface/io.h:16-28).  Binary tables use this
// library's versioned file format, not Boost archives.
#ifndef GENIE_INTERFACE_IO_H_
#define GENIE_INTERFACE_IO_H_

#include <memory>
#include <string>

#include <genie/interface/execution_policy.h>
#include <genie/interface/types.h>

namespace genie {

TableData LoadTableDataFromCsv(const std::string &filename);
std::shared_ptr<genie::table::inv_table> LoadTableFromBinary(const std::string &filename);
void SaveTableToBinary(const std::string &filename, const std::shared_ptr<const genie::table::inv_table> &table);
// The first policy->GetNumOfQueries() rows.
QueryData LoadQueryDataFromCsv(const std::string &filename, const std::shared_ptr<const ExecutionPolicy> &policy);

}  // namespace genie

#endif
