// genie/interface/types.h -- data types of the C++ interface
// (reference src/genie/interface/types.h:12-20).
#ifndef GENIE_INTERFACE_TYPES_H_
#define GENIE_INTERFACE_TYPES_H_

#include <utility>
#include <vector>

namespace genie {

// Row-major table: row i lists object i's value on every dim.
typedef std::vector<std::vector<int> > TableData;
// One row per query: item j asks for dim j's value (within the query range).
typedef std::vector<std::vector<int> > QueryData;
// (ids, counts), k slots per query, row-major q*k + j.
typedef std::pair<std::vector<int>, std::vector<int> > SearchResult;

}  // namespace genie

#endif
