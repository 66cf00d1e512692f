// genie/utility/FileReader.h -- CSV readers of the legacy interface
// (reference src/genie/utility/FileReader.h:29-106).
#ifndef GENIE_UTILITY_FILEREADER_H_
#define GENIE_UTILITY_FILEREADER_H_

#include <vector>

namespace genie {
namespace table {
class inv_table;
}
namespace query {
class Query;
}
}  // namespace genie

namespace genie {
namespace utility {

// One item of a multirange query file: qid, dim, value, selectivity, weight.
typedef struct _GPUGenie_Query_Data {
    int qid;
    int dim;
    int value;
    float sel;
    float weight;
} attr_t;

const unsigned int GPUGENIE_QUERY_QID_INDEX = 0u;
const unsigned int GPUGENIE_QUERY_DIM_INDEX = 1u;
const unsigned int GPUGENIE_QUERY_VALUE_INDEX = 2u;
const unsigned int GPUGENIE_QUERY_SELECTIVITY_INDEX = 3u;
const unsigned int GPUGENIE_QUERY_WEIGHT_INDEX = 4u;
const unsigned int GPUGENIE_QUERY_NUM_OF_FIELDS = 5u;

// Rows of integers separated by ',' or blanks; at most num rows (num < 0: all).
void read_file(std::vector<std::vector<int> > &dest, const char *fname, int num);
// num_of_queries rows as queries over table: item j of a row matches dim j
// within [v - radius, v + radius] (the first num_of_query_dims items).
void read_query(genie::table::inv_table &table, const char *fname, std::vector<genie::query::Query> &queries,
                int num_of_queries, int num_of_query_dims, int radius, int topk, float selectivity);
// Multirange items "qid, dim, value, sel, weight", at most num lines (num < 0: all).
void read_query(std::vector<attr_t> &data, const char *file_name, int num);

}  // namespace utility
}  // namespace genie

#endif
