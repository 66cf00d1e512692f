// genie/original/interface.h -- the reference's legacy C++ interface
// (src/genie/original/interface.h:64-395): GPUGenie_Config, table loading from
// rows (one value per dim, "bijectMap" bags, subsequences, sequences of
// grams), query loading (single range, multirange files, sequences), the
// knn_search entry points, multiload (tables of at most max_data_size rows
// searched in turn and merged), and multi-table search.  Every search runs
// through the C ABI of <genie_gb300.h>.
//
// Results: k slots per query, row-major (q*k + j), sorted by (count desc, id
// asc) and padded with (0, 0) -- the reference's layout, with its unordered
// ties made deterministic.
#ifndef GENIE_ORIGINAL_INTERFACE_H_
#define GENIE_ORIGINAL_INTERFACE_H_

#include <cuda_runtime.h>

#include <iostream>   // the reference's interface header brings it to its callers
#include <string>
#include <vector>

#include <genie/compression/DeviceCodecFactory.h>
#include <genie/exception/exception.h>
#include <genie/query/query.h>
#include <genie/table/inv_table.h>
#include <genie/utility/FileReader.h>
#include <genie/utility/Logger.h>

#define GPUGENIE_DEFAULT_TOPK 10
#define GPUGENIE_DEFAULT_RADIUS 0
#define GPUGENIE_DEFAULT_THRESHOLD 0
#define GPUGENIE_DEFAULT_HASHTABLE_SIZE 1.0f
#define GPUGENIE_DEFAULT_WEIGHT 1
#define GPUGENIE_DEFAULT_DEVICE 0
#define GPUGENIE_DEFAULT_USE_ADAPTIVE_RANGE false
#define GPUGENIE_DEFAULT_SELECTIVITY -1.0f
#define GPUGENIE_DEFAULT_POSTING_LIST_LENGTH 100000
#define GPUGENIE_DEFAULT_LOAD_MULTIPLIER 3.0f
#define GPUGENIE_DEFAULT_USE_LOAD_BALANCE false
#define GPUGENIE_DEFAULT_USE_MULTIRANGE true
#define GPUGENIE_DEFAULT_NUM_OF_QUERIES 0

namespace genie {
namespace original {

// Search configuration (original/interface.h:71-160).  hashtable_size,
// count_threshold, multiplier, posting_list_max_length and use_load_balance
// size the reference's per-query hash table and block load; the counting
// here is exact and sizes itself, so they are accepted and ignored.
typedef struct _GPUGenie_Config {
    int num_of_topk;
    int query_radius;
    int count_threshold;
    float hashtable_size;
    int use_device;
    int dim;
    bool use_adaptive_range;
    float selectivity;
    std::vector<std::vector<int> > *data_points;
    int *data;
    unsigned int *index;
    unsigned int item_num;
    unsigned int row_num;
    int search_type;            // 0: one value per dim, 1: bijectMap bags, 2: sequences of grams
    int data_type;              // 0: rows from csv (1, binary, is rejected as by the reference)
    unsigned int max_data_size; // multiload: rows per table (0: one table)
    bool save_to_gpu;
    std::vector<std::vector<int> > *query_points;
    std::vector<genie::utility::attr_t> *multirange_query_points;
    int posting_list_max_length;
    float multiplier;
    bool use_load_balance;
    bool use_multirange;
    int num_of_queries;
    bool use_subsequence_search;
    int data_gram_length;
    unsigned int num_of_iteration;
    genie::compression::COMPRESSION_TYPE compression;

    _GPUGenie_Config()
        : num_of_topk(GPUGENIE_DEFAULT_TOPK), query_radius(GPUGENIE_DEFAULT_RADIUS),
          count_threshold(GPUGENIE_DEFAULT_THRESHOLD), hashtable_size(GPUGENIE_DEFAULT_HASHTABLE_SIZE),
          use_device(GPUGENIE_DEFAULT_DEVICE), dim(0), use_adaptive_range(GPUGENIE_DEFAULT_USE_ADAPTIVE_RANGE),
          selectivity(GPUGENIE_DEFAULT_SELECTIVITY), data_points(nullptr), data(nullptr), index(nullptr),
          item_num(0), row_num(0), search_type(0), data_type(0), max_data_size(0), save_to_gpu(false),
          query_points(nullptr), multirange_query_points(nullptr),
          posting_list_max_length(GPUGENIE_DEFAULT_POSTING_LIST_LENGTH), multiplier(GPUGENIE_DEFAULT_LOAD_MULTIPLIER),
          use_load_balance(GPUGENIE_DEFAULT_USE_LOAD_BALANCE), use_multirange(GPUGENIE_DEFAULT_USE_MULTIRANGE),
          num_of_queries(GPUGENIE_DEFAULT_NUM_OF_QUERIES), use_subsequence_search(false), data_gram_length(3),
          num_of_iteration(1), compression(genie::compression::DEFAULT_COMPRESSION_TYPE) {}
} GPUGenie_Config;

// Build the table(s) of config.data_points: one table, or with 0 <
// max_data_size < rows, consecutive tables of max_data_size rows (when the
// rows do not divide evenly, the last full table's rows and the remainder are
// split into two tables of about equal size, original/interface.cc:197-277).
// _table receives new inv_table[n]; release it with delete[].  Multiplies
// num_of_topk by num_of_iteration, as the reference does.
bool preprocess_for_knn_csv(GPUGenie_Config &config, genie::table::inv_table *&_table);
// Load the queries against every table of _table, search each, offset the
// ids of table t by the rows of the tables before it, and merge the per-table
// results of each query into its top num_of_topk / num_of_iteration.
void knn_search_after_preprocess(GPUGenie_Config &config, genie::table::inv_table *&_table,
                                 std::vector<int> &result, std::vector<int> &result_count);
void knn_search(std::vector<int> &result, std::vector<int> &result_count, GPUGenie_Config &config);
void knn_search(std::vector<int> &result, GPUGenie_Config &config);
// One table, queries built against it: h_topk/h_topk_count get k slots per
// query (k = the largest topk of the queries).
void knn_search(genie::table::inv_table &table, std::vector<genie::query::Query> &queries,
                std::vector<int> &h_topk, std::vector<int> &h_topk_count, GPUGenie_Config &config);
// Several tables, one query list and configuration each, all searched at once.
void knn_search_MT(std::vector<genie::table::inv_table *> &table,
                   std::vector<std::vector<genie::query::Query> > &queries, std::vector<std::vector<int> > &h_topk,
                   std::vector<std::vector<int> > &h_topk_count, std::vector<GPUGenie_Config> &config);
void knn_search_for_csv_data(std::vector<int> &result, std::vector<int> &result_count, GPUGenie_Config &config);

void load_table(genie::table::inv_table &table, std::vector<std::vector<int> > &data_points, GPUGenie_Config &config);
void load_query(genie::table::inv_table &table, std::vector<genie::query::Query> &queries, GPUGenie_Config &config);
void load_query_singlerange(genie::table::inv_table &table, std::vector<genie::query::Query> &queries,
                            GPUGenie_Config &config);
void load_query_multirange(genie::table::inv_table &table, std::vector<genie::query::Query> &queries,
                           GPUGenie_Config &config);
void load_table_bijectMap(genie::table::inv_table &table, std::vector<std::vector<int> > &data_points,
                          GPUGenie_Config &config);
// Rows given as one value array (row r = data[index[r] - index[0] ..]).
void load_table(genie::table::inv_table &table, int *data, unsigned int item_num, unsigned int *index,
                unsigned int row_num, GPUGenie_Config &config);
void load_table_bijectMap(genie::table::inv_table &table, int *data, unsigned int item_num, unsigned int *index,
                          unsigned int row_num, GPUGenie_Config &config);
void load_table_sequence(genie::table::inv_table &table, std::vector<std::vector<int> > &data_points,
                         GPUGenie_Config &config);
void load_query_sequence(genie::table::inv_table &table, std::vector<genie::query::Query> &queries,
                         GPUGenie_Config &config);
void sequence_to_gram(std::vector<std::vector<int> > &sequences, std::vector<std::vector<int> > &gram_data,
                      int max_value, int gram_length);
void sequence_reduce_to_ground(std::vector<std::vector<int> > &data, std::vector<std::vector<int> > &converted_data,
                               int &min_value, int &max_value);
void reset_device();
// Subsequence results: id = rowID << shift_bits | offset.
void get_rowID_offset(std::vector<int> &result, std::vector<int> &resultID, std::vector<int> &resultOffset,
                      unsigned int shift_bits);
void init_genie(GPUGenie_Config &config);

}  // namespace original
}  // namespace genie

#endif
