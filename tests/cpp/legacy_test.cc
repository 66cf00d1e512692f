// legacy_test.cc -- drives the legacy interface <genie/original/interface.h>
// (libgenie.so over the C ABI) the way the reference's own tests and examples
// drive the reference library, checks the golden values those tests assert
// (test_csv_input_sift_data.cc:65-87, test_csv_input_multiload.cc:70-92,
// test_save2gpu_sift.cc:91-100, test_subsequence_search_csv_input.cc:64-92),
// and prints every result slot as "tag query slot id count" for the caller to
// compare with the oracle.
//
//   legacy_test <mode> <data.csv> [query file]
//   modes: sift, multiload, tweets, tweets_multiload, subseq, multirange,
//          sequence, mt, binary_rows
#include <genie/original/interface.h>
#include <genie/utility/Timing.h>
#include <genie/utility/cuda_macros.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace genie::original;
using namespace genie::table;
using namespace genie::utility;

static int failures = 0;
#define CHECK(c)                                                        \
    do {                                                                \
        if (!(c)) {                                                     \
            std::printf("CHECK failed at line %d: %s\n", __LINE__, #c); \
            ++failures;                                                 \
        }                                                               \
    } while (0)

static void print(const char *tag, const std::vector<int> &ids, const std::vector<int> &counts, int k) {
    for (size_t i = 0; i < ids.size(); ++i)
        std::printf("%s %d %d %d %d\n", tag, (int)(i / k), (int)(i % k), ids[i], counts[i]);
}

// The configuration of the reference's sift_20 tests.
static GPUGenie_Config sift_config(std::vector<std::vector<int> > *data, std::vector<std::vector<int> > *queries) {
    GPUGenie_Config c;
    c.dim = 5;
    c.count_threshold = 14;
    c.num_of_topk = 5;
    c.hashtable_size = 14 * c.num_of_topk * 1.5f;
    c.query_radius = 0;
    c.use_device = 0;
    c.use_adaptive_range = false;
    c.selectivity = 0.0f;
    c.query_points = queries;
    c.data_points = data;
    c.use_load_balance = false;
    c.posting_list_max_length = 6400;
    c.multiplier = 1.5f;
    c.use_multirange = false;
    c.data_type = 0;
    c.search_type = 0;
    c.max_data_size = 0;
    c.num_of_queries = 3;
    return c;
}

static void check_sift_goldens(const std::vector<int> &r, const std::vector<int> &c) {
    CHECK(r.size() == 15);
    CHECK(r[0] == 0 && c[0] == 5);
    CHECK(r[1] == 4 && c[1] == 2);
    CHECK(r[5] == 1 && c[5] == 5);
    CHECK(r[10] == 2 && c[10] == 5);
}

int main(int argc, char **argv) {
    if (argc < 3) {
        std::printf("usage: legacy_test <mode> <data.csv> [query file]\n");
        return 2;
    }
    const std::string mode = argv[1];
    const char *data_file = argv[2];
    std::vector<std::vector<int> > data, queries;
    std::vector<attr_t> multirange;
    std::vector<int> result, result_count;
    read_file(data, data_file, -1);
    GPUGenie_Config config = sift_config(&data, &queries);
    read_file(queries, data_file, config.num_of_queries);
    inv_table *table = nullptr;
    try {
        if (mode == "sift" || mode == "multiload") {
            if (mode == "multiload") config.max_data_size = 10;
            config.save_to_gpu = true;
            init_genie(config);
            preprocess_for_knn_csv(config, table);
            CHECK(table[0].get_total_num_of_table() == (mode == "multiload" ? 2 : 1));
            std::vector<int> &inv = *table[0].inv();
            CHECK(inv[0] == 8 && inv[1] == 9 && inv[2] == 7 && inv[3] == 0 && inv[4] == 2 && inv[5] == 4);
            // the device copy of the postings (test_save2gpu_sift.cc:91-100)
            std::vector<int> dev(inv.size());
            cudaCheckErrors(cudaMemcpy(dev.data(), table->d_inv_p, sizeof(int) * dev.size(), cudaMemcpyDeviceToHost));
            CHECK(dev == inv);
            knn_search_after_preprocess(config, table, result, result_count);
            check_sift_goldens(result, result_count);
            print(mode.c_str(), result, result_count, config.num_of_topk);
            // a second search over the same tables gives the same answer (test_multiple_search.cc)
            std::vector<int> again, again_count;
            knn_search_after_preprocess(config, table, again, again_count);
            CHECK(again == result && again_count == result_count);
        } else if (mode == "tweets" || mode == "tweets_multiload") {
            config.dim = 14;
            config.search_type = 1;
            config.max_data_size = mode == "tweets_multiload" ? 10 : 0;
            init_genie(config);
            preprocess_for_knn_csv(config, table);
            std::vector<int> &inv = *table[0].inv();
            if (mode == "tweets") {
                CHECK(inv[0] == 0 && inv[1] == 11 && inv[2] == 0 && inv[3] == 11 && inv[4] == 0 && inv[5] == 11);
            } else {          // the first of two tables (test_csv_multiload_tweets.cc:64-73)
                CHECK(table[0].get_total_num_of_table() == 2);
                CHECK(inv[0] == 0 && inv[1] == 0 && inv[2] == 0 && inv[3] == 0 && inv[4] == 0 && inv[5] == 7);
            }
            knn_search_after_preprocess(config, table, result, result_count);
            print(mode.c_str(), result, result_count, config.num_of_topk);
        } else if (mode == "subseq") {
            config.search_type = 1;
            config.use_subsequence_search = true;
            init_genie(config);
            preprocess_for_knn_csv(config, table);
            std::vector<int> &inv = *table[0].inv();
            CHECK(inv[0] == 4 && inv[1] == 11 && inv[2] == 36 && inv[3] == 43 && inv[4] == 52 && inv[5] == 67);
            knn_search_after_preprocess(config, table, result, result_count);
            const int bits = (int)table[0]._shift_bits_subsequence();
            CHECK(bits == 3);
            std::vector<int> row, offset;
            get_rowID_offset(result, row, offset, (unsigned)bits);
            CHECK(row[0] == 0 && offset[0] == 0 && result_count[0] == 5);
            CHECK(row[1] == 4 && result_count[1] == 2);
            CHECK(row[5] == 1 && result_count[5] == 5);
            CHECK(row[10] == 2 && result_count[10] == 5);
            print("subseq", result, result_count, config.num_of_topk);
        } else if (mode == "multirange") {
            // example_sift.cc: multirange queries from a qid,dim,value,sel,weight file
            if (argc < 4) return 2;
            config.dim = 128;
            config.num_of_topk = 10;
            config.num_of_queries = 100;
            config.query_radius = 1;
            config.use_adaptive_range = true;
            config.selectivity = 0.2f;
            config.use_multirange = true;
            read_query(multirange, argv[3], -1);
            config.multirange_query_points = &multirange;
            init_genie(config);
            knn_search(result, result_count, config);
            CHECK(result.size() == 1000);
            print("multirange", result, result_count, config.num_of_topk);
        } else if (mode == "sequence") {
            config.search_type = 2;
            config.num_of_topk = 5;
            config.num_of_queries = 3;
            config.data_gram_length = 3;
            init_genie(config);
            knn_search(result, result_count, config);
            CHECK(config.dim == 1);
            print("sequence", result, result_count, config.num_of_topk);
        } else if (mode == "mt") {
            // two tables (the first and last ten rows) searched at once
            std::vector<std::vector<int> > a(data.begin(), data.begin() + 10), b(data.begin() + 10, data.end());
            inv_table t0, t1;
            init_genie(config);
            load_table(t0, a, config);
            load_table(t1, b, config);
            std::vector<genie::query::Query> q0, q1;
            load_query(t0, q0, config);
            load_query(t1, q1, config);
            std::vector<inv_table *> tables{&t0, &t1};
            std::vector<std::vector<genie::query::Query> > qs{q0, q1};
            std::vector<std::vector<int> > ids, counts;
            std::vector<GPUGenie_Config> configs{config, config};
            knn_search_MT(tables, qs, ids, counts, configs);
            CHECK(ids.size() == 2 && counts.size() == 2);
            print("mt0", ids[0], counts[0], config.num_of_topk);
            print("mt1", ids[1], counts[1], config.num_of_topk);
        } else if (mode == "binary_rows") {
            // the (data, index) array form of load_table / load_table_bijectMap
            std::vector<int> flat;
            std::vector<unsigned int> index;
            for (const auto &r : data) {
                index.push_back((unsigned)flat.size());
                flat.insert(flat.end(), r.begin(), r.end());
            }
            inv_table t, tb;
            init_genie(config);
            load_table(t, flat.data(), (unsigned)flat.size(), index.data(), (unsigned)index.size(), config);
            std::vector<int> &inv = *t.inv();
            CHECK(inv[0] == 8 && inv[1] == 9 && inv[2] == 7);
            std::vector<genie::query::Query> qs;
            load_query(t, qs, config);
            knn_search(t, qs, result, result_count, config);
            check_sift_goldens(result, result_count);
            print("binary_rows", result, result_count, config.num_of_topk);
            load_table_bijectMap(tb, flat.data(), (unsigned)flat.size(), index.data(), (unsigned)index.size(), config);
            CHECK(tb.i_size() == (int)data.size() && tb.m_size() == 1);
        } else {
            std::printf("unknown mode %s\n", mode.c_str());
            return 2;
        }
    } catch (std::exception &e) {
        std::printf("exception: %s\n", e.what());
        ++failures;
    }
    delete[] table;
    std::printf(failures ? "FAILED %d\n" : "OK\n", failures);
    return failures ? 1 : 0;
}
