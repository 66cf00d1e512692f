// shim_test.cc -- exercises the C++ interface (<genie/genie.h>) the way the
// reference's examples and tests do (example_1st_level_interface.cc,
// example_2nd_level_interface.cc, test_csv_input_sift_data.cc).
//
//   shim_test host <dir>                    host-only checks (no GPU needed)
//   shim_test gpu <table.csv> <query.csv> <dir>
//
// The gpu mode prints one line per result row, "<case> <q> <j> <id> <count>",
// for the harness to compare with the oracle, and exits non-zero on a failed
// check of its own.
#include <genie/genie.h>

#include <cstdio>
#include <fstream>
#include <iostream>
#include <memory>
#include <string>

using namespace genie;

static int failures = 0;
#define CHECK(cond)                                                          \
    do {                                                                     \
        if (!(cond)) {                                                       \
            std::cerr << "check failed: " #cond " (line " << __LINE__ << ")\n"; \
            ++failures;                                                      \
        }                                                                    \
    } while (0)

template <class E, class F>
static bool throws(F f) {
    try {
        f();
    } catch (const E &) {
        return true;
    } catch (...) {
        return false;
    }
    return false;
}

static void print(const char *tag, const SearchResult &r, int k) {
    for (size_t i = 0; i < r.first.size(); ++i)
        std::cout << tag << " " << i / k << " " << i % k << " " << r.first[i] << " " << r.second[i] << "\n";
}

static int host_checks(const std::string &dir) {
    // configuration errors are InvalidConfigurationException
    CHECK(throws<exception::InvalidConfigurationException>([] { Config().SetNumOfQueries(3).Validate(); }));
    CHECK(throws<exception::InvalidConfigurationException>([] { Config().SetK(3).Validate(); }));
    CHECK(!throws<std::exception>([] { Config().SetK(3).SetNumOfQueries(2).Validate(); }));
    Config c = Config().SetK(7).SetQueryRange(2).SetNumOfQueries(4).SetGpuId(0);
    CHECK(c.GetK() == 7 && c.GetQueryRange() == 2 && c.GetNumOfQueries() == 4 && c.IsQueryRangeSet());
    // configuration file
    {
        std::ofstream f(dir + "/cfg.txt");
        f << "k 9\nnum_of_queries 3\nquery_range 1\n";
    }
    Config lf;
    lf.LoadFromFile(dir + "/cfg.txt");
    CHECK(lf.GetK() == 9 && lf.GetNumOfQueries() == 3 && lf.GetQueryRange() == 1);
    // CSV rows split on commas and blanks
    {
        std::ofstream f(dir + "/t.csv");
        f << "1,2,3\n4, 5 ,6\n7 8 9\n";
    }
    TableData td = LoadTableDataFromCsv(dir + "/t.csv");
    CHECK(td.size() == 3 && td[1][1] == 5 && td[2][2] == 9);
    CHECK(LoadTableDataFromCsv(dir + "/missing.csv").empty());
    // a status code of the C ABI becomes the matching exception type
    CHECK(throws<exception::gpu_runtime_error>([] { exception::throw_on_status(3); }));
    CHECK(throws<exception::NotImplementedException>([] { exception::throw_on_status(4); }));
    CHECK(throws<exception::cpu_runtime_error>([] { exception::throw_on_status(1); }));
    CHECK(throws<exception::gpu_bad_alloc>([] { exception::throw_on_status(8); }));
    std::cout << (failures ? "FAIL" : "OK") << std::endl;
    return failures ? 1 : 0;
}

static int gpu_checks(const std::string &table_csv, const std::string &query_csv, const std::string &dir) {
    // first level: Search (test_csv_input_sift_data.cc:65-87)
    Config config = Config().SetK(5).SetNumOfQueries(5);
    std::shared_ptr<ExecutionPolicy> policy = MakePolicy(config);
    SearchResult r1 = Search(policy, table_csv, query_csv);
    print("search", r1, 5);
    CHECK(r1.first.size() == 25);
    CHECK(r1.first[0] == 0 && r1.second[0] == 5 && r1.first[1] == 4 && r1.second[1] == 2);
    CHECK(r1.first[5] == 1 && r1.second[5] == 5);
    CHECK(r1.first[10] == 2 && r1.second[10] == 5);

    // second level: the same through BuildTable / BuildQuery / Match
    TableData table_data = LoadTableDataFromCsv(table_csv);
    QueryData query_data = LoadQueryDataFromCsv(query_csv, policy);
    CHECK(query_data.size() == 5);
    std::shared_ptr<table::inv_table> table = BuildTable(policy, table_data);
    CHECK(table->i_size() == (int)table_data.size() && table->m_size() == (int)table_data[0].size());
    std::vector<query::Query> queries = BuildQuery(policy, table, query_data);
    SearchResult r2 = Match(policy, table, queries);
    CHECK(r2 == r1);

    // binary save / load gives the same answers
    SaveTableToBinary(dir + "/table.bin", table);
    std::shared_ptr<table::inv_table> loaded = LoadTableFromBinary(dir + "/table.bin");
    CHECK(*loaded->inv() == *table->inv());
    std::vector<query::Query> q2 = BuildQuery(policy, loaded, query_data);
    CHECK(Match(policy, loaded, q2) == r1);

    // several tables at once: results of table t follow those of table t-1
    std::vector<std::shared_ptr<const table::inv_table> > tables{table, loaded};
    std::vector<std::vector<query::Query> > qs{queries, q2};
    SearchResult rm = policy->Match(tables, qs);
    CHECK(rm.first.size() == 50);
    CHECK(std::vector<int>(rm.first.begin(), rm.first.begin() + 25) == r1.first);
    CHECK(std::vector<int>(rm.first.begin() + 25, rm.first.end()) == r1.first);

    // query range: items match [v-1, v+1]
    std::shared_ptr<ExecutionPolicy> ranged = MakePolicy(Config().SetK(5).SetNumOfQueries(5).SetQueryRange(1));
    SearchResult r3 = Match(ranged, table, BuildQuery(ranged, table, query_data));
    print("range1", r3, 5);

    // spans of a built query are the reference's Query::build spans
    query::Query one = queries[0];
    one.build();
    std::vector<query::Query::dim> dims;
    const int nd = one.dump(dims);
    CHECK(nd > 0 && dims[0].end_pos > dims[0].start_pos);

    // errors
    CHECK(throws<exception::cpu_runtime_error>([&] { BuildTable(policy, TableData()); }));
    CHECK(throws<exception::cpu_runtime_error>([&] { Match(policy, table, std::vector<query::Query>()); }));
    CHECK(throws<exception::cpu_runtime_error>([&] { LoadTableFromBinary(dir + "/missing.bin"); }));
    std::cout << (failures ? "FAIL" : "OK") << std::endl;
    return failures ? 1 : 0;
}

int main(int argc, char **argv) {
    const std::string mode = argc > 1 ? argv[1] : "";
    try {
        if (mode == "host" && argc > 2) return host_checks(argv[2]);
        if (mode == "gpu" && argc > 4) return gpu_checks(argv[2], argv[3], argv[4]);
    } catch (const std::exception &e) {
        std::cerr << "uncaught: " << e.what() << std::endl;
        return 2;
    }
    std::cerr << "usage: shim_test host <dir> | shim_test gpu <table.csv> <query.csv> <dir>\n";
    return 2;
}
