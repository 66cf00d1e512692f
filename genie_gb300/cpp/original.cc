// original.cc -- the reference's legacy C++ interface (<genie/original/
// interface.h>, <genie/utility/FileReader.h>, <genie/utility/Logger.h>,
// <genie/utility/Timing.h>) over the C ABI (<genie_gb300.h>).
//
// Reference behaviour kept (file:line in the reference tree):
//   preprocess_for_knn_csv: topk *= num_of_iteration; one table, or multiload
//     tables of max_data_size rows, the last full chunk and the remainder
//     split in two halves                   original/interface.cc:150-279
//   knn_search_after_preprocess: queries loaded per table, ids of table t
//     offset by the rows of tables < t, per-query merge of the tables' slots
//     [q*topk + topk/iter*(iter-1), (q+1)*topk), first topk/iter kept
//                                           original/interface.cc:114-149, 281-312
//   load_table: column j of the rows is dim j   original/interface.cc:313-353
//   load_table_bijectMap: every value of row r lists r (or, for subsequence
//     search, r << bits | offset)           original/interface.cc:621-676
//   load_table_sequence: grams of the values reduced to 0.., each gram's
//     k-th repeat in a row a distinct value (k capped at 63)
//                                           original/interface.cc:678-757, inv_list.cc:87-148
//   load_query_singlerange: item j of row i is dim j (dim 0 for bijectMap)
//     in [v-r, v+r], weight 1, order j     original/interface.cc:473-517
//   load_query_multirange: items grouped by qid in qid order, at most
//     num_of_queries queries, adaptive ranges applied
//                                           original/interface.cc:428-470
//   load_query_sequence                     original/interface.cc:519-616
//   knn_search(config): data_type 0 only, every error mapped to the GENIE
//     exception types                       original/interface.cc:766-818
//   sequence_to_gram, sequence_reduce_to_ground, get_rowID_offset
//                                           original/interface.cc:914-989
//   read_file / read_query: tokens split on ',' and blanks
//                                           utility/FileReader.cc:54-176
// Deliberate differences: results are sorted (count desc, id asc) and the
// multiload merge breaks ties by id (the reference's quicksort leaves them
// in any order); the old-format read_query puts item i of a row on dim i
// (the reference passes the row number as the dim, FileReader.cc:178); the
// hash-table and load-balance settings are accepted and not needed.
#include <genie/original/interface.h>
#include <genie/utility/Timing.h>

#include "../../include/genie_gb300.h"
#include "flat_queries.h"

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <new>
#include <sstream>
#include <string>
#include <unordered_map>

using genie::exception::throw_on_status;
using genie::query::Query;
using genie::table::inv_table;

// ---------------------------------------------------------------- Timing

unsigned long long getTime() {
    return (unsigned long long)std::chrono::duration_cast<std::chrono::microseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

double getInterval(unsigned long long start, unsigned long long stop) { return (double)(stop - start) / 1000.0; }

// ---------------------------------------------------------------- Logger

namespace genie {
namespace utility {

namespace {
int g_log_level = Logger::INFO;
std::string g_log_name;
}  // namespace

void Logger::exit(void) { std::fflush(stderr); }

int Logger::log(int level, const char *fmt, ...) {
    if (level > g_log_level || level <= NONE) return 0;
    va_list ap;
    va_start(ap, fmt);
    const int n = std::vfprintf(stderr, fmt, ap);
    va_end(ap);
    std::fputc('\n', stderr);
    return n;
}

void Logger::set_level(int level) { g_log_level = level; }
int Logger::get_level() { return g_log_level; }
void Logger::set_logfile_name(const char *name) { g_log_name = name ? name : ""; }
const char *Logger::get_logfile_name() { return g_log_name.c_str(); }

// ---------------------------------------------------------------- FileReader

namespace {
std::vector<std::string> tokens(const std::string &line) {
    std::vector<std::string> out;
    std::string cur;
    for (char c : line) {
        if (c == ',' || c == ' ' || c == '\t' || c == '\r' || c == '\n') {
            if (!cur.empty()) out.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}
}  // namespace

void read_file(std::vector<std::vector<int> > &dest, const char *fname, int num) {
    dest.clear();
    std::ifstream in(fname);
    std::string line;
    while ((num < 0 || (int)dest.size() < num) && std::getline(in, line)) {
        std::vector<int> row;
        for (const std::string &t : tokens(line)) row.push_back(std::atoi(t.c_str()));
        dest.push_back(std::move(row));
    }
    Logger::log(Logger::DEBUG, "%d rows are read into memory!", (int)dest.size());
}

void read_query(std::vector<attr_t> &data, const char *file_name, int num) {
    data.clear();
    std::ifstream in(file_name);
    std::string line;
    int left = num;
    while (left != 0 && std::getline(in, line)) {
        const std::vector<std::string> t = tokens(line);
        if (t.size() != GPUGENIE_QUERY_NUM_OF_FIELDS) continue;
        attr_t a;
        a.qid = std::atoi(t[GPUGENIE_QUERY_QID_INDEX].c_str());
        a.dim = std::atoi(t[GPUGENIE_QUERY_DIM_INDEX].c_str());
        a.value = std::atoi(t[GPUGENIE_QUERY_VALUE_INDEX].c_str());
        a.sel = (float)std::atof(t[GPUGENIE_QUERY_SELECTIVITY_INDEX].c_str());
        a.weight = (float)std::atof(t[GPUGENIE_QUERY_WEIGHT_INDEX].c_str());
        data.push_back(a);
        --left;
    }
    Logger::log(Logger::DEBUG, "%d attributes are loaded.", (int)data.size());
}

void read_query(inv_table &table, const char *fname, std::vector<Query> &queries, int num_of_queries,
                int num_of_query_dims, int radius, int topk, float selectivity) {
    queries.clear();
    std::ifstream in(fname);
    std::string line;
    int j = 0;
    while (j < num_of_queries && std::getline(in, line)) {
        const std::vector<std::string> t = tokens(line);
        Query q(table, j);
        for (size_t i = 0; i < t.size() && (int)i < num_of_query_dims; ++i) {
            const int v = std::atoi(t[i].c_str());
            q.attr((int)i, v - radius < 0 ? 0 : v - radius, v + radius, 1.0f, (int)i);
        }
        q.topk(topk);
        if (selectivity > 0.0f) {
            q.selectivity(selectivity);
            q.apply_adaptive_query_range();
        }
        queries.push_back(q);
        ++j;
    }
}

}  // namespace utility
}  // namespace genie

// ---------------------------------------------------------------- original

namespace genie {
namespace original {

namespace {

using Rows = std::vector<std::vector<int> >;

// Row r of a (data, index) array set: data[index[r] - index[0] ..).
Rows rows_of(const int *data, unsigned int item_num, const unsigned int *index, unsigned int row_num) {
    Rows rows(row_num);
    if (row_num == 0) return rows;
    for (unsigned int r = 0; r < row_num; ++r) {
        const size_t a = index[r] - index[0];
        const size_t b = r + 1 < row_num ? index[r + 1] - index[0] : item_num;
        if (b < a || b > item_num) throw exception::cpu_runtime_error("row index outside the data array");
        rows[r].assign(data + a, data + b);
    }
    return rows;
}

void flatten(const Rows &rows, std::vector<int32_t> &vals, std::vector<int64_t> &off) {
    off.assign(1, 0);
    vals.clear();
    for (const auto &r : rows) {
        vals.insert(vals.end(), r.begin(), r.end());
        off.push_back((int64_t)vals.size());
    }
}

// The one table of a configuration's search type over `rows`.
void load_rows(inv_table &table, Rows &rows, GPUGenie_Config &config) {
    switch (config.search_type) {
        case 0: load_table(table, rows, config); break;
        case 1: load_table_bijectMap(table, rows, config); break;
        case 2: load_table_sequence(table, rows, config); break;
        default: throw exception::cpu_runtime_error("Unrecognised search type!");
    }
}

// Gram values of one row, each value's k-th repeat marked in its low `bits`
// bits: the table side keeps repeats past the cap at the cap
// (inv_list.cc:107-121), the query side drops them
// (original/interface.cc:552-566).
std::vector<int> mark_repeats(const std::vector<int> &grams, int bits, bool keep_capped) {
    std::unordered_map<int, int> seen;
    std::vector<int> out;
    const int cap = (1 << bits) - 1;
    for (int g : grams) {
        auto it = seen.find(g);
        if (it == seen.end()) {
            seen.emplace(g, 0);
            out.push_back((int)((unsigned)g << bits));
        } else if (it->second < cap) {
            ++it->second;
            out.push_back((int)(((unsigned)g << bits) + (unsigned)it->second));
        } else if (keep_capped) {
            out.push_back((int)(((unsigned)g << bits) + (unsigned)cap));
        }
    }
    return out;
}

// Result ids of a table as global ids: the rows of the tables before it
// (for a subsequence table, rows << bits, so that offsets stay in place).
int64_t id_span(inv_table &t) {
    const int64_t rows = t.i_size();
    return rows << t._shift_bits_subsequence();
}

}  // namespace

bool preprocess_for_knn_csv(GPUGenie_Config &config, inv_table *&_table) {
    config.num_of_topk = (int)(config.num_of_iteration * (unsigned)config.num_of_topk);
    if (!config.data_points || config.data_points->empty()) throw exception::cpu_runtime_error("no data input!");
    Rows &data = *config.data_points;
    const size_t n = data.size();
    if (config.max_data_size >= n || config.max_data_size == 0) {
        _table = new inv_table[1];
        _table[0].set_table_index(0);
        _table[0].set_total_num_of_table(1);
        load_rows(_table[0], data, config);
        return true;
    }
    if (config.compression != compression::NO_COMPRESSION)
        throw exception::cpu_runtime_error("Compression for multiple tables to yet supported");
    const size_t m = config.max_data_size;
    size_t table_num, full;
    if (n % m == 0) {
        table_num = n / m;
        full = table_num;
    } else {          // the last full chunk and the remainder, halved
        table_num = n / m + 1;
        full = table_num - 2;
    }
    _table = new inv_table[table_num];
    std::vector<std::pair<size_t, size_t> > parts;
    for (size_t i = 0; i < full; ++i) parts.emplace_back(i * m, (i + 1) * m);
    if (table_num != full) {
        const size_t a = full * m, half = (n - a) / 2;
        parts.emplace_back(a, a + half);
        parts.emplace_back(a + half, n);
    }
    for (size_t i = 0; i < table_num; ++i) {
        Rows part(data.begin() + (long)parts[i].first, data.begin() + (long)parts[i].second);
        _table[i].set_table_index((int)i);
        _table[i].set_total_num_of_table((int)table_num);
        load_rows(_table[i], part, config);
    }
    return true;
}

void knn_search_after_preprocess(GPUGenie_Config &config, inv_table *&_table, std::vector<int> &result,
                                 std::vector<int> &result_count) {
    const int table_num = _table[0].get_total_num_of_table();
    std::vector<std::vector<int> > ids(table_num), counts(table_num);
    std::vector<Query> queries;
    int64_t offset = 0;
    for (int t = 0; t < table_num; ++t) {
        queries.clear();
        load_query(_table[t], queries, config);
        knn_search(_table[t], queries, ids[t], counts[t], config);
        if (t > 0)
            for (int &v : ids[t]) v = (int)(v + offset);
        offset += id_span(_table[t]);
    }
    // per-query merge of the tables' slots (merge_knn_results_from_multiload)
    const int topk = config.num_of_topk;
    const int iter = (int)std::max(1u, config.num_of_iteration);
    const int each = topk / iter;
    result.clear();
    result_count.clear();
    for (size_t q = 0; q < queries.size(); ++q) {
        std::vector<std::pair<int, int> > cand;   // (count, id)
        for (int t = 0; t < table_num; ++t) {
            const size_t a = q * (size_t)topk + (size_t)each * (size_t)(iter - 1), b = (q + 1) * (size_t)topk;
            for (size_t j = a; j < b && j < ids[t].size(); ++j) cand.emplace_back(counts[t][j], ids[t][j]);
        }
        std::stable_sort(cand.begin(), cand.end(), [](const std::pair<int, int> &x, const std::pair<int, int> &y) {
            return x.first != y.first ? x.first > y.first : (x.first > 0 && x.second < y.second);
        });
        for (int j = 0; j < each; ++j) {
            const bool have = j < (int)cand.size() && cand[j].first > 0;     // else a (0, 0) pad
            result.push_back(have ? cand[j].second : 0);
            result_count.push_back(have ? cand[j].first : 0);
        }
    }
}

void knn_search(inv_table &table, std::vector<Query> &queries, std::vector<int> &h_topk,
                std::vector<int> &h_topk_count, GPUGenie_Config &config) {
    (void)config;
    h_topk.clear();
    h_topk_count.clear();
    if (queries.empty()) return;
    FlatQueries f(queries);
    const genie_queries g = f.view();
    std::vector<uint32_t> ids((size_t)std::max<int64_t>(1, f.total_k)), cnt(ids.size());
    throw_on_status(genie_search(table.handle(), &g, ids.data(), cnt.data(), nullptr));
    h_topk.assign(ids.begin(), ids.begin() + f.total_k);
    h_topk_count.assign(cnt.begin(), cnt.begin() + f.total_k);
}

void knn_search_MT(std::vector<inv_table *> &tables, std::vector<std::vector<Query> > &queries,
                   std::vector<std::vector<int> > &h_topk, std::vector<std::vector<int> > &h_topk_count,
                   std::vector<GPUGenie_Config> &config) {
    (void)config;
    if (tables.size() != queries.size()) throw exception::cpu_runtime_error("one query list per table is needed");
    std::vector<FlatQueries> fs;
    fs.reserve(tables.size());
    std::vector<genie_queries> gs;
    std::vector<genie_index *> ixs;
    std::vector<int64_t> base{0};
    for (size_t t = 0; t < tables.size(); ++t) {
        fs.emplace_back(queries[t]);
        base.push_back(base.back() + fs.back().total_k);
    }
    for (size_t t = 0; t < tables.size(); ++t) {
        gs.push_back(fs[t].view());
        ixs.push_back(tables[t]->handle());
    }
    std::vector<uint32_t> ids((size_t)std::max<int64_t>(1, base.back())), cnt(ids.size());
    throw_on_status(genie_search_multi(ixs.data(), gs.data(), (int32_t)ixs.size(), ids.data(), cnt.data(), nullptr));
    h_topk.resize(tables.size());
    h_topk_count.resize(tables.size());
    for (size_t t = 0; t < tables.size(); ++t) {
        h_topk[t].assign(ids.begin() + base[t], ids.begin() + base[t + 1]);
        h_topk_count[t].assign(cnt.begin() + base[t], cnt.begin() + base[t + 1]);
    }
}

void knn_search_for_csv_data(std::vector<int> &result, std::vector<int> &result_count, GPUGenie_Config &config) {
    inv_table *table = nullptr;
    preprocess_for_knn_csv(config, table);
    try {
        knn_search_after_preprocess(config, table, result, result_count);
    } catch (...) {
        delete[] table;
        throw;
    }
    delete[] table;
}

void knn_search(std::vector<int> &result, GPUGenie_Config &config) {
    std::vector<int> result_count;
    knn_search(result, result_count, config);
}

void knn_search(std::vector<int> &result, std::vector<int> &result_count, GPUGenie_Config &config) {
    try {
        switch (config.data_type) {
            case 0: knn_search_for_csv_data(result, result_count, config); break;
            case 1: throw exception::cpu_runtime_error("Binary .dat data_type no longer supported\n");
            default: throw exception::cpu_runtime_error("Please check data type in config\n");
        }
    } catch (exception::gpu_bad_alloc &) {
        throw;
    } catch (exception::gpu_runtime_error &) {
        throw;
    } catch (exception::cpu_runtime_error &) {
        throw;
    } catch (exception::cpu_bad_alloc &) {
        throw;
    } catch (exception::InvalidConfigurationException &) {
        throw;
    } catch (exception::NotImplementedException &) {
        throw;
    } catch (std::bad_alloc &e) {
        throw exception::cpu_bad_alloc(e.what());
    } catch (std::exception &e) {
        throw exception::cpu_runtime_error(e.what());
    }
}

void load_table(inv_table &table, std::vector<std::vector<int> > &data_points, GPUGenie_Config &config) {
    if (data_points.empty() || data_points[0].empty()) throw exception::cpu_runtime_error("no data input!");
    const size_t n = data_points.size(), d = data_points[0].size();
    std::vector<int32_t> flat;
    flat.reserve(n * d);
    for (const auto &row : data_points) {
        if (row.size() < d) throw exception::cpu_runtime_error("a row is shorter than the first row");
        flat.insert(flat.end(), row.begin(), row.begin() + (long)d);
    }
    genie_index *ix = nullptr;
    throw_on_status(genie_index_create(flat.data(), (int64_t)n, (int32_t)d, &ix));
    table.adopt(ix);
    table.is_stored_in_gpu = true;      // every table lives on the device (save_to_gpu is implied)
    (void)config;
}

void load_table(inv_table &table, int *data, unsigned int item_num, unsigned int *index, unsigned int row_num,
                GPUGenie_Config &config) {
    if (!data || !index || row_num == 0) throw exception::cpu_runtime_error("no data input!");
    const unsigned int width = row_num == 1 ? item_num : index[1] - index[0];
    Rows rows(row_num);
    for (unsigned int r = 0; r < row_num; ++r) {
        const size_t a = index[r] - index[0];
        if (a + width > item_num) throw exception::cpu_runtime_error("row index outside the data array");
        rows[r].assign(data + a, data + a + width);
    }
    load_table(table, rows, config);
}

void load_table_bijectMap(inv_table &table, std::vector<std::vector<int> > &data_points, GPUGenie_Config &config) {
    std::vector<int32_t> vals;
    std::vector<int64_t> off;
    flatten(data_points, vals, off);
    if (vals.empty()) throw exception::cpu_runtime_error("no data input!");
    genie_index *ix = nullptr;
    if (config.use_subsequence_search)
        throw_on_status(genie_index_create_subsequence(vals.data(), off.data(), (int64_t)data_points.size(), &ix));
    else
        throw_on_status(genie_index_create_bag(vals.data(), off.data(), (int64_t)data_points.size(), &ix));
    table.adopt(ix);
    table.is_stored_in_gpu = true;
}

void load_table_bijectMap(inv_table &table, int *data, unsigned int item_num, unsigned int *index,
                          unsigned int row_num, GPUGenie_Config &config) {
    if (!data || !index || row_num == 0) throw exception::cpu_runtime_error("no data input!");
    Rows rows = rows_of(data, item_num, index, row_num);
    load_table_bijectMap(table, rows, config);
}

void load_table_sequence(inv_table &table, std::vector<std::vector<int> > &data_points, GPUGenie_Config &config) {
    int mn = 0, mx = 0;
    Rows ground, grams;
    sequence_reduce_to_ground(data_points, ground, mn, mx);
    table.set_min_value_sequence(mn);
    table.set_max_value_sequence(mx);
    sequence_to_gram(ground, grams, mx - mn, config.data_gram_length);
    table.set_gram_length_sequence(config.data_gram_length);
    table.shift_bits_sequence = 6;
    config.dim = 1;
    // every marked gram value gets a value id in order of first appearance
    std::unordered_map<int, int> id_of;
    Rows valued(grams.size());
    for (size_t r = 0; r < grams.size(); ++r)
        for (int v : mark_repeats(grams[r], table.shift_bits_sequence, true)) {
            auto it = id_of.find(v);
            if (it == id_of.end()) it = id_of.emplace(v, (int)id_of.size()).first;
            valued[r].push_back(it->second);
        }
    std::vector<std::pair<int, int> > dict(id_of.begin(), id_of.end());
    std::sort(dict.begin(), dict.end());
    table.set_distinct_sequence(std::move(dict));
    std::vector<int32_t> vals;
    std::vector<int64_t> off;
    flatten(valued, vals, off);
    if (vals.empty()) throw exception::cpu_runtime_error("no data input!");
    genie_index *ix = nullptr;
    throw_on_status(genie_index_create_bag(vals.data(), off.data(), (int64_t)valued.size(), &ix));
    table.adopt(ix);
    table.is_stored_in_gpu = true;
}

void load_query(inv_table &table, std::vector<Query> &queries, GPUGenie_Config &config) {
    if (config.search_type == 2) {
        load_query_sequence(table, queries, config);
        return;
    }
    if (config.use_multirange) load_query_multirange(table, queries, config);
    else load_query_singlerange(table, queries, config);
}

void load_query_multirange(inv_table &table, std::vector<Query> &queries, GPUGenie_Config &config) {
    queries.clear();
    if (!config.multirange_query_points) throw exception::cpu_runtime_error("no multirange query input!");
    std::map<int, Query> by_qid;
    for (const utility::attr_t &a : *config.multirange_query_points) {
        auto it = by_qid.find(a.qid);
        if (it == by_qid.end()) {
            Query q(table, a.qid);
            q.topk(config.num_of_topk);
            if (config.selectivity > 0.0f) q.selectivity(config.selectivity);
            it = by_qid.emplace(a.qid, q).first;
        }
        it->second.attr(a.dim, a.value, a.weight, a.sel, it->second.count_ranges());
    }
    for (auto &kv : by_qid) {
        if ((int)queries.size() >= config.num_of_queries) break;
        kv.second.apply_adaptive_query_range();
        queries.push_back(kv.second);
    }
}

void load_query_singlerange(inv_table &table, std::vector<Query> &queries, GPUGenie_Config &config) {
    if (!config.query_points) throw exception::cpu_runtime_error("no query input!");
    const Rows &qp = *config.query_points;
    const int r = config.query_radius;
    for (size_t i = 0; i < qp.size(); ++i) {
        Query q(table, (int)i);
        for (size_t j = 0; j < qp[i].size() && (config.search_type == 1 || (int)j < config.dim); ++j) {
            const int v = qp[i][j];
            q.attr(config.search_type == 1 ? 0 : (int)j, v - r, v + r, (float)GPUGENIE_DEFAULT_WEIGHT, (int)j);
        }
        q.topk(config.num_of_topk);
        q.selectivity(config.selectivity);
        if (config.use_adaptive_range) q.apply_adaptive_query_range();
        queries.push_back(q);
    }
}

void load_query_sequence(inv_table &table, std::vector<Query> &queries, GPUGenie_Config &config) {
    if (!config.query_points) throw exception::cpu_runtime_error("no query input!");
    const int mn = table.get_min_value_sequence(), mx = table.get_max_value_sequence();
    Rows ground;
    for (const auto &row : *config.query_points) {
        std::vector<int> line;
        for (int v : row)
            if (v >= mn && v <= mx) line.push_back(v - mn);
        ground.push_back(std::move(line));
    }
    Rows grams;
    sequence_to_gram(ground, grams, mx - mn, table.get_gram_length_sequence());
    const auto &dict = table.distinct_sequence();
    for (size_t i = 0; i < grams.size(); ++i) {
        Query q(table, (int)i);
        for (int v : mark_repeats(grams[i], table.shift_bits_sequence, false)) {
            if (v < 0) continue;
            auto it = std::lower_bound(dict.begin(), dict.end(), std::make_pair(v, -1));
            if (it == dict.end() || it->first != v) continue;      // a gram no row holds
            q.attr(0, it->second, it->second, (float)GPUGENIE_DEFAULT_WEIGHT, 0);
        }
        q.topk(config.num_of_topk);
        queries.push_back(q);
    }
}

void sequence_to_gram(std::vector<std::vector<int> > &sequences, std::vector<std::vector<int> > &gram_data,
                      int max_value, int gram_length) {
    const int base = max_value + 1;
    for (const auto &seq : sequences) {
        std::vector<int> line;
        const int n = (int)seq.size();
        if (n - gram_length + 1 <= 0) {
            // a sequence shorter than a gram: one gram, padded with its first value
            if (n > 0) {
                unsigned number = 0;
                for (int p = 0; p < gram_length; ++p) number = number * (unsigned)base + (unsigned)(p < n ? seq[p] : seq[0]);
                line.push_back((int)number);
            }
            gram_data.push_back(std::move(line));
            continue;
        }
        for (int j = 0; j + gram_length <= n; ++j) {
            unsigned g = 0;
            for (int t = 0; t < gram_length; ++t) g = g * (unsigned)base + (unsigned)seq[j + t];
            line.push_back((int)g);
        }
        gram_data.push_back(std::move(line));
    }
}

void sequence_reduce_to_ground(std::vector<std::vector<int> > &data, std::vector<std::vector<int> > &converted_data,
                               int &min_value, int &max_value) {
    converted_data.clear();
    bool first = true;
    for (const auto &row : data)
        for (int v : row) {
            if (first || v < min_value) min_value = v;
            if (first || v > max_value) max_value = v;
            first = false;
        }
    if (first) throw exception::cpu_runtime_error("no data input!");
    for (const auto &row : data) {
        std::vector<int> line;
        line.reserve(row.size());
        for (int v : row) line.push_back(v - min_value);
        converted_data.push_back(std::move(line));
    }
}

void reset_device() { throw_on_status(genie_device_reset()); }

void get_rowID_offset(std::vector<int> &result, std::vector<int> &resultID, std::vector<int> &resultOffset,
                      unsigned int shift_bits) {
    for (int v : result) {
        const int row = (int)((unsigned)v >> shift_bits);
        resultID.push_back(row);
        resultOffset.push_back(v - (int)((unsigned)row << shift_bits));
    }
}

void init_genie(GPUGenie_Config &config) { throw_on_status(genie_init(config.use_device)); }

}  // namespace original
}  // namespace genie
