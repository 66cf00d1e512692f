// genie.cc -- the C++ interface (<genie/genie.h>) over the C ABI
// (<genie_gb300.h>): configuration, execution policies, table and query
// objects, CSV/binary I/O and the first/second-level entry points.  Every
// device operation goes through a genie_* call; status codes become the
// reference's exception types.
//
// Reference behaviour kept (file:line in the reference tree):
//   Config validation                      interface/config.cc
//   MakePolicy: single value / single range interface/execution_policy.cc:14-45
//   BuildTable: dim = width of the first row execution_policy/single_value.cc:10-15
//   BuildQuery: item j of row i, [v-r, v+r], weight 1, order j
//                                           original/interface.cc:473-517
//   CSV tokens split on ',' and blanks      utility/FileReader.cc:54-83
//   Search = load + build + match           interface/search.cc:11-22
#include <genie/genie.h>

#include "../../include/genie_gb300.h"
#include "flat_queries.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <iterator>
#include <sstream>
#include <thread>

namespace genie {

// ---------------------------------------------------------------- errors

void exception::throw_on_status(int status) {
    if (status == GENIE_OK) return;
    const std::string msg = genie_last_error();
    switch (status) {
        case GENIE_ERR_GPU_ALLOC:
        case GENIE_ERR_ADMISSION:
            throw gpu_bad_alloc(msg);
        case GENIE_ERR_NOT_IMPLEMENTED:
            throw NotImplementedException();
        case GENIE_ERR_CPU_ALLOC:
            throw cpu_bad_alloc(msg);
        case GENIE_ERR_INVALID_ARG:
        case GENIE_ERR_IO:
            throw cpu_runtime_error(msg);
        default:
            throw gpu_runtime_error(msg);
    }
}

using exception::throw_on_status;

// ---------------------------------------------------------------- Config

uint32_t Config::GetK() const { return k_; }
uint32_t Config::GetQueryRange() const { return query_range_; }
uint32_t Config::GetNumOfQueries() const { return num_of_queries_; }
bool Config::GetSaveToGpu() const { return save_to_gpu_; }
uint8_t Config::GetGpuId() const { return gpu_id_; }

Config &Config::SetK(const uint32_t k) {
    k_ = k;
    k_initialized_ = true;
    return *this;
}
Config &Config::SetQueryRange(const uint32_t query_range) {
    query_range_ = query_range;
    query_range_initialized_ = true;
    return *this;
}
Config &Config::SetNumOfQueries(const uint32_t num_of_queries) {
    num_of_queries_ = num_of_queries;
    num_of_queries_initialized_ = true;
    return *this;
}
Config &Config::SetSaveToGpu(const bool save_to_gpu) {
    save_to_gpu_ = save_to_gpu;
    return *this;
}
Config &Config::SetGpuId(const uint8_t gpu_id) {
    gpu_id_ = gpu_id;
    return *this;
}

Config &Config::LoadFromFile(const std::string &filename) {
    std::ifstream in(filename);
    if (!in) throw exception::cpu_runtime_error("cannot open configuration file " + filename);
    std::string key;
    long long v = 0;
    while (in >> key >> v) {
        if (key == "k") SetK((uint32_t)v);
        else if (key == "query_range") SetQueryRange((uint32_t)v);
        else if (key == "num_of_queries") SetNumOfQueries((uint32_t)v);
        else if (key == "save_to_gpu") SetSaveToGpu(v != 0);
        else if (key == "gpu_id") SetGpuId((uint8_t)v);
        else throw exception::InvalidConfigurationException("unknown configuration key " + key);
    }
    return *this;
}

bool Config::IsKSet() const { return k_initialized_; }
bool Config::IsQueryRangeSet() const { return query_range_initialized_; }
bool Config::IsNumOfQueriesSet() const { return num_of_queries_initialized_; }

void Config::Validate() const {
    if (!k_initialized_) throw exception::InvalidConfigurationException("K is not set.");
    if (!num_of_queries_initialized_) throw exception::InvalidConfigurationException("Number of query is not set.");
}

void Config::DisplayConfiguration() {
    std::cout << "K: " << k_ << "\n"
              << "Query range: " << (query_range_initialized_ ? std::to_string(query_range_) : "unset") << "\n"
              << "Number of queries: " << num_of_queries_ << "\n"
              << "Save to GPU: " << (save_to_gpu_ ? "yes" : "no") << "\n"
              << "GPU id: " << (int)gpu_id_ << std::endl;
}

// ---------------------------------------------------------------- inv_table

namespace table {

inv_table::inv_table() {}
inv_table::inv_table(const int32_t *values, int64_t n_objects, int32_t n_dims) {
    genie_index *ix = nullptr;
    throw_on_status(genie_index_create(values, n_objects, n_dims, &ix));
    adopt(ix);
}
inv_table::inv_table(genie_index *ix) { adopt(ix); }
inv_table::~inv_table() {
    if (ix_) genie_index_destroy(ix_);
}

void inv_table::adopt(genie_index *ix) {
    if (ix_ && ix_ != ix) genie_index_destroy(ix_);
    ix_ = ix;
    d_inv_p = nullptr;
    inv_host_.clear();
    if (!ix_) return;
    const uint32_t *ids = nullptr;
    throw_on_status(genie_index_device_ids(ix_, &ids));
    d_inv_p = (int *)ids;
    int32_t bits = -1;
    throw_on_status(genie_index_subsequence_bits(ix_, &bits));
    shift_bits_subsequence = bits > 0 ? (unsigned)bits : 0u;
}

static genie_index_info info_of(genie_index *ix) {
    genie_index_info inf{};
    if (!ix) throw exception::cpu_runtime_error("the table holds no index (load it first)");
    throw_on_status(genie_index_get_info(ix, &inf));
    return inf;
}

// rows of a subsequence table (its objects are rowID << bits | offset)
int inv_table::i_size() const { return (int)(info_of(ix_).n_objects >> shift_bits_subsequence); }
int inv_table::m_size() const { return (int)info_of(ix_).n_dims; }
int64_t inv_table::inv_size() const { return info_of(ix_).n_ids; }

std::vector<int> *inv_table::inv() {
    const int64_t n = inv_size();
    inv_host_.resize((size_t)n);
    static_assert(sizeof(int) == sizeof(uint32_t), "ids are copied as 32-bit words");
    throw_on_status(genie_index_copy_out(ix_, (uint32_t *)inv_host_.data(), nullptr, nullptr, nullptr, nullptr));
    return &inv_host_;
}

void inv_table::save(const std::string &filename) const { throw_on_status(genie_index_save(ix_, filename.c_str())); }

inv_table *inv_table::load(const std::string &filename) {
    genie_index *ix = nullptr;
    throw_on_status(genie_index_load(filename.c_str(), &ix));
    return new inv_table(ix);
}

}  // namespace table

// ---------------------------------------------------------------- Query

namespace query {

Query::Query(genie::table::inv_table *ref, int index) : ref_(ref), index_(index) {}
Query::Query(genie::table::inv_table &ref, int index) : ref_(&ref), index_(index) {}
Query::Query() {}

genie::table::inv_table *Query::ref_table() { return ref_; }

void Query::attr(int index, int low, int up, float weight, int order) { attr(index, low, up, weight, -1.0f, order); }

void Query::attr(int index, int value, float weight, float selectivity, int order) {
    attr(index, value, value, weight, selectivity, order);
}

void Query::attr(int index, int low, int up, float weight, float selectivity, int order) {
    if (!ref_ || index < 0 || index >= ref_->m_size()) return;
    range r;
    r.query = index_;
    r.order = order;
    r.dim = index;
    r.low = low;
    r.up = up;
    r.weight = weight;
    r.low_offset = 0;
    r.up_offset = 0;
    r.selectivity = selectivity;
    ranges_.push_back(r);
}

void Query::clear_dim(int index) {
    ranges_.erase(std::remove_if(ranges_.begin(), ranges_.end(), [index](const range &r) { return r.dim == index; }),
                  ranges_.end());
}

void Query::selectivity(float s) { selectivity_ = s; }
float Query::selectivity() { return selectivity_; }

void Query::apply_adaptive_query_range() {
    for (range &r : ranges_) {
        const float sel = r.selectivity > 0 ? r.selectivity : selectivity_;
        if (sel <= 0) continue;
        int32_t lo = r.low, hi = r.up;
        throw_on_status(genie_index_adaptive_range(ref_->handle(), r.dim, sel, &lo, &hi));
        r.low = lo;
        r.up = hi;
    }
}

void Query::topk(int k) { topk_ = k; }
int Query::topk() { return topk_; }

void Query::build() {
    dims_.clear();
    for (const range &r : ranges_) {
        int64_t s = 0, e = 0;
        throw_on_status(genie_index_item_span(ref_->handle(), r.dim, r.low, r.up, &s, &e));
        if (e > s) dims_.emplace_back(index_, r.order, (int)s, (int)e, r.weight);
    }
}

int Query::dump(std::vector<dim> &vout) {
    vout.insert(vout.end(), dims_.begin(), dims_.end());
    return (int)dims_.size();
}

int Query::dump(std::vector<range> &ranges) {
    ranges.insert(ranges.end(), ranges_.begin(), ranges_.end());
    return (int)ranges_.size();
}

int Query::index() { return index_; }
int Query::count_ranges() { return (int)ranges_.size(); }

}  // namespace query

// ---------------------------------------------------------------- policies

void ExecutionPolicy::Validate() {
    if (k_ == 0) throw exception::InvalidConfigurationException("K should be larger than 0.");
    if (num_of_queries_ == 0) throw exception::InvalidConfigurationException("Number of query should be larger than 0.");
}
void ExecutionPolicy::SetK(const uint32_t k) { k_ = k; }
void ExecutionPolicy::SetNumOfQueries(const uint32_t num_of_queries) { num_of_queries_ = num_of_queries; }
uint32_t ExecutionPolicy::GetNumOfQueries() const { return num_of_queries_; }

namespace {

SearchResult to_result(const std::vector<uint32_t> &ids, const std::vector<uint32_t> &counts) {
    return SearchResult(std::vector<int>(ids.begin(), ids.end()), std::vector<int>(counts.begin(), counts.end()));
}

class MatchPolicy : public ExecutionPolicy {
  public:
    explicit MatchPolicy(uint32_t query_range) : query_range_(query_range) {}

    std::shared_ptr<genie::table::inv_table> BuildTable(const genie::TableData &table_data) override {
        if (table_data.empty()) throw exception::cpu_runtime_error("no data input!");
        dim_ = (uint32_t)table_data[0].size();
        std::vector<int32_t> flat;
        flat.reserve(table_data.size() * dim_);
        for (const auto &row : table_data) {
            if (row.size() != dim_) throw exception::cpu_runtime_error("table rows differ in width");
            flat.insert(flat.end(), row.begin(), row.end());
        }
        return std::make_shared<genie::table::inv_table>(flat.data(), (int64_t)table_data.size(), (int32_t)dim_);
    }

    std::vector<genie::query::Query> BuildQuery(const std::shared_ptr<const genie::table::inv_table> &table,
                                                const genie::QueryData &query_data) override {
        genie::table::inv_table *t = const_cast<genie::table::inv_table *>(table.get());
        const int d = t->m_size();
        const int r = (int)query_range_;
        std::vector<genie::query::Query> out;
        out.reserve(query_data.size());
        for (size_t i = 0; i < query_data.size(); ++i) {
            genie::query::Query q(t, (int)i);
            for (size_t j = 0; j < query_data[i].size() && (int)j < d; ++j) {
                const int v = query_data[i][j];
                q.attr((int)j, v - r, v + r, 1.0f, (int)j);
            }
            q.topk((int)k_);
            out.push_back(q);
        }
        return out;
    }

    genie::SearchResult Match(const std::shared_ptr<const genie::table::inv_table> &table,
                              const std::vector<genie::query::Query> &queries) override {
        if (queries.empty()) throw exception::cpu_runtime_error("Queries not loaded!");
        FlatQueries f(queries);
        const genie_queries g = f.view();
        std::vector<uint32_t> ids((size_t)std::max<int64_t>(1, f.total_k)), counts(ids.size());
        throw_on_status(genie_search(table->handle(), &g, ids.data(), counts.data(), nullptr));
        ids.resize((size_t)f.total_k);
        counts.resize((size_t)f.total_k);
        return to_result(ids, counts);
    }

    genie::SearchResult Match(const std::vector<std::shared_ptr<const genie::table::inv_table> > &tables,
                              const std::vector<std::vector<genie::query::Query> > &queries) override {
        if (tables.size() != queries.size()) throw exception::cpu_runtime_error("one query list per table is needed");
        std::vector<FlatQueries> fs;
        fs.reserve(queries.size());
        std::vector<genie_queries> gs;
        std::vector<genie_index *> ixs;
        int64_t total = 0;
        for (size_t t = 0; t < tables.size(); ++t) {
            fs.emplace_back(queries[t]);
            total += fs.back().total_k;
        }
        for (size_t t = 0; t < tables.size(); ++t) {
            gs.push_back(fs[t].view());
            ixs.push_back(tables[t]->handle());
        }
        std::vector<uint32_t> ids((size_t)std::max<int64_t>(1, total)), counts(ids.size());
        throw_on_status(genie_search_multi(ixs.data(), gs.data(), (int32_t)ixs.size(), ids.data(), counts.data(),
                                           nullptr));
        ids.resize((size_t)total);
        counts.resize((size_t)total);
        return to_result(ids, counts);
    }

    void Validate() override {
        ExecutionPolicy::Validate();
        if (ranged_ && query_range_ == 0)
            throw exception::InvalidConfigurationException("Query range should be larger than 0.");
    }

    bool ranged_ = false;

  private:
    uint32_t query_range_;
};

}  // namespace

std::shared_ptr<ExecutionPolicy> MakePolicy(const Config &config) {
    config.Validate();
    auto p = std::make_shared<MatchPolicy>(config.IsQueryRangeSet() ? config.GetQueryRange() : 0u);
    p->ranged_ = config.IsQueryRangeSet();
    p->SetK(config.GetK());
    p->SetNumOfQueries(config.GetNumOfQueries());
    p->Validate();
    throw_on_status(genie_init((int)config.GetGpuId()));
    return p;
}

// ---------------------------------------------------------------- I/O

// Integers of one line, separated by ',' or blanks (FileReader.cc:54-83).
static void parse_line(const char *p, const char *e, std::vector<int> &row) {
    auto sep = [](char c) { return c == ',' || c == ' ' || c == '\t' || c == '\r' || c == '\n'; };
    while (p < e) {
        while (p < e && sep(*p)) ++p;
        if (p >= e) break;
        const char *q = p;
        long long v = 0;
        bool neg = false;
        if (*q == '-' || *q == '+') neg = *q++ == '-';
        const char *d = q;
        while (q < e && *q >= '0' && *q <= '9') v = v * 10 + (*q++ - '0');
        if (q > d) row.push_back((int)(neg ? -v : v));
        while (q < e && !sep(*q)) ++q;          // the rest of a token that is not a number
        p = q;
    }
}

// The first `limit` lines (all when < 0) of a CSV file as rows of integers.
// The file is read at once and its lines are parsed in parallel, one block
// of lines per host thread.
static std::vector<std::vector<int> > read_rows(const std::string &filename, long long limit) {
    std::vector<std::vector<int> > rows;
    std::ifstream in(filename, std::ios::binary);
    if (!in) return rows;
    std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    std::vector<size_t> starts;
    for (size_t i = 0; i < text.size(); ++i) {
        if (i == 0 || text[i - 1] == '\n') {
            if (limit >= 0 && (long long)starts.size() >= limit) break;
            starts.push_back(i);
        }
    }
    const size_t n = starts.size();
    rows.resize(n);
    auto line_end = [&](size_t r) {
        if (r + 1 < n) return starts[r + 1];
        const size_t nl = text.find('\n', starts[r]);
        return nl == std::string::npos ? text.size() : nl + 1;
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = std::min<size_t>(hw, std::max<size_t>(1, n / 4096));
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            for (size_t r = n * t / nt; r < n * (t + 1) / nt; ++r)
                parse_line(text.data() + starts[r], text.data() + line_end(r), rows[r]);
        });
    for (auto &x : th) x.join();
    return rows;
}

TableData LoadTableDataFromCsv(const std::string &filename) { return read_rows(filename, -1); }

QueryData LoadQueryDataFromCsv(const std::string &filename, const std::shared_ptr<const ExecutionPolicy> &policy) {
    return read_rows(filename, (long long)policy->GetNumOfQueries());
}

std::shared_ptr<genie::table::inv_table> LoadTableFromBinary(const std::string &filename) {
    return std::shared_ptr<genie::table::inv_table>(genie::table::inv_table::load(filename));
}

void SaveTableToBinary(const std::string &filename, const std::shared_ptr<const genie::table::inv_table> &table) {
    table->save(filename);
}

// ---------------------------------------------------------------- entry points

std::shared_ptr<genie::table::inv_table> BuildTable(std::shared_ptr<genie::ExecutionPolicy> &policy,
                                                    const TableData &table_data) {
    return policy->BuildTable(table_data);
}

std::vector<genie::query::Query> BuildQuery(std::shared_ptr<genie::ExecutionPolicy> &policy,
                                            const std::shared_ptr<genie::table::inv_table> &table,
                                            const QueryData &query_data) {
    return policy->BuildQuery(table, query_data);
}

SearchResult Match(std::shared_ptr<genie::ExecutionPolicy> &policy,
                   const std::shared_ptr<genie::table::inv_table> &table,
                   const std::vector<genie::query::Query> &queries) {
    return policy->Match(table, queries);
}

SearchResult Search(std::shared_ptr<genie::ExecutionPolicy> &policy, const std::string &table_filename,
                    const std::string &query_filename) {
    TableData table_data = LoadTableDataFromCsv(table_filename);
    QueryData query_data = LoadQueryDataFromCsv(query_filename, policy);
    std::shared_ptr<genie::table::inv_table> table = BuildTable(policy, table_data);
    std::vector<genie::query::Query> queries = BuildQuery(policy, table, query_data);
    return Match(policy, table, queries);
}

}  // namespace genie
