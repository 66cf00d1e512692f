// request.cu -- the request protocol over the serving loop: JSON requests
// {"topk": K, "queries": [{"content": [v0, v1, ...], "clusters": [c, ...]}]}
// taken from a TCP socket, each query searched on every index ("cluster") it
// names through a genie_server, the answers merged per query with each
// cluster's id offset, and a JSON answer written back on the socket.
//
// Reference counterparts: dist_genie's request parser and validation
// (dist_genie/parser.cu:128-216; the error messages are kept), its socket
// listener (scheduler.cc:20-64, one request per connection), the per-cluster
// search (search.cu:34-52) and the merge of the clusters' answers with global
// id offsets (sorting.cc:20-64, online.cu:83-105).  The reference writes the
// answer to a CSV file named by the time; here it goes back to the client.
#include "capi_internal.h"

#include <arpa/inet.h>
#include <netinet/in.h>
#include <sys/socket.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cerrno>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

using namespace gg;

namespace {

// ---------------------------------------------------------------- JSON

struct JValue {
    enum Kind { kNull, kBool, kNumber, kString, kArray, kObject } kind = kNull;
    double num = 0;
    bool is_int = false;
    int64_t ival = 0;
    std::string str;
    std::vector<JValue> items;                            // array elements
    std::vector<std::pair<std::string, JValue> > members; // object members
    const JValue *get(const char *key) const {
        for (const auto &m : members)
            if (m.first == key) return &m.second;
        return nullptr;
    }
};

// A recursive-descent parser of one JSON document (RFC 8259; no \u escapes
// beyond ASCII are needed by the protocol and are kept verbatim).
class JParser {
  public:
    explicit JParser(const std::string &s) : s_(s) {}
    bool parse(JValue &out) {
        ws();
        if (!value(out, 0)) return false;
        ws();
        return i_ == s_.size();
    }

  private:
    const std::string &s_;
    size_t i_ = 0;
    void ws() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\t' || s_[i_] == '\n' || s_[i_] == '\r')) ++i_;
    }
    bool lit(const char *w) {
        const size_t n = std::strlen(w);
        if (s_.compare(i_, n, w) != 0) return false;
        i_ += n;
        return true;
    }
    bool value(JValue &v, int depth) {
        if (depth > 64 || i_ >= s_.size()) return false;
        const char c = s_[i_];
        if (c == '{') return object(v, depth);
        if (c == '[') return array(v, depth);
        if (c == '"') {
            v.kind = JValue::kString;
            return string(v.str);
        }
        if (c == 't') { v.kind = JValue::kBool; return lit("true"); }
        if (c == 'f') { v.kind = JValue::kBool; return lit("false"); }
        if (c == 'n') { v.kind = JValue::kNull; return lit("null"); }
        return number(v);
    }
    bool string(std::string &out) {
        if (s_[i_] != '"') return false;
        ++i_;
        while (i_ < s_.size() && s_[i_] != '"') {
            if (s_[i_] == '\\') {
                if (++i_ >= s_.size()) return false;
                const char e = s_[i_];
                out += e == 'n' ? '\n' : e == 't' ? '\t' : e == 'r' ? '\r' : e == 'b' ? '\b' : e == 'f' ? '\f' : e;
            } else {
                out += s_[i_];
            }
            ++i_;
        }
        if (i_ >= s_.size()) return false;
        ++i_;
        return true;
    }
    bool number(JValue &v) {
        const size_t a = i_;
        if (i_ < s_.size() && (s_[i_] == '-' || s_[i_] == '+')) ++i_;
        bool frac = false;
        while (i_ < s_.size() && (std::isdigit((unsigned char)s_[i_]) || s_[i_] == '.' || s_[i_] == 'e' ||
                                  s_[i_] == 'E' || ((s_[i_] == '-' || s_[i_] == '+') && (s_[i_ - 1] == 'e' || s_[i_ - 1] == 'E')))) {
            if (!std::isdigit((unsigned char)s_[i_])) frac = true;
            ++i_;
        }
        if (i_ == a) return false;
        const std::string t = s_.substr(a, i_ - a);
        char *end = nullptr;
        v.kind = JValue::kNumber;
        v.num = std::strtod(t.c_str(), &end);
        if (*end) return false;
        v.is_int = !frac && v.num >= -2147483648.0 && v.num <= 2147483647.0;
        v.ival = v.is_int ? std::strtoll(t.c_str(), nullptr, 10) : 0;
        return true;
    }
    bool array(JValue &v, int depth) {
        v.kind = JValue::kArray;
        ++i_;
        ws();
        if (i_ < s_.size() && s_[i_] == ']') { ++i_; return true; }
        for (;;) {
            JValue e;
            ws();
            if (!value(e, depth + 1)) return false;
            v.items.push_back(std::move(e));
            ws();
            if (i_ >= s_.size()) return false;
            if (s_[i_] == ',') { ++i_; continue; }
            if (s_[i_] == ']') { ++i_; return true; }
            return false;
        }
    }
    bool object(JValue &v, int depth) {
        v.kind = JValue::kObject;
        ++i_;
        ws();
        if (i_ < s_.size() && s_[i_] == '}') { ++i_; return true; }
        for (;;) {
            ws();
            std::string key;
            if (i_ >= s_.size() || !string(key)) return false;
            ws();
            if (i_ >= s_.size() || s_[i_] != ':') return false;
            ++i_;
            ws();
            JValue e;
            if (!value(e, depth + 1)) return false;
            v.members.emplace_back(std::move(key), std::move(e));
            ws();
            if (i_ >= s_.size()) return false;
            if (s_[i_] == ',') { ++i_; continue; }
            if (s_[i_] == '}') { ++i_; return true; }
            return false;
        }
    }
};

std::string jerror(const std::string &msg) {
    std::string out = "{\"error\": \"";
    for (char c : msg) {
        if (c == '"' || c == '\\') out += '\\';
        out += c;
    }
    return out + "\"}";
}

struct ParsedRequest {
    int topk = 0;
    std::vector<std::vector<int32_t> > content;
    std::vector<std::vector<int32_t> > clusters;
};

// ValidateAndParseQuery (dist_genie/parser.cu:128-216), with its messages.
bool parse_request(const std::string &doc, int32_t n_clusters, ParsedRequest &r, std::string &err) {
    JValue j;
    if (!JParser(doc).parse(j) || j.kind != JValue::kObject) {
        err = "Received query is not a valid JSON document";
        return false;
    }
    const JValue *topk = j.get("topk");
    if (!topk) { err = "Entry 'topk' is missing"; return false; }
    if (topk->kind != JValue::kNumber || !topk->is_int) { err = "Entry 'topk' should be an interger"; return false; }
    const JValue *qs = j.get("queries");
    if (!qs) { err = "Entry 'queries' is missing"; return false; }
    if (qs->kind != JValue::kArray) { err = "Entry 'queries' should be an array"; return false; }
    for (const JValue &q : qs->items) {
        const JValue *c = q.kind == JValue::kObject ? q.get("content") : nullptr;
        if (!c) { err = "Some query misses the 'content' section"; return false; }
        if (c->kind != JValue::kArray) { err = "Query's 'content' section should be an array"; return false; }
        const JValue *cl = q.get("clusters");
        if (!cl) { err = "Some query misses the 'clusters' section"; return false; }
        if (cl->kind != JValue::kArray) { err = "Query's 'clusters' section should be an array"; return false; }
    }
    r.topk = (int)topk->ival;
    if (r.topk < 1 || r.topk > kMaxK) { err = "Entry 'topk' should be in [1, " + std::to_string(kMaxK) + "]"; return false; }
    for (const JValue &q : qs->items) {
        std::vector<int32_t> content, clusters;
        for (const JValue &v : q.get("content")->items) {
            if (v.kind != JValue::kNumber || !v.is_int) { err = "Query's 'content' values should be integers"; return false; }
            content.push_back((int32_t)v.ival);
        }
        for (const JValue &v : q.get("clusters")->items) {
            if (v.kind != JValue::kNumber || !v.is_int || v.ival < 0 || v.ival >= n_clusters) {
                err = "Query's 'clusters' should name clusters 0.." + std::to_string(n_clusters - 1);
                return false;
            }
            clusters.push_back((int32_t)v.ival);
        }
        r.content.push_back(std::move(content));
        r.clusters.push_back(std::move(clusters));
    }
    return true;
}

// Search every query on its clusters through the server and merge per query.
int run_request(const genie_request_router *rt, const ParsedRequest &r, std::string &out) {
    const int64_t Q = (int64_t)r.content.size();
    const uint32_t k = (uint32_t)r.topk;
    // per cluster: the queries naming it, as one batch
    std::vector<std::vector<int64_t> > members((size_t)rt->n_clusters);
    for (int64_t q = 0; q < Q; ++q)
        for (int32_t c : r.clusters[(size_t)q]) members[(size_t)c].push_back(q);
    std::vector<std::vector<uint64_t> > tickets((size_t)rt->n_clusters);
    for (int32_t c = 0; c < rt->n_clusters; ++c) {
        if (members[(size_t)c].empty()) continue;
        std::vector<int64_t> off{0};
        std::vector<int32_t> dim, low, up;
        for (int64_t q : members[(size_t)c]) {
            const auto &row = r.content[(size_t)q];
            for (size_t j = 0; j < row.size(); ++j) {     // item j: dim j, [v - r, v + r]
                dim.push_back((int32_t)j);
                low.push_back(row[j] - rt->radius);
                up.push_back(row[j] + rt->radius);
            }
            off.push_back((int64_t)dim.size());
        }
        genie_queries gq{};
        gq.n_queries = (int32_t)members[(size_t)c].size();
        gq.item_off = off.data();
        gq.dim = dim.data();
        gq.low = low.data();
        gq.up = up.data();
        gq.uniform_k = k;
        uint64_t first = 0;
        const int rc = genie_server_submit(rt->server, rt->index_id[c], &gq, nullptr, &first);
        if (rc) return rc;
        for (size_t i = 0; i < members[(size_t)c].size(); ++i) tickets[(size_t)c].push_back(first + i);
    }
    // answers, each cluster's ids offset to global ids
    std::vector<std::vector<std::pair<uint32_t, int64_t> > > cand((size_t)Q);   // (count, global id)
    std::vector<uint32_t> ids(k), cnt(k);
    int first_err = GENIE_OK;
    for (int32_t c = 0; c < rt->n_clusters; ++c)
        for (size_t i = 0; i < tickets[(size_t)c].size(); ++i) {
            const int rc = genie_server_wait(rt->server, tickets[(size_t)c][i], ids.data(), cnt.data(), nullptr, nullptr);
            if (rc) {
                if (!first_err) first_err = rc;
                continue;
            }
            const int64_t q = members[(size_t)c][i];
            for (uint32_t j = 0; j < k; ++j)
                if (cnt[j] > 0) cand[(size_t)q].emplace_back(cnt[j], (int64_t)ids[j] + rt->id_offset[c]);
        }
    if (first_err) return first_err;
    out = "{\"topk\": " + std::to_string(k) + ", \"results\": [";
    for (int64_t q = 0; q < Q; ++q) {
        auto &v = cand[(size_t)q];
        std::sort(v.begin(), v.end(), [](const std::pair<uint32_t, int64_t> &a, const std::pair<uint32_t, int64_t> &b) {
            return a.first != b.first ? a.first > b.first : a.second < b.second;
        });
        std::string sid, scnt;
        for (uint32_t j = 0; j < k; ++j) {
            const bool have = j < v.size();
            sid += (j ? ", " : "") + std::to_string(have ? v[j].second : 0);
            scnt += (j ? ", " : "") + std::to_string(have ? v[j].first : 0u);
        }
        out += (q ? ", " : "") + std::string("{\"ids\": [") + sid + "], \"counts\": [" + scnt + "]}";
    }
    out += "]}";
    return GENIE_OK;
}

std::string handle(const genie_request_router *rt, const std::string &doc) {
    ParsedRequest r;
    std::string err, out;
    if (!parse_request(doc, rt->n_clusters, r, err)) return jerror(err);
    if (!rt->server) return jerror("no server attached");
    const int rc = run_request(rt, r, out);
    return rc ? jerror(genie_last_error()) : out;
}

}  // namespace

struct genie_request_listener {
    genie_request_router router{};
    std::vector<int32_t> index_id;
    std::vector<int64_t> id_offset;
    int fd = -1;
    int port = 0;
    std::atomic<bool> stop{false};
    std::atomic<int64_t> handled{0};
    std::thread th;
};

extern "C" {

int genie_request_handle(const genie_request_router *router, const char *json, char *out, int64_t out_cap,
                         int64_t *out_len) {
    if (!router || !json || (!out && out_cap > 0)) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    if (router->n_clusters < 1 || !router->index_id || !router->id_offset)
        return fail(GENIE_ERR_INVALID_ARG, "the router names no clusters");
    const std::string resp = handle(router, json);
    if (out_len) *out_len = (int64_t)resp.size();
    if ((int64_t)resp.size() + 1 > out_cap) return fail(GENIE_ERR_INVALID_ARG, "answer needs %zu bytes", resp.size() + 1);
    std::memcpy(out, resp.c_str(), resp.size() + 1);
    return GENIE_OK;
}

int genie_request_listen(const genie_request_router *router, const char *host, int32_t port,
                         genie_request_listener **out) {
    if (!router || !out || router->n_clusters < 1 || !router->index_id || !router->id_offset)
        return fail(GENIE_ERR_INVALID_ARG, "NULL argument or no clusters");
    *out = nullptr;
    genie_request_listener *l = new genie_request_listener();
    l->router = *router;
    l->index_id.assign(router->index_id, router->index_id + router->n_clusters);
    l->id_offset.assign(router->id_offset, router->id_offset + router->n_clusters);
    l->router.index_id = l->index_id.data();
    l->router.id_offset = l->id_offset.data();
    l->fd = socket(AF_INET, SOCK_STREAM, 0);
    if (l->fd < 0) {
        delete l;
        return fail(GENIE_ERR_IO, "socket: %s", std::strerror(errno));
    }
    int one = 1;
    setsockopt(l->fd, SOL_SOCKET, SO_REUSEADDR, &one, sizeof(one));
    sockaddr_in a{};
    a.sin_family = AF_INET;
    a.sin_port = htons((uint16_t)port);
    if (inet_pton(AF_INET, host ? host : "127.0.0.1", &a.sin_addr) != 1 ||
        bind(l->fd, (sockaddr *)&a, sizeof(a)) != 0 || listen(l->fd, 16) != 0) {
        const int e = errno;
        close(l->fd);
        delete l;
        return fail(GENIE_ERR_IO, "cannot listen on %s:%d: %s", host ? host : "127.0.0.1", port, std::strerror(e));
    }
    socklen_t al = sizeof(a);
    getsockname(l->fd, (sockaddr *)&a, &al);
    l->port = ntohs(a.sin_port);
    // one request per connection: read until the client ends its side, answer, close
    l->th = std::thread([l] {
        while (!l->stop.load()) {
            const int c = accept(l->fd, nullptr, nullptr);
            if (c < 0) {
                if (l->stop.load()) break;
                continue;
            }
            std::string doc;
            char buf[65536];
            for (;;) {
                const ssize_t n = recv(c, buf, sizeof(buf), 0);
                if (n <= 0) break;
                doc.append(buf, (size_t)n);
                if (doc.size() > ((size_t)1 << 30)) break;
            }
            const std::string resp = handle(&l->router, doc);
            size_t sent = 0;
            while (sent < resp.size()) {
                const ssize_t n = send(c, resp.data() + sent, resp.size() - sent, MSG_NOSIGNAL);
                if (n <= 0) break;
                sent += (size_t)n;
            }
            close(c);
            l->handled.fetch_add(1);
        }
    });
    *out = l;
    return GENIE_OK;
}

int genie_request_listener_port(const genie_request_listener *l, int32_t *port) {
    if (!l || !port) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    *port = l->port;
    return GENIE_OK;
}

int genie_request_listener_handled(const genie_request_listener *l, int64_t *n) {
    if (!l || !n) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    *n = l->handled.load();
    return GENIE_OK;
}

int genie_request_listener_stop(genie_request_listener *l) {
    if (!l) return GENIE_OK;
    l->stop.store(true);
    shutdown(l->fd, SHUT_RDWR);
    close(l->fd);
    if (l->th.joinable()) l->th.join();
    delete l;
    return GENIE_OK;
}

}  // extern "C"
