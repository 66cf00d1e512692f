/*
 * genie_gb300.h -- C ABI of the GB300-native GENIE match-count top-k search.
 *
 * This is the drop-in boundary: plain pointers and sizes, opaque handles,
 * int status codes.  The C++ first/second-level interface (include/genie/)
 * and the Python mirror (genie_gb300/) are thin callers of these entry
 * points.  Each declaration names the reference interface it replaces.
 *
 * Results: query q owns k[q] slots starting at out_off[q] = sum_{p<q} k[p]
 * (q*k for a uniform k, the reference's row-major layout, knn.cu:165-175).
 * Slots are sorted by (primary desc, id asc); primary is the match count of
 * an unweighted query, or the exact fixed-point sum of matched item weights
 * of a weighted one.  Slots beyond the objects with a non-zero primary hold
 * (id 0, count 0, score 0), as the reference pads (heap_count.cu:254-255).
 *
 * Thread safety: an index handle is immutable after creation and may be
 * searched from several threads; a batch or server handle has one owner.
 */
#ifndef GENIE_GB300_H_
#define GENIE_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The C++ shim maps them back to the reference's exception
 * types (src/genie/exception/exception.h:10-46). */
enum genie_status {
    GENIE_OK = 0,
    GENIE_ERR_INVALID_ARG = 1,      /* InvalidConfigurationException / cpu_runtime_error */
    GENIE_ERR_GPU_ALLOC = 2,        /* gpu_bad_alloc */
    GENIE_ERR_CUDA = 3,             /* gpu_runtime_error */
    GENIE_ERR_NOT_IMPLEMENTED = 4,  /* NotImplementedException */
    GENIE_ERR_CPU_ALLOC = 5,        /* cpu_bad_alloc */
    GENIE_ERR_DEVICE_TIMEOUT = 6,   /* a bounded device wait ran out */
    GENIE_ERR_IO = 7,               /* file could not be read or written */
    GENIE_ERR_ADMISSION = 8         /* server: request exceeds the memory budget */
};

/* Codec ids: the reference COMPRESSION_TYPE enum (DeviceCodecFactory.h:38-53). */
enum genie_codec {
    GENIE_NO_COMPRESSION = 0, GENIE_COPY, GENIE_DELTA, GENIE_BP32, GENIE_VARINT,
    GENIE_COMP_BP32_COPY, GENIE_COMP_BP32_VARINT, GENIE_SERIAL_COPY_COPY,
    GENIE_SERIAL_DELTA_COPY, GENIE_SERIAL_DELTA_DELTA, GENIE_SERIAL_DELTA_VARINT,
    GENIE_SERIAL_DELTA_BP32, GENIE_SERIAL_DELTA_COMP_BP32_COPY,
    GENIE_SERIAL_DELTA_COMP_BP32_VARINT, GENIE_N_CODECS
};

typedef struct genie_index genie_index;
typedef struct genie_batch genie_batch;
typedef struct genie_server genie_server;

/* Message of the last failed call on this thread (never NULL). */
const char *genie_last_error(void);
/* ABI version (major*10000 + minor*100 + patch). */
int genie_version(void);

/* Select and initialise a device.  Replaces genie::utility::Init /
 * init_genie (src/genie/utility/init.cu:7-34). */
int genie_init(int device);
/* Reset the current device (cudaDeviceReset): every index, batch and server
 * on it is invalid afterwards and must only be destroyed; the library
 * prepares its kernels again on next use.  Replaces reset_device
 * (original/interface.cc:910-913). */
int genie_device_reset(void);

/* ---------------------------------------------------------------- index */

typedef struct {
    int64_t n_objects;     /* inv_table::i_size (inv_table.cu:93-96) */
    int32_t n_dims;        /* inv_table::m_size (inv_table.cu:87-91) */
    int32_t codec;         /* genie_codec; 0 = uncompressed */
    int64_t n_ids;         /* posting entries (inv_table::inv()->size()) */
    int64_t n_keys;        /* (dim, value) lists */
    int64_t n_words;       /* compressed words (0 when uncompressed) */
    int64_t n_segments;    /* compressed segments (0 when uncompressed) */
    int32_t max_multiplicity; /* most times one id repeats in one list */
    int32_t max_segment;   /* segment length bound of a compressed index */
    int64_t device_bytes;  /* HBM held by the index */
} genie_index_info;

/* Build a resident index from a row-major n_objects x n_dims value matrix.
 * Replaces preprocess_for_knn_csv + load_table + inv_table::build +
 * inv_table::cpy_data_to_gpu (original/interface.cc:150-353,
 * table/inv_table.cu:267-350, table/inv_table.cu:30-45). */
int genie_index_create(const int32_t *values, int64_t n_objects, int32_t n_dims,
                       genie_index **out);

/* Where genie_index_create_with builds the CSR: the device (a stable
 * counting sort per dim, for dims of at most 16384 distinct values) with the
 * host as fallback, the host only, or the device only. */
enum genie_builder { GENIE_BUILD_AUTO = 0, GENIE_BUILD_HOST = 1, GENIE_BUILD_DEVICE = 2 };
/* genie_index_create with a choice of builder; every builder gives the same
 * index.  GENIE_BUILD_DEVICE fails with GENIE_ERR_NOT_IMPLEMENTED when a dim's
 * range is too wide for it.  Replaces the host-side inv_list::invert +
 * inv_table::build (table/inv_list.cc:295-320, table/inv_table.cu:267-350). */
int genie_index_create_with(const int32_t *values, int64_t n_objects, int32_t n_dims, int32_t where,
                            genie_index **out);

/* Single-dim "bag" index (every value of row r lists r).  Replaces
 * load_table_bijectMap (original/interface.cc:621-646, inv_list.cc:51-84). */
int genie_index_create_bag(const int32_t *values, const int64_t *row_off,
                           int64_t n_objects, genie_index **out);

/* Compressed index: each (dim,value) list is cut into segments of at most
 * max_segment ids (<= 1024) and every segment is encoded with `codec`.
 * Replaces inv_compr_table::build (table/inv_compr_table.cu:30-119). */
int genie_index_create_compressed(const int32_t *values, int64_t n_objects, int32_t n_dims,
                                  int32_t codec, int32_t max_segment, genie_index **out);

/* Subsequence index: rows of values (row r = values[row_off[r] ..
 * row_off[r+1])); the object listed for the value at offset o of row r is
 * r << bits | o, bits the least with 2^bits >= the longest row.  A search
 * counts, for every (row, start offset) object, the items i of the query
 * (i = the item's position in its query) whose range holds the row's value at
 * start offset + i.  Searched through genie_search / genie_search_multi only.
 * Replaces load_table_bijectMap with use_subsequence_search
 * (original/interface.cc:650-655, table/inv_list.cc:193-235) and the match
 * kernel's offset shift (matching/match.cu:84-94). */
int genie_index_create_subsequence(const int32_t *values, const int64_t *row_off, int64_t n_rows,
                                   genie_index **out);
/* bits of a subsequence index (-1 for any other index): a result id is
 * rowID << bits | offset (inv_table::_shift_bits_subsequence, inv_table.cu:202-205). */
int genie_index_subsequence_bits(const genie_index *ix, int32_t *bits);
/* Device address of the index's posting ids (read only; n_ids entries, valid
 * while the index lives).  Replaces inv_table::d_inv_p (table/inv_table.h:55). */
int genie_index_device_ids(const genie_index *ix, const uint32_t **ids);

int genie_index_destroy(genie_index *ix);
int genie_index_get_info(const genie_index *ix, genie_index_info *out);

/* Copy the index back to the host (any pointer may be NULL).  ids holds the
 * device posting array, which equals the reference's inv_table::inv()
 * (test_save2gpu_sift.cc:91-100).  key_offsets has n_keys+1 entries, the
 * per-dim arrays n_dims entries, key_base n_dims+1 entries. */
int genie_index_copy_out(const genie_index *ix, uint32_t *ids, int64_t *key_offsets,
                         int64_t *key_base, int32_t *dim_min, int32_t *dim_max);

/* Copy the compressed layout back (any pointer may be NULL): words[n_words],
 * key_seg[n_keys+1], seg_word_off[n_segments+1], seg_first/seg_len[n_segments]. */
int genie_index_copy_compressed(const genie_index *ix, uint32_t *words, int64_t *key_seg,
                                int64_t *seg_word_off, uint32_t *seg_first, uint32_t *seg_len);

/* Span [start,end) of one query item in the posting array; 0 length when the
 * item matches nothing.  Replaces Query::build (query/query.cc:273-333). */
int genie_index_item_span(const genie_index *ix, int32_t dim, int32_t low, int32_t up,
                          int64_t *start, int64_t *end);

/* Widen [low,up] until the covered lists hold ceil(sel*N) ids.  Replaces
 * Query::apply_adaptive_query_range (query/query.cc:196-261). */
int genie_index_adaptive_range(const genie_index *ix, int32_t dim, float selectivity,
                               int32_t *low, int32_t *up);

/* Save / load an index in this library's own versioned file format
 * (header + arrays + checksum).  Replaces SaveTableToBinary /
 * LoadTableFromBinary (interface/io.h:16-28, utility/serialization.cc:23-58). */
int genie_index_save(const genie_index *ix, const char *path);
int genie_index_load(const char *path, genie_index **out);

/* ---------------------------------------------------------------- search */

/* A batch of queries.  Query q owns items [item_off[q], item_off[q+1]);
 * item i matches dim[i] with values in [low[i], up[i]] (inclusive).
 * weight/weighted may be NULL: a query is weighted when weighted[q] != 0,
 * and then every weight of its items must be finite and > 0.  k may be NULL,
 * in which case every query uses uniform_k.  Mirrors Query::range
 * (query/query.h:43-54) and knn_search's topk (knn.cu:158-159). */
typedef struct {
    int32_t n_queries;
    const int64_t *item_off;
    const int32_t *dim;
    const int32_t *low;
    const int32_t *up;
    const float *weight;
    const uint8_t *weighted;
    const uint32_t *k;
    uint32_t uniform_k;
} genie_queries;

/* Plain per-batch search from host buffers to host buffers: query upload,
 * match, top-k, result download, synchronous.  Replaces
 * original::knn_search(table, queries, h_topk, h_topk_count, config)
 * (original/interface.cc:826-857) and matching::knn (knn.cu:106-183).
 * scores may be NULL. */
int genie_search(genie_index *ix, const genie_queries *q, uint32_t *out_ids,
                 uint32_t *out_counts, float *out_scores);

/* Plugin point: the match function genie_search and genie_search_multi use
 * for the indexes of one codec id (0 = uncompressed), as the reference
 * registers a MatchIntegratedFunPtr per COMPRESSION_TYPE
 * (compression/DeviceCodecFactory.h:23-30, DeviceCodecFactory.cu:48-70,
 * looked up in matching/knn.cu:130-140).  A function takes the arguments of
 * genie_search plus the user pointer it was registered with, fills the
 * outputs in the genie_search layout and returns a status.  With no function
 * registered (the default, or fn = NULL) the built-in path runs, which a
 * registered function may call itself through genie_match_builtin.  Batched
 * and served searches always run the built-in kernels. */
typedef int (*genie_match_fn)(genie_index *ix, const genie_queries *q, uint32_t *out_ids, uint32_t *out_counts,
                              float *out_scores, void *user);
int genie_codec_set_match(int32_t codec, genie_match_fn fn, void *user);
int genie_codec_get_match(int32_t codec, genie_match_fn *fn, void **user);
int genie_match_builtin(genie_index *ix, const genie_queries *q, uint32_t *out_ids, uint32_t *out_counts,
                        float *out_scores);

/* Multi-index search, one query batch per index, results concatenated in
 * index order.  Replaces knn_search_MT / knn_MT
 * (original/interface.cc:859-909, matching/knn.cu:185-283). */
int genie_search_multi(genie_index *const *ix, const genie_queries *q, int32_t n_index,
                       uint32_t *out_ids, uint32_t *out_counts, float *out_scores);

/* Search that allocates no memory, for callers that may not call cudaMalloc:
 * a host framework or server that owns every device allocation, or a caller
 * with a hard memory budget or a latency-critical path (cudaMalloc/cudaFree
 * synchronise the device).  No counterpart in the reference: this entry
 * point is this library's own.  All pointers in q, out_off and the outputs
 * are DEVICE pointers (q->n_queries and q->uniform_k are host values);
 * n_items = item_off[n_queries], total_k = sum of k.  The workspace is a
 * fixed 16 MiB device array inside the library, shared by every call: at
 * most 1024 queries, 262144 items, 262144 list units (the items, plus the
 * (dim,value) lists covered by queries whose items cover several lists
 * each) and 32768 results per call, larger batches are rejected with
 * GENIE_ERR_INVALID_ARG.  The first call on a device looks up the array's
 * address (and prepares the kernels).  Every call is blocking: it
 * synchronises `stream` (a cudaStream_t, NULL = legacy default) and reads
 * the device's error word, so no call may be made while any stream is being
 * captured into a CUDA graph.  Calls are serialised; device work that
 * overlaps a call from elsewhere in the process would race on the shared
 * array. */
int genie_search_noalloc(genie_index *ix, const genie_queries *q, const int64_t *out_off,
                         int64_t n_items, int64_t total_k, uint32_t *out_ids, uint32_t *out_counts,
                         float *out_scores, void *stream);

/* ---------------------------------------------------------------- batched */

typedef struct {
    int32_t max_queries;     /* capacity of one run */
    int64_t max_items;
    uint32_t max_k;
    int32_t use_graph;       /* capture the device work as one CUDA graph */
    int64_t max_units;       /* list units: the items, plus the (dim,value) lists covered by queries
                                whose items cover several lists each; 0: 16 * max_items */
} genie_batch_config;

/* Kernel shape knobs picked by the autotuner (0 keeps the current value). */
typedef struct {
    int32_t sparse_slots;       /* hash slots per CTA (4-byte slots; 8-byte get half) */
    int32_t sparse_ctas_per_sm; /* 2: 512-thread CTAs, 1: 1024-thread CTAs */
    int32_t dense_tile;         /* ids per dense tile (1-byte counters; 4-byte get a quarter) */
    int32_t dense_threads;
    int64_t sparse_max_total;   /* queries touching more posting ids go dense */
    int64_t dense_part_work;    /* objects per dense id-range part, in whole tiles (at least one) */
    int32_t sparse_load_pct;    /* posting ids per part <= this % of the hash slots */
    int32_t bitmap_bits;        /* largest id space (objects) of the bitmap kernel; -1: off */
    int32_t dense_bitmaps;      /* dense lists counted from their presence bitmaps: 1 for unweighted
                                   queries, 2 for weighted ones, 3 both, -1 never */
} genie_tuning;

/* Batched search over one resident index: fixed-capacity device buffers,
 * pinned host staging, the batch size read on the device, and the device
 * work (query compile, persistent sparse/dense kernels, top-k, merge)
 * captured once as a CUDA graph.  Beyond the reference, which supports one k
 * per batch (knn.cu:158-159), every query carries its own k and weights. */
int genie_batch_create(genie_index *ix, const genie_batch_config *cfg, genie_batch **out);
int genie_batch_destroy(genie_batch *b);
/* stage + launch + fetch, synchronous. */
int genie_batch_run(genie_batch *b, const genie_queries *q, uint32_t *out_ids,
                    uint32_t *out_counts, float *out_scores);
/* Validate a batch and copy it to the device (returns when it is resident). */
int genie_batch_stage(genie_batch *b, const genie_queries *q);
/* Enqueue the device work of the staged batch on `stream` (a cudaStream_t;
 * NULL = the batch's own stream).  Asynchronous; may be repeated. */
int genie_batch_launch(genie_batch *b, void *stream);
/* Wait for the last launch and copy its results to host buffers. */
int genie_batch_fetch(genie_batch *b, uint32_t *out_ids, uint32_t *out_counts, float *out_scores);
/* Asynchronous genie_batch_run in two calls.  submit waits for the batch's
 * previous work (its pinned staging is reused), validates and copies the
 * queries into that staging, enqueues the upload, the device work and the
 * result download on the batch's stream, and returns.  collect waits for it
 * and copies the results out (out_scores only if submitted with want_scores).
 * Two batches used in turn overlap one batch's host-side staging with the
 * other's device work. */
int genie_batch_submit(genie_batch *b, const genie_queries *q, int32_t want_scores);
int genie_batch_collect(genie_batch *b, uint32_t *out_ids, uint32_t *out_counts, float *out_scores);
/* Time candidate tunings on a sample batch on the device; keeps the fastest. */
int genie_batch_autotune(genie_batch *b, const genie_queries *sample, genie_tuning *chosen);
int genie_batch_get_tuning(const genie_batch *b, genie_tuning *out);
int genie_batch_set_tuning(genie_batch *b, const genie_tuning *t);
/* Statistics of the last launch: kernels launched, device milliseconds
 * (between events around the device work; waits for it to finish). */
int genie_batch_last_stats(const genie_batch *b, int32_t *kernels, float *device_ms);
/* Device milliseconds of each stage of the last launch of a batch created
 * with use_graph = 0: ms[0] plan (+ counter reset), ms[1] presence-bitmap
 * kernel, ms[2] sparse kernel (4- and 8-byte slots), ms[3] dense kernel
 * (1- and 4-byte counters). */
int genie_batch_stage_ms(const genie_batch *b, float *ms);

/* ---------------------------------------------------------------- serving */

/* A request loop over several resident indexes with continuous batching.
 * Requests (one query each) are admitted when a batch slot of their index is
 * free and their memory estimate fits the budget; the requests that have
 * arrived by then form the slot's batch, which runs while other slots' batches
 * are still on the device, so requests that arrive during a run join the next
 * free slot instead of waiting for a whole queue to drain.  A scheduler thread
 * owned by the server does the batching, launches and completions; callers
 * only submit and wait.
 * Reference counterpart: the memory-budget admission loop of knn_MT
 * (matching/knn.cu:206-278) and the request loop of odgenie
 * (dist_genie/online.cu:37-180, scheduler.cc:20-64), which runs one request
 * as one synchronous batch. */
typedef struct {
    int32_t slots_per_index;  /* batches of one index that may be on the device at once (>= 1) */
    int32_t max_queries;      /* requests per batch */
    int64_t max_items;        /* items per batch */
    uint32_t max_k;
    int32_t window_us;        /* while a slot of the index is busy, wait up to this long for more requests */
    int64_t memory_budget;    /* bytes of in-flight request state; 0: bounded by the slots alone */
} genie_server_config;

typedef struct {
    int64_t submitted, completed, rejected, batches;
    double mean_batch;        /* requests per batch */
    double p50_us, p99_us, max_us;   /* arrival -> result ready, completed requests since the last reset */
    double throughput_qps;    /* completed / (last completion - first arrival) */
    int64_t held;             /* requests whose launch waited for in-flight memory under memory_budget */
    int64_t peak_in_flight_bytes;  /* most request state on the device at once (the budget's measure) */
} genie_server_report;

int genie_server_create(const genie_server_config *cfg, genie_server **out);
/* Make an index servable (before genie_server_start); the index must outlive
 * the server. */
int genie_server_add_index(genie_server *s, genie_index *ix, int32_t *index_id);
int genie_server_start(genie_server *s);
/* Submit q->n_queries requests (one per query) to index index_id.  Request i
 * counts as arriving at arrival_ns[i] on the genie_server_now_ns clock
 * (arrival_ns NULL: all now); future times schedule the requests.  Tickets
 * are *first_ticket, +1, ...  A request that can never be admitted (items, k
 * or memory beyond the configuration) fails the whole call with
 * GENIE_ERR_ADMISSION. */
int genie_server_submit(genie_server *s, int32_t index_id, const genie_queries *q, const int64_t *arrival_ns,
                        uint64_t *first_ticket);
/* Block until the request is answered; copy its k ids, counts and (optional)
 * scores; release the ticket.  latency_ns (optional) = completion - arrival. */
int genie_server_wait(genie_server *s, uint64_t ticket, uint32_t *out_ids, uint32_t *out_counts,
                      float *out_scores, int64_t *latency_ns);
/* Block until every submitted request is answered. */
int genie_server_drain(genie_server *s);
int genie_server_stats(genie_server *s, genie_server_report *out);
int genie_server_reset_stats(genie_server *s);
int64_t genie_server_now_ns(void);
int genie_server_destroy(genie_server *s);

/* ---------------------------------------------------------------- requests */

/* The request protocol over a server: a request is one JSON document
 *   {"topk": K, "queries": [{"content": [v0, v1, ...], "clusters": [c, ...]}, ...]}
 * in which value j of a query's content is item j (dim j, values
 * [v - radius, v + radius]) and the query is searched on every cluster it
 * names.  The answer is
 *   {"topk": K, "results": [{"ids": [...], "counts": [...]}, ...]}
 * with K slots per query, the clusters' answers merged by (count desc, id
 * asc) after adding each cluster's id offset, padded (0, 0); an invalid
 * request is answered {"error": "..."} with the reference's messages.
 * Replaces dist_genie's request parser, listener, per-cluster search and
 * merge (dist_genie/parser.cu:128-216, scheduler.cc:20-64, search.cu:34-52,
 * sorting.cc:20-64), which wrote the answer to a file instead. */
typedef struct genie_request_listener genie_request_listener;
typedef struct {
    genie_server *server;       /* a started server holding the clusters' indexes */
    int32_t n_clusters;
    const int32_t *index_id;    /* server index id of each cluster */
    const int64_t *id_offset;   /* global id of each cluster's object 0 */
    int32_t radius;             /* half-width of every item's value range */
} genie_request_router;

/* Answer one request document (no socket): the answer (NUL-terminated) goes
 * to out; *out_len receives its length even when out_cap is too small. */
int genie_request_handle(const genie_request_router *router, const char *json, char *out, int64_t out_cap,
                         int64_t *out_len);
/* Listen on host:port (port 0: any free port) on a thread of its own; each
 * connection carries one request, read until the client shuts its side, and
 * gets the answer back before the connection closes. */
int genie_request_listen(const genie_request_router *router, const char *host, int32_t port,
                         genie_request_listener **out);
int genie_request_listener_port(const genie_request_listener *l, int32_t *port);
int genie_request_listener_handled(const genie_request_listener *l, int64_t *n);
int genie_request_listener_stop(genie_request_listener *l);

/* ---------------------------------------------------------------- shards */

/* Merge the per-shard results of an id-range sharded search: shard s holds
 * objects [id_offset[s], ...) under local ids and answered the same queries
 * (k slots per query, layout as genie_search).  Writes the global top-k per
 * query, sorted (primary desc, id asc), padded (0, 0).  With scores (one
 * array per shard, or NULL for counts only) the primary is the score; exact
 * for unweighted queries, and for weighted ones up to scores equal in float.
 * Host-only.  Replaces the multiload merge (original/interface.cc:114-149)
 * and the MPI gather + sort of dist_genie (sorting.cc:20-64). */
int genie_merge_shards(int32_t n_shards, const uint32_t *const *ids, const uint32_t *const *counts,
                       const float *const *scores, const int64_t *id_offset, int32_t n_queries,
                       const uint32_t *k, uint32_t uniform_k, uint32_t *out_ids, uint32_t *out_counts,
                       float *out_scores);

/* ---------------------------------------------------------------- codecs */

/* Host encoder of the reference byte formats (DeviceCodecFactory.cu:13-48).
 * Returns words written or a negative status. */
int64_t genie_codec_encode(int32_t codec, const uint32_t *in, int64_t n, uint32_t *out, int64_t cap);
/* Worst-case words genie_codec_encode may write for n values. */
int64_t genie_codec_encode_bound(int64_t n);
/* Device decode of independent encoded segments: segment s spans words
 * [word_off[s], word_off[s+1]) and decodes to out[out_off[s] ..).  All
 * pointers are device pointers; out_len[s] receives each decoded length.
 * Replaces g_decodeArrayParallel (DeviceCodecTemplatesImpl.hpp:4-34). */
int genie_codec_decode_device(int32_t codec, const uint32_t *words, const int64_t *word_off,
                              int64_t n_segments, const int64_t *out_off, uint32_t *out,
                              uint32_t *out_len, void *stream);

#ifdef __cplusplus
}
#endif
#endif
