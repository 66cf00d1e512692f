/*
 * genie_oracle.h -- CPU oracle for GENIE's match-count top-k search.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against; it is never linked into, loaded by, or called from
 * the product library (libgenie_gb300).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.
 *
 * It restates, in plain C, the reference algorithm for the search path:
 *   - inverted index build      (src/genie/table/inv_list.cc:295-320,
 *                                src/genie/table/inv_list.cc:51-84,
 *                                src/genie/table/inv_table.cu:267-350)
 *   - query item -> span compile (src/genie/query/query.cc:87-113, 273-333)
 *   - adaptive query range       (src/genie/query/query.cc:196-261)
 *   - dense match-count + top-k  (test/test_compression_query.cu:127-284,
 *                                 the reference's own CPU match oracle)
 *   - posting-list codecs        (src/genie/compression/*.cu host encoders)
 *
 * Parity is pinned by tests against the reference's golden vectors
 * (test/test_csv_input_sift_data.cc:65-87) and against fixtures produced by
 * the reference's own host code (oracle/ref_shim.cu, tests/golden/).
 *
 * Output order is canonical: primary key descending, object id ascending.
 * Unweighted queries rank by match count.  Weighted queries rank by an exact
 * 32-bit fixed-point sum of the matched items' weights (see orc_weight_scale).
 */
#ifndef GENIE_ORACLE_H_
#define GENIE_ORACLE_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* CSR inverted index keyed by (dim, value). */
typedef struct {
    int32_t  n_dims;        /* D */
    int64_t  n_objects;     /* N */
    int64_t  n_ids;         /* total posting entries */
    int32_t *dim_min;       /* [D] smallest value in the dim */
    int32_t *dim_max;       /* [D] largest value in the dim */
    int64_t *key_base;      /* [D+1] first key of each dim; key_base[D] = n_keys */
    int64_t *key_offsets;   /* [n_keys+1] start of each key's list in ids */
    uint32_t *ids;          /* [n_ids] ascending per key */
} orc_index;

/* Build from a row-major N x D value matrix (one value per object per dim). */
int  orc_index_build(const int32_t *values, int64_t n, int32_t d, orc_index *out);
/* Build the single-dim "bag" form: row r holds values[row_off[r] .. row_off[r+1]). */
int  orc_index_build_bag(const int32_t *values, const int64_t *row_off, int64_t n,
                         orc_index *out);
void orc_index_free(orc_index *ix);

/* Span of one query item; returns 0 and start=end=0 if the item matches nothing. */
int  orc_item_span(const orc_index *ix, int32_t dim, int32_t low, int32_t up,
                   int64_t *start, int64_t *end);

/* Widen [low,up] of one item until its lists hold ceil(sel*N) ids
 * (Query::apply_adaptive_query_range).  sel <= 0 leaves the range unchanged. */
void orc_adaptive_range(const orc_index *ix, int32_t dim, float sel,
                        int32_t *low, int32_t *up);

/* Fixed-point scale exponent s for a weighted query of m items: weights are
 * summed as llrint(w * 2^s), s = 31 - e where m * max(w) < 2^e, so every sum
 * fits 32 bits and the scale does not depend on summation order. */
int32_t orc_weight_scale(const float *w, int64_t m);

/*
 * Batched search.  Query q owns items [item_off[q], item_off[q+1]).
 * k[q] results are written at out_off[q] (row-major, canonical order),
 * padded with (0,0,0).  weight/weighted may be NULL (all unweighted).
 * n_threads <= 0 uses all OpenMP threads.  Returns 0 or a negative error.
 */
int orc_search(const orc_index *ix, int32_t n_queries, const int64_t *item_off,
               const int32_t *dim, const int32_t *low, const int32_t *up,
               const float *weight, const uint8_t *weighted,
               const uint32_t *k, const int64_t *out_off,
               uint32_t *out_ids, uint32_t *out_counts, float *out_scores,
               int n_threads);

/* Dense per-object counts of one query (unweighted), for property tests. */
int orc_counts(const orc_index *ix, int64_t m, const int32_t *dim,
               const int32_t *low, const int32_t *up, uint32_t *counts_out);

/* ---- codecs: the reference's COMPRESSION_TYPE byte formats ---- */
enum {
    ORC_NO_COMPRESSION = 0, ORC_COPY, ORC_DELTA, ORC_BP32, ORC_VARINT,
    ORC_COMP_BP32_COPY, ORC_COMP_BP32_VARINT, ORC_SERIAL_COPY_COPY,
    ORC_SERIAL_DELTA_COPY, ORC_SERIAL_DELTA_DELTA, ORC_SERIAL_DELTA_VARINT,
    ORC_SERIAL_DELTA_BP32, ORC_SERIAL_DELTA_COMP_BP32_COPY,
    ORC_SERIAL_DELTA_COMP_BP32_VARINT, ORC_N_CODECS
};
/* Worst-case number of words orc_encode may write for n values. */
int64_t orc_encode_bound(int64_t n);
/* Encode n values; returns the number of 32-bit words written (cap = capacity). */
int64_t orc_encode(int codec, const uint32_t *in, int64_t n, uint32_t *out, int64_t cap);
/* Decode n_words words; returns the number of values written (or -1). */
int64_t orc_decode(int codec, const uint32_t *in, int64_t n_words, uint32_t *out, int64_t cap);

/* Compressed index: each key's list cut into segments of <= max_len ids,
 * every segment encoded independently (inv_compr_table::build). */
typedef struct {
    int32_t  codec;
    int32_t  max_len;
    int64_t  n_segs;
    int64_t  n_words;
    int64_t *key_seg;       /* [n_keys+1] first segment of each key */
    int64_t *seg_word_off;  /* [n_segs+1] word offset of each segment */
    uint32_t *seg_first;    /* [n_segs] first id of each segment */
    uint32_t *seg_len;      /* [n_segs] ids in each segment */
    uint32_t *words;        /* [n_words] */
} orc_compr_index;

int  orc_compress_index(const orc_index *ix, int codec, int32_t max_len, orc_compr_index *out);
void orc_compr_index_free(orc_compr_index *cx);

/* glibc rand() stream of test/test_compression_codecs.cu:174-199 (srand seed). */
void orc_codec_kat_input(uint32_t seed, uint32_t *out, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
