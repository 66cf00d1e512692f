/*
 * genie_oracle.c -- CPU oracle for GENIE's match-count top-k search.
 *
 * TEST INFRASTRUCTURE ONLY (see genie_oracle.h).  Every function names the
 * reference file:line whose behaviour it restates.
 */
#include "genie_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Index build                                                         */
/* ------------------------------------------------------------------ */

static int alloc_index(orc_index *ix, int32_t d, int64_t n) {
    memset(ix, 0, sizeof(*ix));
    ix->n_dims = d;
    ix->n_objects = n;
    ix->dim_min = (int32_t *)calloc((size_t)(d > 0 ? d : 1), sizeof(int32_t));
    ix->dim_max = (int32_t *)calloc((size_t)(d > 0 ? d : 1), sizeof(int32_t));
    ix->key_base = (int64_t *)calloc((size_t)d + 1, sizeof(int64_t));
    return (ix->dim_min && ix->dim_max && ix->key_base) ? 0 : -1;
}

/* inv_list::invert (inv_list.cc:295-320) per column, then inv_table::build
 * (inv_table.cu:267-350): ids ordered by (dim, value - min_dim, id).  A stable
 * counting sort per dim gives exactly that order. */
int orc_index_build(const int32_t *values, int64_t n, int32_t d, orc_index *ix) {
    if (n <= 0 || d <= 0 || !values) return -1;
    if (alloc_index(ix, d, n)) return -1;
    for (int32_t j = 0; j < d; ++j) {
        int32_t mn = values[j], mx = values[j];
        for (int64_t i = 1; i < n; ++i) {
            int32_t v = values[i * d + j];
            if (v < mn) mn = v;
            if (v > mx) mx = v;
        }
        ix->dim_min[j] = mn;
        ix->dim_max[j] = mx;
        ix->key_base[j + 1] = ix->key_base[j] + ((int64_t)mx - mn + 1);
    }
    int64_t n_keys = ix->key_base[d];
    ix->key_offsets = (int64_t *)calloc((size_t)n_keys + 1, sizeof(int64_t));
    ix->n_ids = n * d;
    ix->ids = (uint32_t *)malloc((size_t)ix->n_ids * sizeof(uint32_t) + 64);
    if (!ix->key_offsets || !ix->ids) return -1;
    for (int32_t j = 0; j < d; ++j)
        for (int64_t i = 0; i < n; ++i)
            ix->key_offsets[ix->key_base[j] + (values[i * d + j] - ix->dim_min[j]) + 1]++;
    for (int64_t kk = 0; kk < n_keys; ++kk) ix->key_offsets[kk + 1] += ix->key_offsets[kk];
    int64_t *cur = (int64_t *)malloc((size_t)n_keys * sizeof(int64_t));
    if (!cur) return -1;
    memcpy(cur, ix->key_offsets, (size_t)n_keys * sizeof(int64_t));
    for (int32_t j = 0; j < d; ++j)
        for (int64_t i = 0; i < n; ++i) {
            int64_t key = ix->key_base[j] + (values[i * d + j] - ix->dim_min[j]);
            ix->ids[cur[key]++] = (uint32_t)i;
        }
    free(cur);
    return 0;
}

/* inv_list::invert_bijectMap (inv_list.cc:51-84): one dim, every value of
 * row r adds r to that value's list (duplicates within a row repeat r). */
int orc_index_build_bag(const int32_t *values, const int64_t *row_off, int64_t n,
                        orc_index *ix) {
    if (n <= 0 || !row_off) return -1;
    int64_t total = row_off[n];
    if (total <= 0 || !values) return -1;
    if (alloc_index(ix, 1, n)) return -1;
    int32_t mn = values[0], mx = values[0];
    for (int64_t t = 1; t < total; ++t) {
        if (values[t] < mn) mn = values[t];
        if (values[t] > mx) mx = values[t];
    }
    ix->dim_min[0] = mn;
    ix->dim_max[0] = mx;
    ix->key_base[1] = (int64_t)mx - mn + 1;
    int64_t n_keys = ix->key_base[1];
    ix->key_offsets = (int64_t *)calloc((size_t)n_keys + 1, sizeof(int64_t));
    ix->n_ids = total;
    ix->ids = (uint32_t *)malloc((size_t)total * sizeof(uint32_t) + 64);
    if (!ix->key_offsets || !ix->ids) return -1;
    for (int64_t t = 0; t < total; ++t) ix->key_offsets[values[t] - mn + 1]++;
    for (int64_t kk = 0; kk < n_keys; ++kk) ix->key_offsets[kk + 1] += ix->key_offsets[kk];
    int64_t *cur = (int64_t *)malloc((size_t)n_keys * sizeof(int64_t));
    if (!cur) return -1;
    memcpy(cur, ix->key_offsets, (size_t)n_keys * sizeof(int64_t));
    for (int64_t r = 0; r < n; ++r)
        for (int64_t t = row_off[r]; t < row_off[r + 1]; ++t)
            ix->ids[cur[values[t] - mn]++] = (uint32_t)r;
    free(cur);
    return 0;
}

void orc_index_free(orc_index *ix) {
    if (!ix) return;
    free(ix->dim_min); free(ix->dim_max); free(ix->key_base);
    free(ix->key_offsets); free(ix->ids);
    memset(ix, 0, sizeof(*ix));
}

/* ------------------------------------------------------------------ */
/* Query compile                                                       */
/* ------------------------------------------------------------------ */

/* Query::attr drops dims outside [0, D) (query.cc:87-113); Query::build
 * skips empty / disjoint ranges, clamps to [min,max] and takes the single
 * contiguous span of the covered keys (query.cc:273-333). */
int orc_item_span(const orc_index *ix, int32_t dim, int32_t low, int32_t up,
                  int64_t *start, int64_t *end) {
    *start = *end = 0;
    if (dim < 0 || dim >= ix->n_dims) return 0;
    int32_t mn = ix->dim_min[dim], mx = ix->dim_max[dim];
    if (low > up || low > mx || up < mn) return 0;
    if (low < mn) low = mn;
    if (up > mx) up = mx;
    int64_t k0 = ix->key_base[dim] + ((int64_t)low - mn);
    int64_t k1 = ix->key_base[dim] + ((int64_t)up - mn) + 1;
    *start = ix->key_offsets[k0];
    *end = ix->key_offsets[k1];
    return 1;
}

static int64_t list_size(const orc_index *ix, int32_t dim, int64_t v) {
    /* inv_table::get_posting_list_size (inv_table.cu:164-170) */
    if (v < ix->dim_min[dim] || v > ix->dim_max[dim]) return 0;
    int64_t key = ix->key_base[dim] + (v - ix->dim_min[dim]);
    return ix->key_offsets[key + 1] - ix->key_offsets[key];
}

static int list_contains(const orc_index *ix, int32_t dim, int64_t v) {
    /* inv_table::list_contain (inv_table.cu:173-179) */
    return v <= ix->dim_max[dim] && v >= ix->dim_min[dim];
}

/* Query::apply_adaptive_query_range (query.cc:196-261), one range. */
void orc_adaptive_range(const orc_index *ix, int32_t dim, float sel,
                        int32_t *low, int32_t *up) {
    if (dim < 0 || dim >= ix->n_dims || !(sel > 0.0f)) return;
    float prod = sel * (float)ix->n_objects;     /* float arithmetic, as in the reference */
    uint32_t threshold = (uint32_t)ceilf(prod);
    int64_t lo = *low, hi = *up;
    uint64_t count = 0;
    for (int64_t v = lo; v <= hi; ++v)
        if (list_contains(ix, dim, v)) count += (uint64_t)list_size(ix, dim, v);
    while (count < threshold) {
        if (lo > 0) {
            lo--;
            if (!list_contains(ix, dim, lo)) continue;
            count += (uint64_t)list_size(ix, dim, lo);
        }
        if (!list_contains(ix, dim, hi + 1)) {
            if (lo == 0) break;
        } else {
            hi++;
            count += (uint64_t)list_size(ix, dim, hi);
        }
    }
    *low = (int32_t)lo;
    *up = (int32_t)hi;
}

/* ------------------------------------------------------------------ */
/* Match-count top-k                                                   */
/* ------------------------------------------------------------------ */

int32_t orc_weight_scale(const float *w, int64_t m) {
    float mx = 0.0f;
    for (int64_t i = 0; i < m; ++i) mx = w[i] > mx ? w[i] : mx;
    int e = 0;
    (void)frexp((double)m * (double)mx, &e);   /* any sum of the weights < m*max < 2^e */
    return 31 - e;
}

typedef struct { uint64_t key; } hent;

static void heap_sift_down(uint64_t *h, int64_t n, int64_t i) {
    for (;;) {
        int64_t l = 2 * i + 1, r = l + 1, m = i;
        if (l < n && h[l] < h[m]) m = l;
        if (r < n && h[r] < h[m]) m = r;
        if (m == i) return;
        uint64_t t = h[i]; h[i] = h[m]; h[m] = t;
        i = m;
    }
}

static int cmp_desc_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? 1 : (x > y ? -1 : 0);
}

/* One query: dense per-object accumulation, then the k largest keys
 * key = primary << 32 | (2^32-1 - id): primary desc, id asc.  This is the
 * reference's CPU match oracle (test_compression_query.cu:127-284: dense
 * ++count[id] per listed id, sort by count, take k) with the tie order fixed. */
static int search_one(const orc_index *ix, int64_t m, const int32_t *dim,
                      const int32_t *low, const int32_t *up, const float *w,
                      int weighted, uint32_t k, uint32_t *acc, uint32_t *touched,
                      uint64_t *heap, uint32_t *o_ids, uint32_t *o_cnt, float *o_sc) {
    int32_t s = 0;
    if (weighted) {
        for (int64_t i = 0; i < m; ++i)
            if (!(w[i] > 0.0f) || !isfinite(w[i])) return -2;
        s = orc_weight_scale(w, m);
    }
    int64_t nt = 0;
    for (int64_t i = 0; i < m; ++i) {
        int64_t a, b;
        if (!orc_item_span(ix, dim[i], low[i], up[i], &a, &b)) continue;
        uint32_t inc = 1;
        if (weighted) inc = (uint32_t)llrint(ldexp((double)w[i], s));
        for (int64_t p = a; p < b; ++p) {
            uint32_t id = ix->ids[p];
            if (acc[id] == 0 && inc) touched[nt++] = id;
            acc[id] += inc;
        }
    }
    int64_t hn = 0;
    for (int64_t t = 0; t < nt; ++t) {
        uint32_t id = touched[t];
        uint64_t key = ((uint64_t)acc[id] << 32) | (uint64_t)(0xFFFFFFFFu - id);
        acc[id] = 0;
        if (hn < (int64_t)k) {
            heap[hn++] = key;
            if (hn == (int64_t)k)
                for (int64_t i = hn / 2 - 1; i >= 0; --i) heap_sift_down(heap, hn, i);
        } else if (key > heap[0]) {
            heap[0] = key;
            heap_sift_down(heap, hn, 0);
        }
    }
    qsort(heap, (size_t)hn, sizeof(uint64_t), cmp_desc_u64);
    for (uint32_t j = 0; j < k; ++j) {
        if ((int64_t)j < hn) {
            uint32_t prim = (uint32_t)(heap[j] >> 32);
            uint32_t id = 0xFFFFFFFFu - (uint32_t)(heap[j] & 0xFFFFFFFFu);
            o_ids[j] = id;
            if (weighted) {
                float sc = (float)ldexp((double)prim, -s);
                o_sc[j] = sc;
                o_cnt[j] = (uint32_t)sc;      /* (int) aggregation, knn.cu:54 */
            } else {
                o_cnt[j] = prim;
                o_sc[j] = (float)prim;
            }
        } else {
            o_ids[j] = 0; o_cnt[j] = 0; o_sc[j] = 0.0f;
        }
    }
    return 0;
}

int orc_search(const orc_index *ix, int32_t n_queries, const int64_t *item_off,
               const int32_t *dim, const int32_t *low, const int32_t *up,
               const float *weight, const uint8_t *weighted,
               const uint32_t *k, const int64_t *out_off,
               uint32_t *out_ids, uint32_t *out_counts, float *out_scores,
               int n_threads) {
    if (!ix || n_queries < 0) return -1;
    uint32_t kmax = 0;
    for (int32_t q = 0; q < n_queries; ++q) {
        if (k[q] == 0) return -1;
        if (k[q] > kmax) kmax = k[q];
        if (weighted && weighted[q] && !weight) return -1;
    }
    int err = 0;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
#pragma omp parallel
    {
        uint32_t *acc = (uint32_t *)calloc((size_t)ix->n_objects, sizeof(uint32_t));
        uint32_t *touched = (uint32_t *)malloc((size_t)ix->n_objects * sizeof(uint32_t));
        uint64_t *heap = (uint64_t *)malloc((size_t)(kmax ? kmax : 1) * sizeof(uint64_t));
        if (!acc || !touched || !heap) {
#pragma omp atomic write
            err = -3;
        } else {
#pragma omp for schedule(dynamic, 1)
            for (int32_t q = 0; q < n_queries; ++q) {
                int64_t a = item_off[q], m = item_off[q + 1] - a;
                int wq = weighted ? weighted[q] : 0;
                int r = search_one(ix, m, dim + a, low + a, up + a, weight ? weight + a : NULL,
                                   wq, k[q], acc, touched, heap, out_ids + out_off[q],
                                   out_counts + out_off[q], out_scores + out_off[q]);
                if (r) {
#pragma omp atomic write
                    err = r;
                }
            }
        }
        free(acc); free(touched); free(heap);
    }
    return err;
}

int orc_counts(const orc_index *ix, int64_t m, const int32_t *dim,
               const int32_t *low, const int32_t *up, uint32_t *counts_out) {
    memset(counts_out, 0, (size_t)ix->n_objects * sizeof(uint32_t));
    for (int64_t i = 0; i < m; ++i) {
        int64_t a, b;
        if (!orc_item_span(ix, dim[i], low[i], up[i], &a, &b)) continue;
        for (int64_t p = a; p < b; ++p) counts_out[ix->ids[p]]++;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Codecs                                                              */
/* ------------------------------------------------------------------ */

static uint32_t bits_needed(uint32_t v) { return v ? 32u - (uint32_t)__builtin_clz(v) : 0u; }

/* Lemire-style packing of 32 values at b bits, value j at bit j*b, LSB first
 * (DeviceBitPackingHelpers fastpackwithoutmask / fastunpack layout). */
static void pack32(const uint32_t *in, uint32_t *out, uint32_t b) {
    if (b == 0) return;
    memset(out, 0, b * sizeof(uint32_t));
    for (uint32_t j = 0; j < 32; ++j) {
        uint32_t pos = j * b, w = pos >> 5, sh = pos & 31;
        out[w] |= in[j] << sh;
        if (sh + b > 32) out[w + 1] |= in[j] >> (32 - sh);
    }
}

static void unpack32(const uint32_t *in, uint32_t *out, uint32_t b) {
    for (uint32_t j = 0; j < 32; ++j) {
        if (b == 0) { out[j] = 0; continue; }
        if (b == 32) { out[j] = in[j]; continue; }
        uint32_t pos = j * b, w = pos >> 5, sh = pos & 31;
        uint32_t v = in[w] >> sh;
        if (sh + b > 32) v |= in[w + 1] << (32 - sh);
        out[j] = v & ((1u << b) - 1u);
    }
}

/* DeviceBitPackingCodec::encodeArray (DeviceBitPackingCodec.cu:15-58):
 * [n][w0<<24|w1<<16|w2<<8|w3][w0 words][w1]..[w3] per 128 values; the tail
 * packs ceil(rem/32) zero-padded miniblocks under one more header word. */
static int64_t bp32_encode(const uint32_t *in, int64_t n, uint32_t *out) {
    int64_t o = 0, i = 0;
    out[o++] = (uint32_t)n;
    uint32_t tmp[128];
    while (i < n) {
        int64_t rem = n - i;
        int64_t howmany = rem >= 128 ? 4 : (rem + 31) / 32;
        const uint32_t *src = in + i;
        if (rem < 128) {
            memset(tmp, 0, sizeof(tmp));
            memcpy(tmp, in + i, (size_t)rem * sizeof(uint32_t));
            src = tmp;
        }
        uint32_t B[4] = {0, 0, 0, 0};
        for (int64_t mb = 0; mb < howmany; ++mb) {
            uint32_t acc = 0;
            for (int t = 0; t < 32; ++t) acc |= src[mb * 32 + t];
            B[mb] = bits_needed(acc);
        }
        out[o++] = (B[0] << 24) | (B[1] << 16) | (B[2] << 8) | B[3];
        for (int64_t mb = 0; mb < howmany; ++mb) {
            pack32(src + mb * 32, out + o, B[mb]);
            o += B[mb];
        }
        i += rem >= 128 ? 128 : rem;
    }
    return o;
}

/* DeviceBitPackingCodec::decodeArray (DeviceBitPackingCodec.cu:60-101).
 * *used receives the number of words consumed. */
static int64_t bp32_decode(const uint32_t *in, int64_t n_words, uint32_t *out, int64_t cap,
                           int64_t *used) {
    if (n_words < 1) return -1;
    int64_t n = in[0], p = 1, i = 0;
    if (n > cap) return -1;
    uint32_t tmp[128];
    while (i < n) {
        if (p >= n_words) return -1;
        uint32_t hdr = in[p++];
        uint32_t B[4] = {hdr >> 24, (hdr >> 16) & 255, (hdr >> 8) & 255, hdr & 255};
        int64_t rem = n - i;
        int64_t howmany = rem >= 128 ? 4 : (rem + 31) / 32;
        for (int64_t mb = 0; mb < howmany; ++mb) {
            if (B[mb] > 32 || p + B[mb] > n_words) return -1;
            unpack32(in + p, tmp + mb * 32, B[mb]);
            p += B[mb];
        }
        int64_t take = rem >= 128 ? 128 : rem;
        memcpy(out + i, tmp, (size_t)take * sizeof(uint32_t));
        i += take;
    }
    if (used) *used = p;
    return n;
}

/* DeviceVarintCodec::encodeArray (DeviceVarintCodec.cu:14-78): 7-bit groups,
 * least significant first, the LAST byte of a value has bit 7 set; the byte
 * stream is zero-padded to whole 32-bit words. */
static int64_t varint_encode(const uint32_t *in, int64_t n, uint32_t *out) {
    uint8_t *b = (uint8_t *)out;
    int64_t nb = 0;
    for (int64_t i = 0; i < n; ++i) {
        uint32_t v = in[i];
        int len = v < (1u << 7) ? 1 : v < (1u << 14) ? 2 : v < (1u << 21) ? 3 : v < (1u << 28) ? 4 : 5;
        for (int g = 0; g < len; ++g) {
            uint8_t c = (uint8_t)((v >> (7 * g)) & 0x7F);
            if (g == len - 1) c = (uint8_t)((v >> (7 * g)) | 0x80);
            b[nb++] = c;
        }
    }
    while (nb & 3) b[nb++] = 0;
    return nb / 4;
}

/* DeviceVarintCodec::decodeFromByteArray (DeviceVarintCodec.cu:86-151). */
static int64_t varint_decode(const uint32_t *in, int64_t n_words, uint32_t *out, int64_t cap) {
    const uint8_t *b = (const uint8_t *)in;
    int64_t nb = n_words * 4, o = 0;
    uint32_t v = 0;
    int shift = 0;
    for (int64_t t = 0; t < nb; ++t) {
        uint8_t c = b[t];
        if (shift < 32) v += (uint32_t)(c & 127) << shift;
        shift += 7;
        if (c & 128) {
            if (o >= cap) return -1;
            out[o++] = v;
            v = 0;
            shift = 0;
        }
        if (shift >= 35) shift = 35;      /* malformed: keep shifting out */
    }
    return o;
}

static int64_t enc_simple(int c, const uint32_t *in, int64_t n, uint32_t *out) {
    switch (c) {
    case ORC_COPY: memcpy(out, in, (size_t)n * 4); return n;
    case ORC_DELTA: {   /* DeviceDeltaHelper::delta (DeviceDeltaHelper.h:17-26), init 0 */
        uint32_t prev = 0;
        for (int64_t i = 0; i < n; ++i) { out[i] = in[i] - prev; prev = in[i]; }
        return n;
    }
    case ORC_BP32: return bp32_encode(in, n, out);
    case ORC_VARINT: return varint_encode(in, n, out);
    }
    return -1;
}

static int64_t dec_simple(int c, const uint32_t *in, int64_t nw, uint32_t *out, int64_t cap) {
    switch (c) {
    case ORC_COPY:
        if (nw > cap) return -1;
        memcpy(out, in, (size_t)nw * 4);
        return nw;
    case ORC_DELTA: {
        if (nw > cap) return -1;
        uint32_t acc = 0;
        for (int64_t i = 0; i < nw; ++i) { acc += in[i]; out[i] = acc; }
        return nw;
    }
    case ORC_BP32: {
        int64_t used = 0;
        int64_t r = bp32_decode(in, nw, out, cap, &used);
        return (r >= 0 && used == nw) ? r : -1;
    }
    case ORC_VARINT: return varint_decode(in, nw, out, cap);
    }
    return -1;
}

/* DeviceCompositeCodec::encodeArray (DeviceCompositeCodec.cu:28-58):
 * [len1][BP32 over floor(n/8)*8 values (len1 words)][codec2 over the rest]. */
static int64_t comp_encode(int c2, const uint32_t *in, int64_t n, uint32_t *out) {
    int64_t n1 = (n / 8) * 8, w1 = 0, w2 = 0;
    if (n1) w1 = bp32_encode(in, n1, out + 1);
    if (n - n1) w2 = enc_simple(c2, in + n1, n - n1, out + 1 + w1);
    out[0] = (uint32_t)w1;
    return 1 + w1 + w2;
}

/* DeviceCompositeCodec::decodeArray (DeviceCompositeCodec.cu:60-100). */
static int64_t comp_decode(int c2, const uint32_t *in, int64_t nw, uint32_t *out, int64_t cap) {
    if (nw < 1) return -1;
    int64_t w1 = in[0], n1 = 0;
    if (1 + w1 > nw) return -1;
    if (w1) {
        int64_t used = 0;
        n1 = bp32_decode(in + 1, w1, out, cap, &used);
        if (n1 < 0 || used != w1) return -1;
    }
    int64_t left = nw - 1 - w1;
    if (!left) return n1;
    int64_t n2 = dec_simple(c2, in + 1 + w1, left, out + n1, cap - n1);
    return n2 < 0 ? -1 : n1 + n2;
}

static int64_t enc_c2(int c2, const uint32_t *in, int64_t n, uint32_t *out) {
    if (c2 == ORC_COMP_BP32_COPY) return comp_encode(ORC_COPY, in, n, out);
    if (c2 == ORC_COMP_BP32_VARINT) return comp_encode(ORC_VARINT, in, n, out);
    return enc_simple(c2, in, n, out);
}

static int64_t dec_c2(int c2, const uint32_t *in, int64_t nw, uint32_t *out, int64_t cap) {
    if (c2 == ORC_COMP_BP32_COPY) return comp_decode(ORC_COPY, in, nw, out, cap);
    if (c2 == ORC_COMP_BP32_VARINT) return comp_decode(ORC_VARINT, in, nw, out, cap);
    return dec_simple(c2, in, nw, out, cap);
}

/* Worst-case encoded words: varint needs 5 bytes per value; BP32 packs a
 * zero-padded 32-value miniblock at up to 32 bits even for one value. */
int64_t orc_encode_bound(int64_t n) { return (5 * n) / 4 + 96; }

static void serial_parts(int codec, int *c1, int *c2) {
    switch (codec) {
    case ORC_SERIAL_COPY_COPY: *c1 = ORC_COPY; *c2 = ORC_COPY; break;
    case ORC_SERIAL_DELTA_COPY: *c1 = ORC_DELTA; *c2 = ORC_COPY; break;
    case ORC_SERIAL_DELTA_DELTA: *c1 = ORC_DELTA; *c2 = ORC_DELTA; break;
    case ORC_SERIAL_DELTA_VARINT: *c1 = ORC_DELTA; *c2 = ORC_VARINT; break;
    case ORC_SERIAL_DELTA_BP32: *c1 = ORC_DELTA; *c2 = ORC_BP32; break;
    case ORC_SERIAL_DELTA_COMP_BP32_COPY: *c1 = ORC_DELTA; *c2 = ORC_COMP_BP32_COPY; break;
    case ORC_SERIAL_DELTA_COMP_BP32_VARINT: *c1 = ORC_DELTA; *c2 = ORC_COMP_BP32_VARINT; break;
    default: *c1 = *c2 = -1;
    }
}

/* DeviceSerialCodec::encodeArray (DeviceSerialCodec.cu:47-64): codec1 then
 * codec2 on codec1's output; decodeArray runs them in reverse (:67-96). */
int64_t orc_encode(int codec, const uint32_t *in, int64_t n, uint32_t *out, int64_t cap) {
    if (n <= 0 || !in || !out) return -1;
    if (cap < orc_encode_bound(n)) return -1;
    if (codec >= ORC_COPY && codec <= ORC_VARINT) return enc_simple(codec, in, n, out);
    if (codec == ORC_COMP_BP32_COPY || codec == ORC_COMP_BP32_VARINT) return enc_c2(codec, in, n, out);
    int c1, c2;
    serial_parts(codec, &c1, &c2);
    if (c1 < 0) return -1;
    uint32_t *mid = (uint32_t *)malloc((size_t)orc_encode_bound(n) * 4);
    if (!mid) return -1;
    int64_t m = enc_simple(c1, in, n, mid);
    int64_t r = enc_c2(c2, mid, m, out);
    free(mid);
    return r;
}

int64_t orc_decode(int codec, const uint32_t *in, int64_t n_words, uint32_t *out, int64_t cap) {
    if (n_words <= 0 || !in || !out) return -1;
    if (codec >= ORC_COPY && codec <= ORC_VARINT) return dec_simple(codec, in, n_words, out, cap);
    if (codec == ORC_COMP_BP32_COPY || codec == ORC_COMP_BP32_VARINT) return dec_c2(codec, in, n_words, out, cap);
    int c1, c2;
    serial_parts(codec, &c1, &c2);
    if (c1 < 0) return -1;
    uint32_t *mid = (uint32_t *)malloc((size_t)(cap + 16) * 4);
    if (!mid) return -1;
    int64_t m = dec_c2(c2, in, n_words, mid, cap);
    int64_t r = m < 0 ? -1 : dec_simple(c1, mid, m, out, cap);
    free(mid);
    return r;
}

/* inv_table::build with load balance (inv_table.cu:306-312) cuts each key's
 * list into max_len chunks; inv_compr_table::build (inv_compr_table.cu:30-119)
 * encodes every chunk independently. */
int orc_compress_index(const orc_index *ix, int codec, int32_t max_len, orc_compr_index *cx) {
    memset(cx, 0, sizeof(*cx));
    if (max_len <= 0 || codec <= 0 || codec >= ORC_N_CODECS) return -1;
    int64_t n_keys = ix->key_base[ix->n_dims];
    cx->codec = codec;
    cx->max_len = max_len;
    cx->key_seg = (int64_t *)calloc((size_t)n_keys + 1, sizeof(int64_t));
    int64_t n_segs = 0;
    for (int64_t kk = 0; kk < n_keys; ++kk) {
        int64_t len = ix->key_offsets[kk + 1] - ix->key_offsets[kk];
        cx->key_seg[kk] = n_segs;
        n_segs += (len + max_len - 1) / max_len;
    }
    cx->key_seg[n_keys] = n_segs;
    cx->n_segs = n_segs;
    cx->seg_word_off = (int64_t *)calloc((size_t)n_segs + 1, sizeof(int64_t));
    cx->seg_first = (uint32_t *)calloc((size_t)(n_segs ? n_segs : 1), sizeof(uint32_t));
    cx->seg_len = (uint32_t *)calloc((size_t)(n_segs ? n_segs : 1), sizeof(uint32_t));
    int64_t cap = 0;
    for (int64_t kk = 0; kk < n_keys; ++kk)
        for (int64_t p = ix->key_offsets[kk]; p < ix->key_offsets[kk + 1]; p += max_len) {
            int64_t len = ix->key_offsets[kk + 1] - p;
            cap += orc_encode_bound(len > max_len ? max_len : len);
        }
    cx->words = (uint32_t *)malloc((size_t)cap * 4 + 64);
    if (!cx->key_seg || !cx->seg_word_off || !cx->seg_first || !cx->seg_len || !cx->words) return -1;
    int64_t w = 0, s = 0;
    for (int64_t kk = 0; kk < n_keys; ++kk) {
        for (int64_t p = ix->key_offsets[kk]; p < ix->key_offsets[kk + 1]; p += max_len) {
            int64_t len = ix->key_offsets[kk + 1] - p;
            if (len > max_len) len = max_len;
            cx->seg_word_off[s] = w;
            cx->seg_first[s] = ix->ids[p];
            cx->seg_len[s] = (uint32_t)len;
            int64_t r = orc_encode(codec, ix->ids + p, len, cx->words + w, cap - w);
            if (r <= 0) return -1;
            w += r;
            ++s;
        }
    }
    cx->seg_word_off[s] = w;
    cx->n_words = w;
    return 0;
}

void orc_compr_index_free(orc_compr_index *cx) {
    if (!cx) return;
    free(cx->key_seg); free(cx->seg_word_off); free(cx->seg_first);
    free(cx->seg_len); free(cx->words);
    memset(cx, 0, sizeof(*cx));
}

/* test/test_compression_codecs.cu:174-199: five magnitude classes drawn from
 * glibc rand() after srand(seed). */
void orc_codec_kat_input(uint32_t seed, uint32_t *out, int64_t n) {
    srand(seed);
    for (int64_t i = 0; i < n; ++i) {
        switch (rand() % 5) {
        case 0: out[i] = (uint32_t)((long)rand() % (1 << 7)); break;
        case 1: out[i] = (uint32_t)(((long)rand() + (1 << 7)) % (1 << 15)); break;
        case 2: out[i] = (uint32_t)(((long)rand() + (1 << 14)) % (1 << 22)); break;
        case 3: out[i] = (uint32_t)(((long)rand() + (1 << 21)) % (1 << 28)); break;
        default: out[i] = (uint32_t)((long)rand() + (1 << 28)); break;
        }
    }
}
