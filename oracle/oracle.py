"""ctypes binding of the CPU oracle (oracle/genie_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product library never loads
it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_CODECS = os.path.join(HERE, "_ref", "libref_codecs.so")

CODECS = {
    "COPY": 1, "DELTA": 2, "BP32": 3, "VARINT": 4, "COMP_BP32_COPY": 5,
    "COMP_BP32_VARINT": 6, "SERIAL_COPY_COPY": 7, "SERIAL_DELTA_COPY": 8,
    "SERIAL_DELTA_DELTA": 9, "SERIAL_DELTA_VARINT": 10, "SERIAL_DELTA_BP32": 11,
    "SERIAL_DELTA_COMP_BP32_COPY": 12, "SERIAL_DELTA_COMP_BP32_VARINT": 13,
}


def build(force=False):
    """Compile liboracle.so with gcc (seconds)."""
    src = os.path.join(HERE, "genie_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


class _Index(ctypes.Structure):
    _fields_ = [
        ("n_dims", ctypes.c_int32), ("n_objects", ctypes.c_int64), ("n_ids", ctypes.c_int64),
        ("dim_min", ctypes.POINTER(ctypes.c_int32)), ("dim_max", ctypes.POINTER(ctypes.c_int32)),
        ("key_base", ctypes.POINTER(ctypes.c_int64)), ("key_offsets", ctypes.POINTER(ctypes.c_int64)),
        ("ids", ctypes.POINTER(ctypes.c_uint32)),
    ]


class _ComprIndex(ctypes.Structure):
    _fields_ = [
        ("codec", ctypes.c_int32), ("max_len", ctypes.c_int32), ("n_segs", ctypes.c_int64),
        ("n_words", ctypes.c_int64), ("key_seg", ctypes.POINTER(ctypes.c_int64)),
        ("seg_word_off", ctypes.POINTER(ctypes.c_int64)), ("seg_first", ctypes.POINTER(ctypes.c_uint32)),
        ("seg_len", ctypes.POINTER(ctypes.c_uint32)), ("words", ctypes.POINTER(ctypes.c_uint32)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        _lib.orc_index_build.argtypes = [P, ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(_Index)]
        _lib.orc_index_build_bag.argtypes = [P, P, ctypes.c_int64, ctypes.POINTER(_Index)]
        _lib.orc_index_free.argtypes = [ctypes.POINTER(_Index)]
        _lib.orc_item_span.argtypes = [ctypes.POINTER(_Index), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
        _lib.orc_adaptive_range.argtypes = [ctypes.POINTER(_Index), ctypes.c_int32, ctypes.c_float,
                                            ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
        _lib.orc_search.argtypes = [ctypes.POINTER(_Index), ctypes.c_int32, P, P, P, P, P, P, P, P, P, P, P,
                                    ctypes.c_int]
        _lib.orc_counts.argtypes = [ctypes.POINTER(_Index), ctypes.c_int64, P, P, P, P]
        _lib.orc_encode.restype = ctypes.c_int64
        _lib.orc_encode.argtypes = [ctypes.c_int, P, ctypes.c_int64, P, ctypes.c_int64]
        _lib.orc_decode.restype = ctypes.c_int64
        _lib.orc_decode.argtypes = [ctypes.c_int, P, ctypes.c_int64, P, ctypes.c_int64]
        _lib.orc_compress_index.argtypes = [ctypes.POINTER(_Index), ctypes.c_int, ctypes.c_int32,
                                            ctypes.POINTER(_ComprIndex)]
        _lib.orc_compr_index_free.argtypes = [ctypes.POINTER(_ComprIndex)]
        _lib.orc_codec_kat_input.argtypes = [ctypes.c_uint32, P, ctypes.c_int64]
        _lib.orc_weight_scale.restype = ctypes.c_int32
        _lib.orc_weight_scale.argtypes = [P, ctypes.c_int64]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class Index:
    """CSR inverted index built by the oracle."""

    def __init__(self, values=None, bag=None):
        self._s = _Index()
        L = lib()
        if bag is not None:
            vals, row_off = bag
            vals = np.ascontiguousarray(vals, np.int32)
            row_off = np.ascontiguousarray(row_off, np.int64)
            rc = L.orc_index_build_bag(_p(vals), _p(row_off), len(row_off) - 1, ctypes.byref(self._s))
        else:
            values = np.ascontiguousarray(values, np.int32)
            n, d = values.shape
            rc = L.orc_index_build(_p(values), n, d, ctypes.byref(self._s))
        if rc != 0:
            raise ValueError("oracle index build failed")
        s = self._s
        self.n_dims = s.n_dims
        self.n_objects = s.n_objects
        self.dim_min = _arr(s.dim_min, s.n_dims, np.int32)
        self.dim_max = _arr(s.dim_max, s.n_dims, np.int32)
        self.key_base = _arr(s.key_base, s.n_dims + 1, np.int64)
        self.key_offsets = _arr(s.key_offsets, int(self.key_base[-1]) + 1, np.int64)
        self.ids = _arr(s.ids, s.n_ids, np.uint32)

    def __del__(self):
        try:
            lib().orc_index_free(ctypes.byref(self._s))
        except Exception:
            pass

    def span(self, dim, low, up):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        lib().orc_item_span(ctypes.byref(self._s), dim, low, up, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def adaptive_range(self, dim, sel, low, up):
        lo, hi = ctypes.c_int32(low), ctypes.c_int32(up)
        lib().orc_adaptive_range(ctypes.byref(self._s), dim, ctypes.c_float(sel), ctypes.byref(lo), ctypes.byref(hi))
        return lo.value, hi.value

    def search(self, batch, n_threads=0):
        """batch: dict with item_off, dim, low, up, [weight, weighted], k (array).
        Returns (ids, counts, scores, out_off)."""
        q = len(batch["item_off"]) - 1
        k = np.ascontiguousarray(batch["k"], np.uint32)
        out_off = np.zeros(q + 1, np.int64)
        np.cumsum(k, out=out_off[1:])
        tot = int(out_off[-1])
        ids = np.zeros(tot, np.uint32)
        cnt = np.zeros(tot, np.uint32)
        sc = np.zeros(tot, np.float32)
        item_off = np.ascontiguousarray(batch["item_off"], np.int64)
        dim = np.ascontiguousarray(batch["dim"], np.int32)
        low = np.ascontiguousarray(batch["low"], np.int32)
        up = np.ascontiguousarray(batch["up"], np.int32)
        w = batch.get("weight")
        wf = batch.get("weighted")
        w = None if w is None else np.ascontiguousarray(w, np.float32)
        wf = None if wf is None else np.ascontiguousarray(wf, np.uint8)
        rc = lib().orc_search(ctypes.byref(self._s), q, _p(item_off), _p(dim), _p(low), _p(up), _p(w), _p(wf),
                              _p(k), _p(out_off), _p(ids), _p(cnt), _p(sc), n_threads)
        if rc != 0:
            raise ValueError("oracle search failed (%d)" % rc)
        return ids, cnt, sc, out_off

    def counts(self, dim, low, up):
        out = np.zeros(self.n_objects, np.uint32)
        dim = np.ascontiguousarray(dim, np.int32)
        low = np.ascontiguousarray(low, np.int32)
        up = np.ascontiguousarray(up, np.int32)
        lib().orc_counts(ctypes.byref(self._s), len(dim), _p(dim), _p(low), _p(up), _p(out))
        return out

    def compress(self, codec, max_len):
        c = _ComprIndex()
        if lib().orc_compress_index(ctypes.byref(self._s), codec, max_len, ctypes.byref(c)) != 0:
            raise ValueError("oracle compression failed")
        nk = int(self.key_base[-1])
        out = dict(
            codec=codec, max_len=max_len,
            key_seg=_arr(c.key_seg, nk + 1, np.int64),
            seg_word_off=_arr(c.seg_word_off, c.n_segs + 1, np.int64),
            seg_first=_arr(c.seg_first, c.n_segs, np.uint32),
            seg_len=_arr(c.seg_len, c.n_segs, np.uint32),
            words=_arr(c.words, c.n_words, np.uint32),
        )
        lib().orc_compr_index_free(ctypes.byref(c))
        return out


def encode(codec, values):
    values = np.ascontiguousarray(values, np.uint32)
    cap = (5 * len(values)) // 4 + 96
    out = np.zeros(cap, np.uint32)
    n = lib().orc_encode(codec, _p(values), len(values), _p(out), cap)
    if n < 0:
        raise ValueError("encode failed")
    return out[:n].copy()


def decode(codec, words, cap):
    words = np.ascontiguousarray(words, np.uint32)
    out = np.zeros(cap + 16, np.uint32)
    n = lib().orc_decode(codec, _p(words), len(words), _p(out), cap)
    if n < 0:
        raise ValueError("decode failed")
    return out[:n].copy()


def kat_input(n, seed=666):
    out = np.zeros(n, np.uint32)
    lib().orc_codec_kat_input(seed, _p(out), n)
    return out


def weight_scale(w):
    w = np.ascontiguousarray(w, np.float32)
    return lib().orc_weight_scale(_p(w), len(w))


def ref_codecs():
    """The reference's own host codecs (oracle/_ref), or None where absent."""
    if not os.path.exists(REF_CODECS):
        return None
    r = ctypes.CDLL(REF_CODECS)
    r.ref_encode.restype = ctypes.c_int64
    r.ref_encode.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64]
    r.ref_decode.restype = ctypes.c_int64
    r.ref_decode.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64]
    return r


def _topk(counts, k):
    """(ids, counts) of the k largest counts, ties by ascending id, padded (0, 0)."""
    items = sorted(((c, i) for i, c in counts.items() if c > 0), key=lambda t: (-t[0], t[1]))[:k]
    ids = [i for _, i in items] + [0] * (k - len(items))
    cnt = [c for c, _ in items] + [0] * (k - len(items))
    return ids, cnt


def subsequence_search(rows, queries, k, radius=0):
    """Subsequence search over rows of values, small cases only.  The object
    of row r at offset o is r << bits | o, bits the least with 2^bits >= the
    longest row (inv_list::invert_subsequence, table/inv_list.cc:193-235);
    item j of a query ([v - radius, v + radius] of the query's j-th value)
    adds 1 to object (r, s) when row r holds a value of that range at offset
    s + j (the offset shift of match_AT, matching/match.cu:84-94).  Returns
    (ids, counts) row-major, k slots per query."""
    longest = max(len(r) for r in rows)
    bits = 0
    while (1 << bits) < longest:
        bits += 1
    out_ids, out_cnt = [], []
    for q in queries:
        counts = {}
        for j, v in enumerate(q):
            lo, hi = v - radius, v + radius
            for r, row in enumerate(rows):
                for p, x in enumerate(row):
                    if p >= j and lo <= x <= hi:
                        key = (r << bits) | (p - j)
                        counts[key] = counts.get(key, 0) + 1
        ids, cnt = _topk(counts, k)
        out_ids += ids
        out_cnt += cnt
    return np.array(out_ids, np.int64), np.array(out_cnt, np.int64), bits


def _grams(seq, base, g):
    """sequence_to_gram for one sequence (original/interface.cc:930-975)."""
    n = len(seq)
    if n == 0:
        return []
    if n - g + 1 <= 0:
        num = 0
        for p in range(g):
            num = num * base + (seq[p] if p < n else seq[0])
        return [num]
    out = []
    for j in range(n - g + 1):
        num = 0
        for t in range(g):
            num = num * base + seq[j + t]
        out.append(num)
    return out


def _mark(grams, bits, keep_capped):
    """The k-th repeat of a gram in one row marked in the low bits, capped at
    2^bits - 1: kept at the cap on the table side (inv_list.cc:107-121),
    dropped on the query side (original/interface.cc:552-566)."""
    seen, out, cap = {}, [], (1 << bits) - 1
    for x in grams:
        if x not in seen:
            seen[x] = 0
            out.append(x << bits)
        elif seen[x] < cap:
            seen[x] += 1
            out.append((x << bits) + seen[x])
        elif keep_capped:
            out.append((x << bits) + cap)
    return out


def sequence_search(rows, queries, k, gram_length=3, bits=6):
    """Sequence (gram) search, small cases only: values reduced by the table
    minimum, grams of gram_length values, repeats marked; the count of row r
    is the number of the query's marked grams that r holds, with multiplicity
    (load_table_sequence / load_query_sequence, original/interface.cc:519-616,
    678-757).  Returns (ids, counts) row-major, k slots per query."""
    mn = min(min(r) for r in rows if len(r))
    mx = max(max(r) for r in rows if len(r))
    base = mx - mn + 1
    table = [_mark(_grams([v - mn for v in r], base, gram_length), bits, True) for r in rows]
    out_ids, out_cnt = [], []
    for q in queries:
        qv = _mark(_grams([v - mn for v in q if mn <= v <= mx], base, gram_length), bits, False)
        counts = {}
        for r, marked in enumerate(table):
            c = sum(marked.count(v) for v in qv)
            if c:
                counts[r] = c
        ids, cnt = _topk(counts, k)
        out_ids += ids
        out_cnt += cnt
    return np.array(out_ids, np.int64), np.array(out_cnt, np.int64)
