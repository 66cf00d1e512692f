"""GB300-native GENIE match-count top-k search -- Python host mirror.

This mirrors the reference's first- and second-level interface
(src/genie/interface/{config,execution_policy,search,io,types}.h) over the C
ABI of libgenie_gb300.so:

    cfg = genie_gb300.Config().SetK(5).SetNumOfQueries(3)
    policy = genie_gb300.MakePolicy(cfg)
    ids, counts = genie_gb300.Search(policy, "table.csv", "query.csv")

Results are (ids, counts) lists of length num_queries*k, row-major, sorted by
(count desc, id asc) and padded with (0, 0).
"""
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import GenieQueries, GenieIndexInfo

__all__ = [
    "Config", "MakePolicy", "ExecutionPolicy", "Search", "BuildTable", "BuildQuery", "Match",
    "LoadTableDataFromCsv", "LoadQueryDataFromCsv", "LoadTableFromBinary", "SaveTableToBinary",
    "Table", "Query", "QueryBatch", "Batch", "Server", "poisson_arrivals", "search", "lib",
    "NotImplementedException", "InvalidConfigurationException", "gpu_bad_alloc", "gpu_runtime_error",
    "cpu_bad_alloc", "cpu_runtime_error",
]


# ---------------------------------------------------------------- exceptions
# src/genie/exception/exception.h:10-46
class NotImplementedException(RuntimeError):
    def __init__(self, what="Function is not implemented"):
        super().__init__(what)


class InvalidConfigurationException(ValueError):
    pass


class gpu_bad_alloc(MemoryError):
    pass


class gpu_runtime_error(RuntimeError):
    pass


class cpu_bad_alloc(MemoryError):
    pass


class cpu_runtime_error(RuntimeError):
    pass


_ERR = {1: cpu_runtime_error, 2: gpu_bad_alloc, 3: gpu_runtime_error, 4: NotImplementedException,
        5: cpu_bad_alloc, 6: gpu_runtime_error, 7: cpu_runtime_error, 8: gpu_bad_alloc}


def lib():
    return _lib.load()


def _check(rc):
    if rc != 0:
        msg = lib().genie_last_error().decode(errors="replace")
        exc = _ERR.get(rc, gpu_runtime_error)
        if exc is NotImplementedException:
            raise NotImplementedException(msg or "Function is not implemented")
        raise exc(msg)


def _ptr(a):
    return None if a is None else a.ctypes.data


# ---------------------------------------------------------------- index

class Table:
    """A resident inverted index (the reference's inv_table after
    cpy_data_to_gpu).  Owns a genie_index handle."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)
        self._info = None

    BUILDERS = {"auto": 0, "host": 1, "device": 2}

    @classmethod
    def from_values(cls, values, builder="auto"):
        """builder: "auto" (on the device when every dim spans <= 16384
        values, else on the host), "host" or "device"."""
        values = np.ascontiguousarray(values, dtype=np.int32)
        if values.ndim != 2 or values.size == 0:
            raise cpu_runtime_error("no data input!")
        h = ctypes.c_void_p()
        _check(lib().genie_index_create_with(values.ctypes.data, values.shape[0], values.shape[1],
                                             cls.BUILDERS[builder], ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def from_bag(cls, rows):
        """Single-dim bag index: every value of row r lists r (load_table_bijectMap)."""
        vals = np.concatenate([np.asarray(r, np.int32) for r in rows]) if rows else np.zeros(0, np.int32)
        off = np.zeros(len(rows) + 1, np.int64)
        off[1:] = np.cumsum([len(r) for r in rows])
        return cls.from_bag_arrays(vals, off)

    @classmethod
    def from_bag_arrays(cls, values, row_off):
        values = np.ascontiguousarray(values, np.int32)
        row_off = np.ascontiguousarray(row_off, np.int64)
        h = ctypes.c_void_p()
        _check(lib().genie_index_create_bag(values.ctypes.data, row_off.ctypes.data, len(row_off) - 1,
                                            ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def compressed(cls, values, codec, max_segment=1024):
        values = np.ascontiguousarray(values, dtype=np.int32)
        h = ctypes.c_void_p()
        _check(lib().genie_index_create_compressed(values.ctypes.data, values.shape[0], values.shape[1],
                                                   int(codec), int(max_segment), ctypes.byref(h)))
        return cls(h.value)

    @property
    def handle(self):
        return self._h

    def info(self):
        if self._info is None:
            inf = GenieIndexInfo()
            _check(lib().genie_index_get_info(self._h, ctypes.byref(inf)))
            self._info = inf
        return self._info

    def i_size(self):
        """Number of objects (inv_table::i_size)."""
        return int(self.info().n_objects)

    def m_size(self):
        """Number of dims (inv_table::m_size)."""
        return int(self.info().n_dims)

    def inv(self):
        """Device posting array copied back (inv_table::inv / d_inv_p)."""
        n = int(self.info().n_ids)
        out = np.zeros(n, np.uint32)
        _check(lib().genie_index_copy_out(self._h, out.ctypes.data, None, None, None, None))
        return out

    def layout(self):
        inf = self.info()
        ko = np.zeros(inf.n_keys + 1, np.int64)
        kb = np.zeros(inf.n_dims + 1, np.int64)
        mn = np.zeros(inf.n_dims, np.int32)
        mx = np.zeros(inf.n_dims, np.int32)
        _check(lib().genie_index_copy_out(self._h, None, ko.ctypes.data, kb.ctypes.data, mn.ctypes.data,
                                          mx.ctypes.data))
        return dict(key_offsets=ko, key_base=kb, dim_min=mn, dim_max=mx)

    def ids(self):
        """The device posting array (ids ordered by (dim, value, id))."""
        inf = self.info()
        out = np.zeros(max(1, inf.n_ids), np.uint32)
        _check(lib().genie_index_copy_out(self._h, out.ctypes.data, None, None, None, None))
        return out[: inf.n_ids]

    def compressed_layout(self):
        inf = self.info()
        words = np.zeros(max(1, inf.n_words), np.uint32)
        key_seg = np.zeros(inf.n_keys + 1, np.int64)
        seg_word_off = np.zeros(inf.n_segments + 1, np.int64)
        seg_first = np.zeros(max(1, inf.n_segments), np.uint32)
        seg_len = np.zeros(max(1, inf.n_segments), np.uint32)
        _check(lib().genie_index_copy_compressed(self._h, words.ctypes.data, key_seg.ctypes.data,
                                                 seg_word_off.ctypes.data, seg_first.ctypes.data,
                                                 seg_len.ctypes.data))
        return dict(words=words[: inf.n_words], key_seg=key_seg, seg_word_off=seg_word_off,
                    seg_first=seg_first[: inf.n_segments], seg_len=seg_len[: inf.n_segments])

    def span(self, dim, low, up):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        _check(lib().genie_index_item_span(self._h, dim, low, up, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def adaptive_range(self, dim, selectivity, low, up):
        lo, hi = ctypes.c_int32(low), ctypes.c_int32(up)
        _check(lib().genie_index_adaptive_range(self._h, dim, ctypes.c_float(selectivity), ctypes.byref(lo),
                                                ctypes.byref(hi)))
        return lo.value, hi.value

    def save(self, path):
        _check(lib().genie_index_save(self._h, os.fsencode(path)))

    @classmethod
    def load(cls, path):
        h = ctypes.c_void_p()
        _check(lib().genie_index_load(os.fsencode(path), ctypes.byref(h)))
        return cls(h.value)

    def close(self):
        if self._h is not None and self._h.value:
            lib().genie_index_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- queries

class QueryBatch:
    """Flat SoA query batch (genie_queries).  Query q owns items
    [item_off[q], item_off[q+1]); k is a scalar or one value per query."""

    def __init__(self, item_off, dim, low, up, k, weight=None, weighted=None):
        self.item_off = np.ascontiguousarray(item_off, np.int64)
        self.dim = np.ascontiguousarray(dim, np.int32)
        self.low = np.ascontiguousarray(low, np.int32)
        self.up = np.ascontiguousarray(up, np.int32)
        self.n_queries = len(self.item_off) - 1
        if np.isscalar(k):
            self.k = None
            self.uniform_k = int(k)
            self.k_array = np.full(self.n_queries, int(k), np.uint32)
        else:
            self.k = np.ascontiguousarray(k, np.uint32)
            self.uniform_k = 0
            self.k_array = self.k
        self.weight = None if weight is None else np.ascontiguousarray(weight, np.float32)
        self.weighted = None if weighted is None else np.ascontiguousarray(weighted, np.uint8)
        self.out_off = np.zeros(self.n_queries + 1, np.int64)
        np.cumsum(self.k_array, out=self.out_off[1:])

    @property
    def total_k(self):
        return int(self.out_off[-1])

    def struct(self):
        s = GenieQueries()
        s.n_queries = self.n_queries
        s.item_off = _ptr(self.item_off)
        s.dim, s.low, s.up = _ptr(self.dim), _ptr(self.low), _ptr(self.up)
        s.weight = _ptr(self.weight)
        s.weighted = _ptr(self.weighted)
        s.k = _ptr(self.k)
        s.uniform_k = self.uniform_k
        return s

    def as_oracle_batch(self):
        return dict(item_off=self.item_off, dim=self.dim, low=self.low, up=self.up, k=self.k_array,
                    weight=self.weight, weighted=self.weighted)

    @classmethod
    def from_queries(cls, queries):
        off, dim, low, up, w, wf, ks = [0], [], [], [], [], [], []
        for q in queries:
            for r in q.ranges:
                dim.append(r[0]); low.append(r[1]); up.append(r[2]); w.append(r[3])
            off.append(len(dim))
            wf.append(1 if q.weighted else 0)
            ks.append(q.topk())
        return cls(off, dim, low, up, np.array(ks, np.uint32), np.array(w, np.float32), np.array(wf, np.uint8))


def search(table, batch, scores=False):
    """Plain per-batch search (genie_search).  Returns (ids, counts[, scores])."""
    ids = np.zeros(max(1, batch.total_k), np.uint32)
    cnt = np.zeros(max(1, batch.total_k), np.uint32)
    sc = np.zeros(max(1, batch.total_k), np.float32) if scores else None
    s = batch.struct()
    _check(lib().genie_search(table.handle, ctypes.byref(s), ids.ctypes.data, cnt.ctypes.data, _ptr(sc)))
    n = batch.total_k
    if scores:
        return ids[:n], cnt[:n], sc[:n]
    return ids[:n], cnt[:n]


class Query:
    """One query: ranges (dim, low, up, weight) (query/query.h:43-54)."""

    def __init__(self, table, index=0):
        self.table = table
        self.index = index
        self.ranges = []
        self._topk = 0
        self._selectivity = -1.0
        self.weighted = False

    def attr(self, dim, low, up=None, weight=1.0, selectivity=-1.0, order=0):
        # Query::attr drops dims outside [0, m_size) (query.cc:93-94)
        if up is None:
            up = low
        if dim < 0 or dim >= self.table.m_size():
            return
        self.ranges.append([int(dim), int(low), int(up), float(weight), float(selectivity)])

    def topk(self, k=None):
        if k is None:
            return self._topk
        self._topk = int(k)

    def selectivity(self, s=None):
        if s is None:
            return self._selectivity
        self._selectivity = float(s)

    def count_ranges(self):
        return len(self.ranges)

    def apply_adaptive_query_range(self):
        """query.cc:196-261 -- per-range selectivity, else the query's."""
        for r in self.ranges:
            sel = r[4] if r[4] > 0 else self._selectivity
            if sel > 0:
                r[1], r[2] = self.table.adaptive_range(r[0], sel, r[1], r[2])


# ---------------------------------------------------------------- config / policy

class Config:
    """genie::Config (interface/config.h:20-95)."""

    def __init__(self):
        self._k = None
        self._query_range = None
        self._num_queries = None
        self._save_to_gpu = False
        self._gpu_id = 0

    def SetK(self, k):
        self._k = int(k)
        return self

    def SetQueryRange(self, r):
        self._query_range = int(r)
        return self

    def SetNumOfQueries(self, n):
        self._num_queries = int(n)
        return self

    def SetSaveToGpu(self, b):
        self._save_to_gpu = bool(b)
        return self

    def SetGpuId(self, g):
        self._gpu_id = int(g)
        return self

    def LoadFromFile(self, filename):
        raise NotImplementedException()

    def GetK(self):
        return self._k

    def GetQueryRange(self):
        return self._query_range

    def GetNumOfQueries(self):
        return self._num_queries

    def GetSaveToGpu(self):
        return self._save_to_gpu

    def GetGpuId(self):
        return self._gpu_id

    def IsKSet(self):
        return self._k is not None

    def IsQueryRangeSet(self):
        return self._query_range is not None

    def IsNumOfQueriesSet(self):
        return self._num_queries is not None

    def Validate(self):
        if not self.IsKSet():
            raise InvalidConfigurationException("K is not set.")
        if not self.IsNumOfQueriesSet():
            raise InvalidConfigurationException("Number of query is not set.")


class ExecutionPolicy:
    """genie::ExecutionPolicy (interface/execution_policy.h:21-71)."""

    query_range = 0

    def __init__(self, k, num_queries):
        self.k = k
        self.num_queries = num_queries
        self.dim = 0

    def GetNumOfQueries(self):
        return self.num_queries

    def Validate(self):
        # execution_policy/validation.cc:7-23
        if self.k <= 0:
            raise InvalidConfigurationException("K should be larger than 0.")
        if self.num_queries <= 0:
            raise InvalidConfigurationException("Number of query should be larger than 0.")

    def BuildTable(self, table_data):
        """single_value.cc:10-15: dim = width of the first row."""
        if len(table_data) == 0:
            raise cpu_runtime_error("no data input!")
        self.dim = len(table_data[0])
        return Table.from_values(np.asarray(table_data, np.int32))

    def BuildQuery(self, table, query_data):
        """load_query_singlerange (original/interface.cc:473-517): item j of row i
        matches [v-r, v+r] on dim j for j < dim, weight 1."""
        queries = []
        d = table.m_size()
        r = self.query_range
        for i, row in enumerate(query_data):
            q = Query(table, i)
            for j, v in enumerate(row):
                if j >= d:
                    break
                q.attr(j, v - r, v + r, 1.0, -1.0, j)
            q.topk(self.k)
            queries.append(q)
        return queries

    def Match(self, table, queries):
        if isinstance(table, (list, tuple)):
            raise NotImplementedException()
        if not queries:
            raise cpu_runtime_error("Queries not loaded!")
        batch = QueryBatch.from_queries(queries)
        ids, cnt = search(table, batch)
        return ids.astype(np.int64).tolist(), cnt.astype(np.int64).tolist()


class SingleValueExecutionPolicy(ExecutionPolicy):
    query_range = 0


class SingleRangeExecutionPolicy(ExecutionPolicy):
    def __init__(self, k, num_queries, query_range):
        super().__init__(k, num_queries)
        self.query_range = query_range

    def Validate(self):
        super().Validate()
        if self.query_range <= 0:
            raise InvalidConfigurationException("Query range should be larger than 0.")


def MakePolicy(config):
    """interface/execution_policy.cc:14-45."""
    config.Validate()
    if config.IsQueryRangeSet():
        p = SingleRangeExecutionPolicy(config.GetK(), config.GetNumOfQueries(), config.GetQueryRange())
    else:
        p = SingleValueExecutionPolicy(config.GetK(), config.GetNumOfQueries())
    p.Validate()
    _check(lib().genie_init(config.GetGpuId()))
    return p


def _read_rows(filename, num=-1):
    """utility::read_file (FileReader.cc:54-83): tokens split on ',' and ' '."""
    rows = []
    if not os.path.exists(filename):
        return rows
    with open(filename) as f:
        for line in f:
            if 0 <= num <= len(rows):
                break
            toks = [t for t in line.replace(",", " ").split() if t]
            rows.append([int(t) for t in toks])
    return rows


def LoadTableDataFromCsv(filename):
    return _read_rows(filename, -1)


def LoadQueryDataFromCsv(filename, policy):
    return _read_rows(filename, policy.GetNumOfQueries())


def LoadTableFromBinary(filename):
    return Table.load(filename)


def SaveTableToBinary(filename, table):
    table.save(filename)


def BuildTable(policy, table_data):
    return policy.BuildTable(table_data)


def BuildQuery(policy, table, query_data):
    return policy.BuildQuery(table, query_data)


def Match(policy, table, queries):
    return policy.Match(table, queries)


def Search(policy, table_filename, query_filename):
    """1st-level interface (interface/search.cc:11-22)."""
    table_data = LoadTableDataFromCsv(table_filename)
    query_data = LoadQueryDataFromCsv(query_filename, policy)
    table = BuildTable(policy, table_data)
    queries = BuildQuery(policy, table, query_data)
    return Match(policy, table, queries)


from .batch import Batch  # noqa: E402
from .serve import Server, poisson_arrivals  # noqa: E402
from . import shard  # noqa: E402,F401
