"""ctypes binding of libgenie_gb300.so (the C ABI of include/genie_gb300.h).

The CUDA library is the only implementation: if it cannot be loaded, every
call raises.  There is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgenie_gb300.so")

P = ctypes.c_void_p
I32, I64, U32, F32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32, ctypes.c_float


class GenieQueries(ctypes.Structure):
    _fields_ = [("n_queries", I32), ("item_off", P), ("dim", P), ("low", P), ("up", P),
                ("weight", P), ("weighted", P), ("k", P), ("uniform_k", U32)]


class GenieIndexInfo(ctypes.Structure):
    _fields_ = [("n_objects", I64), ("n_dims", I32), ("codec", I32), ("n_ids", I64), ("n_keys", I64),
                ("n_words", I64), ("n_segments", I64), ("max_multiplicity", I32), ("max_segment", I32),
                ("device_bytes", I64)]


class GenieBatchConfig(ctypes.Structure):
    _fields_ = [("max_queries", I32), ("max_items", I64), ("max_k", U32), ("use_graph", I32),
                ("max_units", I64)]


class GenieTuning(ctypes.Structure):
    _fields_ = [("sparse_slots", I32), ("sparse_ctas_per_sm", I32), ("dense_tile", I32),
                ("dense_threads", I32), ("sparse_max_total", I64), ("dense_part_work", I64),
                ("sparse_load_pct", I32), ("bitmap_bits", I32), ("dense_bitmaps", I32)]


class GenieServerConfig(ctypes.Structure):
    _fields_ = [("slots_per_index", I32), ("max_queries", I32), ("max_items", I64), ("max_k", U32),
                ("window_us", I32), ("memory_budget", I64)]


class GenieRequestRouter(ctypes.Structure):
    _fields_ = [("server", P), ("n_clusters", I32), ("index_id", P), ("id_offset", P), ("radius", I32)]


class GenieServerReport(ctypes.Structure):
    _fields_ = [("submitted", I64), ("completed", I64), ("rejected", I64), ("batches", I64),
                ("mean_batch", ctypes.c_double), ("p50_us", ctypes.c_double), ("p99_us", ctypes.c_double),
                ("max_us", ctypes.c_double), ("throughput_qps", ctypes.c_double), ("held", I64),
                ("peak_in_flight_bytes", I64)]


# name -> (restype, argtypes); mirrors include/genie_gb300.h
PROTOTYPES = {
    "genie_last_error": (ctypes.c_char_p, []),
    "genie_version": (ctypes.c_int, []),
    "genie_init": (ctypes.c_int, [ctypes.c_int]),
    "genie_device_reset": (ctypes.c_int, []),
    "genie_index_create": (ctypes.c_int, [P, I64, I32, P]),
    "genie_index_create_with": (ctypes.c_int, [P, I64, I32, I32, P]),
    "genie_index_create_bag": (ctypes.c_int, [P, P, I64, P]),
    "genie_index_create_compressed": (ctypes.c_int, [P, I64, I32, I32, I32, P]),
    "genie_index_destroy": (ctypes.c_int, [P]),
    "genie_index_create_subsequence": (ctypes.c_int, [P, P, I64, P]),
    "genie_index_subsequence_bits": (ctypes.c_int, [P, P]),
    "genie_index_device_ids": (ctypes.c_int, [P, P]),
    "genie_index_get_info": (ctypes.c_int, [P, P]),
    "genie_index_copy_out": (ctypes.c_int, [P, P, P, P, P, P]),
    "genie_index_copy_compressed": (ctypes.c_int, [P, P, P, P, P, P]),
    "genie_index_item_span": (ctypes.c_int, [P, I32, I32, I32, P, P]),
    "genie_index_adaptive_range": (ctypes.c_int, [P, I32, F32, P, P]),
    "genie_index_save": (ctypes.c_int, [P, ctypes.c_char_p]),
    "genie_index_load": (ctypes.c_int, [ctypes.c_char_p, P]),
    "genie_search": (ctypes.c_int, [P, P, P, P, P]),
    "genie_search_multi": (ctypes.c_int, [P, P, I32, P, P, P]),
    "genie_codec_set_match": (ctypes.c_int, [I32, P, P]),
    "genie_codec_get_match": (ctypes.c_int, [I32, P, P]),
    "genie_match_builtin": (ctypes.c_int, [P, P, P, P, P]),
    "genie_search_noalloc": (ctypes.c_int, [P, P, P, I64, I64, P, P, P, P]),
    "genie_batch_create": (ctypes.c_int, [P, P, P]),
    "genie_batch_destroy": (ctypes.c_int, [P]),
    "genie_batch_run": (ctypes.c_int, [P, P, P, P, P]),
    "genie_batch_stage": (ctypes.c_int, [P, P]),
    "genie_batch_launch": (ctypes.c_int, [P, P]),
    "genie_batch_fetch": (ctypes.c_int, [P, P, P, P]),
    "genie_batch_submit": (ctypes.c_int, [P, P, I32]),
    "genie_batch_collect": (ctypes.c_int, [P, P, P, P]),
    "genie_batch_autotune": (ctypes.c_int, [P, P, P]),
    "genie_batch_get_tuning": (ctypes.c_int, [P, P]),
    "genie_batch_set_tuning": (ctypes.c_int, [P, P]),
    "genie_batch_last_stats": (ctypes.c_int, [P, P, P]),
    "genie_batch_stage_ms": (ctypes.c_int, [P, P]),
    "genie_server_create": (ctypes.c_int, [P, P]),
    "genie_server_add_index": (ctypes.c_int, [P, P, P]),
    "genie_server_start": (ctypes.c_int, [P]),
    "genie_server_submit": (ctypes.c_int, [P, I32, P, P, P]),
    "genie_server_wait": (ctypes.c_int, [P, ctypes.c_uint64, P, P, P, P]),
    "genie_server_drain": (ctypes.c_int, [P]),
    "genie_server_stats": (ctypes.c_int, [P, P]),
    "genie_server_reset_stats": (ctypes.c_int, [P]),
    "genie_server_now_ns": (I64, []),
    "genie_server_destroy": (ctypes.c_int, [P]),
    "genie_request_handle": (ctypes.c_int, [P, ctypes.c_char_p, P, I64, P]),
    "genie_request_listen": (ctypes.c_int, [P, ctypes.c_char_p, I32, P]),
    "genie_request_listener_port": (ctypes.c_int, [P, P]),
    "genie_request_listener_handled": (ctypes.c_int, [P, P]),
    "genie_request_listener_stop": (ctypes.c_int, [P]),
    "genie_merge_shards": (ctypes.c_int, [I32, P, P, P, P, I32, P, U32, P, P, P]),
    "genie_codec_encode": (I64, [I32, P, I64, P, I64]),
    "genie_codec_encode_bound": (I64, [I64]),
    "genie_codec_decode_device": (ctypes.c_int, [I32, P, P, I64, P, P, P, P]),
}

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "GPU_ALLOC", 3: "CUDA", 4: "NOT_IMPLEMENTED", 5: "CPU_ALLOC",
          6: "DEVICE_TIMEOUT", 7: "IO", 8: "ADMISSION"}

_lib = None


def load(path=None):
    """Load the CUDA library (raises OSError when it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError("libgenie_gb300.so is missing (%s); run genie_gb300.build.build() first" % p)
    lib = ctypes.CDLL(p)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
