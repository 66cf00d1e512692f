"""The library's own host encoders (genie_codec_encode) reproduce the
reference codecs byte for byte (fixtures from the reference's encoders), and
the compressed layout equals the oracle's."""
import ctypes
import json
import os
import zlib

import numpy as np

from conftest import GOLDEN


def _encode(lib, codec, x):
    cap = lib.genie_codec_encode_bound(len(x))
    out = np.zeros(cap, np.uint32)
    n = lib.genie_codec_encode(codec, x.ctypes.data, len(x), out.ctypes.data, cap)
    assert n > 0, lib.genie_last_error()
    return out[:n]


def test_host_encoders_match_reference_kat(oracle):
    import genie_gb300 as g
    lib = g.lib()
    with open(os.path.join(GOLDEN, "codecs_kat.json")) as f:
        kat = json.load(f)
    x = oracle.kat_input(1024, kat["input_seed"])
    for name, e in kat["codecs"].items():
        for n in range(1, 1025):
            w = _encode(lib, e["id"], np.ascontiguousarray(x[:n]))
            assert len(w) == e["words"][n - 1] and zlib.crc32(w.tobytes()) == e["crc32"][n - 1], (name, n)


def test_encoder_rejects_bad_arguments():
    import genie_gb300 as g
    lib = g.lib()
    x = np.arange(10, dtype=np.uint32)
    out = np.zeros(4, np.uint32)
    assert lib.genie_codec_encode(99, x.ctypes.data, 10, out.ctypes.data, 4) < 0
    assert lib.genie_codec_encode(1, x.ctypes.data, 10, out.ctypes.data, 4) < 0      # capacity
    assert lib.genie_codec_encode_bound(1) >= 34
