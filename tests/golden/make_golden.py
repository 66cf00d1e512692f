"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

Run in a container that has the reference tree (read-only) and nvcc:

    python tests/golden/make_golden.py /path/to/reference

It compiles the reference's own host code into oracle/_ref/ (oracle/Makefile,
target `ref`), then records:

* sift20.npz / sift1k.npz / tweets20.npz -- the input tables of the reference's
  tests (static/*.csv), the reference-built posting array (`inv`), and the
  reference's spans for a set of query items (including out-of-range,
  clamped, empty and adaptive-range items);
* codecs_kat.json -- for all 13 reference codecs and every length 1..1024 of
  the test_compression_codecs.cu input stream, the reference encoder's word
  count and CRC32, plus the full encoding for a few lengths.

The fixtures are small; the GPU machine has no reference tree, so tests only read
these files there.
"""
import ctypes
import json
import os
import subprocess
import sys
import zlib

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(REPO, "tests", "golden")


def read_csv_rows(path, limit=-1):
    """utility::read_file (FileReader.cc:54-83): strtok on ", ", atoi."""
    rows = []
    with open(path) as f:
        for line in f:
            if 0 <= limit <= len(rows):
                break
            toks = [t for t in line.replace(",", " ").split() if t]
            rows.append([int(float(t)) if "." in t else int(t) for t in toks])
    return rows


def read_multirange(path):
    """utility::read_query (FileReader.cc:91-125): qid, dim, value, sel, weight."""
    out = []
    with open(path) as f:
        for line in f:
            toks = [t for t in line.replace(",", " ").split() if t]
            if len(toks) == 5:
                out.append((int(toks[0]), int(toks[1]), int(toks[2]), float(toks[3]), float(toks[4])))
    return out


def ref_index_lib():
    r = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libref_index.so"))
    P = ctypes.c_void_p
    r.ref_index_spans.argtypes = [P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, P, ctypes.c_int32,
                                  P, P, P, P, P, P, P, P]
    return r


def ref_spans(values, bag_off, dim, low, up, sel):
    r = ref_index_lib()
    if bag_off is None:
        n, d = values.shape
        total = n * d
        row_off = None
    else:
        n, d = len(bag_off) - 1, 1
        total = int(bag_off[-1])
        row_off = np.ascontiguousarray(bag_off, np.int64)
    vals = np.ascontiguousarray(values, np.int32).ravel()
    m = len(dim)
    ids = np.zeros(total + 16, np.uint32)
    nid = np.zeros(1, np.int64)
    st = np.zeros(m, np.int64)
    en = np.zeros(m, np.int64)
    arrs = [np.ascontiguousarray(a, t) for a, t in ((dim, np.int32), (low, np.int32), (up, np.int32), (sel, np.float32))]
    r.ref_index_spans(vals.ctypes.data, n, d, 0 if bag_off is None else 1,
                      None if row_off is None else row_off.ctypes.data, m,
                      arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data, arrs[3].ctypes.data,
                      ids.ctypes.data, nid.ctypes.data, st.ctypes.data, en.ctypes.data)
    return ids[: int(nid[0])].copy(), st, en


def probe_items(values, n_dims, rng, n=400):
    """Query items covering exact, ranged, clamped, empty and invalid cases."""
    lo_all, hi_all = int(values.min()), int(values.max())
    dim = rng.integers(-1, n_dims + 1, n)
    low = rng.integers(lo_all - 5, hi_all + 5, n)
    width = rng.choice([0, 0, 0, 1, 2, 5, 40, -1], n)
    up = low + width
    return dim.astype(np.int32), low.astype(np.int32), up.astype(np.int32)


def table_case(name, values, rng, queries_multirange=None):
    n, d = values.shape
    dim, low, up = probe_items(values, d, rng)
    sel = np.zeros(len(dim), np.float32)
    if queries_multirange is not None:
        mq = np.array([(a[1], a[2], a[3]) for a in queries_multirange])
        dim = np.concatenate([dim, mq[:, 0].astype(np.int32)])
        low = np.concatenate([low, mq[:, 1].astype(np.int32)])
        up = np.concatenate([up, mq[:, 1].astype(np.int32)])
        sel = np.concatenate([sel, mq[:, 2].astype(np.float32)])
    inv, st, en = ref_spans(values, None, dim, low, up, sel)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), values=values.astype(np.int32), inv=inv,
                        dim=dim, low=low, up=up, sel=sel, start=st, end=en)
    print(name, values.shape, "inv", len(inv), "items", len(dim))


def bag_case(name, rows, rng):
    vals = np.concatenate([np.array(r, np.int32) for r in rows])
    off = np.zeros(len(rows) + 1, np.int64)
    off[1:] = np.cumsum([len(r) for r in rows])
    m = 200
    dim = rng.integers(-1, 2, m).astype(np.int32)
    low = rng.integers(int(vals.min()) - 3, int(vals.max()) + 3, m).astype(np.int32)
    up = (low + rng.choice([0, 0, 1, 3, -1], m)).astype(np.int32)
    sel = np.zeros(m, np.float32)
    inv, st, en = ref_spans(vals, off, dim, low, up, sel)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), values=vals, row_off=off, inv=inv,
                        dim=dim, low=low, up=up, sel=sel, start=st, end=en)
    print(name, len(rows), "inv", len(inv))


def codec_kat():
    r = O.ref_codecs()
    x = O.kat_input(1024)
    full_lengths = [1, 2, 7, 8, 9, 31, 32, 33, 100, 127, 128, 129, 255, 256]
    out = {"input_seed": 666, "codecs": {}}
    for name, c in O.CODECS.items():
        entry = {"id": c, "words": [], "crc32": [], "full": {}}
        for n in range(1, 1025):
            buf = np.zeros(4 * n + 128, np.uint32)
            m = r.ref_encode(c, x[:n].ctypes.data, n, buf.ctypes.data, len(buf))
            w = buf[:m]
            entry["words"].append(int(m))
            entry["crc32"].append(int(zlib.crc32(w.tobytes())))
            if n in full_lengths:
                entry["full"][str(n)] = [int(v) for v in w]
        out["codecs"][name] = entry
    with open(os.path.join(OUT, "codecs_kat.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("codecs_kat.json written")


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GENIE_REFERENCE")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py <reference tree>")
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + ref])
    rng = np.random.default_rng(20240601)
    static = os.path.join(ref, "static")
    sift20 = np.array(read_csv_rows(os.path.join(static, "sift_20.csv")), np.int32)
    table_case("sift20", sift20, rng)
    sift1k = np.array(read_csv_rows(os.path.join(static, "sift_1k.csv")), np.int32)
    mq = read_multirange(os.path.join(static, "sift_1k_query.csv"))
    table_case("sift1k", sift1k, rng, queries_multirange=mq)
    np.save(os.path.join(OUT, "sift1k_multirange.npy"),
            np.array([(a[0], a[1], a[2]) for a in mq], np.int32))
    with open(os.path.join(OUT, "sift1k_multirange_selw.json"), "w") as f:
        json.dump({"sel": sorted(set(a[3] for a in mq)), "weight": sorted(set(a[4] for a in mq))}, f)
    tweets = read_csv_rows(os.path.join(static, "tweets_20.csv"))
    bag_case("tweets20", tweets, rng)
    # synthetic table with negative values, gaps and a wide range
    syn = rng.integers(-300, 60000, size=(300, 6)).astype(np.int32)
    syn[:, 2] = rng.integers(5, 9, 300)
    table_case("synthetic_wide", syn, rng)
    codec_kat()


if __name__ == "__main__":
    main()
