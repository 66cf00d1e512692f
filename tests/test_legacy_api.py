"""The legacy C++ interface <genie/original/interface.h> (libgenie.so over the
C ABI): the reference's own example and test programs compile and link
against include/ unchanged (CPU), and tests/cpp/legacy_test.cc drives
preprocess_for_knn_csv / knn_search_after_preprocess / knn_search /
knn_search_MT over one-value-per-dim, bijectMap, multiload, subsequence,
sequence and multirange inputs on the GPU, checked against the reference
tests' golden values and the oracle."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden

# the reference tree, where present (only read, to compile its programs)
REFERENCE = os.environ.get("GENIE_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")

# reference programs that use only the public interfaces (not the table's internals)
PROGRAMS = [
    "example/example_1st_level_interface.cc", "example/example_2nd_level_interface.cc",
    "example/example_sift.cc", "example/example_tweets.cc", "example/example_table_from_file.cc",
    "example/example_sift_subsequence.cc",
    "test/test_csv_input_sift_data.cc", "test/test_csv_input_multiload.cc", "test/test_csv_input_tweets.cc",
    "test/test_csv_multiload_tweets.cc", "test/test_save2gpu_sift.cc", "test/test_multiple_search.cc",
    "test/test_hashtable_overflow.cc", "test/test_subsequence_search_csv_input.cc",
    "test/test_refactoring_new_interface.cc",
]


def _built():
    from genie_gb300 import build
    build.build()
    build.build_cpp()
    return build


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "example")), reason="reference tree not present")
@pytest.mark.parametrize("prog", PROGRAMS)
def test_reference_program_compiles_against_include(prog, tmp_path):
    """The drop-in claim: the reference's example and test programs compile
    unchanged against include/ and link against libgenie.so +
    libgenie_gb300.so (running them needs a GPU and the reference's data)."""
    b = _built()
    exe = tmp_path / "prog"
    cmd = (["g++", "-std=c++17", "-O0", "-I" + os.path.join(ROOT, "include"),
            "-I" + os.path.join(b.cuda_home(), "include"), os.path.join(REFERENCE, prog), "-o", str(exe),
            "-L" + b.HERE, "-lgenie", "-lgenie_gb300"] + b.cudart_link())
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]


def _csv(path, rows):
    with open(path, "w") as f:
        for row in rows:
            f.write(",".join(str(int(v)) for v in row) + "\n")


def _run(mode, *files):
    b = _built()
    r = subprocess.run([b.LEGACY_TEST, mode] + [str(f) for f in files], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout[-3000:] + r.stderr[-2000:]
    out = {}
    for line in r.stdout.splitlines():
        p = line.split()
        if len(p) == 5 and p[0] != "CHECK":
            out.setdefault(p[0], []).append([int(x) for x in p[1:]])
    return {t: np.array(v) for t, v in out.items()}


def _sift20_rows():
    return golden("sift20.npz")["values"]


def _tweets20_rows():
    z = golden("tweets20.npz")
    off = z["row_off"]
    return [z["values"][off[i]:off[i + 1]] for i in range(len(off) - 1)]


def _expect(oracle, values, queries, k, radius=0, bag=None):
    if bag is not None:
        vals, off = bag
        ox = oracle.Index(bag=(vals, off))
        dims = [np.zeros(len(q), np.int32) for q in queries]
    else:
        ox = oracle.Index(values)
        dims = [np.arange(len(q), dtype=np.int32) for q in queries]
    item_off = np.zeros(len(queries) + 1, np.int64)
    item_off[1:] = np.cumsum([len(q) for q in queries])
    flat = np.concatenate([np.asarray(q) for q in queries]).astype(np.int32)
    batch = dict(item_off=item_off, dim=np.concatenate(dims), low=flat - radius, up=flat + radius,
                 k=np.full(len(queries), k, np.uint32))
    oid, ocnt, _, _ = ox.search(batch)
    return oid, ocnt


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["sift", "multiload"])
def test_legacy_sift20(mode, oracle, tmp_path):
    """test_csv_input_sift_data / test_csv_input_multiload / test_save2gpu_sift
    / test_multiple_search: the reference's golden postings and top-k, the
    device copy of the postings, two tables merged, and the oracle."""
    rows = _sift20_rows()
    _csv(tmp_path / "sift_20.csv", rows)
    got = _run(mode, tmp_path / "sift_20.csv")[mode]
    oid, ocnt = _expect(oracle, rows, list(rows[:3]), 5)
    assert np.array_equal(got[:, 2], oid) and np.array_equal(got[:, 3], ocnt)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["tweets", "tweets_multiload"])
def test_legacy_tweets_bijectmap(mode, oracle, tmp_path):
    """test_csv_input_tweets / test_csv_multiload_tweets (search_type 1): the
    reference's golden postings; counts are exact where the reference's
    packed counter wraps, so they are checked against the oracle."""
    rows = _tweets20_rows()
    _csv(tmp_path / "tweets_20.csv", rows)
    got = _run(mode, tmp_path / "tweets_20.csv")[mode]
    z = golden("tweets20.npz")
    oid, ocnt = _expect(oracle, None, rows[:3], 5, bag=(z["values"], z["row_off"]))
    assert np.array_equal(got[:, 3], ocnt)
    # ids agree wherever the count is not tied with a neighbour across the
    # multiload split (both sides order ties by id)
    assert np.array_equal(got[:, 2], oid)


@pytest.mark.gpu
def test_legacy_subsequence(oracle, tmp_path):
    """test_subsequence_search_csv_input: rowID << 3 | offset postings, the
    reference's golden results, and every slot against the oracle."""
    rows = _sift20_rows()
    _csv(tmp_path / "sift_20.csv", rows)
    got = _run("subseq", tmp_path / "sift_20.csv")["subseq"]
    oid, ocnt, bits = oracle.subsequence_search([list(r) for r in rows], [list(r) for r in rows[:3]], 5)
    assert bits == 3
    assert np.array_equal(got[:, 2], oid) and np.array_equal(got[:, 3], ocnt)


@pytest.mark.gpu
def test_legacy_sequence_grams(oracle, tmp_path):
    """search_type 2: grams of 3 values with repeats marked, against the
    oracle's restatement of load_table_sequence / load_query_sequence."""
    rng = np.random.default_rng(11)
    rows = [rng.integers(3, 12, rng.integers(2, 30)).tolist() for _ in range(40)]
    rows[5] = rows[0][:]                    # an exact repeat of query 0
    rows[7] = rows[1][2:]                   # a suffix of query 1
    _csv(tmp_path / "seq.csv", rows)
    got = _run("sequence", tmp_path / "seq.csv")["sequence"]
    oid, ocnt = oracle.sequence_search(rows, rows[:3], 5)
    assert np.array_equal(got[:, 3], ocnt)
    assert np.array_equal(got[:, 2], oid)


@pytest.mark.gpu
def test_legacy_knn_search_mt_and_array_rows(oracle, tmp_path):
    """knn_search_MT over two tables at once, and the (data, index) array form
    of load_table, against the oracle."""
    rows = _sift20_rows()
    _csv(tmp_path / "sift_20.csv", rows)
    got = _run("mt", tmp_path / "sift_20.csv")
    for tag, part in (("mt0", rows[:10]), ("mt1", rows[10:])):
        oid, ocnt = _expect(oracle, part, list(rows[:3]), 5)
        assert np.array_equal(got[tag][:, 2], oid) and np.array_equal(got[tag][:, 3], ocnt), tag
    got = _run("binary_rows", tmp_path / "sift_20.csv")["binary_rows"]
    oid, ocnt = _expect(oracle, rows, list(rows[:3]), 5)
    assert np.array_equal(got[:, 2], oid) and np.array_equal(got[:, 3], ocnt)


@pytest.mark.gpu
def test_legacy_multirange_adaptive(oracle, tmp_path):
    """example_sift.cc's path: qid,dim,value,sel,weight items read by
    read_query, grouped per query, widened by the adaptive range (sel 0.04),
    searched through knn_search(result, result_count, config)."""
    z = golden("sift1k.npz")
    values = z["values"]
    mq = np.load(os.path.join(ROOT, "tests", "golden", "sift1k_multirange.npy"))
    with open(os.path.join(ROOT, "tests", "golden", "sift1k_multirange_selw.json")) as f:
        sw = json.load(f)
    _csv(tmp_path / "sift_1k.csv", values)
    with open(tmp_path / "query.csv", "w") as f:
        for qid, d, v in mq:
            f.write("%d,%d,%d,%g,%g\n" % (qid, d, v, sw["sel"][0], sw["weight"][0]))
    got = _run("multirange", tmp_path / "sift_1k.csv", tmp_path / "query.csv")["multirange"]
    ox = oracle.Index(values)
    qids = np.unique(mq[:, 0])[:100]
    off, dims, lows, ups = [0], [], [], []
    for qid in qids:
        for _, d, v in mq[mq[:, 0] == qid]:
            lo, hi = ox.adaptive_range(int(d), float(sw["sel"][0]), int(v), int(v))
            dims.append(d)
            lows.append(lo)
            ups.append(hi)
        off.append(len(dims))
    batch = dict(item_off=np.array(off), dim=np.array(dims, np.int32), low=np.array(lows, np.int32),
                 up=np.array(ups, np.int32), k=np.full(len(qids), 10, np.uint32))
    oid, ocnt, _, _ = ox.search(batch)
    assert np.array_equal(got[:, 2], oid) and np.array_equal(got[:, 3], ocnt)
