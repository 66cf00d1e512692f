"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference's own benchmark datasets (SIFT 4.5M, tweets, ocr, adult) are not
available; these generators stand in for them with the stated shapes and value
distributions.  Seeds are 1234 + config id; every size can be scaled down for
tests.  Each generator returns (values, QueryBatch-compatible dict).

  cfg0  plain small     N x 128 uint8, half-normal(sigma 40) with 30% zeros;
                        queries = perturbed objects (+N(0,8)), exact items, k=10
  cfg1  LSH buckets     N x 240 uniform in [0, 8192); half the queries derived
                        from stored objects with 60% of items redrawn; k=100
  cfg2  short text      N x 32 Zipf(1.1) over 65,536 terms; 32 Zipf items; k=32
  cfg3  uneven batch    as cfg0 values; 8..128 items on distinct dims, half-width
                        r in {0,1,2,4}, half the queries weighted U[0.5,2]; k in {10,100}
"""
import numpy as np


def _halfnormal_u8(rng, shape, sigma=40.0, zero_frac=0.30):
    v = np.rint(np.abs(rng.normal(0.0, sigma, size=shape)))
    v = np.clip(v, 0, 255)
    v[rng.random(shape) < zero_frac] = 0
    return v.astype(np.int32)


def _batch(item_off, dim, low, up, k, weight=None, weighted=None):
    return dict(item_off=np.asarray(item_off, np.int64), dim=np.asarray(dim, np.int32),
                low=np.asarray(low, np.int32), up=np.asarray(up, np.int32), k=np.asarray(k, np.uint32),
                weight=None if weight is None else np.asarray(weight, np.float32),
                weighted=None if weighted is None else np.asarray(weighted, np.uint8))


def config0(n=1000, d=128, q=100, k=10, seed=1234):
    rng = np.random.default_rng(seed)
    values = _halfnormal_u8(rng, (n, d))
    src = rng.integers(0, n, q)
    qv = np.clip(values[src] + np.rint(rng.normal(0, 8, size=(q, d))), 0, 255).astype(np.int32)
    dims = np.tile(np.arange(d, dtype=np.int32), q)
    flat = qv.ravel()
    return values, _batch(np.arange(q + 1) * d, dims, flat, flat, np.full(q, k))


def config1(n=1_000_000, d=240, q=1024, k=100, buckets=8192, seed=1235):
    rng = np.random.default_rng(seed)
    values = rng.integers(0, buckets, size=(n, d), dtype=np.int32)
    return values, config1_queries(values, q, k, buckets, rng=rng)


def config1_queries(values, q=1024, k=100, buckets=8192, seed=None, rng=None):
    """A config1 query batch over given values: half the queries derived from
    stored objects with 60% of their items redrawn, half uniform."""
    rng = rng if rng is not None else np.random.default_rng(seed)
    n, d = values.shape
    qv = rng.integers(0, buckets, size=(q, d), dtype=np.int32)
    derived = np.arange(q) < q // 2
    src = rng.integers(0, n, q)
    keep = rng.random((q, d)) >= 0.60          # 60% of items redrawn
    qv[derived] = np.where(keep[derived], values[src[derived]], qv[derived])
    dims = np.tile(np.arange(d, dtype=np.int32), q)
    flat = qv.ravel()
    return _batch(np.arange(q + 1) * d, dims, flat, flat, np.full(q, k))


def zipf_ranks(rng, size, s=1.1, n_terms=65536):
    p = np.arange(1, n_terms + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(p)
    cdf /= cdf[-1]
    return np.minimum(np.searchsorted(cdf, rng.random(size), side="right"), n_terms - 1).astype(np.int32)


def config2(n=10_000_000, d=32, q=4096, k=32, n_terms=65536, seed=1236):
    rng = np.random.default_rng(seed)
    values = np.empty((n, d), np.int32)
    step = 1 << 20
    for a in range(0, n, step):
        b = min(n, a + step)
        values[a:b] = zipf_ranks(rng, (b - a, d), n_terms=n_terms)
    qv = zipf_ranks(rng, (q, d), n_terms=n_terms)
    dims = np.tile(np.arange(d, dtype=np.int32), q)
    flat = qv.ravel()
    return values, _batch(np.arange(q + 1) * d, dims, flat, flat, np.full(q, k))


def config3(n=10_000_000, d=128, q=16384, seed=1237, min_items=8, max_items=128, ks=(10, 100)):
    rng = np.random.default_rng(seed)
    values = np.empty((n, d), np.int32)
    step = 1 << 20
    for a in range(0, n, step):
        b = min(n, a + step)
        values[a:b] = _halfnormal_u8(rng, (b - a, d))
    m = rng.integers(min_items, max_items + 1, q)
    off = np.zeros(q + 1, np.int64)
    off[1:] = np.cumsum(m)
    dims = np.empty(off[-1], np.int32)
    centre = np.empty(off[-1], np.int32)
    radius = rng.choice(np.array([0, 1, 2, 4], np.int32), q)
    src = rng.integers(0, n, q)
    for i in range(q):
        dd = rng.choice(d, m[i], replace=False).astype(np.int32)
        dims[off[i]:off[i + 1]] = dd
        centre[off[i]:off[i + 1]] = values[src[i], dd]
    r_item = np.repeat(radius, m)
    low = centre - r_item
    up = centre + r_item
    weighted = (np.arange(q) % 2 == 1).astype(np.uint8)
    weight = rng.uniform(0.5, 2.0, off[-1]).astype(np.float32)
    k = rng.choice(np.array(ks, np.uint32), q)
    return values, _batch(off, dims, low, up, k, weight, weighted)


def algorithmic_bytes(key_offsets, key_base, dim_min, dim_max, batch, bytes_per_id=4):
    """Posting-list bytes a batch touches: sum over items of the clamped span
    lengths times bytes per id (the roofline's algorithmic traffic)."""
    dim = batch["dim"]
    lo = batch["low"].astype(np.int64)
    hi = batch["up"].astype(np.int64)
    ok = (dim >= 0) & (dim < len(dim_min))
    d = np.where(ok, dim, 0)
    mn = dim_min[d].astype(np.int64)
    mx = dim_max[d].astype(np.int64)
    ok &= ~((lo > hi) | (lo > mx) | (hi < mn))
    lo = np.maximum(lo, mn)
    hi = np.minimum(hi, mx)
    k0 = key_base[d] + (lo - mn)
    k1 = key_base[d] + (hi - mn) + 1
    k0 = np.where(ok, k0, 0)
    k1 = np.where(ok, k1, 0)
    spans = np.where(ok, key_offsets[k1] - key_offsets[k0], 0)
    return int(spans.sum()) * bytes_per_id


def take_queries(batch, qs):
    """The batch made of queries qs (indices, repeats allowed) of `batch`."""
    qs = np.asarray(qs, np.int64)
    off = batch["item_off"]
    lens = off[qs + 1] - off[qs]
    new_off = np.zeros(len(qs) + 1, np.int64)
    np.cumsum(lens, out=new_off[1:])
    src = np.repeat(off[qs] - new_off[:-1], lens) + np.arange(new_off[-1])
    out = dict(item_off=new_off, dim=batch["dim"][src], low=batch["low"][src], up=batch["up"][src],
               k=batch["k"][qs], weight=None, weighted=None)
    if batch.get("weight") is not None:
        out["weight"] = batch["weight"][src]
        out["weighted"] = batch["weighted"][qs]
    return out

