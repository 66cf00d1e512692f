"""The device index builder gives exactly the host builder's index (posting
order = the reference's inv_table::_inv), and searches on it match."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _same_index(genie, values):
    th = genie.Table.from_values(values, builder="host")
    td = genie.Table.from_values(values, builder="device")
    lh, ld = th.layout(), td.layout()
    for key in ("key_offsets", "key_base", "dim_min", "dim_max"):
        assert np.array_equal(lh[key], ld[key]), key
    assert np.array_equal(th.ids(), td.ids())
    return th, td


@pytest.mark.parametrize("case", ["config1", "config3", "config0", "odd", "negative"])
def test_device_build_equals_host_build(genie, oracle, case):
    from genie_gb300 import workloads
    rng = np.random.default_rng(3)
    if case == "config1":
        values, batch = workloads.config1(n=100_000, q=16, k=10)
    elif case == "config3":
        values, batch = workloads.config3(n=150_000, q=16)
    elif case == "config0":
        values, batch = workloads.config0(n=1000, q=16, k=10)
    elif case == "odd":         # n not a multiple of the chunk, d not of the tile
        values = rng.integers(0, 37, size=(10_007, 37), dtype=np.int32)
        _, batch = workloads.config0(n=10, q=1, k=5)
        batch = None
    else:                       # negative values and a range near the device limit
        values = rng.integers(-9000, 7000, size=(20_000, 5), dtype=np.int32)
        batch = None
    th, td = _same_index(genie, values)
    if batch is not None:
        qb = genie.QueryBatch(batch["item_off"], batch["dim"], batch["low"], batch["up"], batch["k"],
                              batch.get("weight"), batch.get("weighted"))
        a = genie.search(th, qb)
        b = genie.search(td, qb)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_device_build_sift_goldens(genie):
    for name in ("sift20", "sift1k"):
        z = golden(name + ".npz")
        _, td = _same_index(genie, z["values"])
        assert np.array_equal(td.ids(), z["inv"]), name


def test_wide_range_falls_back_to_host(genie):
    rng = np.random.default_rng(4)
    values = rng.integers(0, 1 << 20, size=(5000, 3), dtype=np.int32)
    with pytest.raises(genie.NotImplementedException):
        genie.Table.from_values(values, builder="device")
    ta = genie.Table.from_values(values)                 # auto: host
    th = genie.Table.from_values(values, builder="host")
    assert np.array_equal(ta.ids(), th.ids())
