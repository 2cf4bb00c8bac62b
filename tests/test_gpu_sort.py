"""The update kernel's batch sort (the stable sort_by_key of gpma.cuh:977):
the bucket sort, its fall-back to digit passes for crowded buckets, and the
digit passes alone all leave the structure bit-identical to the oracle.

Batches here hold new keys several times with different non-zero values: all
copies are inserted, in batch order (a stable sort), so the layout's values
show the order among equal keys. (Repeats of a key already present are not
used: their in-place writes race in the reference's kernel as in this one.)"""
import numpy as np
import pytest

from oracle.oracle import OracleGPMA

pytestmark = pytest.mark.gpu


@pytest.fixture
def sort_mode(built_lib):
    import gpma_bfs_gb300 as G

    old = G.get_tuning()
    yield G
    G.set_tuning(**old)


def _same(g, o, ctx):
    for a, b, name in zip(g.export_layout(), o.export_layout(), ("keys", "values", "row_offset")):
        assert np.array_equal(a, b), f"{ctx}: {name}"


def _batch_with_repeats(rng, n, size, step, rows=None):
    """`size` random keys, distinct (random 0/1 values, column below n - 8), and
    (from 16 rows) up to size // 16 new keys in column n - 1 - step (step < 8),
    each two or three times with the values 2, 3, 4 in batch order, shuffled
    together."""
    src = rng.integers(0, n, size) if rows is None else rng.choice(rows, size)
    dst = rng.integers(0, max(1, n - 8), size)
    keys = np.unique((src.astype(np.uint64) << np.uint64(32)) | dst.astype(np.uint64))
    keys = keys[rng.permutation(len(keys))]
    vals = rng.integers(0, 2, len(keys)).astype(np.uint8)
    fresh = np.unique(rng.integers(0, n, size // 16 if n >= 16 else 0)).astype(np.uint64)
    fresh = (fresh << np.uint64(32)) | np.uint64(max(0, n - 1 - step))
    copies = rng.integers(2, 4, len(fresh))
    rk = np.repeat(fresh, copies)
    rv = np.concatenate([np.arange(2, 2 + c, dtype=np.uint8) for c in copies]) if len(fresh) else np.zeros(0, np.uint8)
    # interleave: the copies keep their relative order, at random batch positions
    total = len(keys) + len(rk)
    slots = np.sort(rng.choice(total, len(rk), replace=False))
    out_k = np.empty(total, np.uint64)
    out_v = np.empty(total, np.uint8)
    mask = np.zeros(total, bool)
    mask[slots] = True
    out_k[mask], out_v[mask] = rk, rv
    out_k[~mask], out_v[~mask] = keys, vals
    return out_k, out_v


@pytest.mark.parametrize("mode", [0, 1])
def test_spread_batches_match_oracle(sort_mode, mode):
    G = sort_mode
    G.set_tuning(update_sort=mode)
    rng = np.random.default_rng(40 + mode)
    n = 50000
    g, o = G.GPMA(n), OracleGPMA(n, threads=4)
    g.set_profiling(True)
    for step, size in enumerate((200000, 3000, 40000, 1, 70000, 900)):
        k, v = _batch_with_repeats(rng, n, size, step)
        G.update_gpma(g, k, v)
        o.update(k, v)
        _same(g, o, f"mode {mode} step {step}")
    p = g.profile()
    assert p["update_kernels"] == 6
    assert p["sort_fallbacks"] == 0  # keys spread like the rows' slots: no crowded bucket
    g.close()


def test_crowded_bucket_falls_back_to_digit_passes(sort_mode):
    G = sort_mode
    G.set_tuning(update_sort=0)
    rng = np.random.default_rng(43)
    n = 1 << 16
    g, o = G.GPMA(n), OracleGPMA(n, threads=4)
    g.set_profiling(True)
    k, v = _batch_with_repeats(rng, n, 20000, 0)
    G.update_gpma(g, k, v)
    o.update(k, v)
    # 12000 keys into three rows: their slots (a few dozen) lie in one or two
    # buckets, which then hold far more than 1024 keys
    k, v = _batch_with_repeats(rng, n, 12000, 1, rows=np.array([7, 8, 9]))
    G.update_gpma(g, k, v)
    o.update(k, v)
    _same(g, o, "crowded")
    assert g.profile()["sort_fallbacks"] == 1
    # and the next spread batch takes the bucket sort again
    k, v = _batch_with_repeats(rng, n, 30000, 2)
    G.update_gpma(g, k, v)
    o.update(k, v)
    _same(g, o, "after the crowded batch")
    assert g.profile()["sort_fallbacks"] == 1
    g.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_many_graphs_one_launch(sort_mode, mode):
    """Graphs of different sizes (and one with an empty batch) in one launch:
    buckets and items never mix graphs."""
    G = sort_mode
    G.set_tuning(update_sort=mode)
    rng = np.random.default_rng(50 + mode)
    sizes = [3, 100, 5000, 1 << 14, 777, 1 << 16]
    gs = [G.GPMA(n) for n in sizes]
    os_ = [OracleGPMA(n, threads=2) for n in sizes]
    b = G.Batch()
    for step in range(4):
        ks, vs = [], []
        for i, n in enumerate(sizes):
            size = 0 if (i == 2 and step == 1) else int(rng.integers(1, 4 * n))
            k, v = _batch_with_repeats(rng, n, size, step) if size else (np.zeros(0, np.uint64), np.zeros(0, np.uint8))
            ks.append(k)
            vs.append(v)
        b.update(gs, ks, vs)
        for i, o in enumerate(os_):
            o.update(ks[i], vs[i])
            _same(gs[i], o, f"mode {mode} step {step} graph {i}")
    b.close()
    for g in gs:
        g.close()


def test_update_sort_setting_is_checked(sort_mode):
    G = sort_mode
    with pytest.raises(G.GPMAError):
        G.set_tuning(update_sort=2)
