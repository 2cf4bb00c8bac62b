"""Autotuner logic with synthetic probes (host only: tuning is host state)."""
import pytest


@pytest.fixture
def T(built_lib):
    import gpma_bfs_gb300 as G
    import gpma_bfs_gb300.autotune as T

    old = G.get_tuning()
    yield T
    G.set_tuning(**old)


def test_picks_fastest_setting_and_leaves_it_in_force(T):
    import gpma_bfs_gb300 as G

    def probe():
        t = G.get_tuning()
        # fastest at 4 CTAs/SM and a switch at n/8
        ms = abs(t["bfs_blocks_per_sm"] - 4) + abs(t["bfs_dense_div"] - 8) * 0.1 + 1.0
        return ms, "same"

    r = T.tune_group("bfs", probe, repeats=1)
    assert r.best == {"bfs_blocks_per_sm": 4, "bfs_dense_div": 8}
    assert G.get_tuning()["bfs_blocks_per_sm"] == 4 and G.get_tuning()["bfs_dense_div"] == 8
    assert len(r.trials) == 12 and r.best_ms == 1.0


def test_keeps_current_setting_when_nothing_is_faster(T):
    import gpma_bfs_gb300 as G

    G.set_tuning(ms_blocks_per_sm=8, ms_dense_div=8)
    r = T.tune_group("ms", lambda: (1.0, "x"), repeats=2)
    assert r.best == {"ms_blocks_per_sm": 8, "ms_dense_div": 8}


def test_result_changing_setting_is_an_error(T):
    import gpma_bfs_gb300 as G

    def probe():
        return 1.0, "a" if G.get_tuning()["update_blocks_per_sm"] != 3 else "b"

    before = G.get_tuning()
    with pytest.raises(RuntimeError, match="changed the result"):
        T.tune_group("update", probe, repeats=1)
    assert G.get_tuning() == before  # restored


def test_autotune_report_and_save_load(T, tmp_path):
    import gpma_bfs_gb300 as G

    report = T.autotune({"bfs": lambda: (2.0 - 0.1 * G.get_tuning()["bfs_blocks_per_sm"], "d")}, repeats=1)
    assert report["bfs"]["best"]["bfs_blocks_per_sm"] == 8
    path = tmp_path / "tuning.json"
    T.save(str(path), report)
    G.set_tuning(bfs_blocks_per_sm=2)
    T.load(str(path))
    assert G.get_tuning()["bfs_blocks_per_sm"] == 8
