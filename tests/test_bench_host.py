"""bench.py's host-side accounting: algorithmic bytes per query and the DRAM
traffic figure read from the committed ncu summaries (no GPU)."""
import numpy as np


def test_algorithmic_bytes_accounting():
    import bench
    # expanded, scanned, relaxed, phases, bfs reached, bfs scanned
    st = np.array([[10, 80, 60, 3, 0, 0], [1, 8, 4, 1, 0, 0]], np.int64)
    lm64x8 = bench.algorithmic_bytes(st, 64, 8)
    lm32x16 = bench.algorithmic_bytes(st, 32, 16)
    # 12 B per expanded node, 12 B per scanned arc, 16 B + the landmark row
    # (2 L entries of bits / 8 bytes) per relaxation
    assert lm64x8.tolist() == [12 * 10 + 12 * 80 + (16 + 128) * 60, 12 * 1 + 12 * 8 + (16 + 128) * 4]
    assert np.array_equal(lm64x8, lm32x16)  # both rows are 128 B
    assert bench.algorithmic_bytes(st, 32, 8)[0] == 12 * 10 + 12 * 80 + (16 + 64) * 60
    hops = np.array([[10, 80, 60, 3, 500, 4000]], np.int64)
    assert bench.algorithmic_bytes(hops)[0] == 12 * 10 + 16 * 80 + 16 * 60 + 12 * 500 + 8 * 4000


def test_traffic_scales_with_algorithmic_bytes():
    import bench
    r = bench.TRAFFIC_PER_ALG_BYTE[("c4", "bidir")]
    assert 1.0 < r < 20.0
    assert bench.traffic_per_launch("c4", "bidir", 1e9) == r * 1e9
    assert bench.traffic_per_launch("c4-small", "bidir", 10.0) == r * 10.0
    assert bench.traffic_per_launch("c4", "landmark", 1e9) is None


def test_fixture_check_needs_matching_inputs(tmp_path, monkeypatch):
    import bench
    g = type("G", (), {})()
    g.off = np.arange(5, dtype=np.int32)
    g.col = np.arange(4, dtype=np.int32)
    g.w = np.ones(4, np.uint32)
    S = np.array([0, 1], np.int32)
    T = np.array([2, 3], np.int32)
    np.savez(tmp_path / "c4_costs.npz", costs=np.array([5, 7], np.int32),
             graph_digest=bench._digest(g.off, g.col, g.w), pairs_digest=bench._digest(S, T))
    monkeypatch.setattr(bench, "FIXTURES", str(tmp_path))
    ok = bench.check_fixture({}, 2, 0, g, S, T, np.array([5, 7], np.int32))
    assert ok["exact"] is True and ok["checked"] == 2
    bad = bench.check_fixture({}, 2, 0, g, S, T, np.array([5, 8], np.int32))
    assert bad["exact"] is False and bad["first_mismatch"] == 1
    other = bench.check_fixture({}, 2, 0, g, T, S, np.array([5, 7], np.int32))
    assert other["exact"] is None
