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


def test_traffic_read_from_profile_for_its_table_only():
    import bench
    per_query = None
    covers = None
    for line in open(f"{bench.ROOT}/profiles/k_batch_c4_landmark.md"):
        if line.startswith("traffic_bytes_per_query:"):
            per_query = float(line.split(":")[1])
        elif line.startswith("traffic_table:"):
            covers = line.split(":", 1)[1].strip()
    assert per_query and covers
    assert bench.traffic_per_launch("c4", 4096, "landmark", covers) == per_query * 4096
    assert bench.traffic_per_launch("c4", 4096, "landmark", "16 x 16-bit") is None
    assert bench.traffic_per_launch("c4", 100, "capped") > 0  # summary without a table line
    assert bench.traffic_per_launch("nonexistent", 100, "landmark", covers) is None
