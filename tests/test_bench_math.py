"""The bench's byte counts (host arithmetic, no GPU): the fused step's
algorithmic bytes per particle and the whole-step figure with the list build
amortised, as the measurement definitions give them."""

import pytest

import bench


def test_fused_step_bytes():
    # FP32: 156 + 4 n + 8 n_b; FP64: 188 + 4 n + 8 n_b
    assert bench.algorithmic_bytes(10.0, 2.0, "fp32") == 156 + 40 + 16
    assert bench.algorithmic_bytes(10.0, 2.0, "fp64") == 188 + 40 + 16


def test_step_bytes_amortise_the_list_build():
    N, n, nb = 1000, 9.9, 1.98
    no_build = bench.step_bytes(N, n, nb, 0.0)
    assert no_build == N * bench.algorithmic_bytes(n, nb, "fp32")
    # one build every 6 steps adds N (16 + 4 n) / 6
    assert bench.step_bytes(N, n, nb, 1.0 / 6.0) - no_build == pytest.approx(N * (16 + 4 * n) / 6.0, rel=1e-12)
