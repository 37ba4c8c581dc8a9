"""CPU: the arithmetic behind the bench line -- the gather bytes of the sparse
product, the reference arm's sample schedule and rate, the workload config
both arms share, and the peak the roofline divides by.  No GPU and no solve."""
import importlib.util
import json
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Ham:
    def __init__(self, D, Z):
        self.D, self.nnz_offdiag = D, Z


def test_spmm_gather_counts_one_x_row_per_entry(bench):
    # two launches of a CSR product: 16 and 48 columns (FP32), D rows, Z entries
    D, Z, s = 1000, 20000, 4.0
    op = Z * (4.0 + s) + (D + 1) * 8.0 + D * s
    cols = [16, 48]
    alg = sum(op + 2 * D * B * s for B in cols)  # what the library records
    prof = {"k_spmm": {"launches": 2, "ms": 2.0, "bytes": alg}}
    g = bench._spmm_gather(prof, _Ham(D, Z), False)
    want = sum(op + (Z + 2 * D) * B * s for B in cols)
    assert g["gather_bytes_per_launch"] == round(want / 2)
    assert g["mean_columns"] == 32.0
    assert abs(g["achieved"] - want / 2e-3 / 1e9) < 0.1
    # matrix-free: the operator is one packed state per row
    prof = {"k_spmm_mf": {"launches": 1, "ms": 1.0, "bytes": D * 8.0 + 2 * D * 8 * s}}
    g = bench._spmm_gather(prof, _Ham(D, Z), True)
    assert g["gather_bytes_per_launch"] == round(D * 8.0 + (Z + 2 * D) * 8 * s)
    assert bench._spmm_gather({}, _Ham(D, Z), False) is None


def test_reference_arm_schedule_and_rate(bench):
    ref = object.__new__(bench.CpuReference)  # the schedule needs no oracle
    ref.threads = 16
    ref.ops = {n: (None, None, None, np.zeros(d)) for n, d in
               zip(bench.SECTORS, [24310, 48620, 92378, 167960, 293930])}
    assert ref.shape(8) == (16, 1) and ref.shape(9) == (16, 1)
    assert ref.shape(10) == (4, 4) and ref.shape(12) == (4, 4)
    seen = set()
    for k in range(10):
        n, bs = ref.points(k)
        assert n == bench.SECTORS[k % 5]
        assert len(bs) == ref.shape(n)[0]
        assert all(8 <= b < bench.NJ for b in bs)  # the eight smallest J are left out
        seen.update(bs)
    assert len(seen) > 30  # waves spread over the J grid
    # equal seconds per solve in every sector: rate = 1 / that
    assert abs(bench.CpuReference.rate({n: [0.5] for n in bench.SECTORS}) - 2.0) < 1e-12
    # the grid's rate weighs every sector equally
    per = {8: [0.1], 9: [0.2], 10: [0.3], 11: [0.4], 12: [1.0]}
    assert abs(bench.CpuReference.rate(per) - 5 / 2.0) < 1e-12


def test_both_arms_describe_the_same_workload(bench):
    c1 = bench.workload_config(1)
    assert c1["sectors"] == [8, 9, 10, 11, 12] and c1["j_points"] == 64 and c1["nev"] == 10
    assert c1["parallelism"] == "one GPU"
    c2 = bench.workload_config(2)
    assert "2 ranks" in c2["parallelism"]
    assert {k: v for k, v in c1.items() if k != "parallelism"} == \
           {k: v for k, v in c2.items() if k != "parallelism"}


def test_measured_peak_is_read_from_the_peaks_file(bench, tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.measured_peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6674.8}))
    assert bench.measured_peaks() == (6674.8, "measured")
