"""Host logic of bench.py that needs no GPU: block plans, the clock record of
the timed window, the DRAM-traffic file parser and the index-load leg's error
path."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_block_plan_plain_and_per_bucket():
    assert bench.block_plan(10, 4, None) == [(0, 4, "stream16"), (4, 4, "stream16"), (8, 2, "stream16")]
    tuned = {"buckets": [{"first": 0, "reads": 5, "block": 4, "verify": "head32"},
                         {"first": 5, "reads": 3, "block": 8, "verify": "pair16"}]}
    assert bench.block_plan(8, 4, tuned) == [(0, 4, "head32"), (4, 1, "head32"), (5, 3, "pair16")]


class _FakeProc:
    def __init__(self, out):
        self.out = out

    def terminate(self):
        pass

    def communicate(self, timeout=None):
        return self.out, ""


def _sampler(lines):
    s = bench.ClockSampler(0)
    s.proc = _FakeProc("\n".join(lines))
    return s


def test_clock_record_keeps_the_timed_window():
    ts = bench.ClockSampler._stamp("2026/12/04 10:00:00.000")
    rows = ["2026/12/04 10:00:00.000, 1500, 2070, 300.0, Not Active, Not Active, Not Active, Not Active",
            "2026/12/04 10:00:00.200, 2070, 2070, 900.0, Not Active, Not Active, Not Active, Active",
            "2026/12/04 10:00:00.400, 2070, 2070, 950.0, Not Active, Not Active, Not Active, Not Active",
            "2026/12/04 10:00:00.600, 1000, 2070, 200.0, Active, Not Active, Not Active, Not Active"]
    rec = _sampler(rows).stop(ts + 0.1, ts + 0.5)
    assert rec["window"] == "timed region" and rec["samples"] == 2
    assert rec["sm_mhz"] == 2070 and rec["sm_max_mhz"] == 2070 and rec["reasons"] == ["sw_power_cap"]
    # a window between two samples keeps the nearest one on each side
    rec = _sampler(rows).stop(ts + 0.05, ts + 0.1)
    assert rec["window"] == "nearest" and rec["samples"] == 2 and rec["sm_mhz"] == (1500 + 2070) / 2


def test_profile_traffic_reads_the_committed_figures():
    tr = bench.profile_traffic("k_cand_table")
    assert tr and tr["dram_bytes_per_item_human"] > 0
    assert bench.profile_traffic("no_such_kernel") is None


class _Info:
    n_seeds, n_words2, n_words3 = 10, 4, 2


class _FailingIndex:
    def info(self):
        return _Info()

    def save(self, prefix):
        raise RuntimeError("swm_index_save: no space left on device")


class _Runtime:
    def cudaDeviceSynchronize(self):
        return 0


def test_index_load_reports_a_failure_instead_of_raising():
    out = bench.index_load(None, _Runtime(), _FailingIndex(), 2, 0)
    assert "skipped" in out and "no space left" in out["skipped"]
