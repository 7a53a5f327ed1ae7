"""bench.py reads the roofline's `traffic` (DRAM bytes per launch) from the
committed ncu summary profiles/dram_traffic.md: every kernel the bench can
name as the dominant one has a row there, and the row gives bytes per cell
in the range the summary's own B/cell column states."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_for_traffic", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b


def test_traffic_rows_parse_to_bytes_per_cell():
    b = _bench()
    cells = 512 * 512 * 80
    for kernel, lo, hi in (("k_mx_hevi_tmad", 40.0, 60.0), ("k_mx_fix", 30.0, 45.0), ("k_mx_finish", 200.0, 240.0)):
        t = b.traffic_of(kernel, cells)
        assert t is not None, kernel
        assert lo <= t / cells <= hi, (kernel, t / cells)
