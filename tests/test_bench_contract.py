"""bench.py's reporting arithmetic (CPU): the LCC algorithmic bytes per pass."""
import importlib.util
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_lcc_pass_bytes_per_entry():
    b = _bench()
    # k = 6: 4 + 1/8 + 1/8 + 1 + 1 = 6.25 B per listed entry
    assert b.lcc_pass_bytes(1000, 0, 6) == 6250.0
    assert b.lcc_pass_bytes(1000, 80, 6) == 6260.0
    # k = 12: two bytes of roles
    assert b.lcc_pass_bytes(8, 0, 12) == 8 * 7.25
    assert b.lcc_pass_bytes(0, 0, 6) == 0.0
