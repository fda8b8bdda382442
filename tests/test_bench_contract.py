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


def test_poisson_stream_reports_rates_and_percentiles():
    """The arrival loop against a stand-in server (no GPU): more requests at
    the higher rate, every ticket released, p99 >= p50."""
    import random
    import types

    b = _bench()
    released = []

    class Result:
        def __init__(self, lat):
            self.latency_ms = lat
            self.status = 0

    class Server:
        def __init__(self, graph, slots):
            self.n, self.done = 0, {}

        def __enter__(self):
            return self

        def __exit__(self, *exc):
            return False

        def submit(self, tmpl):
            self.n += 1
            self.done[self.n] = Result(random.uniform(5, 50))
            return self.n

        def wait(self, ticket):
            return self.done[ticket]

        def release(self, ticket):
            released.append(ticket)

    pm = types.SimpleNamespace(PM_SUCCESS=0, PM_E_TIMEOUT=-7, Server=Server)
    lo = b.poisson_stream(None, pm, list(range(15)), 40.0, 0.4, 4, seed=3)
    hi = b.poisson_stream(None, pm, list(range(15)), 400.0, 0.4, 4, seed=4)
    assert hi["requests"] > lo["requests"] > 0
    assert lo["failed"] == 0 and lo["timed_out"] == 0 and lo["completed"] == lo["requests"]
    assert lo["latency_ms_p99"] >= lo["latency_ms_p50"]
    assert len(released) == lo["requests"] + hi["requests"] + 8  # + the warm-up requests
