"""The bench reads figures from the committed ncu summaries: each summary it
cites exists and has the line the bench parses."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_profiled_traffic_lines_parse():
    bench = load_bench()
    for name in ("pathtrace_config1.txt", "raycast_config0.txt"):
        t = bench.profiled_traffic(name)
        assert t is not None and t > 0, name


def test_profiled_issue_metrics_parse():
    bench = load_bench()
    issue = bench.profiled_metric("pathtrace_config1.txt",
                                  "smsp__issue_active.avg.pct_of_peak_sustained_active")
    lanes = bench.profiled_metric("pathtrace_config1.txt",
                                  "smsp__thread_inst_executed_per_inst_executed.ratio")
    assert issue is not None and 0 < issue <= 100
    assert lanes is not None and 0 < lanes <= 32
    assert bench.profiled_metric("pathtrace_config1.txt", "no_such_metric") is None


def test_every_profile_names_its_command():
    for name in os.listdir(os.path.join(ROOT, "profiles")):
        with open(os.path.join(ROOT, "profiles", name)) as f:
            text = f.read()
        assert "python bench.py" in text and "ncu " in text, name


def test_issue_roofline_from_profile():
    """frac = thread instructions per second / lane-issue peak; with the
    profile's own launch time (scaled to 64 spp) it equals issue-active share x active
    lanes / 32 up to the elapsed-vs-active difference, so it lies in (0, 1]."""
    bench = load_bench()
    t1 = bench.profiled_metric("pathtrace_config1.txt", "gpu__time_duration.sum")
    pspp = bench.profiled_value("pathtrace_config1.txt", "profiled_spp_per_launch") or 1.0
    r = bench.issue_roofline(t1 * 1e-3 * 64 / pspp, 64, 1024, sms=152)
    assert r is not None and r["bound"] == "issue" and r["unit"] == "Gthread-inst/s"
    assert 0 < r["frac"] <= 1.0
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert bench.issue_roofline(1.0, 64, 512, sms=152) is None  # other sizes: no profile
