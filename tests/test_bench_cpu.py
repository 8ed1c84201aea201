"""bench.py's host-side pieces on the CPU: the seeded ensemble workload, the order of the
JSON line's sections with the summary last, and the DRAM-traffic lookup of the roofline."""
import importlib.util
import os

from compact3d_gb300.grid import C3D_MIXED

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_cpu_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_ensemble_grids_seeded_and_in_range():
    """32 channels drawn from Nx, Nz in {48, 64, 96, 128} and Ny in {33, 49, 65, 97} points,
    RE = 3/4 of a bulk Reynolds number in [3000, 12000], the same draw for the same seed."""
    b = load_bench()
    a, dt = b.ensemble_grids(32, 7, C3D_MIXED)
    c, _ = b.ensemble_grids(32, 7, C3D_MIXED)
    d, _ = b.ensemble_grids(32, 8, C3D_MIXED)
    key = lambda gs: [(g.n1m, g.n2m, g.n3m, g.re) for g in gs]
    assert key(a) == key(c) and key(a) != key(d)
    assert len(a) == 32 and dt == 0.002
    for g in a:
        assert g.n1m in (48, 64, 96, 128) and g.n3m in (48, 64, 96, 128)
        assert g.n2m + 1 in (33, 49, 65, 97)
        assert 0.75 * 3000.0 <= g.re <= 0.75 * 12000.0


def test_with_summary_orders_sections():
    """Plain keys first, then the long tables, then a summary of every headline figure."""
    b = load_bench()
    errs = {k: 1e-7 for k in ("u", "v", "w", "p", "p_mean", "p_fluct", "divmax", "bulk_rel", "wsm_rel")}
    res = {"metric": "m", "value": 1.0e10, "ms_per_step": 3.6, "kernels": {"zE": {"ms": 0.5}},
           "fp64": {"value": 1.0e9}, "batched": {"value": 8.0e9, "streams_form": {"value": 7.0e9}},
           "err_vs_fp64": {"mixed": errs, "steps": 20}, "roofline": {"frac": 0.87},
           "e2e": {"value": 1.6e9}, "cpu_baseline": {"value": 6.7e6}}
    out = b.with_summary(res)
    keys = list(out)
    assert keys[-1] == "summary"
    assert keys.index("e2e") < keys.index("kernels") < keys.index("summary")
    assert keys.index("cpu_baseline") < keys.index("batched")
    s = out["summary"]
    assert s["mixed"] == 1.0e10 and s["ms_per_step"] == 3.6 and s["fp64"] == 1.0e9
    assert s["batched"] == 8.0e9 and s["batched_streams_form"] == 7.0e9
    assert s["err_vs_fp64"]["steps"] == 20 and s["err_vs_fp64"]["p"] == 1e-7
    assert s["roofline_frac"] == 0.87 and s["e2e"] == 1.6e9 and s["cpu_baseline"] == 6.7e6


def test_traffic_lookup():
    """The roofline's traffic comes from the committed ncu summary: the dominant kernel of
    channel384 has an entry near its algorithmic bytes (3.02 GB per launch), an unknown
    kernel none."""
    b = load_bench()
    t = b.traffic_for("channel384", "mixed", "zE")
    assert t is not None and 2.9e9 < t < 3.6e9
    assert b.traffic_for("channel384", "mixed", "no_such_kernel") is None
