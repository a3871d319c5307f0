"""bench.py's reference arm on the CPU: the JSON line of `--impl reference`
(the reference algorithm's CPU path, oracle port, on the host cores) and the
timing of its non-solve functions, on small grids."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    """The reference arm prints one JSON line with the base contract's keys,
    impl "reference", a cpu_baseline describing the run and an e2e block with
    no host-device copies; the ladder fit is labelled an extrapolation."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "3",
                        "--warmup", "1", "--no-ref-nonsolve"], cwd=ROOT, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["steps"] == 3 and d["warmup"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert "extrapolated" in d["config"]["value_is"]
    assert set(d["config"]["ladder"]) == {"16x8x8", "24x12x12", "32x16x16"}
    assert d["config"]["nonsolve_at_workload"] is None


def test_nonsolve_timing_small_grid():
    """The non-solve functions of one design iteration, timed at a small grid:
    every part present and timed, the OC bisection's step count that of the
    oracle's bisection (optimality_criterion.py:59-79, tolerance 1e-3)."""
    sys.path.insert(0, ROOT)
    import bench
    t = bench._ref_nonsolve_at_workload((12, 6, 6))
    assert t["grid"] == "12x6x6" and t["cores"] == 1
    assert set(t["seconds"]) == {"edofmat", "assembly", "dirichlet_slicing",
                                 "compliance_and_sensitivities", "filter_matrix",
                                 "sensitivity_filter", "oc_bisection", "density_filter"}
    assert all(np.isfinite(v) and v >= 0 for v in t["seconds"].values())
    assert 10 <= t["oc_steps"] <= 60
    assert t["seconds_per_design_iteration_without_solve"] > 0
