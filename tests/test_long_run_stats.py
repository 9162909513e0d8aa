"""Long-run statistics of config 1's periodic compression to 100 kPa (tests/compression_protocol.py):
the GPU engine against the CPU oracle over five seeds each.

The dynamics are chaotic, so the two engines are compared statistically: for each outcome
(steps to 100 kPa, solid fraction, coordination number and deviatoric stress at 100 kPa, and the
bulk stiffness of the packing there) the
means over the seeds must agree within three standard errors of the difference plus 2%.  The
oracle's runs are a committed fixture (tests/golden/compression_stats.json, written by
tests/golden/make_compression_stats.py), together with runs of an oracle with a planted mistake
(contact stiffness x 1.3: 30% more stress at a given strain), which the same rule must tell
apart from the correct oracle.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
STATS = os.path.join(HERE, "golden", "compression_stats.json")
SEEDS = (1, 2, 3, 4, 5)
METRICS = ("steps_to_100kPa", "solid_fraction", "coordination", "deviatoric_stress", "bulk_stiffness")
REL_TOL = 0.02


def _load(prefix=""):
    if not os.path.exists(STATS):
        pytest.skip("tests/golden/compression_stats.json missing (tests/golden/make_compression_stats.py)")
    d = json.load(open(STATS))
    need = [f"{prefix}{lab}/{s}" for lab in ("oracle", "oracle_kn_x1.3") for s in SEEDS]
    metrics = SERVO_METRICS if prefix == "servo_" else METRICS
    if not all(k in d and all(m in d[k] for m in metrics) for k in need):
        pytest.skip("tests/golden/compression_stats.json is incomplete (tests/golden/make_compression_stats.py)")
    return d


SERVO_METRICS = ("axial_stress", "lateral_stress", "porosity", "coordination", "mean_depth")


def agree(a, b, metrics=METRICS):
    """Per metric: (ok, |mean difference|, allowed) for two lists of per-seed results."""
    out = {}
    for m in metrics:
        x = np.array([r[m] for r in a], dtype=float)
        y = np.array([r[m] for r in b], dtype=float)
        se = np.sqrt(x.var(ddof=1) / len(x) + y.var(ddof=1) / len(y))
        allowed = 3.0 * se + REL_TOL * abs(y.mean())
        out[m] = (abs(x.mean() - y.mean()) <= allowed, abs(x.mean() - y.mean()), allowed)
    return out


def test_rule_detects_a_30_percent_stiffness_gap():
    d = _load()
    good = [d[f"oracle/{s}"] for s in SEEDS]
    bad = [d[f"oracle_kn_x1.3/{s}"] for s in SEEDS]
    assert all(r["reached"] for r in good + bad)
    res = agree(bad, good)
    for m, (ok, diff, allowed) in res.items():
        print(f"kn x1.3 vs oracle: {m}: |diff| {diff:.4g}, allowed {allowed:.4g}, {'agree' if ok else 'DIFFER'}")
    assert not all(ok for ok, _, _ in res.values())


@pytest.mark.gpu
def test_gpu_compression_statistics_match_oracle(gpu):
    import compression_protocol as CP
    from sudodem_gb300 import Engine
    d = _load()
    oracle_runs = [d[f"oracle/{s}"] for s in SEEDS]
    runs = []
    for s in SEEDS:
        spec = CP.spec_for(s)
        e = Engine(device=0)
        e.load(spec)
        e.set_periodic_fix(True)
        runs.append(CP.Run(spec, e))
    while not all(r.done for r in runs):
        live = [r for r in runs if not r.done]
        for r in live:
            r.advance()        # asynchronous: the five engines' chunks overlap on the GPU
        for r in live:
            r.check()
    gpu_runs = [r.result for r in runs]
    assert all(r["reached"] for r in gpu_runs)
    res = agree(gpu_runs, oracle_runs)
    for m, (ok, diff, allowed) in res.items():
        g = np.mean([r[m] for r in gpu_runs])
        o = np.mean([r[m] for r in oracle_runs])
        print(f"{m}: gpu {g:.6g} oracle {o:.6g} |diff| {diff:.4g} allowed {allowed:.4g}")
    assert all(ok for ok, _, _ in res.values())


def test_servo_rule_detects_a_30_percent_stiffness_gap():
    d = _load("servo_")
    good = [d[f"servo_oracle/{s}"] for s in SEEDS]
    bad = [d[f"servo_oracle_kn_x1.3/{s}"] for s in SEEDS]
    res = agree(bad, good, SERVO_METRICS)
    for m, (ok, diff, allowed) in res.items():
        print(f"servo, kn x1.3 vs oracle: {m}: |diff| {diff:.4g}, allowed {allowed:.4g}, {'agree' if ok else 'DIFFER'}")
    assert not all(ok for ok, _, _ in res.values())


@pytest.mark.gpu
def test_gpu_servo_statistics_match_oracle(gpu):
    """Config 2's servo-controlled specimen (tests/servo_protocol.py), five seeds."""
    import servo_protocol as SP
    from sudodem_gb300 import Engine
    d = _load("servo_")
    oracle_runs = [d[f"servo_oracle/{s}"] for s in SEEDS]
    runs = []
    for s in SEEDS:
        spec, cfg = SP.spec_and_config(s)
        e = Engine(device=0)
        e.load(spec)
        runs.append(SP.Run(spec, e, cfg))
    while not all(r.done for r in runs):
        live = [r for r in runs if not r.done]
        for r in live:
            r.advance()
        for r in live:
            r.check()
    gpu_runs = [r.result for r in runs]
    res = agree(gpu_runs, oracle_runs, SERVO_METRICS)
    for m, (ok, diff, allowed) in res.items():
        g = np.mean([r[m] for r in gpu_runs])
        o = np.mean([r[m] for r in oracle_runs])
        print(f"servo {m}: gpu {g:.6g} oracle {o:.6g} |diff| {diff:.4g} allowed {allowed:.4g}")
    assert all(ok for ok, _, _ in res.values())
