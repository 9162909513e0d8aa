"""The mixed-precision form on the GPU (double-float searches on the FP32 pipes, deferred
searches in FP64) against the CPU oracle.

Bar (per touching contact, relative error of the force normal + shear after one step from
identical states): at least 99.9% of contacts within 1e-6, median below 1e-9, on dense states
whose exponents reach the ill-conditioned ends of the configurations (walled eps 0.3-1.8; the
polydisperse slice of config 4, r 0.5-2 mm, eps 0.2-1.0; a periodic cell compressed to
100 kPa).  A contact above 1e-6 counts as within the bar when its error is within three times
the reference's own spread at the double-float level: how far the oracle's force moves when its
transcendental results change by 2^-47 relative (parity_util.oracle_spread), i.e. a contact
whose answer the reference's own arithmetic does not determine to 1e-6 at that precision.
Those contacts are counted and printed.  Also: the device computes exactly the host model of
the double-float searches (tests/ff_host.cu), and the searches it defers get the FP64 kernel's
results bit for bit.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import OracleScene
from parity_util import by_pair, oracle_spread, rel_force_errors, snapshot_into, touching_common
from sudodem_gb300 import Engine, assemblies

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TILE = os.path.join(HERE, "golden", "config1_tile.npz")


def one_step(spec, orc, precision, periodic=False, spread=True):
    eng = Engine(device=0, precision=precision)
    eng.load(spec)
    eng.set_lm_spread(spread)
    snapshot_into(eng, orc, periodic=periodic)
    eng.step(1)
    rep = eng.sync()
    return eng, rep


FF_REL = 2.0 ** -47      # relative rounding of a double-float value


def compare(spec, orc, label, periodic=False):
    state = (orc.bodies(), orc.interactions(), orc.scalars(), orc.cell() if periodic else None)
    spread = oracle_spread(spec, state, rel=FF_REL, threads=os.cpu_count())
    mixed, rep_m = one_step(spec, orc, "mixed", periodic)
    fp64, rep_d = one_step(spec, orc, "fp64", periodic)
    orc.step(1)
    Gm, R, km = touching_common(mixed.interactions(True), orc.interactions())
    Gd, Rd, kd = touching_common(fp64.interactions(True), orc.interactions())
    em, ed = rel_force_errors(Gm, R), rel_force_errors(Gd, Rd)
    sp = np.array([spread.get(k, 0.0) for k in km])
    D = by_pair(fp64.interactions(True))
    for n in np.nonzero(em > 1e-6)[0]:
        g, r, d = Gm[n], R[n], D.get(km[n])
        print(f"  outlier {km[n]}: err {em[n]:.2e} oracle spread {sp[n]:.2e} depth oracle {r[4]:.6e} mixed {g[4]:.6e} fp64 "
              f"{d[4] if d is not None else float('nan'):.6e}; |Fn| {np.linalg.norm(r[26:29]):.3e} "
              f"|Fs| oracle {np.linalg.norm(r[29:32]):.6e} mixed {np.linalg.norm(g[29:32]):.6e}; angles oracle "
              f"{r[5:7]} mixed {g[5:7]} fp64 {d[5:7] if d is not None else None}; shearNew {r[22]} {g[22]}")
    q = lambda x, p: float(np.quantile(x, p))
    print(f"{label}: touching {len(em)}; mixed err median {q(em, .5):.2e} p99 {q(em, .99):.2e} p99.9 "
          f"{q(em, .999):.2e} max {em.max():.2e} frac<=1e-6 {np.mean(em <= 1e-6):.5f} (deferred to FP64: "
          f"{rep_m['fallback_fp64']}, double-float evaluations {rep_m['evals_fp32']}, FP64 {rep_m['evals_fp64']}); "
          f"fp64 err median {q(ed, .5):.2e} max {ed.max():.2e} frac<=1e-6 {np.mean(ed <= 1e-6):.5f}")
    ok = (em <= 1e-6) | (em <= 3 * sp)
    print(f"  above 1e-6: {np.sum(em > 1e-6)}, of which within 3x the oracle's own double-float-level spread: "
          f"{np.sum((em > 1e-6) & ok)}; within the bar {ok.mean():.5f}")
    return em, ed, rep_m, state, ok


def test_mixed_dense_walled_wide_exponents(gpu):
    spec = assemblies.walled_lattice(2000, seed=3, box=0.03, per_side=12, spacing=2.1e-3, eps_range=(0.3, 1.8))
    orc = OracleScene.from_spec(spec, threads=os.cpu_count())
    orc.step(5)
    em, ed, rep, _, ok = compare(spec, orc, "walled 2000 eps 0.3-1.8")
    assert len(em) > 1000
    assert ok.mean() >= 0.999 and np.median(em) < 1e-9
    assert rep["evals_fp32"] > 10 * rep["evals_fp64"]


def test_mixed_polydisperse_config4_slice(gpu):
    spec = assemblies.config4(seed=1, n=5000)
    orc = OracleScene.from_spec(spec, threads=os.cpu_count())
    orc.step(20)
    em, ed, rep, _, ok = compare(spec, orc, "config4 slice 5000")
    assert len(em) > 300
    assert ok.mean() >= 0.999 and np.median(em) < 1e-9


def test_mixed_dense_periodic_100kpa(gpu):
    if not os.path.exists(TILE):
        pytest.skip("tests/golden/config1_tile.npz missing (tests/golden/make_config1_tile.py)")
    spec = assemblies.config1_dense(TILE, tiles=1)
    orc = OracleScene.from_spec(spec, threads=os.cpu_count())
    orc.step(3)
    em, ed, rep, _, ok = compare(spec, orc, "periodic 1600 at 100 kPa", periodic=True)
    assert len(em) > 1000
    assert ok.mean() >= 0.999 and np.median(em) < 1e-9


def _host_model():
    import test_ff_host
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    lib = test_ff_host.LIB
    if not os.path.exists(lib) or any(os.path.getmtime(s) > os.path.getmtime(lib) for s in test_ff_host.SOURCES):
        os.makedirs(test_ff_host.BUILD, exist_ok=True)
        cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--fmad=false",
               "-diag-suppress", "1444", "-shared", "-o", lib + ".tmp", test_ff_host.SOURCES[0]]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        assert r.returncode == 0, r.stdout.decode(errors="replace")
        os.replace(lib + ".tmp", lib)
    return C.CDLL(lib)


def test_device_searches_equal_host_model_and_deferred_equal_fp64(gpu):
    """The angles every double-float search returns on the device equal, bit for bit, those of
    the host build of the same routines from the same start; the searches the host model defers
    (itmax reached) carry on the device the FP64 kernel's angles, bit for bit."""
    spec = assemblies.walled_lattice(2000, seed=3, box=0.03, per_side=12, spacing=2.1e-3, eps_range=(0.3, 1.8))
    orc = OracleScene.from_spec(spec, threads=os.cpu_count())
    orc.step(5)
    b, recs = orc.bodies(), orc.interactions()
    mixed, _ = one_step(spec, orc, "mixed")
    fp64, _ = one_step(spec, orc, "fp64")
    M, D = by_pair(mixed.interactions(True)), by_pair(fp64.interactions(True))
    lib = _host_model()
    dp = C.POINTER(C.c_double)
    P = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(dp)
    same = deferred_same = deferred = searched = 0
    for rec in recs:
        i, j = int(rec[0]), int(rec[1])
        if spec.kind[i] or spec.kind[j] or rec[3] == 0 or (i, j) not in M:
            continue
        sA, sB = spec.shape5[i], spec.shape5[j]
        if np.linalg.norm(b[i, 0:3] - b[j, 0:3]) > assemblies.shape_props(*sA)[4] + assemblies.shape_props(*sB)[4]:
            continue
        out = np.zeros(16)
        lib.ffh_lmder2(P(sA), P(b[i, 3:7]), P(b[i, 0:3]), P(sB), P(b[j, 3:7]), P(b[j, 0:3]), P(rec[5:7]), P(out), 0)
        searched += 1
        if out[13] == 9 and out[12] == 0:
            # the search ends at its first evaluation (separated at the start point): the FP64
            # pre-pass settles it before the double-float kernel and keeps the start angles
            same += np.array_equal(M[(i, j)][5:7], rec[5:7])
            continue
        if out[15] == 2:
            deferred += 1
            deferred_same += np.array_equal(M[(i, j)][5:7], D[(i, j)][5:7])
        else:
            eq = np.array_equal(M[(i, j)][5:7], out[0:2])
            same += eq
            if not eq and searched - same - deferred <= 5:
                print(f"  differs {(i, j)}: start {rec[5:7].tolist()} host {out[0:2].tolist()} (stop {int(out[13])}, k "
                      f"{int(out[12])}, evals {int(out[14])}) device {M[(i, j)][5:7].tolist()} fp64 {D[(i, j)][5:7].tolist()}")
    print(f"searches {searched}: device = host model {same}, deferred {deferred} (= FP64 kernel {deferred_same})")
    assert searched > 5000
    assert deferred_same == deferred
    # a search that ends in a restart from the centre line (Superquadrics_Ig2.cpp:2013-2053) runs
    # a second call on the device that the single-call host model does not
    assert same >= 0.995 * (searched - deferred)


def test_mixed_spare_lane_evaluations_change_nothing(gpu):
    spec = assemblies.walled_lattice(2000, seed=3, box=0.03, per_side=12, spacing=2.1e-3, eps_range=(0.3, 1.8))
    orc = OracleScene.from_spec(spec, threads=os.cpu_count())
    orc.step(5)
    a, _ = one_step(spec, orc, "mixed", spread=True)
    b, _ = one_step(spec, orc, "mixed", spread=False)
    assert np.array_equal(a.interactions(True), b.interactions(True))
    assert np.array_equal(a.body_state(), b.body_state())
