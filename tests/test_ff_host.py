"""The mixed form's double-float arithmetic on the host, against the oracle (no GPU).

`tests/ff_host.cu` builds sq_ff.cuh / sq_lmff.cuh (the __host__ __device__ routines the mixed
kernels run) for the host; they use only IEEE float operations and fmaf, so the host build
computes what the device computes.  Checked here: the elementary functions against float64
libm, one Disfunction evaluation against the oracle's FP64 one, and whole lmder2 searches
against the oracle's lmder2 from the same inputs (the searches of a dense state: same stop code
and iteration count, depth within the stated tolerance).  Test infrastructure only.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from sudodem_gb300 import assemblies

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libff_host.so")
SOURCES = [os.path.join(HERE, "ff_host.cu")] + [os.path.join(ROOT, "sudodem_gb300", "csrc", f)
                                                 for f in ("sq_ff.cuh", "sq_lmff.cuh", "sq_device.cuh")]
DP = C.POINTER(C.c_double)


def _p(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(DP)


@pytest.fixture(scope="module")
def ffh():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc is needed to build the host copy of the double-float routines")
    if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in SOURCES):
        os.makedirs(BUILD, exist_ok=True)
        cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--fmad=false",
               "-diag-suppress", "1444", "-shared", "-o", LIB + ".tmp", SOURCES[0]]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        assert r.returncode == 0, r.stdout.decode(errors="replace")
        os.replace(LIB + ".tmp", LIB)
    return C.CDLL(LIB)


def _elem(lib, op, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    lib.ffh_elem(op, _p(x), C.c_long(len(x)), _p(out))
    return out


def test_elementary_functions(ffh):
    rng = np.random.default_rng(1)
    x = rng.uniform(0.5, 2, 100000)
    assert np.max(np.abs(_elem(ffh, 0, x) - np.log2(x))) < 1e-14          # log2 near 1: absolute
    x = np.exp(rng.uniform(-60, 60, 100000))
    r = np.log2(x)
    assert np.max(np.abs(_elem(ffh, 0, x) - r) / np.maximum(np.abs(r), 1)) < 1e-14
    x = rng.uniform(-1, 1, 100000)
    assert np.max(np.abs(_elem(ffh, 1, x) / np.exp2(x) - 1)) < 5e-14
    x = rng.uniform(-100, 20, 100000)
    assert np.max(np.abs(_elem(ffh, 1, x) / np.exp2(x) - 1)) < 5e-13
    x = rng.uniform(-4, 4, 100000)
    assert np.max(np.abs(_elem(ffh, 2, x) - np.sin(x))) < 1e-14
    assert np.max(np.abs(_elem(ffh, 3, x) - np.cos(x))) < 1e-14
    x = rng.uniform(-1e-4, 1e-4, 100000)
    assert np.max(np.abs(_elem(ffh, 2, x) / np.sin(x) - 1)) < 1e-14


def _rq(rng):
    q = rng.standard_normal(4)
    return q / np.linalg.norm(q)


def test_disfunction_against_oracle_fp64(ffh):
    """Support points within the FP64 rounding of the global positions (~1e-17 m), including
    angles next to multiples of pi/2 where the FP64 rounding of the reference is reproduced."""
    rng = np.random.default_rng(2)
    errs, flags = [], 0
    for _ in range(4000):
        sA = np.r_[rng.uniform(0.8e-3, 1.2e-3, 3), rng.uniform(0.3, 1.8, 2)]
        sB = np.r_[rng.uniform(0.8e-3, 1.2e-3, 3), rng.uniform(0.3, 1.8, 2)]
        qA, qB = _rq(rng), _rq(rng)
        pA = rng.uniform(0, 0.1, 3)
        pB = pA + rng.standard_normal(3) * 1.2e-3
        pa0, pa1 = rng.uniform(-3.2, 3.2), rng.uniform(-1.6, 1.6)
        out = np.zeros(14)
        ffh.ffh_disfunction(_p(sA), _p(qA), _p(pA), _p(sB), _p(qB), _p(pB), C.c_double(pa0), C.c_double(pa1), _p(out))
        p1, p2, stop = O.disfunction(sA, qA, pA, sB, qB, pB, pa0, pa1)
        assert out[10] == 0   # no evaluation needs the FP64 path here
        errs.append(max(np.max(np.abs(out[0:3] + pA - p1)), np.max(np.abs(out[3:6] + pA - p2))))
        flags += (out[9] > 0) != stop
    errs = np.array(errs)
    assert flags == 0
    assert np.median(errs) < 1e-17 and np.quantile(errs, 0.999) < 1e-15 and errs.max() < 1e-13


def _searches(lib, spec, o):
    b, r = o.bodies(), o.interactions()
    rows = []
    for rec in r:
        i, j = int(rec[0]), int(rec[1])
        if spec.kind[i] or spec.kind[j] or rec[3] == 0:
            continue
        sA, sB = spec.shape5[i], spec.shape5[j]
        pA, pB = b[i, 0:3], b[j, 0:3]
        if np.linalg.norm(pA - pB) > assemblies.shape_props(*sA)[4] + assemblies.shape_props(*sB)[4]:
            continue
        ref = O.lmder2(sA, b[i, 3:7], pA, sB, b[j, 3:7], pB, rec[5:7])
        out = np.zeros(16)
        lib.ffh_lmder2(_p(sA), _p(b[i, 3:7]), _p(pA), _p(sB), _p(b[j, 3:7]), _p(pB), _p(rec[5:7]), _p(out), 1)
        rows.append((ref, out, pA))
    return rows


def test_searches_follow_the_oracles_lmder2(ffh):
    """Whole lmder2 searches of a dense state (2,000 superellipsoids, eps in [0.3, 1.8], a 2.1 mm
    lattice five steps in): every search not deferred to FP64 takes the oracle's stop code and
    iteration count, and the depth of every touching result is within 1e-6 of the oracle's
    (measured: median ~2e-12, max ~3e-8).  Deferred: only searches that reach itmax."""
    spec = assemblies.walled_lattice(2000, seed=3, box=0.03, per_side=12, spacing=2.1e-3, eps_range=(0.3, 1.8))
    o = O.OracleScene.from_spec(spec, threads=os.cpu_count())
    o.step(5)
    rows = _searches(ffh, spec, o)
    assert len(rows) > 5000
    deferred = [r for r in rows if r[1][15] == 2]
    assert len(deferred) <= 0.002 * len(rows)
    assert all(r[0]["iters"] >= 50 or r[0]["stop"] == 3 for r in deferred)
    ended = [r for r in rows if r[1][15] == 1]
    assert all(r[0]["stop"] == int(r[1][13]) and r[0]["iters"] == int(r[1][12]) for r in ended)
    errs = []
    for ref, out, pA in ended:
        assert ref["touching"] == bool(out[11])
        if ref["touching"]:
            dr = np.dot(ref["p1"] - ref["p2"], ref["contact"])
            dm = np.dot(out[2:5] - out[5:8], out[8:11])
            errs.append(abs(dm - dr) / dr)
    errs = np.array(errs)
    assert len(errs) > 1000
    assert np.median(errs) < 1e-10 and errs.max() < 1e-6
