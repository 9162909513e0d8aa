"""The double-float routines compute the same on the GPU as in the host build, bit for bit
(tests/ff_device_probe.cu against tests/ff_host.cu): the elementary functions and whole
Disfunction evaluations on random inputs.  The CPU tests of the mixed form (test_ff_host.py)
rely on this equality."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import test_ff_host

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
PROBE = os.path.join(test_ff_host.BUILD, "libff_device_probe.so")
DP = C.POINTER(C.c_double)


def _p(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(DP)


def _build(out, srcs, flags):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out) for s in srcs):
        os.makedirs(test_ff_host.BUILD, exist_ok=True)
        r = subprocess.run([nvcc, *flags, "-shared", "-o", out + ".tmp", srcs[0]], stdout=subprocess.PIPE,
                           stderr=subprocess.STDOUT)
        assert r.returncode == 0, r.stdout.decode(errors="replace")
        os.replace(out + ".tmp", out)
    return C.CDLL(out)


@pytest.fixture(scope="module")
def libs(gpu):
    host = _build(test_ff_host.LIB, test_ff_host.SOURCES,
                  ["-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--fmad=false",
                   "-diag-suppress", "1444"])
    dev = _build(PROBE, [os.path.join(HERE, "ff_device_probe.cu")] + test_ff_host.SOURCES[1:],
                 ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--fmad=false", "-Xcompiler",
                  "-fPIC", "-diag-suppress", "1444"])
    return host, dev


def test_elementary_functions_device_equals_host(libs):
    host, dev = libs
    rng = np.random.default_rng(5)
    cases = {0: np.exp(rng.uniform(-60, 60, 20000)), 1: rng.uniform(-100, 20, 20000),
             2: rng.uniform(-20, 20, 20000), 3: rng.uniform(-20, 20, 20000)}
    for op, x in cases.items():
        a, b = np.zeros_like(x), np.zeros_like(x)
        host.ffh_elem(op, _p(x), C.c_long(len(x)), _p(a))
        assert dev.ffd_elem(op, _p(x), C.c_long(len(x)), _p(b)) == 0
        bad = np.nonzero(a != b)[0]
        assert len(bad) == 0, (op, len(bad), x[bad[:3]], a[bad[:3]], b[bad[:3]])


def test_disfunction_device_equals_host(libs):
    host, dev = libs
    rng = np.random.default_rng(6)
    n = 20000
    rows = []
    for _ in range(n):
        qA = rng.standard_normal(4); qA /= np.linalg.norm(qA)
        qB = rng.standard_normal(4); qB /= np.linalg.norm(qB)
        pA = rng.uniform(0, 0.1, 3)
        rows.append(np.r_[rng.uniform(0.8e-3, 1.2e-3, 3), rng.uniform(0.3, 1.8, 2), qA, pA,
                          rng.uniform(0.8e-3, 1.2e-3, 3), rng.uniform(0.3, 1.8, 2), qB,
                          pA + rng.standard_normal(3) * 1.2e-3, rng.uniform(-3.2, 3.2), rng.uniform(-1.6, 1.6)])
    inp = np.array(rows)
    a, b = np.zeros((n, 14)), np.zeros((n, 14))
    host.ffh_disfunction_raw(_p(inp), C.c_long(n), _p(a))
    assert dev.ffd_disfunction(_p(inp), C.c_long(n), _p(b)) == 0
    bad = np.nonzero(np.any(a != b, axis=1))[0]
    assert len(bad) == 0, (len(bad), inp[bad[0]].tolist(), a[bad[0]].tolist(), b[bad[0]].tolist())
