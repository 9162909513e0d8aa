"""The adjoint's arithmetic on the host, against the oracle's frozen-pair window (no GPU).

`tests/adjoint_host.cu` builds the __host__ __device__ functions that the CUDA kernels of
`sqdem_adjoint.cu` run (geometry, law and integrator templates on double and on dual numbers,
the per-pair and per-body reverse steps) for the host and runs a whole window with them.  With
the host's libm on both sides the forward equals the oracle's bit for bit, and the reverse pass
is checked against central differences of the oracle, as the GPU tests check the kernels.  Test
infrastructure only: the package never loads this build.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from adjoint_scene import compressed_specimen, lid_weights, oracle_window, params_of

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libadjoint_host.so")
SOURCES = [os.path.join(HERE, "adjoint_host.cu"), os.path.join(ROOT, "sudodem_gb300", "csrc", "sqdem_adjoint.cu"),
           os.path.join(ROOT, "sudodem_gb300", "csrc", "sq_dual.cuh"), os.path.join(ROOT, "include", "sqdem.h")]
NSTEPS = 60
TOL = 1e-5


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


@pytest.fixture(scope="module")
def host():
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc is needed to build the host copy of the adjoint's functions")
    if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in SOURCES):
        os.makedirs(BUILD, exist_ok=True)
        cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--fmad=false",
               "-diag-suppress", "1444", "-Xcompiler", "-Wno-deprecated-declarations", "-shared",
               "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB + ".tmp", SOURCES[0]]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        assert r.returncode == 0, r.stdout.decode(errors="replace")
        os.replace(LIB + ".tmp", LIB)
    lib = C.CDLL(LIB)
    lib.adjh_set_branches.restype = C.c_int
    lib.adjh_set_branches.argtypes = [C.c_int]
    lib.adjh_branch_report.restype = None
    lib.adjh_branch_report.argtypes = [C.POINTER(C.c_double)]
    lib.adjh_run.restype = C.c_double
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    lib.adjh_run.argtypes = [C.c_int, ip, dp, ip, ip, dp, C.c_long, dp, C.c_double, dp, C.c_double, C.c_int, dp, dp,
                             dp, dp, C.c_int, dp, dp, dp, dp, dp, dp, dp, C.POINTER(C.c_ulonglong),
                             C.POINTER(C.c_longlong)]
    return lib


def _run(lib, spec, bodies, recs, eps, mu, Kn, Ks, nsteps, wF, wX):
    """(loss, signature, replay mismatches, gradients, final state) of the host window."""
    n = spec.n_bodies
    nm = len(Kn)

    def d(a):
        return np.ascontiguousarray(a, dtype=np.float64)

    def i(a):
        return np.ascontiguousarray(a, dtype=np.int32)

    arrs = dict(kind=i(spec.kind), shape5=d(spec.shape5), was=i(spec.wall_axis_sense), mat=i(spec.mat),
                st=d(bodies), recs=d(recs), g=d(spec.params["gravity"]), Kn=d(Kn), Ks=d(Ks), fa=d(np.arctan(mu)),
                eps=d(eps), wF=d(wF), wX=d(wX))
    gE, gKn, gKs, gMu, fin = np.zeros((n, 2)), np.zeros(nm), np.zeros(nm), np.zeros(nm), np.zeros((n, 16))
    sig, mism = C.c_ulonglong(), C.c_longlong()
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    Q = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
    L = lib.adjh_run(n, Q(arrs["kind"]), P(arrs["shape5"]), Q(arrs["was"]), Q(arrs["mat"]), P(arrs["st"]),
                     len(recs), P(arrs["recs"]), float(spec.params["dt"]), P(arrs["g"]),
                     float(spec.params["damping"]), nm, P(arrs["Kn"]), P(arrs["Ks"]), P(arrs["fa"]), P(arrs["eps"]),
                     int(nsteps), P(arrs["wF"]), P(arrs["wX"]), P(gE), P(gKn), P(gKs), P(gMu), P(fin), C.byref(sig),
                     C.byref(mism))
    return L, sig.value, mism.value, {"eps": gE, "Kn": gKn, "Ks": gKs, "mu": gMu}, fin


@pytest.fixture(scope="module")
def scene():
    return compressed_specimen()


def test_host_forward_is_the_oracles_bit_for_bit(host, scene):
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF, wX = lid_weights(n), np.zeros((n, 3))
    for nsteps in (1, NSTEPS):
        L, _, _, _, fin = _run(host, spec, bodies, recs, eps, mu, Kn, Ks, nsteps, wF, wX)
        Lo, _, ob = oracle_window(spec, bodies, recs, eps, mu, Kn, Ks, nsteps, wF, wX)
        assert L != 0
        assert np.array_equal(fin[:, 0:3], ob[:, 0:3])
        assert np.array_equal(fin[:, 7:10], ob[:, 7:10])
        assert L == Lo


def test_host_reverse_pass_matches_oracle_central_differences(host, scene):
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF, wX = lid_weights(n), np.zeros((n, 3))
    L0, _, mism, gr, _ = _run(host, spec, bodies, recs, eps, mu, Kn, Ks, NSTEPS, wF, wX)
    assert mism == 0
    _, s0, _ = oracle_window(spec, bodies, recs, eps, mu, Kn, Ks, NSTEPS, wF, wX)
    rng = np.random.default_rng(11)
    part = (spec.kind == 0)[:, None]
    checked = {}
    for trial in range(5):   # 20 seeded directions, five per parameter kind
        dirs = [("eps", (rng.normal(size=eps.shape) * eps * part, 0 * mu, 0 * Kn, 0 * Ks), 3e-8),
                ("mu", (0 * eps, rng.normal(size=mu.shape) * mu, 0 * Kn, 0 * Ks), 3e-5),
                ("Kn", (0 * eps, 0 * mu, rng.normal(size=Kn.shape) * Kn, 0 * Ks), 3e-5),
                ("Ks", (0 * eps, 0 * mu, 0 * Kn, rng.normal(size=Ks.shape) * Ks), 3e-5)]
        for name, (dE, dmu, dKn, dKs), h in dirs:
            vals, sigs = [], []
            for s in (1, -1):
                Ls, ss, _ = oracle_window(spec, bodies, recs, eps + s * h * dE, mu + s * h * dmu, Kn + s * h * dKn,
                                          Ks + s * h * dKs, NSTEPS, wF, wX)
                vals.append(Ls)
                sigs.append(ss)
            if not (sigs[0] == sigs[1] == s0):
                continue
            fd = (vals[0] - vals[1]) / (2 * h)
            ad = float(np.sum(gr["eps"] * dE) + np.sum(gr["mu"] * dmu) + np.sum(gr["Kn"] * dKn) +
                       np.sum(gr["Ks"] * dKs))
            assert abs(fd - ad) <= TOL * abs(ad), (name, trial, fd, ad)
            checked[name] = checked.get(name, 0) + 1
    assert all(checked.get(k, 0) >= 3 for k in ("eps", "mu", "Kn", "Ks")), checked


def _branch_report(lib):
    out = np.zeros(5)
    lib.adjh_branch_report(out.ctypes.data_as(C.POINTER(C.c_double)))
    return dict(zip(("decisions", "disagreements", "unforced", "steps", "surface_sign_changes"),
                    out.astype(np.int64).tolist()))


def test_host_forced_branches_central_differences_at_the_relative_step_1e_6(host, scene):
    """Finite differences within the recorded branches (sqdem_adj_set_branches): the base run
    records every decision, the +h and -h runs take the recorded outcomes.  At the relative step
    1e-6 of the differentiation check the natural runs leave the base run's branches (a
    Levenberg-Marquardt stopping test, a contact gate, a damping sign), the forced ones do not,
    and their central differences match the reverse pass along 20 seeded directions within 1e-5
    relative, or within the loss's rounding noise (measured from runs perturbed by 1e-13, at
    which the linear change is below it) divided by h where the directional derivative is so
    small that the noise dominates the difference; at least 15 of the 20 within 1e-5."""
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF, wX = lid_weights(n), np.zeros((n, 3))
    assert host.adjh_set_branches(2) != 0            # nothing recorded yet
    assert host.adjh_set_branches(1) == 0
    L0, s0, mism, gr, _ = _run(host, spec, bodies, recs, eps, mu, Kn, Ks, NSTEPS, wF, wX)
    rec = _branch_report(host)
    assert mism == 0 and rec["decisions"] > 0 and rec["disagreements"] == 0 and rec["steps"] == NSTEPS
    h = 1e-6
    rng = np.random.default_rng(7)
    part = (spec.kind == 0)[:, None]
    natural_left, within, worst = 0, 0, 0.0
    try:
        assert host.adjh_set_branches(2) == 0
        L1, s1, _, _, _ = _run(host, spec, bodies, recs, eps, mu, Kn, Ks, NSTEPS, wF, wX)
        rep = _branch_report(host)
        assert L1 == L0 and s1 == s0 and rep["disagreements"] == 0 and rep["decisions"] == rec["decisions"]
        noise = 0.0
        for k in range(4):
            d = rng.normal(size=mu.shape) * mu
            Ls, _, _, _, _ = _run(host, spec, bodies, recs, eps, mu + 1e-13 * d, Kn, Ks, NSTEPS, wF, wX)
            noise = max(noise, abs(Ls - L0 - 1e-13 * float(np.sum(gr["mu"] * d))))
        for trial in range(5):
            dirs = [("eps", (rng.normal(size=eps.shape) * eps * part, 0 * mu, 0 * Kn, 0 * Ks)),
                    ("mu", (0 * eps, rng.normal(size=mu.shape) * mu, 0 * Kn, 0 * Ks)),
                    ("Kn", (0 * eps, 0 * mu, rng.normal(size=Kn.shape) * Kn, 0 * Ks)),
                    ("Ks", (0 * eps, 0 * mu, 0 * Kn, rng.normal(size=Ks.shape) * Ks))]
            for name, (dE, dmu, dKn, dKs) in dirs:
                vals, dis = [], 0
                for sgn in (1, -1):
                    args = (eps + sgn * h * dE, mu + sgn * h * dmu, Kn + sgn * h * dKn, Ks + sgn * h * dKs)
                    Ls, _, _, _, _ = _run(host, spec, bodies, recs, *args, NSTEPS, wF, wX)
                    vals.append(Ls)
                    dis += _branch_report(host)["disagreements"]
                natural_left += dis > 0
                fd = (vals[0] - vals[1]) / (2 * h)
                ad = float(np.sum(gr["eps"] * dE) + np.sum(gr["mu"] * dmu) + np.sum(gr["Kn"] * dKn) +
                           np.sum(gr["Ks"] * dKs))
                err = abs(fd - ad)
                worst = max(worst, err / abs(ad))
                within += err <= TOL * abs(ad)
                assert err <= TOL * abs(ad) + 2 * noise / h, (name, trial, fd, ad, dis, noise)
    finally:
        host.adjh_set_branches(0)
    print(f"forced central differences at h=1e-6: {within}/20 within 1e-5 (worst {worst:.2e}, rounding noise of "
          f"the loss {noise:.1e}); {natural_left}/20 directions left a recorded branch when evaluated naturally")
    assert within >= 15 and natural_left > 0


def test_host_forced_differences_converge_as_h_squared(host, scene):
    """On the recorded branch the map is smooth: the error of forced central differences along
    an exponent direction falls as h^2 (the central difference's own truncation) while the
    natural runs would have changed hundreds of decisions at the larger steps."""
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF, wX = lid_weights(n), np.zeros((n, 3))
    try:
        assert host.adjh_set_branches(1) == 0
        _, _, _, gr, _ = _run(host, spec, bodies, recs, eps, mu, Kn, Ks, NSTEPS, wF, wX)
        assert host.adjh_set_branches(2) == 0
        dE = np.random.default_rng(7).normal(size=eps.shape) * eps * (spec.kind == 0)[:, None]
        ad = float(np.sum(gr["eps"] * dE))
        errs, dis = [], []
        for h in (1e-4, 1e-5):
            vals = []
            for sgn in (1, -1):
                Ls, _, _, _, _ = _run(host, spec, bodies, recs, eps + sgn * h * dE, mu, Kn, Ks, NSTEPS, wF, wX)
                vals.append(Ls)
                dis.append(_branch_report(host)["disagreements"])
            errs.append(abs((vals[0] - vals[1]) / (2 * h) - ad) / abs(ad))
    finally:
        host.adjh_set_branches(0)
    print(f"forced central differences along eps: rel. error {errs[0]:.2e} at h=1e-4, {errs[1]:.2e} at 1e-5; "
          f"decisions forced against their natural outcome {dis}")
    assert max(dis[:2]) > 100
    assert 1e-2 / 3 <= errs[1] / errs[0] <= 3e-2
