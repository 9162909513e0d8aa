"""The C-ABI library loads and exports every symbol include/sqdem.h declares (no GPU needed)."""
import os
import re

import numpy as np

import oracle as O
from sudodem_gb300 import _native, build, shapes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "sqdem.h")).read()
    return sorted(set(re.findall(r"\b(sqdem_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_header_symbols():
    build.build()
    lib = _native.load_library()
    decl = declared_symbols()
    assert len(decl) >= 20
    for name in decl:
        assert hasattr(lib, name), name
    assert set(decl) == set(_native.exported_symbols())


def test_shape_props_host_helper_matches_oracle_bitwise():
    rng = np.random.default_rng(3)
    for _ in range(50):
        s = [*rng.uniform(0.5e-3, 2e-3, 3), *rng.uniform(0.2, 1.8, 2)]
        a = _native.shape_props(*s)
        b = O.shape_props(*s)
        c = np.asarray(shapes.shape_props(*s))
        assert np.array_equal(a, b)
        assert np.array_equal(a, c)


def test_building_inputs_loads_no_native_library():
    """Scene generation (the inputs of every benchmark arm) must not map libsqdem_gpu.so."""
    import subprocess
    import sys
    code = ("import sudodem_gb300.assemblies as a; a.periodic_cell(50, seed=1); a.walled_lattice(40, seed=2); "
            "import sys; print(any(n.endswith('libsqdem_gpu.so') for n in open('/proc/self/maps').read().split()))")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, check=True)
    assert out.stdout.strip() == "False", out.stdout + out.stderr


def test_engine_without_gpu_fails_loudly():
    import pytest
    try:
        import torch
        has = torch.cuda.is_available()
    except Exception:
        has = False
    if has:
        pytest.skip("a GPU is present")
    with pytest.raises(_native.SqdemError):
        _native.Engine(device=0)


def test_adjoint_without_gpu_fails_loudly():
    import pytest
    try:
        import torch
        has = torch.cuda.is_available()
    except Exception:
        has = False
    if has:
        pytest.skip("a GPU is present")
    from sudodem_gb300.adjoint import AdjointWindow
    with pytest.raises(_native.SqdemError):
        AdjointWindow(0)
