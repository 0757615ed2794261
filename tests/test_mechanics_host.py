"""Mechanics::compute_stress (include/prismspf/utilities/mechanics.h) on the CPU: the Voigt
product sigma = C epsilon of the reference (include/prismspf/utilities/mechanics.h:18-109, a dense
deal.II contraction) equals, bit for bit, the same dense sum in the same order, whether the
stiffness is orthotropic (the products of its zero blocks skipped) or general."""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


@pytest.fixture(scope="module")
def ms(tmp_path_factory):
    out = tmp_path_factory.mktemp("ms_shim") / "libms_shim.so"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "mechanics_shim.cc"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(str(out))
    P = C.POINTER(C.c_double)
    lib.ms_stress3.argtypes = [P, P, P]
    lib.ms_stress2.argtypes = [P, P, P]
    return lib


def dense(Cm, e):
    """The reference's order: s_i = ((C_i0 e_0 + C_i1 e_1) + ...)."""
    n = len(e)
    out = np.empty(n)
    for i in range(n):
        s = Cm[i, 0] * e[0]
        for j in range(1, n):
            s = s + Cm[i, j] * e[j]
        out[i] = s
    return out


def call(fn, Cm, e):
    c = np.ascontiguousarray(Cm, dtype=np.float64)
    ee = np.ascontiguousarray(e, dtype=np.float64)
    s = np.zeros(len(e))
    P = C.POINTER(C.c_double)
    fn(c.ctypes.data_as(P), ee.ctypes.data_as(P), s.ctypes.data_as(P))
    return s


def cubic(c11, c12, c44, n=6):
    Cm = np.zeros((n, n))
    nn = 3 if n == 6 else 2
    Cm[:nn, :nn] = c12
    np.fill_diagonal(Cm[:nn, :nn], c11)
    for i in range(nn, n):
        Cm[i, i] = c44
    return Cm


def test_orthotropic_and_general_stiffness_match_the_dense_product(ms):
    rng = np.random.default_rng(3)
    mats = [cubic(250.0, 150.0, 100.0), cubic(3.7, 1.1, 0.3)]
    ortho = np.zeros((6, 6))
    ortho[:3, :3] = rng.uniform(1, 5, (3, 3))
    ortho[3:, 3:] = np.diag(rng.uniform(1, 5, 3))
    mats.append(ortho)
    general = rng.uniform(-1, 5, (6, 6))
    mats.append(general)
    nearly = cubic(250.0, 150.0, 100.0)
    nearly[0, 4] = 1e-300  # one non-zero coupling: the dense product
    mats.append(nearly)
    for Cm in mats:
        for _ in range(200):
            e = rng.standard_normal(6) * 10.0 ** rng.integers(-8, 3)
            got = call(ms.ms_stress3, Cm, e)
            want = dense(Cm, e)
            assert np.array_equal(got, want), (Cm, e)
    for Cm in (cubic(250.0, 150.0, 100.0, n=3), rng.uniform(-1, 5, (3, 3))):
        for _ in range(200):
            e = rng.standard_normal(3)
            assert np.array_equal(call(ms.ms_stress2, Cm, e), dense(Cm, e))
