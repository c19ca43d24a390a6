"""The host FP64 symmetric eigensolver used by the PCA basis's Rayleigh-Ritz
step (scarf_gb300/csrc/symeig.cpp), compiled with the host compiler and
checked against numpy's LAPACK eigh (no GPU)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "scarf_gb300", "csrc")


@pytest.fixture(scope="module")
def symeig(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("symeig")
    wrap = d / "wrap.cpp"
    wrap.write_text('#include "symeig.h"\n'
                    'extern "C" int symeig(int n, const double* a, double* w, double* v) '
                    '{ return sg::symeig_host(n, a, w, v); }\n')
    so = d / "libsymeig.so"
    subprocess.run([cxx, "-O2", "-shared", "-fPIC", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(CSRC, "symeig.cpp"), str(wrap), "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))

    def run(A):
        n = A.shape[0]
        a = np.asfortranarray(A, dtype=np.float64)
        w = np.zeros(n)
        v = np.zeros((n, n), order="F")
        p = ctypes.c_void_p
        rc = lib.symeig(n, p(a.ctypes.data), p(w.ctypes.data), p(v.ctypes.data))
        return rc, w, v
    return run


def cases():
    rng = np.random.default_rng(5)
    m = rng.standard_normal((67, 67))
    near = np.diag(np.sort(rng.uniform(1e5, 1.3e5, 67))) + 1e-2 * (m + m.T)
    near[5, 5] = near[6, 6] + 1e-3                      # a near-degenerate pair
    m2 = rng.standard_normal((40, 40))
    low = m2[:, :3] @ m2[:, :3].T                      # rank 3: a 37-fold zero eigenvalue
    return {"1x1": np.array([[3.0]]), "2x2": np.array([[2.0, 1.0], [1.0, 2.0]]),
            "diagonal": np.diag([3.0, -1.0, 2.0, 2.0, 0.0]), "zero": np.zeros((6, 6)),
            "dense": (m + m.T) / 2, "nearly_diagonal": near, "rank3": low}


@pytest.mark.parametrize("name", sorted(cases()))
def test_symeig_matches_lapack(symeig, name):
    A = cases()[name]
    rc, w, v = symeig(A)
    assert rc == 0
    n = A.shape[0]
    ref = np.linalg.eigvalsh(A)
    scale = max(1.0, np.abs(ref).max())
    assert np.all(np.diff(w) >= 0)                                   # ascending
    assert np.abs(w - ref).max() <= 1e-13 * scale
    assert np.abs(v.T @ v - np.eye(n)).max() <= 1e-13 * n
    assert np.abs(A @ v - v * w).max() <= 1e-13 * scale * n


def test_symeig_reads_the_lower_triangle_only(symeig):
    rng = np.random.default_rng(2)
    m = rng.standard_normal((9, 9))
    A = (m + m.T) / 2
    junk = A + np.triu(rng.standard_normal((9, 9)), 1)               # garbage above the diagonal
    assert np.array_equal(symeig(A)[1], symeig(junk)[1])
