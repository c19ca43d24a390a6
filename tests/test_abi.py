"""The C ABI library builds, loads and exports every entry point the header
declares; without a GPU every entry point fails loudly (no CPU fallback)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "scarf_gb300.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*|size_t|unsigned long long|double)\s+(sg_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from scarf_gb300 import build
    try:
        return str(build.build())
    except RuntimeError as e:  # pragma: no cover - nvcc absent
        pytest.skip(f"cannot build: {e}")


def test_header_declares_entry_points():
    names = declared()
    for n in ("sg_normalize_csr", "sg_zstats", "sg_covariance", "sg_pca_basis", "sg_project", "sg_knn",
              "sg_smooth", "sg_fuzzy_union", "sg_kmeans_minibatch", "sg_blosc_decode", "sg_blosc_encode", "sg_calc_snn", "sg_merge_graphs", "sg_umap_layout", "sg_create", "sg_destroy", "sg_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (sg_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing


def test_library_loads_and_binding_matches(lib_path):
    from scarf_gb300 import _lib
    lib = _lib.load()
    assert lib.sg_version() >= 1
    assert set(_lib.exported_symbols()) == set(declared())
    # a call without a GPU reports an error instead of computing anything
    h = ctypes.c_void_p()
    rc = lib.sg_create(0, 0, ctypes.byref(h))
    assert rc != 0
    assert lib.sg_last_error()


def test_python_entry_points_refuse_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from scarf_gb300 import kernels
    with pytest.raises(RuntimeError):
        kernels.handle()


def _declared_arities():
    """Parameter count of every sg_ declaration in the header."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"(sg_\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_table_matches_header_arity():
    """Every ctypes signature has as many arguments as its C declaration."""
    from scarf_gb300 import _lib
    arity = _declared_arities()
    bad = {n: (len(args), arity.get(n)) for n, (_, args) in _lib.SIGNATURES.items() if arity.get(n) != len(args)}
    assert not bad, bad
