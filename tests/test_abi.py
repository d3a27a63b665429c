"""The C-ABI library loads and exports every entry point include/lbffs_cuda.h declares (CPU only)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "lbffs_cuda.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(lbffs_\w+)\s*\(", txt, re.M)))


def test_header_declares_entry_points():
    names = _declared()
    assert "lbffs_create" in names and "lbffs_step" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(cuda_lib):
    lib = ctypes.CDLL(os.path.join(ROOT, "lbffs_gb300", "liblbffs_cuda.so"))
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_create_rejects_bad_descriptors_without_gpu_calls(cuda_lib):
    import lbffs_gb300 as L
    lib = L.load_library()
    h = ctypes.c_void_p()
    for bad in (L.Desc(0, 4, 4, 19, 0, 0, 0, 0, 0, 0.1), L.Desc(4, 4, 4, 23, 0, 0, 0, 0, 0, 0.1),
                L.Desc(4, 4, 4, 19, 0, 1, 0, 0, 0, 0.1), L.Desc(4, 4, 4, 19, 7, 0, 0, 0, 0, 0.1),
                L.Desc(4, 4, 4, 19, 0, 0, 0, 0, 0, 0.0), L.Desc(4, 4, 4, 19, 0, 0, 0, 0, 0, 0.1, 3)):
        assert lib.lbffs_create(ctypes.byref(bad), ctypes.byref(h)) == L.E_ARG
        assert lib.lbffs_last_error(None)


def test_no_product_code_imports_the_oracle():
    pat = re.compile(r"import oracle|from oracle|liboracle|oracle/_ref|ref_driver")
    for dirpath, _, files in os.walk(os.path.join(ROOT, "lbffs_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                assert not pat.search(open(os.path.join(dirpath, f)).read()), f
