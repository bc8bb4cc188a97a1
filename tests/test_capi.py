"""The C-ABI library loads without a GPU and exports every function include/*.h declares."""
import ctypes
import glob
import os
import re

from randomwalk_nmr_gb300 import engine as eng
from randomwalk_nmr_gb300 import host

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(rwnmr_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "rwnmr_cpmg_run" in names and "rwnmr_place_walkers" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_match_headers(built_lib):
    declared = declared_functions()
    assert set(eng.EXPORTS) | set(host.HOST_EXPORTS) <= declared


def test_version_string(built_lib):
    lib = eng.load_library()
    assert b"sm_103a" in lib.rwnmr_version()


def test_null_context_is_rejected_without_gpu(built_lib):
    lib = eng.load_library()
    assert lib.rwnmr_ctx_create(None, 0) == 1  # RWNMR_ERR_INVALID before touching CUDA
    assert lib.rwnmr_last_error(None) == b"null context"
