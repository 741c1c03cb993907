"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares."""
import glob
import os
import re

import _golden  # noqa: F401  (sets up sys.path through conftest)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(eh_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_boundary():
    names = declared()
    for must in ("eh_matrix_build", "eh_count_triangles", "eh_count_cliques", "eh_count_lollipops",
                 "eh_similar_nodes", "eh_hgraph_read_binary", "eh_last_error"):
        assert must in names


def test_every_declared_symbol_is_exported(eh):
    import ctypes
    lib = ctypes.CDLL(eh.lib_path())
    missing = [n for n in sorted(declared()) if not hasattr(lib, n)]
    assert not missing, missing


def test_errors_without_gpu_work(eh):
    # Argument errors are reported as status codes with a message, never a crash.
    import ctypes as C
    L = eh.load()
    h = C.c_void_p()
    assert L.eh_matrix_get_info(None, None) == 1
    assert b"NULL" in L.eh_last_error()
    assert L.eh_hgraph_read_binary(b"/nonexistent/graph.bin", C.byref(h)) == 5
    assert L.eh_status_string(3) == b"EH_ERR_OUT_OF_MEMORY"
