"""The C-ABI library loads without a GPU and exports every entry point include/dsrg.h declares."""
import ctypes as C
import os
import re

from conftest import ROOT


def declared_entry_points():
    text = open(os.path.join(ROOT, "include", "dsrg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*|void \*)\s*(dsrg_\w+)\s*\(", text, re.M)))


def test_header_declares_the_python_list(built):
    import dfpsr_gb300 as d
    assert sorted(d.EXPORTED) == declared_entry_points()


def test_library_exports_every_declared_symbol(built):
    import dfpsr_gb300 as d
    lib = C.CDLL(d.LIB_PATH)
    missing = [name for name in declared_entry_points() if not hasattr(lib, name)]
    assert not missing


def test_context_create_reports_status_without_gpu(built):
    """With no GPU present the ABI returns a status instead of crashing; with a GPU it succeeds."""
    import dfpsr_gb300 as d
    lib = d.lib()
    h = C.c_void_p()
    status = lib.dsrg_context_create(0, C.byref(h))
    if status == 0:
        assert lib.dsrg_context_destroy(h) == 0
    else:
        assert status == 2 and not h.value


def test_null_arguments_are_rejected(built):
    import dfpsr_gb300 as d
    lib = d.lib()
    assert lib.dsrg_context_create(0, None) == 1
    assert lib.dsrg_model_render(None, None, None, None, None, None) == 1
    assert lib.dsrg_renderer_end(None) == 1
