"""The C-ABI library loads and exports every entry point include/rstsr_cuda.h declares (CPU only)."""

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(rstsr_cuda_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "rstsr_cuda_assign_arbitrary" in names
    assert "rstsr_cuda_reduce_axes" in names
    assert "rstsr_cuda_gemm" in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in declared_symbols() if not hasattr(built_lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_every_declared_symbol():
    from rstsr_gb300 import _lib

    bound = set(_lib.exported_names())
    missing = [n for n in declared_symbols() if n not in bound]
    assert not missing, f"no ctypes signature for: {missing}"


def test_version_and_error_plumbing(built_lib):
    from rstsr_gb300 import _lib

    assert b"sm_103a" in built_lib.rstsr_cuda_version()
    # a host-only call that fails sets the thread-local message
    bad = _lib.Layout.make((2, 3), (3, 1))
    out = _lib.Layout()
    rc = built_lib.rstsr_cuda_layout_for_array_copy(C.byref(bad), b"X", C.byref(out))
    assert rc == 2
    assert b"CFK" in built_lib.rstsr_cuda_last_error()


def test_null_context_is_an_error_not_a_crash(built_lib):
    rc = built_lib.rstsr_cuda_ctx_sync(None)
    assert rc != 0


@pytest.mark.parametrize("lang,std", [("c", "c99"), ("c++", "c++17")])
def test_header_is_plain_c_and_cxx(tmp_path, lang, std):
    """include/rstsr_cuda.h is the boundary for any FFI: it compiles as strict
    C99 and as C++17 without warnings (plain pointers, sizes and enums only)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / "use_header.c"
    src.write_text('#include <string.h>\n#include "rstsr_cuda.h"\nint main(void) {\n'
                   '    const char* (*version)(void) = rstsr_cuda_version;\n'
                   '    rstsr_layout l;\n'
                   '    memset(&l, 0, sizeof l);\n'
                   '    (void)version;\n'
                   '    return l.ndim;\n}\n')
    flags = ["-std=" + std, "-Wall", "-Wextra", "-Werror"] + (["-pedantic"] if lang == "c" else ["-x", "c++"])
    res = subprocess.run([cc, *flags, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(tmp_path / "o.o")],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
