"""The C-ABI libraries load and export every function their headers declare
(no compute calls: this runs without a GPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
LIB = ROOT / "gpugi_gb300" / "lib"

HEADERS = {
    "gpugi_cuda.h": "libgpugi_cuda.so",
    "gpugi_bvhmake.h": "libgpugi_bvhmake.so",
}


def declared_functions(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = set()
    for m in re.finditer(r"(?:^|;|\})\s*(?!typedef)[A-Za-z_][\w\s\*]*?\b(gpugi_\w+)\s*\(", text, flags=re.M):
        names.add(m.group(1))
    return sorted(names)


@pytest.mark.parametrize("header,libname", sorted(HEADERS.items()))
def test_exports_every_declared_symbol(built, header, libname):
    names = declared_functions(ROOT / "include" / header)
    assert len(names) >= 5
    lib = C.CDLL(str(LIB / libname))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"{libname} lacks {missing}"


def test_checked_library_exports_the_same_symbols(built):
    """The bounds-checked build (-DGPUGI_CHECKED=1) is the same C ABI."""
    names = declared_functions(ROOT / "include" / "gpugi_cuda.h")
    lib = C.CDLL(str(LIB / "libgpugi_cuda_checked.so"))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"libgpugi_cuda_checked.so lacks {missing}"
    lib.gpugi_version.restype = C.c_char_p
    assert lib.gpugi_version().endswith(b"checked")
    plain = C.CDLL(str(LIB / "libgpugi_cuda.so"))
    plain.gpugi_version.restype = C.c_char_p
    assert not plain.gpugi_version().endswith(b"checked")


def test_all_headers_covered():
    for h in (ROOT / "include").glob("*.h"):
        assert h.name in HEADERS, f"{h.name} has no library mapping in this test"

