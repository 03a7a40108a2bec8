"""The public headers on their own (CPU, no device code runs): every C header
compiles as C99 with warnings as errors, alone and all together, and the C++
class's check program compiles and links against the library."""
import os
import shutil
import subprocess

import pytest

from crystalgrowth_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
C_HEADERS = sorted(h for h in os.listdir(INC) if h.endswith(".h"))


@pytest.mark.parametrize("header", C_HEADERS + ["(all)"])
def test_c_header_compiles_as_c99(tmp_path, header):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    names = C_HEADERS if header == "(all)" else [header]
    src = tmp_path / "use.c"
    src.write_text("".join('#include "%s"\n' % h for h in names) + "int main(void) { return 0; }\n")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only", "-I", INC, str(src)],
                   check=True)


def test_cpp_class_check_program_compiles_and_links(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no C++ compiler")
    libdir = os.path.dirname(_lib.LIB_PATH)
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    subprocess.run([gxx, "-std=c++14", "-Wall", "-Werror", "-O1", "-I", INC,
                    os.path.join(ROOT, "tests", "cpp", "kobayashi_hpp_check.cpp"), "-o", str(tmp_path / "check"),
                    "-L", libdir, "-lkobayashi_gpu", "-Wl,-rpath," + libdir], check=True)
