"""The C example of INTEGRATION.md compiles and links against
include/euler2d.h and the built libeuler2d.so (not run: it needs a GPU and
the reference's mesh file)."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_integration_c_example_compiles(lib, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        text = f.read()
    blocks = re.findall(r"```c\n(.*?)```", text, re.S)
    assert len(blocks) == 1
    lines = blocks[0].splitlines()
    includes = [l for l in lines if l.startswith("#include")]
    body = [l for l in lines if not l.startswith("#include")]
    src = tmp_path / "example.c"
    src.write_text("\n".join(includes) + "\nint main(void) {\n" + "\n".join(body) + "\nreturn 0;\n}\n")
    libdir = os.path.join(ROOT, "gpueularsolver2d_gb300", "lib")
    res = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-Wno-unused-variable",
                          f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", str(tmp_path / "example"),
                          f"-L{libdir}", "-leuler2d", f"-Wl,-rpath,{libdir}"],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
