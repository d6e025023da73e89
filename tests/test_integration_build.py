"""CPU: a complete CVODE user program with the GB300 modules plugged in
(tests/integration/cvode_heat2d_gb300.c) compiles against the reference's own
headers -- the GB300 headers deferring to them -- and links against the
reference's CVODE library and libsundials_gb300.so: the drop-in works at the
source and link level.  (Running it needs a GB300 and the reference library
built for that machine; the GPU tests drive the same objects through the
CVODE restatement instead.)"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF_INCLUDE = Path("/root/reference/include")
REF_LIB = ROOT / "oracle" / "_ref" / "libsundials_ref.so"


@pytest.mark.skipif(not (REF_INCLUDE.exists() and REF_LIB.exists()),
                    reason="reference headers / library not on this machine")
def test_cvode_user_program_compiles_and_links(gb300_lib, tmp_path):
    from sundials_gb300 import build
    cc = shutil.which("gcc")
    assert cc
    exe = tmp_path / "cvode_heat2d_gb300"
    cmd = [cc, "-O1", "-Wall", "-Werror", "-Wno-unused-parameter",
           "-I", str(ROOT / "oracle" / "ref_config"), "-I", str(REF_INCLUDE),
           "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "integration" / "cvode_heat2d_gb300.c"),
           "-o", str(exe), str(REF_LIB), str(build.LIB), "-lm",
           f"-Wl,-rpath,{REF_LIB.parent}", f"-Wl,-rpath,{build.LIB.parent}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert exe.exists()
