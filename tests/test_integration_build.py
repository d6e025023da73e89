"""CPU: complete CVODE and ARKODE user programs with the GB300 modules plugged
in (tests/integration/cvode_heat2d_gb300.c, arkode_bruss3d_gb300.c) compile
against the reference's own headers -- the GB300 headers deferring to them --
and link against the reference's integrator library and libsundials_gb300.so:
the drop-in works at the source and link level.  (Running them needs a GB300
and the reference library built for that machine; the GPU tests drive the
same objects through the CVODE and ARKStep restatements instead.)"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF_LIB = ROOT / "oracle" / "_ref" / "libsundials_ref.so"


def _ref_include():
    from sundials_gb300 import build
    return build.REFERENCE_SRC / "include"


@pytest.mark.skipif(not (_ref_include().exists() and REF_LIB.exists()),
                    reason="reference headers / library not on this machine")
@pytest.mark.parametrize("program", ["cvode_heat2d_gb300", "arkode_bruss3d_gb300"])
def test_user_program_compiles_and_links(program, gb300_lib, tmp_path):
    from sundials_gb300 import build
    cc = shutil.which("gcc")
    assert cc
    exe = tmp_path / program
    cmd = [cc, "-O1", "-Wall", "-Werror", "-Wno-unused-parameter",
           "-I", str(ROOT / "oracle" / "ref_config"), "-I", str(_ref_include()),
           "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "integration" / (program + ".c")),
           "-o", str(exe), str(REF_LIB), str(build.LIB), "-lm",
           f"-Wl,-rpath,{REF_LIB.parent}", f"-Wl,-rpath,{build.LIB.parent}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert exe.exists()
