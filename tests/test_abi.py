"""CPU checks of the drop-in boundary: the C-ABI library loads, exports every
function declared in include/*.h, and its object layouts match the
reference's SUNDIALS v7.5.0 headers (no GPU work is done here)."""
import ctypes as ct
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
INCLUDE = ROOT / "include"
from sundials_gb300 import build as _build  # noqa: E402

REF_INCLUDE = _build.REFERENCE_SRC / "include"


def declared_functions():
    names = []
    for h in sorted(INCLUDE.glob("*.h")):
        text = h.read_text()
        for m in re.finditer(r"SUNGB300_EXPORT[^;{]*?\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            if not m.group(1).startswith("__"):
                names.append(m.group(1))
    return sorted(set(names))


def test_headers_declare_api():
    names = declared_functions()
    assert "N_VNew_GB300" in names and "N_VLinearCombination_GB300" in names
    assert len(names) > 60


def test_library_exports_every_declared_symbol(gb300_lib):
    missing = [n for n in declared_functions() if not hasattr(gb300_lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_ops_table_layout_matches_python_mirror():
    from sundials_gb300 import _lib
    # 56 function pointers: sundials_nvector.h:101-195
    assert ct.sizeof(_lib.NVectorOps) == 56 * 8
    assert ct.sizeof(_lib.GenericNVector) == 3 * 8


def _layout_program(include_dirs, defines):
    src = r"""
#include <stddef.h>
#include <stdio.h>
#include "sundials_gb300_abi.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n",
         sizeof(struct _generic_N_Vector_Ops),
         offsetof(struct _generic_N_Vector_Ops, nvlinearcombination),
         offsetof(struct _generic_N_Vector_Ops, nvdotprodlocal),
         offsetof(struct _generic_N_Vector_Ops, nvprintfile),
         sizeof(struct _generic_SUNMatrix_Ops),
         sizeof(struct _generic_SUNLinearSolver_Ops),
         offsetof(struct _generic_SUNLinearSolver_Ops, solve),
         sizeof(struct _generic_N_Vector));
  return 0;
}
"""
    return src


def test_abi_header_matches_reference_headers(tmp_path):
    """Compile the same layout probe against include/sundials_gb300_abi.h
    alone and against the reference's own headers (when present): identical
    output."""
    src = tmp_path / "layout.c"
    src.write_text(_layout_program(None, None))
    out_own = tmp_path / "own"
    subprocess.run(["gcc", "-I", str(INCLUDE), str(src), "-o", str(out_own)], check=True)
    own = subprocess.run([str(out_own)], capture_output=True, text=True, check=True).stdout
    assert own.split()[0] == str(56 * 8)
    if not REF_INCLUDE.exists():
        pytest.skip("reference headers not on this machine")
    out_ref = tmp_path / "ref"
    subprocess.run(["gcc", "-DSUNGB300_WITH_SUNDIALS", "-I", str(INCLUDE),
                    "-I", str(ROOT / "oracle" / "ref_config"), "-I", str(REF_INCLUDE),
                    str(src), "-o", str(out_ref)], check=True)
    ref = subprocess.run([str(out_ref)], capture_output=True, text=True, check=True).stdout
    assert own == ref
