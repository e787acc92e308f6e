"""The C ABI (CPU): libmafem.so loads and exports exactly the functions include/mafem.h declares."""
import os
import re
import subprocess

from _cases import M, ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "mafem.h")).read()
    return sorted(set(re.findall(r"\b(mafem_[A-Za-z_0-9]+)\s*\(", src)))


def test_symbols_exported():
    M.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", M.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (mafem_[A-Za-z_0-9]+)", out))
    declared = _declared()
    assert "mafem_calc_r_K" in declared
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    undeclared = sorted(exported - set(declared))
    assert not undeclared, undeclared


def test_no_device_needed_for_host_calls():
    p = M.Params(motion=M.ALEVB, scenario=M.F_PULL, num1el=6, num2el=6, length=1.0)
    mesh = M.Mesh(p)
    assert M.footprint_bytes(mesh) > 0
    assert M.footprint_bytes(mesh, M.FP32_REFINE) < 2 * M.footprint_bytes(mesh)
