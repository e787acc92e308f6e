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


# ---- struct layouts: the ctypes mirrors against the header, compiled by gcc ----------
_STRUCTS = {"mafem_params": "_CParams", "mafem_args": "_CArgs", "mafem_mesh_desc": "MeshDesc",
            "mafem_step_stats": "StepStats", "mafem_request": "_CRequest", "mafem_server_stats": "ServerStats",
            "mafem_kernel_times": "KernelTimes", "mafem_batch_stats": "BatchStats"}


def test_struct_layouts_match_the_header(tmp_path):
    """Every struct of include/mafem.h, as the C compiler lays it out, against
    the ctypes mirror in mafem.py: size, and each field's name and offset."""
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "mafem.h"', "int main(void) {"]
    for cname, pyname in _STRUCTS.items():
        st = getattr(M, pyname)
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in st._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, field, v = line.split()
        got[(cname, field)] = int(v)
    for cname, pyname in _STRUCTS.items():
        st = getattr(M, pyname)
        assert got[(cname, "size")] == C_sizeof(st), cname
        for fname, _ in st._fields_:
            assert got[(cname, fname)] == getattr(st, fname).offset, (cname, fname)


def C_sizeof(st):
    import ctypes
    return ctypes.sizeof(st)


def test_create_rejects_a_mesh_the_kernels_would_misread():
    """mafem_create checks the connectivity and index ranges before it touches
    the device (so this runs without a GPU): an IX other than construct_IX's
    tensor-product numbering (Mesh.jl:574-593), or an out-of-range ID / uel_ids
    entry, is MAFEM_ERR_ARG."""
    import ctypes
    import numpy as np
    p = M.Params(motion=M.ALEVB, scenario=M.F_PULL, num1el=4, num2el=4, length=1.0)
    mesh = M.Mesh(p)
    cp, ca = p.c_params(), p.c_args()

    def create_with(field, arr):
        d = M.MeshDesc.from_buffer_copy(mesh.desc)
        setattr(d, field, arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        h = ctypes.c_void_p()
        rc = M.lib().mafem_create(ctypes.byref(d), ctypes.byref(cp), ctypes.byref(ca), M.PLAIN_FP64, ctypes.byref(h))
        return rc, M.lib().mafem_last_error(None).decode()

    ix = np.ascontiguousarray(mesh.IX.T.reshape(-1))  # 9 x numel column-major
    bad = ix.copy()
    bad[[0, 1]] = bad[[1, 0]]  # two nodes of element 1 exchanged
    rc, msg = create_with("IX", bad)
    assert rc == M.ERR_ARG and "tensor-product" in msg
    bad = ix.copy()
    bad[9 * 5 + 4] = mesh.numnp + 7  # a node that does not exist
    rc, msg = create_with("IX", bad)
    assert rc == M.ERR_ARG
    ID = np.ascontiguousarray(mesh.ID.T.reshape(-1))
    bad = ID.copy()
    bad[3] = mesh.nmdf + 1
    rc, msg = create_with("ID", bad)
    assert rc == M.ERR_ARG and "ID" in msg
    uel = np.ascontiguousarray(mesh.area_tables()[0])
    bad = uel.copy()
    bad[2] = 0
    rc, msg = create_with("uel_ids", bad)
    assert rc == M.ERR_ARG and "uel_ids" in msg
