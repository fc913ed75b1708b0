"""The C-ABI library builds for sm_103a, loads, and exports every function
declared in include/ionization_gb300.h (no compute calls: runs without a GPU)."""

import ctypes
import os
import re

import pytest

from .conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ionization_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*\*?\s*\*?\s*\b(ion_[A-Za-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "ion_tdma_c128" in names and "ion_sh_split_run_c64" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    from ionization_gb300 import _build, _native

    path = _build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    # the Python binding covers the same set
    assert set(declared_functions()) == set(_native.exported_symbols())


def test_size_queries_without_gpu():
    from ionization_gb300 import _native as nat

    assert nat.value("ion_version") >= 100
    assert nat.value("ion_tdma_scratch_bytes_c128", 100) == 0  # fits one CTA: no scratch
    assert nat.value("ion_tdma_scratch_bytes_c128", 1_000_000) > 16 * 3 * 1_000_000
    assert nat.value("ion_sh_max_n_r_c128") >= 4000
    assert nat.value("ion_line_max_n_c64") >= 4096


def test_struct_layouts_match_header():
    """ctypes mirrors: sizes follow the C layout of the header structs."""
    from ionization_gb300 import _native as nat

    # 8-byte pointers, fields in header order
    assert ctypes.sizeof(nat.ShPlan) == 8 + 4 * 4 + 8 + 4 + 4 + 8 + 4 + 4 + 4 + 4 + 24 * 4
    assert nat.ShSim.g.offset == 0 and nat.ShSim.t.offset == 16
    assert nat.LineSim.t.offset == 16
    assert ctypes.sizeof(nat.CylMesh) == 8 + 9 * 8 + 8 + 2 * 8


def test_struct_offsets_match_the_c_compiler(tmp_path):
    """Every field of every ctypes mirror sits where the C compiler puts the
    header's field of the same name (sizes too)."""
    import shutil
    import subprocess

    from ionization_gb300 import _native as nat

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"ion_sh_sim": nat.ShSim, "ion_sh_plan": nat.ShPlan, "ion_line_sim": nat.LineSim,
               "ion_line_plan": nat.LinePlan, "ion_cyl_mesh": nat.CylMesh, "ion_hop": nat.Hop,
               "ion_psi_row": nat.PsiRow}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ionization_gb300.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "abi"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    seen = 0
    for line in filter(None, out):
        cname, fname, value = line.split()
        py = mirrors[cname]
        got = ctypes.sizeof(py) if fname == "sizeof" else getattr(py, fname).offset
        assert got == int(value), f"{cname}.{fname}: ctypes {got}, C {value}"
        seen += 1
    assert seen == sum(len(p._fields_) + 1 for p in mirrors.values())
