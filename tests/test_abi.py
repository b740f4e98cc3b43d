"""The C-ABI library: loads, exports every symbol include/fsi_mg.h declares,
and its parameter struct matches the header (no GPU needed)."""
import ctypes
import re
from pathlib import Path

from flow_structure_interaction_fem_ibm_gb300 import _native
from flow_structure_interaction_fem_ibm_gb300.build import build_all
from flow_structure_interaction_fem_ibm_gb300.params import FsiMgParams

HEADER = Path(__file__).resolve().parents[1] / "include" / "fsi_mg.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fsi_mg_\w+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    build_all()
    lib = ctypes.CDLL(str(_native.solver_lib_path()))
    names = declared_functions()
    assert "fsi_mg_solve" in names and "fsi_mg_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared_functions()) <= set(_native.SOLVER_SYMBOLS)


def test_params_struct_matches_header():
    text = HEADER.read_text()
    body = text[text.index("typedef struct {"):text.index("} fsi_mg_params;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl or decl.startswith("typedef"):
            decl = decl.replace("typedef struct {", "").strip()
            if not decl:
                continue
        parts = decl.split(None, 1)
        for name in parts[1].split(","):
            fields.append(re.sub(r"\[.*\]", "", name).strip())
    assert fields == [f[0] for f in FsiMgParams._fields_]


def test_geometry_library_exports():
    g = _native.geometry()
    for n in _native.GEOM_SYMBOLS:
        assert hasattr(g, n)
