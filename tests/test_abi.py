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


# ---------------------------------------------------------- C host driver --
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = HEADER.parents[1]
DRIVER_SRC = ROOT / "tests" / "abi_driver" / "fsi_mg_driver.c"


def _cc():
    return shutil.which("gcc") or shutil.which("cc")


def test_header_compiles_as_c99_and_cpp():
    for cmd in ([_cc(), "-std=c99", "-x", "c"], [shutil.which("g++") or "g++", "-std=c++11", "-x", "c++"]):
        subprocess.run(cmd + ["-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only", str(HEADER)], check=True)


def build_driver(out_dir: Path) -> Path:
    build_all()
    lib_dir = _native.solver_lib_path().parent
    exe = out_dir / "fsi_mg_driver"
    cuda_lib = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "lib64"
    subprocess.run([_cc(), "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I", str(HEADER.parent),
                    str(DRIVER_SRC), "-o", str(exe), "-L", str(lib_dir), "-lfsi_mg",
                    f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath-link,{cuda_lib}"], check=True)
    return exe


def test_c_driver_builds_against_the_library(tmp_path):
    assert build_driver(tmp_path).exists()


def write_driver_input(path: Path, pr):
    """The driver's input file: the parameter struct, then every array of the
    hand-over in the driver's read order (Fortran memory order)."""
    g = pr.geom
    f = lambda a, t: np.asarray(a, dtype=t).ravel(order="F").tobytes()
    with open(path, "wb") as fh:
        fh.write(bytes(pr.params.to_c()))
        for c in (pr.x, pr.y, pr.z):
            fh.write(f(c, np.float64))
        fh.write(f(g.iblank, np.int8)); fh.write(f(g.ghost, np.int8))
        for a in g.flags:
            fh.write(f(a, np.int8))
        fh.write(np.int32(g.nGhost).tobytes())
        for a in (g.iG, g.jG, g.kG, g.iCI, g.jCI, g.kCI):
            fh.write(f(a if g.nGhost else [], np.int32))
        fh.write(f(g.coeff if g.nGhost else [], np.float64))
        fh.write(f(g.probe if g.nGhost else [], np.float64))
        fh.write(f(g.pgrad, np.float64))
        fh.write(f(pr.nlu0, np.float64))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere16_tanh", "box2d_32"])
def test_c_driver_solves_like_the_python_binding(gpu_built, tmp_path, case):
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    from flow_structure_interaction_fem_ibm_gb300.poisson import solve
    from tests.helpers import sphere_problem
    pr = sphere_problem(16, stretch=1.5) if case == "sphere16_tanh" else P.box2d(32, seed=9)
    pr.params.iterMax_Poisson = 60
    pr.params.restol_Poisson = 1e-9 * float(np.abs(pr.nlu0).max())
    exe = build_driver(tmp_path)
    write_driver_input(tmp_path / "in.bin", pr)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    raw = (tmp_path / "out.bin").read_bytes()
    st, it = np.frombuffer(raw[:8], np.int32)
    maxres = np.frombuffer(raw[8:16], np.float64)[0]
    n = int(np.prod(pr.shape))
    p = np.frombuffer(raw[28:28 + 8 * n], np.float64).reshape(pr.shape, order="F")
    mean = np.frombuffer(raw[28 + 8 * n:], np.float64)[0]
    ref = solve(pr)
    assert (st, it) == (ref["status"], ref["iters"]) and maxres == ref["maxres"]
    assert np.array_equal(p, ref["p"])
    from tests.helpers import cell_volumes, interior
    I = interior(pr)
    fl = 1.0 - pr.geom.iblank[I]
    vol = cell_volumes(pr) * fl
    assert abs(mean - float((ref["p"][I] * vol).sum() / vol.sum())) <= 1e-12 * max(1.0, np.abs(ref["p"]).max())


# ------------------------------------------------- parameter validation --
import pytest

from flow_structure_interaction_fem_ibm_gb300.grid import make_grid
from flow_structure_interaction_fem_ibm_gb300.params import SolverParams
from flow_structure_interaction_fem_ibm_gb300.poisson import FsiMgError, PoissonSolver

BAD_PARAMS = [
    ("periodic", dict(bc=(5, 5, 1, 1, 1, 1)), "periodic"),
    ("pbc", dict(pbc=(2, 2, 2, 2, 2, 3)), "pbc"),
    ("omega_high", dict(omega=2.0), "omega"),
    ("omega_zero", dict(omega=0.0), "omega"),
    ("krylov", dict(outer_krylov=61), "outer_krylov"),
    ("lsor", dict(pp_solver_type=1), "pp_solver_type"),
    ("cycle", dict(mgcycle=(1, 4, 1)), "mgcycle"),
    ("precision", dict(precision_mode=2), "precision_mode"),
    ("ndim", dict(ndim=4), "ndim"),
    ("2d_nz", dict(ndim=2, nz=3), "nz = 2"),
    ("tiny", dict(nx=2), "too small"),
]


@pytest.mark.parametrize("change,match", [(c, m) for _, c, m in BAD_PARAMS], ids=[b[0] for b in BAD_PARAMS])
def test_create_rejects_bad_parameters_before_any_device_call(change, match):
    """fsi_mg_create validates every parameter on the host and returns -1
    with the reason before it looks for a device (no GPU needed)."""
    p = SolverParams(ndim=3, nx=9, ny=9, nz=9)
    for k, v in change.items():
        setattr(p, k, v)
    x, y, z = make_grid(max(p.nx, 3), max(p.ny, 3), max(p.nz, 2))
    with pytest.raises(FsiMgError, match=match):
        PoissonSolver(p, x, y, z)


# ------------------------------------------- Fortran shim vs the header --
SHIM = Path(__file__).resolve().parents[1] / "flow_structure_interaction_fem_ibm_gb300" / "fortran" / "fsi_mg_shim.F90"


def _c_struct(name):
    """(field name, kind, element count) in memory order of a struct of the header."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    end = re.search(r"\}\s*" + name + r"\s*;", text).start()
    body = text[text.rindex("typedef struct {", 0, end) + len("typedef struct {"):end]
    out = []
    for decl in filter(None, (d.strip() for d in body.split(";"))):
        base = "double" if "double" in decl.split()[0:2] or decl.startswith("const double") else "int"
        names = re.sub(r"^(const\s+)?(double|int)\s+", "", decl)
        for item in (n.strip() for n in names.split(",")):
            kind = "ptr" if item.startswith("*") else base
            dims = [int(v) for v in re.findall(r"\[(\d+)\]", item)]
            count = 1
            for v in dims:
                count *= v
            out.append((re.sub(r"[\*\s]|\[.*", "", item).lower(), kind, count))
    return out


def _f_type(name):
    text = "\n".join(l.split("!")[0] for l in SHIM.read_text().splitlines())
    body = re.search(r"TYPE, BIND\(C\) :: " + name + r"\n(.*?)END TYPE " + name, text, flags=re.S).group(1)
    kinds = {"INTEGER(C_INT)": "int", "REAL(C_DOUBLE)": "double", "TYPE(C_PTR)": "ptr"}
    out = []
    for line in filter(None, (l.strip() for l in body.splitlines())):
        decl, names = line.split("::")
        kind = kinds[decl.strip()]
        for item in re.findall(r"\w+(?:\([\d,\s]+\))?", names):
            dims = [int(v) for v in re.findall(r"\d+", item[item.index("("):])] if "(" in item else []
            count = 1
            for v in dims:
                count *= v
            out.append((item.split("(")[0].lower(), kind, count))
    return out


@pytest.mark.parametrize("name", ["fsi_mg_params", "fsi_mg_rhs_ad_fields", "fsi_mg_bc_values"])
def test_fortran_shim_types_match_the_header(name):
    """The shim's BIND(C) types have the C structs' fields, in order, with
    the same kinds and element counts (no Fortran compiler here or on the GPU
    host, so this textual check is what keeps the two layouts together)."""
    assert _f_type(name) == _c_struct(name)


def _c_prototypes():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(fsi_mg_\w+)\s*\(([^)]*)\)\s*;", text):
        args = m.group(2).strip()
        protos[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    return protos


def test_fortran_shim_interfaces_match_the_header():
    """Every BIND(C) interface of the shim binds a declared entry point with
    the same number of arguments."""
    text = re.sub(r"&\s*\n\s*", "", SHIM.read_text())
    found = re.findall(r"FUNCTION\s+\w+\s*\(([^)]*)\)\s*BIND\(C,\s*NAME='(fsi_mg_\w+)'\)", text)
    found += [(a, n) for a, n in re.findall(r"SUBROUTINE\s+\w+\s*\(([^)]*)\)\s*BIND\(C,\s*NAME='(fsi_mg_\w+)'\)", text)]
    protos = _c_prototypes()
    assert len(found) >= 10
    for args, cname in found:
        assert cname in protos, cname
        nargs = 0 if not args.strip() else len(args.split(","))
        assert nargs == protos[cname], (cname, nargs, protos[cname])
