"""Readers of the reference's input decks: param.in, mat.in and system.in.

Host-side set-up, restated from src/heatflow/mod_inputs.f90 (read_param :204-360, check_param
:366-596, read_system :602-649, read_mat :654-721, assignD/I/L/S :728-814, val :819-826) and the
material table of src/heatflow/mod_material.f90:54-267.  The result is a
:class:`heatflow_gb300.problem.Problem` that the CUDA path consumes through the C ABI.
"""
from __future__ import annotations

import os
import re
from dataclasses import dataclass, field

import numpy as np

from .problem import Problem

# read_param keywords in readvar order (mod_inputs.f90:283-327); kind: I, D, L, S
PARAM_KEYS = [
    ("IVERB", "I"), ("ntime", "I"), ("time_step", "D"), ("freq", "D"), ("iboundary", "I"),
    ("icattaneo", "I"), ("isteady", "I"), ("power_in", "D"), ("kappaBoundx1", "D"),
    ("kappaBoundy1", "D"), ("kappaBoundz1", "D"), ("_Check_Sparse_Full", "L"),
    ("_Check_Stability", "L"), ("_WriteToTxt", "L"), ("_Percentage_Completion", "L"),
    ("_Test_Run", "L"), ("_InputTempDis", "L"), ("_RunName", "S"), ("_FullRestart", "L"),
    ("T_Bathx1", "D"), ("T_Bathx2", "D"), ("T_Bathy1", "D"), ("T_Bathy2", "D"),
    ("T_Bathz1", "D"), ("T_Bathz2", "D"), ("T_System", "D"), ("T_Bath", "D"),
    ("kappaBound", "D"), ("kappaBoundNx", "D"), ("kappaBoundNy", "D"), ("kappaBoundNz", "D"),
    ("start_ix", "I"), ("end_ix", "I"), ("start_iy", "I"), ("end_iy", "I"), ("start_iz", "I"),
    ("end_iz", "I"), ("write_every", "I"), ("TempDepProp", "I"), ("Periodic", "S"),
    ("heattime", "I"), ("T_BathCG", "D"), ("BR", "D"), ("T_BathCC", "L"), ("CG_dir", "S"),
]


class InputError(ValueError):
    """The reference prints an error and executes `stop` for these inputs."""


def _fortran_real(tok: str) -> float:
    return float(tok.strip().rstrip(",").replace("d", "e").replace("D", "E"))


def _fortran_int(tok: str) -> int:
    return int(tok.strip().rstrip(","))


def _strip_comment(line: str) -> str:
    k = line.find("!")
    return line[:k] if k >= 0 else line


def _keyword_value(line: str):
    """(keyword, value) as assignD/I/L/S see them: keyword = text before the first '=',
    value = text after the last '=' (val, mod_inputs.f90:819-826)."""
    if "=" not in line:
        return None, None
    key = line[: line.index("=")].strip()
    value = line[line.rindex("=") + 1:].strip()
    return key, value


def read_param(text: str) -> dict:
    """read_param + check_param (mod_inputs.f90:204-596).  Returns the parameter dictionary."""
    p = dict(IVERB=1, _Check_Sparse_Full=False, _Check_Stability=False,
             _Percentage_Completion=False, _Test_Run=False, _InputTempDis=False,
             _FullRestart=False, _RunName="default", _WriteToTxt=False, ntime=10, heattime=0,
             write_every=1, time_step=1.0, freq=1.0, iboundary=1, icattaneo=1, isteady=0,
             T_System=300.0, T_Bath=0.0, T_BathCG=0.0, T_BathCC=False, BR=1.0, CG_dir="",
             power_in=0.0, Periodic="", kappaBound=0.0, kappaBoundx1=0.0, kappaBoundy1=0.0,
             kappaBoundz1=0.0, kappaBoundNx=0.0, kappaBoundNy=0.0, kappaBoundNz=0.0,
             TempDepProp=0, start_ix=1, end_ix=0, start_iy=1, end_iy=0, start_iz=1, end_iz=0)
    # T_Bath is read after these defaults are taken (mod_inputs.f90:234-239): all 0 here.
    for k in ("T_Bathx1", "T_Bathx2", "T_Bathy1", "T_Bathy2", "T_Bathz1", "T_Bathz2"):
        p[k] = 0.0
    readvar = [0] * len(PARAM_KEYS)
    for raw in text.splitlines():
        line = _strip_comment(raw)
        if not line.strip():
            continue
        key, value = _keyword_value(line)
        if key is None or value == "":
            continue
        for idx, (name, kind) in enumerate(PARAM_KEYS):
            if key != name:
                continue
            readvar[idx] += 1
            if kind == "I":
                p[name] = _fortran_int(value.split()[0])
            elif kind == "D":
                p[name] = _fortran_real(value.split()[0])
            elif kind == "L":
                if "T" in value or "t" in value:
                    p[name] = True
                if "F" in value or "f" in value:
                    p[name] = False
            else:
                p[name] = value.split()[0] if value.split() else ""
    per = p["Periodic"]
    p["Periodicx"] = "x" in per or "X" in per
    p["Periodicy"] = "y" in per or "Y" in per
    p["Periodicz"] = "z" in per or "Z" in per
    cg = p["CG_dir"]
    p["CG_x_m"], p["CG_x_p"] = "-x" in cg, "+x" in cg
    p["CG_y_m"], p["CG_y_p"] = "-y" in cg, "+y" in cg
    p["CG_z_m"], p["CG_z_p"] = "-z" in cg, "+z" in cg
    _check_param(p, readvar)
    return p


def _check_param(p: dict, rv: list):
    """check_param, mod_inputs.f90:366-596 (warnings are silent; errors raise)."""
    if any(v > 1 for v in rv):
        raise InputError("ERROR: same KEYWORD apears more than once")
    kb = rv[8:11]
    kbn = rv[28:31]
    if not (p["Periodicx"] and p["Periodicy"] and p["Periodicz"]):
        if (0 in kb or 0 in kbn) and rv[27] == 0:
            raise InputError("ERROR: KappaBoundx,y,z and KappaBound are not set")
        if (all(v == 1 for v in kb) or all(v == 1 for v in kbn)) and rv[27] == 0:
            rv[27] = 1
        if (0 in kb or 0 in kbn) and rv[27] == 1:
            for k in ("kappaBoundx1", "kappaBoundy1", "kappaBoundz1", "kappaBoundNx",
                      "kappaBoundNy", "kappaBoundNz"):
                p[k] = p["kappaBound"]
    if rv[41] == 1 and p["T_BathCG"] > 0:
        for k in range(19, 25):
            rv[k] = 1
        rv[26] = 1
    if any(rv[k] == 0 for k in range(19, 25)):
        for k in ("T_Bathx1", "T_Bathx2", "T_Bathy1", "T_Bathy2", "T_Bathz1", "T_Bathz2"):
            p[k] = p["T_Bath"]
    if rv[41] == 0:
        p["T_BathCG"] = 0.0


@dataclass
class Material:
    index: int
    heat_capacity: float = 0.0
    h_conv: float = 0.0
    kappa: float = 0.0
    kappa3D: float = 0.0
    rho: float = 0.0
    sound_speed: float = 0.0
    tau: float = 0.0
    em: float = 0.0


MAT_KEYS = ["heat_capacity", "h_conv", "kappa", "kappa3D", "rho", "sound_speed", "tau", "em"]


def read_mat(text: str) -> list[Material]:
    """read_mat, mod_inputs.f90:654-721."""
    mats: list[Material] = []
    found = [0] * 8
    cur = None
    for raw in text.splitlines():
        line = _strip_comment(raw)
        if not line.strip():
            continue
        first = line.split()[0]
        if re.fullmatch(r"[+-]?\d+", first.rstrip(",")):
            idx = int(first.rstrip(","))
            if idx == 0:
                if any(v != 1 for v in found):
                    raise InputError(f"Error in parameters : material {found}")
                found = [0] * 8
            else:
                cur = Material(index=idx)
                mats.append(cur)
                if len(mats) == 101:
                    raise InputError("Error: code does not suporrt over 100 materials")
            continue
        key, value = _keyword_value(line)
        if key is None or cur is None:
            continue
        for k, name in enumerate(MAT_KEYS):
            if key == name and value != "":
                found[k] += 1
                setattr(cur, name, _fortran_real(value.split()[0]))
    seen = set()
    for m in mats:
        if m.index in seen:
            raise InputError(f"Error: Duplicate material index {m.index}")
        seen.add(m.index)
    return mats


@dataclass
class System:
    nx: int
    ny: int
    nz: int
    lx: float
    ly: float
    lz: float
    imaterial: np.ndarray = field(repr=False)
    iheater: np.ndarray = field(repr=False)


def read_system(text: str) -> System:
    """read_system, mod_inputs.f90:602-649: dims, box lengths, then per z-plane one separator
    line followed by ny lines of nx `material:heater` tokens."""
    lines = text.splitlines()
    nx, ny, nz = (int(t) for t in lines[0].split()[:3])
    lx, ly, lz = (_fortran_real(t) for t in lines[1].split()[:3])
    imat = np.zeros(nx * ny * nz, np.int64)
    iheat = np.zeros(nx * ny * nz, np.int64)
    pos = 2
    for iz in range(nz):
        pos += 1  # the line before each plane
        for iy in range(ny):
            if pos >= len(lines):
                raise InputError("Error: Unexpected EOF system.in")
            toks = lines[pos].split()
            pos += 1
            for ix in range(nx):
                m, h = toks[ix].split(":")
                I = ix + nx * (iy + ny * iz)
                imat[I] = int(m)
                iheat[I] = int(h)
    return System(nx, ny, nz, lx, ly, lz, imat, iheat)


# Built-in materials, mod_material.f90:116-265.  tau/em are left unchanged by the reference for
# the entries that do not set them; here they default to 0.
BUILTIN = {
    100: dict(heat_capacity=1.0, h_conv=21.4, kappa=1.0, kappa3D=0.02587, rho=1.0, tau=0.0),
    140: dict(heat_capacity=4200.0, h_conv=0.0, kappa=130.0, kappa3D=130.0, rho=2328.0, sound_speed=8433.0),
    3001: dict(heat_capacity=840.0, kappa=0.19, kappa3D=0.19, rho=941.0, sound_speed=1000.0),
    3002: dict(heat_capacity=1100.0, kappa=1.42, kappa3D=1.42, rho=1700.0, sound_speed=1000.0),
    3003: dict(heat_capacity=1400.0, kappa=1.59, kappa3D=1.59, rho=1800.0, sound_speed=1000.0),
    3004: dict(heat_capacity=2300.0, kappa=1.25, kappa3D=1.25, rho=2300.0, sound_speed=1000.0),
    9001: dict(heat_capacity=3421.0, kappa=0.6, kappa3D=0.0, rho=1090.0, sound_speed=3.0),
    9002: dict(heat_capacity=3391.0, kappa=0.209, kappa3D=0.0, rho=1109.0, sound_speed=3.0),
    9003: dict(heat_capacity=2348.0, kappa=0.317, kappa3D=0.0, rho=911.0, sound_speed=3.0),
    310: dict(heat_capacity=700.0, kappa=130.0, kappa3D=130.0, rho=2329.0, sound_speed=8433.0),
    320: dict(heat_capacity=720.0, kappa=1.4, kappa3D=1.4, rho=2400.0, sound_speed=5970.0, tau=1.0),
    330: dict(heat_capacity=236.0, kappa=427.0, kappa3D=429.0, rho=10524.0, sound_speed=3650.0),
    340: dict(heat_capacity=1500.0, kappa=0.2, kappa3D=0.2, rho=1153.0, sound_speed=8433.0, tau=1.0),
    350: dict(heat_capacity=361.0, kappa=10.2, kappa3D=10.2, rho=7140.0, sound_speed=3650.0, tau=1.0),
}


def material(imaterial: int, mats: list[Material]) -> Material:
    """material(), mod_material.f90:54-267."""
    if imaterial <= 0:
        raise InputError(f"Error: imaterial_type not recognized: {imaterial}")
    if imaterial <= 99:
        for m in mats:
            if m.index == imaterial:
                return m
        raise InputError(f"Error: imaterial_type not recognized: {imaterial}")
    if imaterial not in BUILTIN:
        raise InputError(f"Error: imaterial_type not recognized: {imaterial}")
    return Material(index=imaterial, **BUILTIN[imaterial])


def build_problem(param: dict, mats: list[Material], system: System) -> Problem:
    """set_global_variables' per-cell part (mod_setup.f90:53-68) as a Problem."""
    N = system.nx * system.ny * system.nz
    cache = {}
    kappa = np.empty(N)
    rho = np.empty(N)
    hc = np.empty(N)
    tau = np.empty(N)
    em = np.empty(N)
    for I in range(N):
        im = int(system.imaterial[I])
        if im not in cache:
            cache[im] = material(im, mats)
        m = cache[im]
        kappa[I], rho[I], hc[I], tau[I], em[I] = m.kappa, m.rho, m.heat_capacity, m.tau, m.em
    cg = (param["CG_x_m"], param["CG_x_p"], param["CG_y_m"], param["CG_y_p"], param["CG_z_m"],
          param["CG_z_p"])
    return Problem(
        nx=system.nx, ny=system.ny, nz=system.nz, lx=system.lx, ly=system.ly, lz=system.lz,
        kappa=kappa, rho=rho, heat_capacity=hc, tau=tau, em=em, iheater=system.iheater,
        power_in=param["power_in"], freq=param["freq"], time_step=param["time_step"],
        heated_steps=param["heattime"], icattaneo=param["icattaneo"], isteady=param["isteady"],
        periodic=(int(param["Periodicx"]), int(param["Periodicy"]), int(param["Periodicz"])),
        cg_face=tuple(int(c) for c in cg),
        kappa_bound=(param["kappaBoundx1"], param["kappaBoundNx"], param["kappaBoundy1"],
                     param["kappaBoundNy"], param["kappaBoundz1"], param["kappaBoundNz"]),
        t_bath_face=(param["T_Bathx1"], param["T_Bathx2"], param["T_Bathy1"], param["T_Bathy2"],
                     param["T_Bathz1"], param["T_Bathz2"]),
        t_bath=param["T_Bath"], t_bath_cg=param["T_BathCG"], br=param["BR"],
        t_system=param["T_System"])


def read_all_files(param_text: str, mat_text: str, system_text: str):
    """read_all_files (mod_inputs.f90:116-196) on in-memory decks: (param, Problem)."""
    param = read_param(param_text)
    mats = read_mat(mat_text)
    system = read_system(system_text)
    return param, build_problem(param, mats, system)


def read_input_dir(path: str):
    """The three files of an ./inputs/ directory."""
    def rd(name):
        fn = os.path.join(path, name)
        if not os.path.exists(fn):
            raise InputError(f"Error cannot find file: {name}")
        return open(fn).read()
    return read_all_files(rd("param.in"), rd("mat.in"), rd("system.in"))


# ---- temperature tables (TempDepProp = 1, mod_tempdep.f90) ------------------------------------
def parse_property_table(text: str, name: str = "table") -> np.ndarray:
    """One material's table in the format of the reference's test/data/tempdep.in: one row per
    line, T (ascending), kappa, rho, heat capacity.  Returns a (rows, 4) array."""
    rows = []
    for line in text.splitlines():
        t = line.split()
        if not t:
            continue
        if len(t) != 4:
            raise InputError(f"Error: {name}: each row needs 4 values (T, kappa, rho, c), got {len(t)}")
        rows.append([_fortran_real(v) for v in t])
        if len(rows) > 1 and not rows[-1][0] > rows[-2][0]:
            raise InputError(f"Error: {name}: temperatures must ascend")
    if len(rows) < 2:
        raise InputError(f"Error: {name}: a table needs at least two rows")
    return np.asarray(rows, dtype=np.float64)


def material_tables(inputs_dir: str, imaterial) -> tuple[list, np.ndarray]:
    """ChangeProp's lookup (mod_tempdep.f90:44-55): every material of the grid that has a file
    <inputs_dir>/MatTable<imaterial> gets that table (materials in ascending index order); the
    others keep fixed properties.  Returns (tables, cell_table) for HeatFlow.set_property_tables
    (cell_table: the table of each cell, or -1).  The reference builds the name with
    char(imaterial), the character whose code is the index -- evidently meant as the decimal
    index, which is what is used here."""
    imaterial = np.asarray(imaterial, dtype=np.int64)
    tables, index = [], {}
    for m in sorted(set(int(v) for v in np.unique(imaterial))):
        path = os.path.join(inputs_dir, f"MatTable{m}")
        index[m] = -1
        if os.path.exists(path):
            with open(path) as f:
                tables.append(parse_property_table(f.read(), path))
            index[m] = len(tables) - 1
    cell_table = np.array([index[int(v)] for v in imaterial], dtype=np.int32)
    return tables, cell_table


# ---- restart / output formats (mod_output.f90:225-237, mod_init_evolve.f90:66-140) ----------
def format_temp_file(values) -> str:
    """final_print's layout: 6 values per line, ES16.8 with 1X separators, two blank lines."""
    out = []
    vals = list(values)
    for k in range(0, len(vals), 6):
        out.append("".join(_es16_8(v) + " " for v in vals[k:k + 6]))
    out.append("")
    out.append("")
    return "\n".join(out) + "\n"


def _es16_8(v: float) -> str:
    s = f"{v:.8E}"
    mant, exp = s.split("E")
    e = int(exp)
    return f"{mant}E{'+' if e >= 0 else '-'}{abs(e):02d}".rjust(16)


def parse_temp_file(text: str, na: int) -> np.ndarray:
    """read_temp_file: exactly `na` values, 6 per line (errors as the reference's)."""
    vals = []
    for line in text.splitlines():
        toks = line.split()
        if not toks:
            continue
        vals.extend(_fortran_real(t) for t in toks)
    if len(vals) < na:
        raise InputError(f"Error: File contains fewer values than expected ({len(vals)} out of {na}).")
    if len(vals) > na:
        raise InputError("Error: File contains more values than expected.")
    return np.asarray(vals, np.float64)
