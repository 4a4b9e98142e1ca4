"""Readers and writers for the reference solver's ``data/*.dat`` input files.

The formats are kept exactly so that the reference program and this solver
consume identical inputs (reference ``src/NmrRelaxationSolve.cpp``):

* ``Nmr_start.dat`` — three integers (ik, jk, kk), each followed by the rest of
  its line (cpp:68-93; CRLF tolerated).
* ``Nmr_data.dat`` — exactly 61 lines ``value<TAB>comment``; a parameter is the
  value of the FIRST line whose comment contains its token (cpp:175-723).
* ``Nmr_grad.dat`` — a count, then one gradient per line (cpp:727-778).
* ``Poro.dat`` — one header line, then ik*jk*kk characters ``'0'``/``'1'`` read
  with ``>> char``; k outermost, then j, then i (cpp:859-872).
* ``Vx.dat`` / ``Vy.dat`` / ``Vz.dat`` — one header line, then (ik+1)*jk*kk,
  ik*(jk+1)*kk, ik*jk*(kk+1) doubles, i outermost, then j, then k
  (cpp:1466-1536); the solver multiplies them by VEL_MULT.
* ``SurfRel{1,2}{Water,Oil}{X,Y,Z}.dat`` — face relaxivities in the layout of
  the velocity files (cpp:1035-1434), read when nSurfRelWater / nSurfRelOil is 1.
* ``n1_init.dat`` — one header line, then ik*jk*kk values read as float, i
  outermost, then j, then k (cpp:974-1006): the first concentration of NCOMP 2.

Array conventions of this package: ``mask[k, j, i]`` (1 = pore), face
velocities ``vx[k, j, i]`` with i in [0, nx] (face i is the low face of cell i),
``vy[k, j, i]`` with j in [0, ny], ``vz[k, j, i]`` with k in [0, nz].
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field, fields

import numpy as np

# Token of each of the 61 lines of Nmr_data.dat, in file order. The attribute
# name is what NmrData calls the parameter.
_DATA_LINES = [
    ("key", "KEY", 1), ("i_print", "IPRINT", 1), ("j_print", "JPRINT", 1), ("k_print", "KPRINT", 1),
    ("nd_print", "Printing on console", 500), ("nd_write", "NDWRIT", 1), ("nd_vid", "NDVID", 1),
    ("nd_ampl", "NDAMPL", 1), ("n_poro", "NPOR", 1), ("n_components", "NCOMP", 1), ("n_fluid", "NFLUID", 1),
    ("n_surf_rel_water", "nSurfRelWater", 0), ("n_surf_rel_oil", "nSurfRelOil", 0),
    ("n_vector_mult", "NVECTOR", 0), ("n_velocity", "NVELOC", 0), ("n_diffusion", "NDIFFUS", 1),
    ("n_direction_field", "NDIRECT_FIELD", 1), ("n_sequence", "NSEQUENCE", 0),
    ("nb1", "NB1", 1), ("nb2", "NB2", 1), ("nb3", "NB3", 1), ("nb4", "NB4", 1), ("nb5", "NB5", 1), ("nb6", "NB6", 1),
    ("dx", "DX", 1e-6), ("dy", "DY", 1e-6), ("dz", "DZ", 1e-6),
    ("bx0", "BX0", 1.0), ("by0", "BY0", 0.0), ("bz0", "BZ0", 0.0),
    ("bdx0", "BDX0", 0.0), ("bdy0", "BDY0", 0.0), ("bdz0", "BDZ0", 0.0),
    ("time1", "TIME1", 0.0), ("time2", "TIME2", 70e-3),
    ("grad_x", "GRAD_X", 0.0), ("grad_y", "GRAD_Y", 0.0), ("grad_z", "GRAD_Z", 0.0),
    ("ampl_noise", "AMPL_NOISE", 0.0), ("vel_mult", "VEL_MULT", 1.0),
    ("d_oil", "D_OIL", 2.1e-10), ("d_water", "D_WAT", 2.3e-9),
    ("r1_oil", "R1_OIL", 0.0), ("r1_water", "R1_WAT", 0.0), ("r2_oil", "R2_OIL", 0.0), ("r2_water", "R2_WAT", 0.0),
    ("t1_oil", "T1_OIL", 2.5), ("t1_water", "T1_WAT", 2.5), ("t2_oil", "T2_OIL", 2.0), ("t2_water", "T2_WAT", 2.0),
    ("temperature", "T0", 300.0), ("an1", "AN(1)", 1.0), ("an2", "AN(2)", 0.0), ("bn1", "BN(1)", 0.0),
    ("bn2", "BN(2)", 1.0), ("cfl", "CFL", 0.002), ("cfl1", "CFL1", 0.002), ("step0", "TIMEW(1)", 1e-6),
    ("buffer_x", "bufferX", 0), ("buffer_y", "bufferY", 0), ("buffer_z", "bufferZ", 0),
]
assert len(_DATA_LINES) == 61


@dataclass
class NmrData:
    """The 61 parameters of ``Nmr_data.dat`` (defaults: one water phase, no flow)."""
    key: int = 1
    i_print: int = 1
    j_print: int = 1
    k_print: int = 1
    nd_print: int = 500
    nd_write: int = 1
    nd_vid: int = 1
    nd_ampl: int = 1
    n_poro: int = 1
    n_components: int = 1
    n_fluid: int = 1
    n_surf_rel_water: int = 0
    n_surf_rel_oil: int = 0
    n_vector_mult: int = 0
    n_velocity: int = 0
    n_diffusion: int = 1
    n_direction_field: int = 1
    n_sequence: int = 0
    nb1: int = 1
    nb2: int = 1
    nb3: int = 1
    nb4: int = 1
    nb5: int = 1
    nb6: int = 1
    dx: float = 1e-6
    dy: float = 1e-6
    dz: float = 1e-6
    bx0: float = 1.0
    by0: float = 0.0
    bz0: float = 0.0
    bdx0: float = 0.0
    bdy0: float = 0.0
    bdz0: float = 0.0
    time1: float = 0.0
    time2: float = 70e-3
    grad_x: float = 0.0
    grad_y: float = 0.0
    grad_z: float = 0.0
    ampl_noise: float = 0.0
    vel_mult: float = 1.0
    d_oil: float = 2.1e-10
    d_water: float = 2.3e-9
    r1_oil: float = 0.0
    r1_water: float = 0.0
    r2_oil: float = 0.0
    r2_water: float = 0.0
    t1_oil: float = 2.5
    t1_water: float = 2.5
    t2_oil: float = 2.0
    t2_water: float = 2.0
    temperature: float = 300.0
    an1: float = 1.0
    an2: float = 0.0
    bn1: float = 0.0
    bn2: float = 1.0
    cfl: float = 0.002
    cfl1: float = 0.002
    step0: float = 1e-6
    buffer_x: int = 0
    buffer_y: int = 0
    buffer_z: int = 0


def _fmt(v) -> str:
    if isinstance(v, (int, np.integer)) and not isinstance(v, bool):
        return str(int(v))
    return repr(float(v))


def write_data(path: str, data: NmrData) -> None:
    with open(path, "w") as f:
        for attr, token, _ in _DATA_LINES:
            f.write(f"{_fmt(getattr(data, attr))}\t{token}\n")


def read_data(path: str) -> NmrData:
    """First-substring-match lookup over the first 61 lines (cpp:189-723)."""
    lines = []
    with open(path, "r", newline="") as f:
        text = f.read()
    rest = text
    for _ in range(61):
        tab = rest.find("\t")
        if tab < 0:
            raise ValueError(f"{path}: fewer than 61 value<TAB>comment lines")
        value = rest[:tab]
        nl = rest.find("\n", tab + 1)
        comment = rest[tab + 1:] if nl < 0 else rest[tab + 1:nl]
        rest = "" if nl < 0 else rest[nl + 1:]
        lines.append((value, comment))
    d = NmrData()
    types = {f.name: f.type for f in fields(NmrData)}
    for attr, token, _ in _DATA_LINES:
        for value, comment in lines:
            if token in comment:
                if types[attr] in ("int", int):
                    setattr(d, attr, _atoi(value))
                else:
                    setattr(d, attr, _atof(value))
                break
    return d


def _atoi(s: str) -> int:
    s = s.strip()
    n = 0
    while n < len(s) and (s[n].isdigit() or (n == 0 and s[n] in "+-")):
        n += 1
    try:
        return int(s[:n])
    except ValueError:
        return 0


def _atof(s: str) -> float:
    s = s.strip()
    for end in range(len(s), 0, -1):
        try:
            return float(s[:end])
        except ValueError:
            continue
    return 0.0


def write_start(path: str, nx: int, ny: int, nz: int) -> None:
    with open(path, "w") as f:
        f.write(f"{nx}\n{ny}\n{nz}\n")


def read_start(path: str) -> tuple[int, int, int]:
    with open(path, "r") as f:
        vals = [int(line.split()[0]) for line in f.read().splitlines()[:3]]
    return vals[0], vals[1], vals[2]


def write_grad(path: str, values) -> None:
    values = list(values)
    with open(path, "w") as f:
        f.write(f"{len(values)}\n")
        for v in values:
            f.write(f"{float(v):.9f}\n")


def write_poro(path: str, mask: np.ndarray) -> None:
    """mask[k, j, i] -> one header line, then rows of '0'/'1' (k, j outer; i inner)."""
    nz, ny, nx = mask.shape
    rows = np.where(mask.reshape(nz * ny, nx) != 0, ord("1"), ord("0")).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"Poro\n")
        nl = np.full((nz * ny, 1), ord("\n"), np.uint8)
        f.write(np.concatenate([rows, nl], axis=1).tobytes())


def read_poro(path: str, nx: int, ny: int, nz: int) -> np.ndarray:
    with open(path, "rb") as f:
        f.readline()
        raw = np.frombuffer(f.read(), np.uint8)
    raw = raw[(raw > 32)]
    if raw.size < nx * ny * nz:
        raise ValueError(f"{path}: expected {nx * ny * nz} cells, found {raw.size}")
    return (raw[: nx * ny * nz] == ord("1")).astype(np.uint8).reshape(nz, ny, nx)


def _write_doubles(path: str, header: str, arr_ijk: np.ndarray) -> None:
    with open(path, "w") as f:
        f.write(header + "\n")
        np.savetxt(f, arr_ijk.reshape(-1, 1), fmt="%.17g")


def write_velocity(dirpath: str, vx: np.ndarray, vy: np.ndarray, vz: np.ndarray) -> None:
    """Face velocities in this package's [k, j, i] layout -> Vx/Vy/Vz.dat (i outer, k inner)."""
    _write_doubles(os.path.join(dirpath, "Vx.dat"), "Vx", np.transpose(vx, (2, 1, 0)))
    _write_doubles(os.path.join(dirpath, "Vy.dat"), "Vy", np.transpose(vy, (2, 1, 0)))
    _write_doubles(os.path.join(dirpath, "Vz.dat"), "Vz", np.transpose(vz, (2, 1, 0)))


def _read_doubles(path: str, n: int) -> np.ndarray:
    with open(path, "r") as f:
        f.readline()
        a = np.array(f.read().split(), dtype=np.float64)
    if a.size < n:
        raise ValueError(f"{path}: expected {n} values, found {a.size}")
    return a[:n]


def read_velocity(dirpath: str, nx: int, ny: int, nz: int):
    vx = _read_doubles(os.path.join(dirpath, "Vx.dat"), (nx + 1) * ny * nz).reshape(nx + 1, ny, nz)
    vy = _read_doubles(os.path.join(dirpath, "Vy.dat"), nx * (ny + 1) * nz).reshape(nx, ny + 1, nz)
    vz = _read_doubles(os.path.join(dirpath, "Vz.dat"), nx * ny * (nz + 1)).reshape(nx, ny, nz + 1)
    t = (2, 1, 0)
    return (np.ascontiguousarray(np.transpose(vx, t)), np.ascontiguousarray(np.transpose(vy, t)),
            np.ascontiguousarray(np.transpose(vz, t)))


SURFREL_KEYS = ("1Water", "2Water", "1Oil", "2Oil")


def write_surfrel(dirpath: str, key: str, fx: np.ndarray, fy: np.ndarray, fz: np.ndarray) -> None:
    """Face relaxivities in this package's [k, j, i] face layout -> SurfRel<key>X/Y/Z.dat."""
    for ax, a in zip("XYZ", (fx, fy, fz)):
        _write_doubles(os.path.join(dirpath, f"SurfRel{key}{ax}.dat"), f"SurfRel{key}{ax}", np.transpose(a, (2, 1, 0)))


def read_surfrel(dirpath: str, key: str, nx: int, ny: int, nz: int):
    dims = {"X": (nx + 1, ny, nz), "Y": (nx, ny + 1, nz), "Z": (nx, ny, nz + 1)}
    out = []
    for ax in "XYZ":
        n = int(np.prod(dims[ax]))
        a = _read_doubles(os.path.join(dirpath, f"SurfRel{key}{ax}.dat"), n).reshape(dims[ax])
        out.append(np.ascontiguousarray(np.transpose(a, (2, 1, 0))))
    return tuple(out)


def write_n1(path: str, n1: np.ndarray) -> None:
    """n1[k, j, i] -> n1_init.dat (i outer, k inner), each value exactly a float."""
    a = np.transpose(np.asarray(n1, dtype=np.float32), (2, 1, 0)).reshape(-1)
    with open(path, "w") as f:
        f.write("n1\n")
        for x in a:
            f.write(repr(float(x)) + "\n")


def read_n1(path: str, nx: int, ny: int, nz: int) -> np.ndarray:
    with open(path, "r") as f:
        f.readline()
        a = np.array(f.read().split(), dtype=np.float32)
    if a.size < nx * ny * nz:
        raise ValueError(f"{path}: expected {nx * ny * nz} values, found {a.size}")
    return np.ascontiguousarray(np.transpose(a[: nx * ny * nz].reshape(nx, ny, nz), (2, 1, 0)))


def write_case(dirpath: str, data: NmrData, mask: np.ndarray, vel=None, grads=(0.0,), surfrel=None,
               n1=None) -> None:
    """Write a complete reference input directory (``dirpath/data/*.dat``)."""
    d = os.path.join(dirpath, "data")
    os.makedirs(d, exist_ok=True)
    nz, ny, nx = mask.shape
    write_start(os.path.join(d, "Nmr_start.dat"), nx, ny, nz)
    write_data(os.path.join(d, "Nmr_data.dat"), data)
    write_grad(os.path.join(d, "Nmr_grad.dat"), grads)
    write_poro(os.path.join(d, "Poro.dat"), mask)
    if vel is not None:
        write_velocity(d, *vel)
    for key, faces in (surfrel or {}).items():
        write_surfrel(d, key, *faces)
    if n1 is not None:
        write_n1(os.path.join(d, "n1_init.dat"), n1)
