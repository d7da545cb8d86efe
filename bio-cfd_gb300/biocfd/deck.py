"""The reference's input deck, restart and output formats, and a driver that
runs a deck through the GB300 path with the reference's output cadence.

Input (src/ReadInput.f90:25-456): ``input_data.nml`` (namelist
``&input_data``), ``body_search.dat``, ``grid_shift.dat``, ``shift.dat``,
``flap_amp.dat``, ``butter_move.dat``, ``block_details.dat``, the grid files
``{x,y,z}grid_bk{g:03d}_{n+1}.txt``, ``interface_details.dat`` and the gmsh
surface ``geometries/butterflyMedium.msh``.  Lengths are millimetres in the
files; the unit conversions and derived quantities follow ReadInput.f90
operation for operation (``0.001_dp * x + shift``, ``mu_f * 1e-5``,
``u0 = re*mu_f/(rho_f*l_c)``, ``deltat = 1/(4*freq*dt_order)``, ...).

Restart (src/LastConditions.f90:12-49): ``out/aorta_chkpt.{id:03d}.{re:6.1f}.dat``,
one line ``u v w p totime ita ita1`` per point, x fastest.  The checkpoint
writer of the reference (src/WriteOutput_corner1.F90:116-138) writes the same
layout under another name (``out/Chkpt/{char_f}_butter_chkpt.{id:03d}.{re:6.1f}.{dx:8.6f}.dat``),
so a run cannot restart from its own checkpoints without renaming them;
``run_deck`` writes its checkpoints under both names.

Field output (src/WriteOutput_corner1.F90:74-104): the ASCII zone file
``out/{char_f}_butter_fielddata.{ita:09d}.{id:03d}.{re:7.1f}.{dx:8.6f}.{nblocks:03d}.dat``
with cell-centred velocities, every 200 steps and at steps 0-2; the surface
file ``out/butterfly_{id:03d}.dat`` at step 1.  With ``output_format="hdf5"``
the field files are the reference's HDF5 build's instead
(src/WriteOutput_corner1.F90:21-78, ``out/timestep_{ita:05d}_block_{id:05d}.h5``,
written by ``h5io``) at the same cadence.  Files are written by a background
thread from host copies, so the time loop does not wait for them.
"""
from __future__ import annotations

import dataclasses
import os
import re as _re
import threading
import queue
from dataclasses import dataclass
from pathlib import Path
from typing import Dict, List, Optional

import numpy as np

from . import h5io, synth

BLK_START = 2  # the first fine block (src/ReadInput.f90:10)

NML_KEYS = ("nblocks", "intflines", "itamax", "epsi", "pcItaMax", "omega1", "omega2", "omega3", "omega4",
            "re", "rho_f", "mu_f", "l_c", "u0", "surGeoPoints", "phase_angle", "freq", "aoa", "piv_pt",
            "alpha_m", "theta_m", "istart", "dt_order", "inor", "dxmin")


# ---------------------------------------------------------------------------
# Fortran namelist and list-directed records
# ---------------------------------------------------------------------------

def _fortran_number(tok: str):
    t = tok.strip().rstrip(",")
    if _re.fullmatch(r"[+-]?\d+", t):
        return int(t)
    return float(t.replace("d", "e").replace("D", "E"))


def read_namelist(path, group: str = "input_data") -> Dict[str, object]:
    """Values of one namelist group (keys case-insensitive; `!` comments;
    Fortran `d` exponents)."""
    text = Path(path).read_text()
    lines = [ln.split("!", 1)[0] for ln in text.splitlines()]
    body = " ".join(lines)
    m = _re.search(r"&\s*" + group + r"\b(.*?)(?<![\w.])/", body, flags=_re.IGNORECASE | _re.DOTALL)
    if not m:
        raise ValueError(f"namelist group &{group} not found in {path}")
    out: Dict[str, object] = {}
    for key, val in _re.findall(r"(\w+)\s*=\s*([^=]+?)(?=(?:,?\s*\w+\s*=)|\s*$)", m.group(1).strip()):
        out[key.lower()] = _fortran_number(val)
    return out


def write_namelist(path, values: Dict[str, object], group: str = "input_data") -> None:
    with open(path, "w") as f:
        f.write(f"&{group}\n")
        for k in NML_KEYS:
            if k.lower() in values:
                v = values[k.lower()]
                f.write(f"  {k} = {v!r},\n" if isinstance(v, float) else f"  {k} = {int(v)},\n")
        f.write("/\n")


def _records(path) -> List[List[str]]:
    """Whitespace/comma separated tokens per non-empty line (list-directed input)."""
    rows = []
    for ln in Path(path).read_text().splitlines():
        toks = [t for t in _re.split(r"[\s,]+", ln.strip()) if t]
        if toks:
            rows.append(toks)
    return rows


def _num(t: str) -> float:
    return float(t.replace("d", "e").replace("D", "E"))


# ---------------------------------------------------------------------------
# the deck
# ---------------------------------------------------------------------------

@dataclass
class DeckBlock:
    search: tuple            # i_start, i_end, j_start, j_end, k_start, k_end (body_search.dat)
    gshift: tuple            # grid shift, metres (grid_shift.dat x 0.001)
    shift: tuple             # body shift, metres (shift.dat x 0.001)
    extent_mm: tuple         # xstart, xend, ystart, yend, zstart, zend (block_details.dat, unused by the solver)
    n: tuple                 # nx, ny, nz
    fineg: float             # block_details dx as read (the reference keeps it as `fineg`)
    d: tuple                 # (1/dx)*0.001 etc. as the reference stores them
    x1: np.ndarray           # x1(1..nx+3), metres
    y1: np.ndarray
    z1: np.ndarray
    omega: float
    a0: float = 0.0          # flap_amp.dat (blocks >= 2)
    yamp: float = 0.0        # butter_move.dat x dxmin (blocks >= 2)
    bfreq: float = 0.0


@dataclass
class Deck:
    nml: Dict[str, object]   # input_data.nml as read
    # derived as src/ReadInput.f90:149-158
    mu_f: float
    rho_f: float
    l_c: float
    u0: float
    uc: float
    re: float
    freq: float
    deltat: float
    dxmin: float
    char_f: str
    blocks: List[DeckBlock]
    interfaces: List[dict]
    mesh: Optional[synth.Mesh] = None
    directory: str = "."


def _grid(path, n: int, shift: float):
    """x1(1..n+3) from the n+1 face values x1(2..n+2) in mm (src/ReadInput.f90:250-265)."""
    vals = [_num(r[0]) for r in _records(path)][: n + 1]
    if len(vals) != n + 1:
        raise ValueError(f"{path}: expected {n + 1} values, got {len(vals)}")
    x1 = np.zeros(n + 3)
    for i, v in enumerate(vals):
        x1[i + 1] = 0.001 * v
        x1[i + 1] = x1[i + 1] + shift
    dl = x1[2] - x1[1]
    dr = x1[n + 1] - x1[n]
    x1[0] = x1[1] - dl
    x1[n + 2] = x1[n + 1] + dr
    return x1


def grid_file(d: str, axis: str, g: int, n: int) -> str:
    return os.path.join(d, f"{axis}grid_bk{g:03d}_{n + 1}.txt")


def read_gmsh(path, sur_geo_points: int, inor: int = 1) -> synth.Mesh:
    """The surface mesh as src/ReadInput.f90:365-426 reads it: 4 lines, the node
    count, nodes `id x y z` (mm), 2 lines, the element count, surGeoPoints
    point elements to skip, then `id type ntags surf_id tag p1 p2 p3`."""
    lines = [ln for ln in Path(path).read_text().splitlines()]
    pos = 4
    nn = int(lines[pos].split()[0])
    pos += 1
    nodes = np.zeros((nn, 3))
    for n in range(nn):
        t = lines[pos + n].split()
        nodes[n] = [0.001 * _num(t[1]), 0.001 * _num(t[2]), 0.001 * _num(t[3])]
    pos += nn + 2
    ne = int(lines[pos].split()[0]) - sur_geo_points
    pos += 1 + sur_geo_points
    tris = np.zeros((ne, 3), np.int64)
    sid = np.zeros(ne, np.int64)
    for n in range(ne):
        t = lines[pos + n].split()
        sid[n] = int(t[3])
        tris[n] = [int(t[5]), int(t[6]), int(t[7])]
    return synth.Mesh(nodes=nodes, tris=tris, surf_id=sid, inor=inor)


def write_gmsh(path, mesh: synth.Mesh, sur_geo_points: int = 0) -> None:
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n")
        f.write(f"{len(mesh.nodes)}\n")
        for n, (x, y, z) in enumerate(mesh.nodes, 1):
            f.write(f"{n} {float(x) * 1000.0!r} {float(y) * 1000.0!r} {float(z) * 1000.0!r}\n")
        f.write("$EndNodes\n$Elements\n")
        f.write(f"{len(mesh.tris) + sur_geo_points}\n")
        for n in range(sur_geo_points):
            f.write(f"{n + 1} 15 2 0 {n + 1} {n + 1}\n")
        for n, (tri, s) in enumerate(zip(mesh.tris, mesh.surf_id), sur_geo_points + 1):
            f.write(f"{n} 2 2 {int(s)} 1 {int(tri[0])} {int(tri[1])} {int(tri[2])}\n")
        f.write("$EndElements\n")


def read_deck(directory, mesh_file: str = "geometries/butterflyMedium.msh") -> Deck:
    d = str(directory)
    nml = read_namelist(os.path.join(d, "input_data.nml"))
    nb = int(nml["nblocks"])
    search = [tuple(int(x) for x in r[:6]) for r in _records(os.path.join(d, "body_search.dat"))[:nb]]
    gshift = [tuple(_num(x) * 0.001 for x in r[:3]) for r in _records(os.path.join(d, "grid_shift.dat"))[:nb]]
    shift = [tuple(_num(x) * 0.001 for x in r[:3]) for r in _records(os.path.join(d, "shift.dat"))[:nb]]
    alpha_m, theta_m = float(nml.get("alpha_m", 0.0)), float(nml.get("theta_m", 0.0))
    char_f = "   "
    if alpha_m != 0 and theta_m != 0:
        char_f = "bot"
    if alpha_m == 0 and theta_m != 0:
        char_f = "amp"
    if alpha_m != 0 and theta_m == 0:
        char_f = "ang"
    dxmin = 0.001 * float(nml["dxmin"])
    a0 = [0.0] * nb
    for g, r in enumerate(_records(os.path.join(d, "flap_amp.dat"))[: nb - 1], BLK_START):
        a0[g - 1] = _num(r[0])
    mu_f = float(nml["mu_f"]) * 1e-5
    rho_f = float(nml["rho_f"])
    l_c = 0.001 * float(nml["l_c"])
    u0 = float(nml["re"]) * mu_f / (rho_f * l_c)
    uc = u0
    re = rho_f / mu_f
    freq = float(nml["freq"]) * u0 / l_c
    deltat = 1.0 / (4.0 * freq * float(nml["dt_order"]))
    yamp = [0.0] * nb
    bfreq = [0.0] * nb
    for g, r in enumerate(_records(os.path.join(d, "butter_move.dat"))[: nb - 1], BLK_START):
        yamp[g - 1] = dxmin * _num(r[0])
        bfreq[g - 1] = _num(r[1])
    details = _records(os.path.join(d, "block_details.dat"))[:nb]
    omegas = [float(nml.get(f"omega{min(g, 4)}", 1.0)) for g in range(1, nb + 1)]
    blocks = []
    for g in range(1, nb + 1):
        r = details[g - 1]
        ext = tuple(_num(x) for x in r[:6])
        nx, ny, nz = (int(x) for x in r[6:9])
        ddx = tuple(_num(x) for x in r[9:12])
        gs = gshift[g - 1]
        blocks.append(DeckBlock(
            search=search[g - 1], gshift=gs, shift=shift[g - 1], extent_mm=ext, n=(nx, ny, nz), fineg=ddx[0],
            d=tuple((1.0 / v) * 0.001 for v in ddx),
            x1=_grid(grid_file(d, "x", g, nx), nx, gs[0]), y1=_grid(grid_file(d, "y", g, ny), ny, gs[1]),
            z1=_grid(grid_file(d, "z", g, nz), nz, gs[2]), omega=omegas[g - 1],
            a0=a0[g - 1], yamp=yamp[g - 1], bfreq=bfreq[g - 1]))
    interfaces = []
    for r in _records(os.path.join(d, "interface_details.dat"))[: int(nml["intflines"])]:
        interfaces.append({"a_blk": int(r[0]), "a_msh": int(r[1]), "a_intf": int(r[2]), "b_blk": int(r[3]),
                           "b_msh": int(r[4]), "b_intf": int(r[5]),
                           "box": tuple(_num(x) * 0.001 for x in r[6:12])})
    mesh = None
    mp = os.path.join(d, mesh_file)
    if nb > 1 and os.path.exists(mp):
        mesh = read_gmsh(mp, int(nml.get("surgeopoints", 0)), int(nml.get("inor", 1)))
    return Deck(nml=nml, mu_f=mu_f, rho_f=rho_f, l_c=l_c, u0=u0, uc=uc, re=re, freq=freq, deltat=deltat,
                dxmin=dxmin, char_f=char_f, blocks=blocks, interfaces=interfaces, mesh=mesh, directory=d)


def deck_to_case(deck: Deck, name: str = "deck") -> synth.Case:
    """The case app/main.F90 builds from the deck: block 1 coarse with the
    domain BCs, every block g >= 2 carrying the surface (placed by
    shiftSurfaceNodesInitial with its shift and the deck's kinematics),
    omega by block number, uniform initial field u = uc (initialConditions)."""
    nml = deck.nml
    specs = []
    for g, b in enumerate(deck.blocks, 1):
        nx, ny, nz = b.n
        spec = synth.BlockSpec(nx, ny, nz, b.x1[1:nx + 2].copy(), b.y1[1:ny + 2].copy(), b.z1[1:nz + 2].copy(),
                               omega=b.omega, is_coarse=(g == 1))
        spec.search_box = tuple(b.search)
        if g >= BLK_START and deck.mesh is not None:
            spec.mesh = dataclasses.replace(deck.mesh, nodes=deck.mesh.nodes.copy())
            spec.motion = synth.Motion(a0_deg=b.a0, bfreq=b.bfreq, yamp=b.yamp, shift=tuple(b.shift))
        specs.append(spec)
    ifs = [synth.InterfaceSpec(a_blk=it["a_blk"], b_blk=it["b_blk"], a_msh=it["a_msh"], b_msh=it["b_msh"],
                               box=it["box"]) for it in deck.interfaces]
    case = synth.Case(name=name, blocks=specs, interfaces=ifs, dt=deck.deltat, re=deck.re, uc=deck.uc,
                      epsi=float(nml["epsi"]), pc_ita_max=int(nml["pcitamax"]), n_steps=int(nml["itamax"]))
    if any(s.motion is not None for s in specs):
        case.motion = synth.MotionInputs(aoa_deg=float(nml.get("aoa", 0.0)),
                                         phase_deg=float(nml.get("phase_angle", 0.0)),
                                         piv_pt=float(nml.get("piv_pt", 0.0)), freq=deck.freq, dxmin=deck.dxmin)
    case.init = [uniform_initial(s, deck.uc) for s in specs]
    return case


def uniform_initial(spec: synth.BlockSpec, uc: float) -> dict:
    """initialConditions (src/InitialConditions.f90:10-35): u = uc, v = w = p = 0."""
    shp = spec.shape
    return {"u": np.full(shp, uc, order="F"), "v": np.zeros(shp, order="F"), "w": np.zeros(shp, order="F"),
            "p": np.zeros(shp, order="F")}


def write_deck(directory, case: synth.Case, *, mu_f_in: float, rho_f: float, l_c_mm: float, re_in: float,
               freq_in: float, dt_order: float, itamax: Optional[int] = None, istart: int = 0,
               dxmin_mm: float = 0.0, aoa: float = 0.0, phase_angle: float = 0.0, piv_pt: float = 0.0,
               inor: int = 1, shift_mm=None, flap_amp=None, butter_move=None) -> None:
    """Write the reference's input files for a case (lengths in mm).  The
    namelist's re/mu_f/rho_f/l_c/freq/dt_order are the reference's raw inputs:
    it derives mu = mu_f_in 1e-5, u0 = re_in mu/(rho_f l_c), re = rho_f/mu,
    freq = freq_in u0/l_c, deltat = 1/(4 freq dt_order)."""
    d = Path(directory)
    (d / "geometries").mkdir(parents=True, exist_ok=True)
    nb = len(case.blocks)
    omegas = [b.omega for b in case.blocks] + [1.0] * 4
    nml = {"nblocks": nb, "intflines": len(case.interfaces), "itamax": itamax if itamax is not None else case.n_steps,
           "epsi": float(case.epsi), "pcitamax": int(case.pc_ita_max),
           "omega1": float(omegas[0]), "omega2": float(omegas[1]), "omega3": float(omegas[2]),
           "omega4": float(omegas[3]), "re": float(re_in), "rho_f": float(rho_f), "mu_f": float(mu_f_in),
           "l_c": float(l_c_mm), "u0": 0.0, "surgeopoints": 0, "phase_angle": float(phase_angle),
           "freq": float(freq_in), "aoa": float(aoa), "piv_pt": float(piv_pt), "alpha_m": 0.0, "theta_m": 0.0,
           "istart": int(istart), "dt_order": float(dt_order), "inor": int(inor), "dxmin": float(dxmin_mm)}
    write_namelist(d / "input_data.nml", nml)

    def rows(name, vals):
        with open(d / name, "w") as f:
            for v in vals:
                f.write(" ".join(repr(float(x)) if isinstance(x, float) else str(int(x)) for x in v) + "\n")

    rows("body_search.dat", [b.search_box for b in case.blocks])
    rows("grid_shift.dat", [(0.0, 0.0, 0.0)] * nb)
    shifts = shift_mm or [tuple(1000.0 * x for x in (b.motion.shift if b.motion else (0.0, 0.0, 0.0)))
                          for b in case.blocks]
    rows("shift.dat", shifts)
    rows("flap_amp.dat", flap_amp or [(float(b.motion.a0_deg if b.motion else 0.0),) for b in case.blocks[1:]])
    rows("butter_move.dat", butter_move or [(0.0, 0.0)] * (nb - 1))
    det = []
    for g, b in enumerate(case.blocks, 1):
        xs = (b.x_faces[0], b.x_faces[-1], b.y_faces[0], b.y_faces[-1], b.z_faces[0], b.z_faces[-1])
        det.append(tuple(1000.0 * float(v) for v in xs) + (b.nx, b.ny, b.nz) +
                   tuple(float(1.0 / (1000.0 * (f[1] - f[0]))) for f in (b.x_faces, b.y_faces, b.z_faces)))
    rows("block_details.dat", det)
    for g, b in enumerate(case.blocks, 1):
        for axis, faces, n in (("x", b.x_faces, b.nx), ("y", b.y_faces, b.ny), ("z", b.z_faces, b.nz)):
            rows(os.path.basename(grid_file(str(d), axis, g, n)), [(1000.0 * float(v),) for v in faces])
    with open(d / "interface_details.dat", "w") as f:
        for it in case.interfaces:
            box = " ".join(repr(1000.0 * float(v)) for v in it.box)
            f.write(f"{it.a_blk} {it.a_msh} 1 {it.b_blk} {it.b_msh} 1 {box}\n")
    mesh = next((b.mesh for b in case.blocks[1:] if b.mesh is not None), None)
    if mesh is not None:
        write_gmsh(d / "geometries" / "butterflyMedium.msh", mesh)


# ---------------------------------------------------------------------------
# restart and output files
# ---------------------------------------------------------------------------

def restart_name(block_id: int, re: float) -> str:
    """The file lastConditions reads (src/LastConditions.f90:27-28)."""
    return f"out/aorta_chkpt.{block_id:03d}.{re:6.1f}.dat"


def checkpoint_name(char_f: str, block_id: int, re: float, dx: float) -> str:
    """The file writeResult writes (src/WriteOutput_corner1.F90:125-126)."""
    return f"out/Chkpt/{char_f}_butter_chkpt.{block_id:03d}.{re:6.1f}.{dx:8.6f}.dat"


def field_name(char_f: str, ita: int, block_id: int, re: float, dx: float, nblocks: int) -> str:
    """The file write_output_ascii writes (src/WriteOutput_corner1.F90:84-85)."""
    return f"out/{char_f}_butter_fielddata.{ita:09d}.{block_id:03d}.{re:7.1f}.{dx:8.6f}.{nblocks:03d}.dat"


def write_restart(path, fields: dict, totime: float, ita: int, ita1: int) -> None:
    """One line `u v w p totime ita ita1` per point, x fastest (exact FP64 text)."""
    u, v, w, p = (np.asarray(fields[k], dtype=np.float64).ravel(order="F") for k in ("u", "v", "w", "p"))
    n = u.size
    cols = np.empty((n, 5))
    cols[:, 0], cols[:, 1], cols[:, 2], cols[:, 3] = u, v, w, p
    cols[:, 4] = totime
    Path(path).parent.mkdir(parents=True, exist_ok=True)
    with open(path, "w") as f:
        tail = f" {int(ita)} {int(ita1)}\n"
        for row in cols:
            f.write(" ".join(repr(float(x)) for x in row) + tail)


def read_restart(path, nx: int, ny: int, nz: int):
    """Fields (u, v, w, p) of shape (nx+2, ny+2, nz+2) and the (totime, ita,
    ita1) of the last record, as lastConditions leaves them."""
    shp = (nx + 2, ny + 2, nz + 2)
    n = shp[0] * shp[1] * shp[2]
    recs = _records(path)
    if len(recs) < n:
        raise ValueError(f"{path}: {len(recs)} records, expected {n}")
    a = np.array([[_num(t) for t in r[:5]] for r in recs[:n]])
    last = recs[n - 1]
    fields = {k: np.asfortranarray(a[:, q].reshape(shp, order="F")) for q, k in enumerate(("u", "v", "w", "p"))}
    return fields, float(_num(last[4])), int(last[5]), int(last[6])


def _centres(a: np.ndarray) -> np.ndarray:
    return 0.5 * (a[1:] + a[:-1])


def write_fields_ascii(path, x1, y1, z1, fields: dict, tags: dict, totime: float) -> None:
    """The zone file of write_output_ascii: header, then per interior cell
    x y z u v w p totime cell cell_n cell_pr with cell-centred velocities
    u1 = (u(i)+u(i-1))/2 etc."""
    u, v, w, p = (np.asarray(fields[k]) for k in ("u", "v", "w", "p"))
    nx, ny, nz = u.shape[0] - 2, u.shape[1] - 2, u.shape[2] - 2
    xp, yp, zp = _centres(np.asarray(x1))[1:nx + 1], _centres(np.asarray(y1))[1:ny + 1], _centres(np.asarray(z1))[1:nz + 1]
    u1 = 0.5 * (u[1:-1, 1:-1, 1:-1] + u[:-2, 1:-1, 1:-1])
    v1 = 0.5 * (v[1:-1, 1:-1, 1:-1] + v[1:-1, :-2, 1:-1])
    w1 = 0.5 * (w[1:-1, 1:-1, 1:-1] + w[1:-1, 1:-1, :-2])
    X, Y, Z = np.meshgrid(xp, yp, zp, indexing="ij")
    cols = [X, Y, Z, u1, v1, w1, p[1:-1, 1:-1, 1:-1], np.full(u1.shape, totime)]
    cols += [np.asarray(tags[k])[1:-1, 1:-1, 1:-1] for k in ("cell", "cell_n", "cell_pr")]
    table = np.stack([c.ravel(order="F") for c in cols], axis=1)
    Path(path).parent.mkdir(parents=True, exist_ok=True)
    with open(path, "w") as f:
        f.write(' variables="x","y","z","u","v","w","p","totime","cellid","cell_n","cell_pr"\n')
        f.write(f" zone, i = {nx} j = {ny} k = {nz}\n")
        np.savetxt(f, table, fmt=["%.17g"] * 8 + ["%d"] * 3)


def write_surface(path, nodes: np.ndarray, tris: np.ndarray) -> None:
    """body_plot (src/WriteOutput_corner1.F90:141-161): FE triangle zone."""
    Path(path).parent.mkdir(parents=True, exist_ok=True)
    with open(path, "w") as f:
        f.write(' TITLE = "FEstressplot"\n VARIABLES= "x", "y", "z","bd_n"\n')
        f.write(f" ZONE NODES= {len(nodes)},ELEMENTS={len(tris)},DATAPACKING=POINT, ZONETYPE=FETRIANGLE\n")
        for x, y, z in nodes:
            f.write(f"{float(x)!r} {float(y)!r} {float(z)!r} 99\n")
        for t in tris:
            f.write(f"{int(t[0])} {int(t[1])} {int(t[2])}\n")


class AsyncWriter:
    """Writes files on a background thread (the time loop hands over host
    copies and continues)."""

    def __init__(self):
        self.q: "queue.Queue" = queue.Queue()
        self.errors: List[BaseException] = []
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def _run(self):
        while True:
            job = self.q.get()
            if job is None:
                return
            fn, args = job
            try:
                fn(*args)
            except BaseException as e:  # reported by close()
                self.errors.append(e)

    def submit(self, fn, *args):
        self.q.put((fn, args))

    def close(self):
        self.q.put(None)
        self.t.join()
        if self.errors:
            raise self.errors[0]


# ---------------------------------------------------------------------------
# the driver
# ---------------------------------------------------------------------------

def run_deck(directory, n_steps: Optional[int] = None, precision: int = 0, div_tol: float = 1e-6,
             out_dir: Optional[str] = None, outputs: bool = True, mesh_file: str = "geometries/butterflyMedium.msh",
             output_format: str = "ascii"):
    """app/main.F90 on the GB300 path: read the deck, set up (restart fields
    when istart = 1), write the step-0 output, run n_steps (default itamax)
    with field output at steps <= 2 and every 200 (ASCII zone files, or the
    HDF5 files of the reference's USE_HDF5 build with output_format="hdf5"),
    checkpoints every 500 and the surface at step 1.  Returns the Solver
    (blocks left on the device)."""
    if output_format not in ("ascii", "hdf5"):
        raise ValueError(f"output_format {output_format!r}: 'ascii' or 'hdf5'")
    from .solver import Solver
    deck = read_deck(directory, mesh_file)
    case = deck_to_case(deck)
    out = Path(out_dir or directory)
    nb = len(case.blocks)
    ita0, tot0 = 0, 0.0
    if int(deck.nml.get("istart", 0)) == 1:
        for g, spec in enumerate(case.blocks, 1):
            f, tot0, ita0, _ = read_restart(os.path.join(directory, restart_name(g, deck.re)), spec.nx, spec.ny, spec.nz)
            case.init[g - 1] = f
    s = Solver(case)
    s.setup()
    if ita0 or tot0:
        s.set_time(ita0, tot0 + case.dt)
    writer = AsyncWriter() if outputs else None

    def emit(ita: int, totime: float):
        for g, (h, spec, b) in enumerate(zip(s.handles, case.blocks, deck.blocks), 1):
            if ita <= 2 or ita % 200 == 0:
                f = s.fields(h)
                t = s.tags(h)
                tags = {"cell": t["cell"], "cell_n": t["cell_n"], "cell_pr": t["cell_pr"][:-1, :-1, :-1]}
                if output_format == "hdf5":
                    writer.submit(h5io.write_fields_hdf5, out / h5io.field_name_hdf5(ita, g),
                                  b.x1, b.y1, b.z1, f, tags, totime)
                else:
                    writer.submit(write_fields_ascii, out / field_name(deck.char_f, ita, g, deck.re, b.d[0], nb),
                                  b.x1, b.y1, b.z1, f, tags, totime)
            if ita % 500 == 0 and ita > 0:
                f = s.fields(h)
                for name in (checkpoint_name(deck.char_f, g, deck.re, b.d[0]), restart_name(g, deck.re)):
                    writer.submit(write_restart, out / name, f, totime, ita, 0)
            if ita == 1 and spec.mesh is not None:
                nodes = np.stack([s.read(h, k, len(spec.mesh.nodes)) for k in ("xnode1", "ynode1", "znode1")], axis=1)
                writer.submit(write_surface, out / f"out/butterfly_{g:03d}.dat", nodes, spec.mesh.tris)

    steps = int(n_steps if n_steps is not None else deck.nml["itamax"])
    try:
        if writer:
            emit(ita0, s.time()[1])
        for _ in range(steps):
            s.run(1, precision=precision, div_tol=div_tol)
            ita, totime = s.time()
            if writer:
                emit(ita, totime)
    finally:
        if writer:
            writer.close()
    return s
