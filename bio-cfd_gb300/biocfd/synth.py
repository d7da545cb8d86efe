"""Seeded synthetic inputs for the Bio-CFD hot path.

The reference reads its grids, surface mesh and restart fields from files
that are not part of its repository (`.gitignore` excludes them), so every
workload here is generated: uniform tensor-product grids, a Fibonacci-sphere
surface triangulated by its convex hull (or an ellipsoidal plate), interface
boxes, and the initial field u = uc plus N(0, 1e-3) noise on u, v, w drawn
from ``numpy.random.default_rng(20261203)``.

Coordinates are in metres (the reference converts its millimetre inputs with
a factor 0.001 in src/ReadInput.f90:142-351; here they are generated directly
in the converted units).  Grid conventions follow src/ReadInput.f90:250-351:
a block with ``n`` interior cells along x has face coordinates
``x1(2..n+2)``; the ghosts ``x1(1)``/``x1(n+3)`` and the spacings are
derived by the same rules on the device side and in the oracle.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

SEED = 20261203


@dataclass
class Mesh:
    """Triangulated immersed surface (the gmsh file of src/ReadInput.f90:365-426)."""
    nodes: np.ndarray          # (n_nodes, 3) float64, world coordinates (xnode1 ...)
    tris: np.ndarray           # (n_elems, 3) int64, 1-based node indices (ibElP1..3)
    surf_id: np.ndarray        # (n_elems,) int64 physical tag: 50 static, 51/52 rotating
    inor: int = 1              # normal orientation factor of computeSurfaceNorm


@dataclass
class Motion:
    """Rigid-body motion of a block's surface (Block_t members read by
    src/Search.F90:49-208): pitch amplitude a0 in degrees, heave frequency and
    amplitude, body placement.  With a motion the mesh nodes are in the body
    frame."""
    a0_deg: float = 0.0
    bfreq: float = 0.0
    yamp: float = 0.0
    shift: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    # phase lag (degrees) of this body's heave and pitch behind the shared
    # kinematics (bcfd_block_set_body_lag); 0 = the reference's kinematics
    lag_deg: float = 0.0


@dataclass
class MotionInputs:
    """The app/main.F90 inputs of the motion: initial angle of attack (deg),
    phase angle (deg), pivot offset, pitch frequency, dxmin."""
    aoa_deg: float = 0.0
    phase_deg: float = 0.0
    piv_pt: float = 0.0
    freq: float = 0.0
    dxmin: float = 0.0


@dataclass
class BlockSpec:
    nx: int
    ny: int
    nz: int
    x_faces: np.ndarray        # nx+1 face coordinates = x1(2..nx+2)
    y_faces: np.ndarray
    z_faces: np.ndarray
    omega: float = 1.7
    is_coarse: bool = False    # domain BCs (velocityBC) and coarse Poisson folding
    mesh: Optional[Mesh] = None
    search_box: Tuple[int, int, int, int, int, int] = (0, -1, 0, -1, 0, -1)
    # rigid-body kinematics read by the forcing routines
    xdot: float = 0.0
    ydot: float = 0.0
    yddot: float = 0.0
    piv: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    motion: Optional["Motion"] = None

    @property
    def has_body(self) -> bool:
        return self.mesh is not None

    @property
    def shape(self) -> Tuple[int, int, int]:
        """Array extents of the cell-centred fields, (nx+2, ny+2, nz+2)."""
        return (self.nx + 2, self.ny + 2, self.nz + 2)

    @property
    def n_interior(self) -> int:
        return self.nx * self.ny * self.nz


@dataclass
class InterfaceSpec:
    """One coarse/fine coupling (interface_details.dat, src/ReadInput.f90:430-456)."""
    a_blk: int                 # coarse block number (1-based)
    b_blk: int                 # fine block number
    a_msh: int
    b_msh: int
    box: Tuple[float, float, float, float, float, float]  # xs, xe, ys, ye, zs, ze


@dataclass
class Case:
    name: str
    blocks: List[BlockSpec]
    interfaces: List[InterfaceSpec] = field(default_factory=list)
    dt: float = 0.0
    re: float = 100.0          # the reference's `re` argument: 1/nu (src/ReadInput.f90:155)
    uc: float = 1.0
    epsi: float = 1e-6
    pc_ita_max: int = 5000
    n_steps: int = 1
    init: List[dict] = field(default_factory=list)   # per block: {"u","v","w","p"} arrays
    motion: Optional["MotionInputs"] = None

    @property
    def n_interior(self) -> int:
        return sum(b.n_interior for b in self.blocks)


# ---------------------------------------------------------------------------
# surfaces
# ---------------------------------------------------------------------------

def _canonical_hull(pts: np.ndarray, center: np.ndarray) -> np.ndarray:
    """Convex-hull triangles, oriented outward, in a platform-independent order."""
    from scipy.spatial import ConvexHull
    tri = np.asarray(ConvexHull(pts).simplices, dtype=np.int64)
    a, b, c = pts[tri[:, 0]], pts[tri[:, 1]], pts[tri[:, 2]]
    nrm = np.cross(b - a, c - a)
    out = np.einsum("ij,ij->i", nrm, (a + b + c) / 3.0 - center) > 0
    tri[~out] = tri[~out][:, [0, 2, 1]]
    # rotate each triangle so its smallest node comes first (keeps orientation)
    r = np.argmin(tri, axis=1)
    idx = (np.arange(3)[None, :] + r[:, None]) % 3
    tri = np.take_along_axis(tri, idx, axis=1)
    order = np.lexsort((tri[:, 2], tri[:, 1], tri[:, 0]))
    return tri[order]


def fibonacci_sphere(center, diameter: float, spacing: float, surf_id: int = 50) -> Mesh:
    """Markers on a sphere at roughly `spacing`, triangulated by the convex hull."""
    center = np.asarray(center, dtype=np.float64)
    n = max(12, int(round(np.pi * (diameter / spacing) ** 2)))
    i = np.arange(n, dtype=np.float64)
    z = 1.0 - (2.0 * i + 1.0) / n
    r = np.sqrt(1.0 - z * z)
    phi = i * (np.pi * (3.0 - np.sqrt(5.0)))
    pts = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1) * (0.5 * diameter) + center
    tri = _canonical_hull(pts, center)
    return Mesh(nodes=pts, tris=tri + 1, surf_id=np.full(len(tri), surf_id, dtype=np.int64))


def ellipsoid_plate(center, semi_axes, spacing: float, surf_id: int = 51) -> Mesh:
    """A rigid ellipsoidal plate: Fibonacci directions mapped onto the ellipsoid."""
    center = np.asarray(center, dtype=np.float64)
    ax = np.asarray(semi_axes, dtype=np.float64)
    area = 4 * np.pi * ((ax[0] * ax[1]) ** 1.6 + (ax[0] * ax[2]) ** 1.6 + (ax[1] * ax[2]) ** 1.6) ** (1 / 1.6) / 3 ** (1 / 1.6)
    n = max(12, int(round(area / spacing ** 2)))
    i = np.arange(n, dtype=np.float64)
    z = 1.0 - (2.0 * i + 1.0) / n
    r = np.sqrt(1.0 - z * z)
    phi = i * (np.pi * (3.0 - np.sqrt(5.0)))
    unit = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    tri = _canonical_hull(unit, np.zeros(3))
    pts = unit * ax + center
    return Mesh(nodes=pts, tris=tri + 1, surf_id=np.full(len(tri), surf_id, dtype=np.int64))


def search_box_for(spec: BlockSpec, lo, hi, margin_cells: int = 3):
    """Cell-index box (body_search.dat) covering [lo, hi] plus a margin, clamped to 2..n+1."""
    out = []
    for faces, n, a, b in ((spec.x_faces, spec.nx, lo[0], hi[0]),
                           (spec.y_faces, spec.ny, lo[1], hi[1]),
                           (spec.z_faces, spec.nz, lo[2], hi[2])):
        # cell i (1-based, interior 2..n+1) spans faces[i-2] .. faces[i-1]
        i0 = int(np.searchsorted(faces, a, side="right")) + 1 - margin_cells
        i1 = int(np.searchsorted(faces, b, side="left")) + 1 + margin_cells
        out += [max(2, i0), min(n + 1, i1)]
    return tuple(out)


def uniform_faces(x0: float, x1: float, n: int) -> np.ndarray:
    return x0 + (x1 - x0) * np.arange(n + 1, dtype=np.float64) / n


def noisy_initial(spec: BlockSpec, uc: float, rng: np.random.Generator, sigma: float = 1e-3) -> dict:
    """u = uc, v = w = p = 0 plus N(0, sigma) on u, v, w at every point (restart path)."""
    shp = spec.shape
    u = np.full(shp, uc, dtype=np.float64, order="F") + rng.normal(0.0, sigma, shp)
    v = rng.normal(0.0, sigma, shp)
    w = rng.normal(0.0, sigma, shp)
    p = np.zeros(shp)
    return {k: np.asfortranarray(a) for k, a in (("u", u), ("v", v), ("w", w), ("p", p))}


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

def sphere_single_block(n: int = 64, n_steps: int = 100, diameter: float = 0.25,
                        center=(0.4, 0.5, 0.5), omega: float = 1.7, pc_ita_max: int = 5000,
                        reynolds: float = 100.0, seed: int = SEED) -> Case:
    """Single uniform n^3 block on the unit cube with a stationary sphere.

    Re = U D / nu = 100 with U = uc = 1 -> the reference's `re` argument is
    1/nu = Re / D; dt from CFL 0.3 (dt = 0.3 dx / U); SOR omega 1.7 to 1e-6.
    The block carries both the domain BCs and the body (composed by the
    harness; the reference driver applies IB only to blocks g >= 2).
    """
    f = uniform_faces(0.0, 1.0, n)
    dx = 1.0 / n
    spec = BlockSpec(n, n, n, f, f.copy(), f.copy(), omega=omega, is_coarse=True)
    spec.mesh = fibonacci_sphere(center, diameter, dx)
    c = np.asarray(center)
    spec.search_box = search_box_for(spec, c - diameter / 2, c + diameter / 2)
    rng = np.random.default_rng(seed)
    case = Case(name=f"sphere{n}", blocks=[spec], dt=0.3 * dx / 1.0, re=reynolds / diameter,
                uc=1.0, epsi=1e-6, pc_ita_max=pc_ita_max, n_steps=n_steps)
    case.init = [noisy_initial(spec, case.uc, rng)]
    return case


def plate_single_block(n: int = 32, n_steps: int = 2, semi_axes=(0.25, 0.125, 0.0125),
                       center=(0.45, 0.5, 0.5), reynolds: float = 300.0, omega: float = 1.7,
                       pc_ita_max: int = 5000, seed: int = SEED, surf_id: int = 51) -> Case:
    """Single uniform n^3 block on the unit cube with a stationary rigid
    ellipsoidal plate (surface 51) thinner than a cell, so that its IB cells are
    thin-surface cells and the momentum predictor's ghost substitution runs.
    Re = U c / nu on the chord c = 2 * semi_axes[0]."""
    f = uniform_faces(0.0, 1.0, n)
    dx = 1.0 / n
    spec = BlockSpec(n, n, n, f, f.copy(), f.copy(), omega=omega, is_coarse=True)
    spec.mesh = ellipsoid_plate(center, semi_axes, 0.5 * dx, surf_id=surf_id)
    c = np.asarray(center)
    ax = np.asarray(semi_axes)
    spec.search_box = search_box_for(spec, c - ax, c + ax)
    rng = np.random.default_rng(seed)
    chord = 2.0 * semi_axes[0]
    case = Case(name=f"plate{n}", blocks=[spec], dt=0.3 * dx, re=reynolds / chord, uc=1.0, epsi=1e-6,
                pc_ita_max=pc_ita_max, n_steps=n_steps)
    case.init = [noisy_initial(spec, case.uc, rng)]
    return case


def moving_plate_single_block(n: int = 32, n_steps: int = 3, semi_axes=(0.25, 0.125, 0.0125),
                              center=(0.45, 0.5, 0.5), a0_deg: float = 10.0, yamp: float = 0.05,
                              freq: float = 0.25, phase_deg: float = 90.0, reynolds: float = 300.0,
                              seed: int = SEED) -> Case:
    """The plate of plate_single_block heaving (yamp sin(2 pi freq t)) and
    pitching about x (a0 sin(2 pi freq t + phase)), towed in -x by the
    reference's fixed 0.05 dxmin per step (src/Search.F90:12)."""
    f = uniform_faces(0.0, 1.0, n)
    dx = 1.0 / n
    spec = BlockSpec(n, n, n, f, f.copy(), f.copy(), omega=1.7, is_coarse=True)
    spec.mesh = ellipsoid_plate((0.0, 0.0, 0.0), semi_axes, 0.5 * dx, surf_id=51)
    spec.motion = Motion(a0_deg=a0_deg, bfreq=freq, yamp=yamp, shift=tuple(center))
    c = np.asarray(center)
    ax = np.asarray(semi_axes)
    reach = np.array([0.0, yamp + ax[1], ax[1]]) + ax
    spec.search_box = search_box_for(spec, c - reach, c + reach)
    rng = np.random.default_rng(seed)
    chord = 2.0 * semi_axes[0]
    case = Case(name=f"moving_plate{n}", blocks=[spec], dt=0.3 * dx, re=reynolds / chord, uc=1.0,
                epsi=1e-6, pc_ita_max=5000, n_steps=n_steps)
    case.motion = MotionInputs(aoa_deg=0.0, phase_deg=phase_deg, piv_pt=0.0, freq=freq, dxmin=dx)
    case.init = [noisy_initial(spec, case.uc, rng)]
    return case


def heaving_sphere_single_block(n: int = 24, n_steps: int = 6, diameter: float = 0.3,
                                center=(0.45, 0.5, 0.5), yamp: float = 0.05, bfreq: float = 0.5,
                                a0_deg: float = 10.0, freq: float = 0.5, phase_deg: float = 90.0,
                                piv_pt: float = 0.1, reynolds: float = 100.0, seed: int = SEED) -> Case:
    """The sphere of sphere_single_block (surface 50) on the motion of
    src/Search.F90:49-208: heave yamp sin(2 pi bfreq t), tow in -x by
    0.05 dxmin per step, pitch a0 sin(2 pi freq t + phase) about x through
    z = piv_pt.  Surface-50 nodes only translate, so the body has no
    thin-surface cells and its IB cells are ordinary forcing cells."""
    f = uniform_faces(0.0, 1.0, n)
    dx = 1.0 / n
    spec = BlockSpec(n, n, n, f, f.copy(), f.copy(), omega=1.7, is_coarse=True)
    spec.mesh = fibonacci_sphere((0.0, 0.0, 0.0), diameter, dx)
    spec.motion = Motion(a0_deg=a0_deg, bfreq=bfreq, yamp=yamp, shift=tuple(center))
    c = np.asarray(center)
    reach = np.full(3, 0.5 * diameter) + np.array([0.05 * dx * n_steps, yamp, 0.0])
    spec.search_box = search_box_for(spec, c - reach, c + reach)
    rng = np.random.default_rng(seed)
    case = Case(name=f"heaving_sphere{n}", blocks=[spec], dt=0.3 * dx, re=reynolds / diameter, uc=1.0,
                epsi=1e-6, pc_ita_max=5000, n_steps=n_steps)
    case.motion = MotionInputs(aoa_deg=0.0, phase_deg=phase_deg, piv_pt=piv_pt, freq=freq, dxmin=dx)
    case.init = [noisy_initial(spec, case.uc, rng)]
    return case


def sphere_two_block(nf: int = 64, n_steps: int = 200, diameter: float = 0.5,
                     reynolds: float = 300.0, omega_c: float = 1.7, omega_f: float = 1.7,
                     pc_ita_max: int = 5000, seed: int = SEED, coarse=(96, 64, 64),
                     domain=(3.0, 2.0, 2.0), fine_box=((1.0, 2.0), (0.5, 1.5), (0.5, 1.5)),
                     center=None) -> Case:
    """Coarse 96x64x64 over 3x2x2 plus a nested fine nf^3 block at ratio 2 around a sphere.

    The fine block spans `fine_box` (a unit cube) at half the coarse spacing;
    the interface box equals the fine block's extent.  Re = 300 on D = 0.5.
    """
    cnx, cny, cnz = coarse
    L = domain
    dxc = L[0] / cnx
    cs = BlockSpec(cnx, cny, cnz, uniform_faces(0, L[0], cnx), uniform_faces(0, L[1], cny),
                   uniform_faces(0, L[2], cnz), omega=omega_c, is_coarse=True)
    (x0, x1), (y0, y1), (z0, z1) = fine_box
    ratio = 2
    nfx = int(round((x1 - x0) / dxc)) * ratio
    nfy = int(round((y1 - y0) / (L[1] / cny))) * ratio
    nfz = int(round((z1 - z0) / (L[2] / cnz))) * ratio
    assert (nfx, nfy, nfz) == (nf, nf, nf), (nfx, nfy, nfz)
    fs = BlockSpec(nfx, nfy, nfz, uniform_faces(x0, x1, nfx), uniform_faces(y0, y1, nfy),
                   uniform_faces(z0, z1, nfz), omega=omega_f, is_coarse=False)
    if center is None:
        center = (0.5 * (x0 + x1), 0.5 * (y0 + y1), 0.5 * (z0 + z1))
    c = np.asarray(center, dtype=np.float64)
    fs.mesh = fibonacci_sphere(c, diameter, (x1 - x0) / nfx)
    fs.search_box = search_box_for(fs, c - diameter / 2, c + diameter / 2)
    it = InterfaceSpec(1, 2, 1, ratio, (x0, x1, y0, y1, z0, z1))
    rng = np.random.default_rng(seed)
    dxf = (x1 - x0) / nfx
    case = Case(name=f"two_block_{cnx}x{cny}x{cnz}+{nf}^3", blocks=[cs, fs], interfaces=[it],
                dt=0.3 * dxf, re=reynolds / diameter, uc=1.0, epsi=1e-6,
                pc_ita_max=pc_ita_max, n_steps=n_steps)
    case.init = [noisy_initial(b, case.uc, rng) for b in case.blocks]
    return case


def multi_block(coarse=(48, 32, 32), domain=(3.0, 2.0, 2.0),
                fine_boxes=(((0.5, 1.0), (0.5, 1.0), (0.5, 1.0)),
                            ((1.5, 2.25), (0.75, 1.25), (1.0, 1.5)),
                            ((2.375, 2.75), (1.0, 1.5), (0.375, 0.75))),
                body=0, diameter: float = 0.25, reynolds: float = 300.0, n_steps: int = 2,
                omega: float = 1.7, pc_ita_max: int = 5000, seed: int = SEED, plate: bool = False,
                plate_axes=None, motion: Optional[Motion] = None,
                motion_inputs: Optional[MotionInputs] = None, lags_deg=None) -> Case:
    """A coarse block with several nested fine blocks of uneven sizes at ratio 2
    (one interface per fine block), a stationary sphere (or, with `plate`, a
    thin plate of surface 51) centred in fine block `body` (an index, or a
    tuple of indices for one body in each of several blocks).  Box edges must
    lie on coarse faces.  With a `motion`, `lags_deg` gives each body (in the
    order of `body`) its phase lag behind the shared kinematics."""
    bodies = (body,) if isinstance(body, int) else tuple(body)
    cnx, cny, cnz = coarse
    L = domain
    d = (L[0] / cnx, L[1] / cny, L[2] / cnz)
    cs = BlockSpec(cnx, cny, cnz, uniform_faces(0, L[0], cnx), uniform_faces(0, L[1], cny),
                   uniform_faces(0, L[2], cnz), omega=omega, is_coarse=True)
    blocks, ifs = [cs], []
    ratio = 2
    for q, box in enumerate(fine_boxes):
        n = []
        for ax in range(3):
            cells = (box[ax][1] - box[ax][0]) / d[ax]
            assert abs(cells - round(cells)) < 1e-9, (box, ax)
            n.append(int(round(cells)) * ratio)
        fs = BlockSpec(n[0], n[1], n[2], uniform_faces(*box[0], n[0]), uniform_faces(*box[1], n[1]),
                       uniform_faces(*box[2], n[2]), omega=omega, is_coarse=False)
        if q in bodies:
            c = np.array([0.5 * (box[a][0] + box[a][1]) for a in range(3)])
            dxf = (box[0][1] - box[0][0]) / n[0]
            if plate:
                ax = np.array([0.4, 0.3, 0.1]) * diameter if plate_axes is None else np.asarray(plate_axes)
                if motion is not None:
                    # body-frame mesh placed by the motion; the search box
                    # covers the heave and the pitch
                    fs.mesh = ellipsoid_plate((0.0, 0.0, 0.0), ax, 0.5 * dxf)
                    lag = 0.0 if lags_deg is None else float(lags_deg[bodies.index(q)])
                    fs.motion = dataclasses.replace(motion, shift=tuple(c), lag_deg=lag)
                    reach = ax + np.array([0.0, motion.yamp + ax[1], ax[1]])
                    fs.search_box = search_box_for(fs, c - reach, c + reach)
                else:
                    fs.mesh = ellipsoid_plate(c, ax, 0.5 * dxf)
                    fs.search_box = search_box_for(fs, c - ax, c + ax)
            else:
                fs.mesh = fibonacci_sphere(c, diameter, dxf)
                fs.search_box = search_box_for(fs, c - diameter / 2, c + diameter / 2)
        blocks.append(fs)
        ifs.append(InterfaceSpec(1, q + 2, 1, ratio, (box[0][0], box[0][1], box[1][0], box[1][1],
                                                      box[2][0], box[2][1])))
    rng = np.random.default_rng(seed)
    dxf = d[0] / ratio
    case = Case(name=f"multi_{len(blocks)}", blocks=blocks, interfaces=ifs, dt=0.3 * dxf,
                re=reynolds / diameter, uc=1.0, epsi=1e-6, pc_ita_max=pc_ita_max, n_steps=n_steps)
    case.motion = motion_inputs
    case.init = [noisy_initial(b, case.uc, rng) for b in case.blocks]
    return case


def flapping_plate_pair(n_steps: int = 200, size: str = "full", seed: int = SEED) -> Case:
    """A coarse block with one nested fine block at ratio 2 around a flapping
    plate (surface 51): heave yamp sin(2 pi 0.25 t), pitch 30 deg
    sin(2 pi 0.25 t + 90 deg) about x, Re 300 on the chord, towed by 0.05
    fine cells per step.  "full": coarse 128x96x96 over 8x6x6 + fine
    128x128x128 over 4^3 (dx 1/32), plate 0.5x0.125x0.0125, yamp 0.5;
    "small": coarse 64x48x48 over 4x3x3 + fine 80x80x64 (dx 1/32), plate
    0.15x0.0625x0.01, yamp 0.1.  The fine block is wide enough that the
    reference's block-move margins (src/Search.F90:1013-1040) never trigger."""
    if size == "full":
        coarse, domain, box = (128, 96, 96), (8.0, 6.0, 6.0), ((2.0, 6.0), (1.0, 5.0), (1.0, 5.0))
        axes, yamp = (0.5, 0.125, 0.0125), 0.5
    else:
        coarse, domain, box = (64, 48, 48), (4.0, 3.0, 3.0), ((0.75, 3.25), (0.25, 2.75), (0.5, 2.5))
        axes, yamp = (0.15, 0.0625, 0.01), 0.1
    chord = 2.0 * axes[0]
    mo = Motion(a0_deg=30.0, bfreq=0.25, yamp=yamp)
    mi = MotionInputs(aoa_deg=0.0, phase_deg=90.0, piv_pt=0.0, freq=0.25, dxmin=1.0 / 32)
    case = multi_block(coarse=coarse, domain=domain, fine_boxes=(box,), body=0, plate=True, plate_axes=axes,
                       diameter=chord, reynolds=300.0, motion=mo, motion_inputs=mi, n_steps=n_steps, seed=seed)
    # the search box also covers the tow in -x (0.05 dxmin per step)
    fs = case.blocks[1]
    c = np.array(fs.motion.shift)
    ax = np.asarray(axes)
    reach = ax + np.array([0.0, yamp + ax[1], ax[1]])
    lo = c - reach
    lo[0] -= 0.05 * mi.dxmin * (n_steps + 2)
    fs.search_box = search_box_for(fs, lo, c + reach)
    return replace(case, name=f"flapping_plate_pair_{size}")


def moving_plate_block_move(n_steps: int = 3, seed: int = SEED) -> Case:
    """A coarse 48x32x32 block over 1.5x1x1 (dx 1/32) with one fine block at
    ratio 2 around a heaving, pitching, towed plate, sized so that the
    reference's block-move margins (src/Search.F90:1013-1040: 4.5, 5 and 1.52
    times 3 coarse cells in x, y and z) hold from the first step: the fine
    block moves by whole cells every step."""
    mo = Motion(a0_deg=10.0, bfreq=0.25, yamp=0.02)
    mi = MotionInputs(aoa_deg=0.0, phase_deg=90.0, piv_pt=0.0, freq=0.25, dxmin=1.0 / 64)
    return multi_block(coarse=(48, 32, 32), domain=(1.5, 1.0, 1.0),
                       fine_boxes=(((0.25, 1.0), (0.25, 0.75), (0.25, 0.75)),), body=0, plate=True,
                       plate_axes=(0.1, 0.075, 0.02), motion=mo, motion_inputs=mi, n_steps=n_steps, seed=seed)


# the 12-block layout: a coarse 256x192x192 block over 8x6x6 (dx 1/32) with 11
# fine blocks at ratio 2 in the sizes 160x96x96, 128x64x64, 96x64x64,
# 64x48x48, 48^3, 32^3 and repeats of the last five (13.3M cells in all)
TWELVE_BLOCK_BOXES = (
    ((0.5, 3.0), (0.5, 2.0), (0.5, 2.0)),      # 160x96x96, holds the plate
    ((3.5, 5.5), (0.5, 1.5), (0.5, 1.5)),      # 128x64x64
    ((6.0, 7.5), (0.5, 1.5), (0.5, 1.5)),      # 96x64x64
    ((3.5, 4.5), (2.0, 2.75), (0.5, 1.25)),    # 64x48x48
    ((5.0, 5.75), (2.0, 2.75), (0.5, 1.25)),   # 48^3
    ((6.5, 7.0), (2.25, 2.75), (0.5, 1.0)),    # 32^3
    ((0.5, 2.5), (0.5, 1.5), (3.0, 4.0)),      # 128x64x64
    ((3.0, 4.5), (0.5, 1.5), (3.0, 4.0)),      # 96x64x64
    ((5.0, 6.0), (0.5, 1.25), (3.0, 3.75)),    # 64x48x48
    ((6.5, 7.25), (0.5, 1.25), (3.0, 3.75)),   # 48^3
    ((0.5, 1.0), (3.0, 3.5), (3.0, 3.5)),      # 32^3
)


def twelve_block(n_steps: int = 10, seed: int = SEED, moving: bool = False) -> Case:
    """Twelve blocks of uneven sizes around a rigid ellipsoidal plate (semi-axes
    0.5 x 0.125 x 0.0125, surface 51), Re = 500 on the chord: a coarse
    320x224x224 block over 10x7x7 (dx 1/32, 16.1M cells) and the eleven fine
    blocks of TWELVE_BLOCK_BOXES at ratio 2 (3.9M cells), 20.0M cells in all.
    With `moving` the plate heaves h(t) = 0.5 sin(2 pi 0.25 t) and pitches
    about x theta(t) = 30 deg sin(2 pi 0.25 t + 90 deg) (plus the reference's
    fixed tow); its block is then 160x144x96 (20.7M cells in all), tall enough
    that the heave stays inside the reference's block-move margins
    (src/Search.F90:1010-1024)."""
    boxes = list(TWELVE_BLOCK_BOXES)
    motion = inputs = None
    if moving:
        boxes[0] = ((0.5, 3.0), (0.25, 2.5), (0.5, 2.0))
        motion = Motion(a0_deg=30.0, bfreq=0.25, yamp=0.5)
        inputs = MotionInputs(aoa_deg=0.0, phase_deg=90.0, piv_pt=0.0, freq=0.25, dxmin=1.0 / 64.0)
    return multi_block(coarse=(320, 224, 224), domain=(10.0, 7.0, 7.0), fine_boxes=tuple(boxes),
                       body=0, diameter=1.0, reynolds=500.0, n_steps=n_steps, seed=seed, plate=True,
                       plate_axes=(0.5, 0.125, 0.0125), motion=motion, motion_inputs=inputs)


def tandem_plates(n_steps: int = 2, seed: int = SEED, moving: bool = False, lag_deg: float = 90.0,
                  size: str = "full") -> Case:
    """Two thin plates in tandem on the 44M-cell layout: a coarse 384x256x256
    block over 6x4x4 (dx 1/64) and two fine 256x192x192 blocks at ratio 2
    (dx 1/128), each holding a rigid ellipsoidal plate of semi-axes
    0.5 x 0.125 x 0.0125 (surface 51) at its centre; the plates are 1.5 chords
    apart (centres at x = 1.75 and 4.25), Re = 1000 on the chord.  With
    `moving` the leading plate heaves 0.125 sin(2 pi 0.25 t) and pitches about
    x 15 deg sin(2 pi 0.25 t + 90 deg), starting at its t = 0 angle of attack
    (15 deg); the trailing plate does the same `lag_deg` behind
    (bcfd_block_set_body_lag), starting at its own t = 0 state.  The
    amplitudes keep each plate inside its block's move margins
    (src/Search.F90:1010-1040).  "small": the same arrangement at test size --
    coarse 96x48x24 over 6x3x1.5 (dx 1/16), two fine 64x72x24 blocks (dx
    1/32) just wide enough for the move margins, plates 0.1 x 0.05 x 0.008
    (thinner than a fine cell), heave 0.05, pitch 10 deg, Re 300."""
    if size == "small":
        boxes = (((0.5, 2.5), (0.375, 2.625), (0.375, 1.125)),
                 ((3.0, 5.0), (0.375, 2.625), (0.375, 1.125)))
        motion = inputs = None
        if moving:
            motion = Motion(a0_deg=10.0, bfreq=0.25, yamp=0.05)
            inputs = MotionInputs(aoa_deg=10.0, phase_deg=90.0, piv_pt=0.0, freq=0.25, dxmin=1.0 / 32.0)
        case = multi_block(coarse=(96, 48, 24), domain=(6.0, 3.0, 1.5), fine_boxes=boxes, body=(0, 1),
                           diameter=0.2, reynolds=300.0, n_steps=n_steps, seed=seed, plate=True,
                           plate_axes=(0.1, 0.05, 0.008), motion=motion, motion_inputs=inputs,
                           lags_deg=(0.0, lag_deg) if moving else None)
        return replace(case, name="tandem_plates_small")
    boxes = (((0.75, 2.75), (1.25, 2.75), (1.25, 2.75)),
             ((3.25, 5.25), (1.25, 2.75), (1.25, 2.75)))
    motion = inputs = None
    if moving:
        motion = Motion(a0_deg=15.0, bfreq=0.25, yamp=0.125)
        inputs = MotionInputs(aoa_deg=15.0, phase_deg=90.0, piv_pt=0.0, freq=0.25, dxmin=1.0 / 128.0)
    return multi_block(coarse=(384, 256, 256), domain=(6.0, 4.0, 4.0), fine_boxes=boxes, body=(0, 1),
                       diameter=1.0, reynolds=1000.0, n_steps=n_steps, seed=seed, plate=True,
                       plate_axes=(0.5, 0.125, 0.0125), motion=motion, motion_inputs=inputs,
                       lags_deg=(0.0, lag_deg) if moving else None)


def plate_block(n=(256, 192, 192), n_steps: int = 2, seed: int = SEED) -> Case:
    """One block of the tandem plates' fine-block size (dx 1/128) with the
    domain BCs and a stationary plate of semi-axes 0.5 x 0.125 x 0.0125 at its
    centre, Re = 1000 on the chord: the momentum stencil, forcing and Search
    of the large workload on ~1 GB of device memory (profiler captures)."""
    nx, ny, nz = n
    L = (nx / 128.0, ny / 128.0, nz / 128.0)
    spec = BlockSpec(nx, ny, nz, uniform_faces(0, L[0], nx), uniform_faces(0, L[1], ny),
                     uniform_faces(0, L[2], nz), omega=1.7, is_coarse=True)
    c = np.array([0.5 * L[0], 0.5 * L[1], 0.5 * L[2]])
    ax = np.array([0.5, 0.125, 0.0125])
    dx = 1.0 / 128.0
    spec.mesh = ellipsoid_plate(c, ax, 0.5 * dx)
    spec.search_box = search_box_for(spec, c - ax, c + ax)
    case = Case(name=f"plate_block{nx}", blocks=[spec], dt=0.3 * dx, re=1000.0, uc=1.0, epsi=1e-6,
                pc_ita_max=5000, n_steps=n_steps)
    case.init = [noisy_initial(spec, case.uc, np.random.default_rng(seed))]
    return case


def uniform_block(n=(384, 256, 256), lengths=(3.0, 2.0, 2.0), seed: int = SEED,
                  noise: bool = True) -> Case:
    """One body-free uniform block with the domain BCs (384x256x256 is the
    coarse block size of the tandem-plate workload); used to measure the
    Poisson sweeps at sizes far above the 129 MB L2."""
    nx, ny, nz = n
    spec = BlockSpec(nx, ny, nz, uniform_faces(0, lengths[0], nx), uniform_faces(0, lengths[1], ny),
                     uniform_faces(0, lengths[2], nz), omega=1.7, is_coarse=True)
    dx = lengths[0] / nx
    case = Case(name=f"block{nx}x{ny}x{nz}", blocks=[spec], dt=0.3 * dx, re=1000.0, uc=1.0)
    if noise:
        case.init = [noisy_initial(spec, case.uc, np.random.default_rng(seed))]
    else:
        shp = spec.shape
        case.init = [{"u": np.ones(shp), "v": np.zeros(shp), "w": np.zeros(shp), "p": np.zeros(shp)}]
    return case


def small_two_block(n_steps: int = 2, seed: int = SEED) -> Case:
    """A 24x16x16 coarse + 16^3 fine version of the two-block case for fast parity tests."""
    return sphere_two_block(nf=16, n_steps=n_steps, diameter=0.5, coarse=(24, 16, 16),
                            domain=(3.0, 2.0, 2.0), fine_box=((1.0, 2.0), (0.5, 1.5), (0.5, 1.5)),
                            pc_ita_max=2000, seed=seed)


def mixed_omega(nx: int, ny: int, nz: int) -> float:
    """The relaxation factor the mixed path's FP32 sweeps use by default: the
    classical red-black SOR optimum 2 / (1 + sqrt(1 - rho^2)) for the 7-point
    Laplacian on an nx x ny x nz box with Dirichlet boundaries, rho = (cos(pi/nx)
    + cos(pi/ny) + cos(pi/nz)) / 3, at most 1.99 (the library's expression)."""
    import math
    pi = 3.14159265358979323846

    def s2(n):
        x = math.sin(pi / (2.0 * n))
        return 2.0 * x * x

    e = (s2(nx) + s2(ny) + s2(nz)) / 3.0
    return min(1.99, max(1.0, 2.0 / (1.0 + math.sqrt(e * (2.0 - e)))))


def with_mixed_omega(case: Case) -> Case:
    """A copy of `case` whose blocks relax with the factor the mixed path's FP32
    sweeps use by default (`mixed_omega`) instead of the input's omega: the
    plain FP64 solve at the same relaxation separates the gain of the precision
    from that of the factor."""
    blocks = [dataclasses.replace(b, omega=mixed_omega(b.nx, b.ny, b.nz)) for b in case.blocks]
    return dataclasses.replace(case, blocks=blocks)


def replace(case: Case, **kw) -> Case:
    return dataclasses.replace(case, **kw)
