"""Synthetic workload layouts (no GPU): block sizes, bodies and interface boxes
of the 44M-cell tandem-plate layout, and the block sizes, bodies, motion and
run parameters of the other benchmark configurations (the 64^3 sphere, the
two-block sphere, the twelve-block and two-block flapping plates)."""
import numpy as np

from biocfd import synth


def test_tandem_plates_layout():
    case = synth.tandem_plates(n_steps=1)
    sizes = [(b.nx, b.ny, b.nz) for b in case.blocks]
    assert sizes == [(384, 256, 256), (256, 192, 192), (256, 192, 192)]
    assert sum(b.nx * b.ny * b.nz for b in case.blocks) == 44_040_192
    coarse, f1, f2 = case.blocks
    assert coarse.is_coarse and not coarse.has_body
    assert f1.has_body and f2.has_body
    for f in (f1, f2):
        # one stationary surface-51 plate centred in its block, 1/128 cells
        assert f.motion is None
        assert np.all(f.mesh.surf_id == 51)
        assert np.allclose(np.diff(f.x_faces), 1.0 / 128)
    c1 = f1.mesh.nodes.mean(axis=0)
    c2 = f2.mesh.nodes.mean(axis=0)
    # chord 1, centres 2.5 apart: a gap of 1.5 chords
    assert abs((c2[0] - c1[0]) - 2.5) < 1e-9
    assert np.ptp(f1.mesh.nodes[:, 0]) <= 1.0 + 1e-12
    # interface boxes lie on coarse faces and match the fine grids
    dxc = 6.0 / 384
    for it, f in zip(case.interfaces, (f1, f2)):
        box = np.array(it.box)
        assert np.allclose(box / dxc, np.round(box / dxc))
        assert np.isclose(box[0], f.x_faces[0]) and np.isclose(box[1], f.x_faces[-1])
    assert case.re == 1000.0


def _cells(case):
    return sum(b.nx * b.ny * b.nz for b in case.blocks)


def test_sphere_configurations():
    # one 64^3 block on the unit cube, sphere D 0.25 at (0.4, 0.5, 0.5):
    # nu = 0.0025 (re argument 400), dt = 0.3 dx, omega 1.7, epsi 1e-6, 100 steps
    c1 = synth.sphere_single_block()
    (b,) = c1.blocks
    assert (b.nx, b.ny, b.nz) == (64, 64, 64) and b.x_faces[0] == 0.0 and b.x_faces[-1] == 1.0
    assert np.allclose(b.mesh.nodes.mean(axis=0), (0.4, 0.5, 0.5), atol=1e-3)
    assert abs(np.ptp(b.mesh.nodes[:, 0]) - 0.25) < 1e-3 and set(b.mesh.surf_id.tolist()) == {50}
    assert (c1.re, c1.dt, b.omega, c1.epsi, c1.n_steps) == (400.0, 0.3 / 64, 1.7, 1e-6, 100)
    # coarse 96x64x64 over 3x2x2 + fine 64^3 at ratio 2 around a D 0.5 sphere, re argument 600
    c2 = synth.sphere_two_block()
    assert [(b.nx, b.ny, b.nz) for b in c2.blocks] == [(96, 64, 64), (64, 64, 64)]
    assert c2.blocks[0].is_coarse and c2.blocks[1].has_body and len(c2.interfaces) == 1
    assert abs(np.ptp(c2.blocks[1].mesh.nodes[:, 0]) - 0.5) < 1e-3
    assert (c2.re, c2.n_steps) == (600.0, 200)


def test_moving_plate_configurations():
    # twelve blocks, ~20.7M cells, one heaving (0.5) and pitching (30 deg) plate at 0.25 Hz, Re 500
    c3 = synth.twelve_block(moving=True)
    assert len(c3.blocks) == 12 and len(c3.interfaces) == 11 and _cells(c3) == 20_684_800
    movers = [b for b in c3.blocks if b.motion is not None]
    assert len(movers) == 1 and c3.re == 500.0
    m = movers[0].motion
    assert (m.yamp, m.a0_deg, m.bfreq, m.lag_deg) == (0.5, 30.0, 0.25, 0.0)
    assert np.allclose(np.ptp(movers[0].mesh.nodes, axis=0), (1.0, 0.25, 0.025), atol=1e-3)
    # coarse 128x96x96 + fine 128^3, 3.28M cells, the same plate and motion
    c4 = synth.flapping_plate_pair()
    assert [(b.nx, b.ny, b.nz) for b in c4.blocks] == [(128, 96, 96), (128, 128, 128)]
    assert _cells(c4) == 3_276_800 and c4.n_steps == 200
    assert (c4.blocks[1].motion.yamp, c4.blocks[1].motion.a0_deg) == (0.5, 30.0)
    # the tandem plates moving: the trailing plate 90 deg behind the leading one
    c5 = synth.tandem_plates(moving=True)
    lead, trail = c5.blocks[1].motion, c5.blocks[2].motion
    assert (lead.lag_deg, trail.lag_deg) == (0.0, 90.0)
    assert (lead.yamp, lead.a0_deg, lead.bfreq) == (trail.yamp, trail.a0_deg, trail.bfreq) == (0.125, 15.0, 0.25)
