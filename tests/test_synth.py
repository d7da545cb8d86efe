"""Synthetic workload layouts (no GPU): block sizes, bodies and interface boxes
of the 45M-cell tandem-plate layout."""
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
