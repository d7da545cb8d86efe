"""The reference's input deck, restart and output formats (CPU): namelist
parsing, the unit conversions of src/ReadInput.f90, deck -> case round trips
of grids, blocks, interfaces and the gmsh surface, restart round trips, and
the zone-file layout of the field output."""
import os

import numpy as np
import pytest

from biocfd import deck, synth


def test_namelist_parsing(tmp_path):
    p = tmp_path / "input_data.nml"
    p.write_text("! comment line\n&INPUT_DATA nblocks = 2, intflines=1,\n  epsi = 1.0d-6 ! tol\n"
                 "  re=100.0, mu_f = 250., dt_order = 8.0D0, istart = 0 /\n")
    v = deck.read_namelist(p)
    assert v["nblocks"] == 2 and v["intflines"] == 1 and v["istart"] == 0
    assert v["epsi"] == 1e-6 and v["re"] == 100.0 and v["mu_f"] == 250.0 and v["dt_order"] == 8.0
    q = tmp_path / "out.nml"
    deck.write_namelist(q, {"nblocks": 3, "epsi": 2.5e-7, "pcitamax": 40})
    w = deck.read_namelist(q)
    assert w == {"nblocks": 3, "epsi": 2.5e-7, "pcitamax": 40}


def _sphere_deck(tmp_path, n=16):
    """The single-sphere workload written as a two-block deck the reference
    can read: coarse block 1 and the body block 2 (lengths in mm)."""
    case = synth.sphere_two_block(nf=n, n_steps=2, diameter=0.5, coarse=(24, 16, 16), domain=(3.0, 2.0, 2.0),
                                  fine_box=((1.0, 2.0), (0.5, 1.5), (0.5, 1.5)))
    # mu_f 250 (x1e-5), rho_f 1, l_c 250 mm, re 100 -> u0 = 1, re = 400; dt_order = 1/(16 dt)
    dt = case.dt
    deck.write_deck(tmp_path, case, mu_f_in=250.0, rho_f=1.0, l_c_mm=250.0, re_in=100.0, freq_in=1.0,
                    dt_order=1.0 / (16.0 * dt), shift_mm=[(0.0, 0.0, 0.0)] * len(case.blocks))
    return case


def test_deck_units_and_round_trip(tmp_path):
    case = _sphere_deck(tmp_path)
    d = deck.read_deck(tmp_path)
    assert d.mu_f == 250.0 * 1e-5 and d.l_c == 0.001 * 250.0
    assert d.u0 == 100.0 * d.mu_f / (1.0 * d.l_c) and d.uc == d.u0
    assert abs(d.u0 - 1.0) < 1e-15 and d.re == 1.0 / d.mu_f
    assert abs(d.deltat - case.dt) < 1e-15 * case.dt / 1e-3
    c2 = deck.deck_to_case(d)
    assert len(c2.blocks) == len(case.blocks) and c2.blocks[0].is_coarse and not c2.blocks[1].is_coarse
    for a, b in zip(case.blocks, c2.blocks):
        assert (a.nx, a.ny, a.nz) == (b.nx, b.ny, b.nz)
        assert a.search_box == b.search_box and a.omega == b.omega
        for fa, fb in ((a.x_faces, b.x_faces), (a.y_faces, b.y_faces), (a.z_faces, b.z_faces)):
            # ReadInput's own arithmetic on the mm values: 0.001 * x + shift
            np.testing.assert_allclose(fb, fa, rtol=0, atol=1e-15)
    # block g >= 2 carries the surface, as main.F90 reads it into every fine block
    m0, m1 = case.blocks[1].mesh, c2.blocks[1].mesh
    np.testing.assert_allclose(m1.nodes, m0.nodes, rtol=0, atol=1e-15)
    assert np.array_equal(m1.tris, m0.tris) and np.array_equal(m1.surf_id, m0.surf_id)
    assert len(c2.interfaces) == 1 and c2.interfaces[0].b_blk == 2
    np.testing.assert_allclose(c2.interfaces[0].box, case.interfaces[0].box, atol=1e-15)
    # uniform initial field (initialConditions)
    assert np.all(c2.init[0]["u"] == d.uc) and np.all(c2.init[1]["p"] == 0.0)


def test_grid_arithmetic_matches_readinput(tmp_path):
    vals = [0.0, 0.7, 1.9, 3.3]
    p = tmp_path / "xgrid_bk001_4.txt"
    p.write_text("".join(f"{v}\n" for v in vals))
    x1 = deck._grid(p, 3, 0.25)
    ref = np.array([0.001 * v + 0.25 for v in vals])
    assert np.array_equal(x1[1:5], ref)
    assert x1[0] == x1[1] - (x1[2] - x1[1]) and x1[5] == x1[4] + (x1[4] - x1[3])


def test_restart_round_trip_and_names(tmp_path):
    rng = np.random.default_rng(3)
    shp = (6, 5, 4)
    f = {k: np.asfortranarray(rng.normal(size=shp)) for k in ("u", "v", "w", "p")}
    path = tmp_path / deck.restart_name(2, 400.0)
    deck.write_restart(path, f, 1.25e-2, 37, 5)
    g, tot, ita, ita1 = deck.read_restart(path, 4, 3, 2)
    for k in f:
        assert np.array_equal(g[k], f[k])
    assert (tot, ita, ita1) == (1.25e-2, 37, 5)
    assert deck.restart_name(2, 400.0) == "out/aorta_chkpt.002. 400.0.dat"
    assert deck.checkpoint_name("amp", 1, 400.0, 0.0625) == "out/Chkpt/amp_butter_chkpt.001. 400.0.0.062500.dat"
    assert deck.field_name("bot", 200, 3, 400.0, 0.03125, 12) == "out/bot_butter_fielddata.000000200.003.  400.0.0.031250.012.dat"


def test_field_output_layout(tmp_path):
    nx, ny, nz = 3, 2, 2
    shp = (nx + 2, ny + 2, nz + 2)
    rng = np.random.default_rng(1)
    f = {k: np.asfortranarray(rng.normal(size=shp)) for k in ("u", "v", "w", "p")}
    tags = {k: np.zeros(shp, np.int64, order="F") for k in ("cell", "cell_n", "cell_pr")}
    x1 = np.arange(nx + 3, dtype=float)
    y1 = np.arange(ny + 3, dtype=float) * 2
    z1 = np.arange(nz + 3, dtype=float) * 3
    path = tmp_path / "zone.dat"
    deck.write_fields_ascii(path, x1, y1, z1, f, tags, 0.5)
    lines = path.read_text().splitlines()
    assert lines[0].strip().startswith('variables="x"') and "i = 3 j = 2 k = 2" in lines[1]
    rows = np.loadtxt(lines[2:])
    assert rows.shape == (nx * ny * nz, 11)
    # first interior cell (i,j,k) = (2,2,2): centre and averaged velocities
    r = rows[0]
    assert r[0] == 0.5 * (x1[1] + x1[2]) and r[1] == 0.5 * (y1[1] + y1[2])
    assert r[3] == 0.5 * (f["u"][1, 1, 1] + f["u"][0, 1, 1])
    assert r[4] == 0.5 * (f["v"][1, 1, 1] + f["v"][1, 0, 1])
    assert r[6] == f["p"][1, 1, 1] and r[7] == 0.5
    # x fastest
    assert rows[1][0] == 0.5 * (x1[2] + x1[3])
