"""A deck in the reference's file formats run through the native driver
(run_deck): the fields after three steps are bitwise those of the oracle on
the same deck-derived case, and the step-0..2 field files and the step-1
surface file are written."""
import os

import numpy as np
import pytest

from biocfd import deck, synth
from oracle.bridge import Oracle
from parity_util import compare_fields

pytestmark = pytest.mark.gpu


def test_run_deck_matches_oracle(tmp_path):
    case = synth.sphere_two_block(nf=16, n_steps=3, diameter=0.5, coarse=(24, 16, 16), domain=(3.0, 2.0, 2.0),
                                  fine_box=((1.0, 2.0), (0.5, 1.5), (0.5, 1.5)))
    deck.write_deck(tmp_path, case, mu_f_in=250.0, rho_f=1.0, l_c_mm=250.0, re_in=100.0, freq_in=1.0,
                    dt_order=1.0 / (16.0 * case.dt), itamax=3, shift_mm=[(0.0, 0.0, 0.0)] * len(case.blocks))
    s = deck.run_deck(tmp_path, n_steps=3, out_dir=str(tmp_path))
    d = deck.read_deck(tmp_path)
    o = Oracle()
    o.setup(deck.deck_to_case(d))
    for _ in range(3):
        o.step()
    compare_fields(o, s, "deck, 3 steps")
    for g in (1, 2):
        for ita in (0, 1, 2):
            assert os.path.exists(tmp_path / deck.field_name(d.char_f, ita, g, d.re, d.blocks[g - 1].d[0], 2))
    assert os.path.exists(tmp_path / "out" / "butterfly_002.dat")
    rows = np.loadtxt(tmp_path / deck.field_name(d.char_f, 2, 1, d.re, d.blocks[0].d[0], 2), skiprows=2)
    assert rows.shape == (24 * 16 * 16, 11) and np.all(np.isfinite(rows))


def test_run_deck_hdf5_field_files(tmp_path):
    """The HDF5 build's field files (write_output_hdf5): after two steps the
    step-2 file holds the solver's fields and tags, and steps 0 and 1 have
    files too."""
    from biocfd import h5io
    case = synth.sphere_two_block(nf=16, n_steps=2, diameter=0.5, coarse=(24, 16, 16), domain=(3.0, 2.0, 2.0),
                                  fine_box=((1.0, 2.0), (0.5, 1.5), (0.5, 1.5)))
    deck.write_deck(tmp_path, case, mu_f_in=250.0, rho_f=1.0, l_c_mm=250.0, re_in=100.0, freq_in=1.0,
                    dt_order=1.0 / (16.0 * case.dt), itamax=2, shift_mm=[(0.0, 0.0, 0.0)] * len(case.blocks))
    s = deck.run_deck(tmp_path, n_steps=2, out_dir=str(tmp_path), output_format="hdf5")
    d = deck.read_deck(tmp_path)
    i = (slice(1, -1),) * 3
    for g, h in enumerate(s.handles, 1):
        for ita in (0, 1):
            assert os.path.exists(tmp_path / h5io.field_name_hdf5(ita, g))
        fn = tmp_path / h5io.field_name_hdf5(2, g)
        f, t = s.fields(h), s.tags(h)
        u = f["u"]
        assert np.array_equal(h5io.hdf5_read_real_3d(fn, "/", "u1"), 0.5 * (u[i] + u[:-2, 1:-1, 1:-1]))
        assert np.array_equal(h5io.hdf5_read_real_3d(fn, "/", "p"), f["p"][i])
        assert np.array_equal(h5io.hdf5_read_int_3d(fn, "/", "cell"), t["cell"][i])
        assert np.array_equal(h5io.hdf5_read_int_3d(fn, "/", "cell_pr"), t["cell_pr"][:-1, :-1, :-1][i])
        b = d.blocks[g - 1]
        xp = 0.5 * (np.asarray(b.x1)[1:] + np.asarray(b.x1)[:-1])[1:u.shape[0] - 1]
        assert np.array_equal(h5io.hdf5_read_real_1d(fn, "/", "xp"), xp)
        assert h5io.hdf5_read_real_scalar(fn, "/", "totime") == s.time()[1]
        assert h5io.hdf5_read_int_scalar(fn, "/", "zonek") == u.shape[2] - 2
    s.close()
