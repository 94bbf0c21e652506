"""Reference-compatible INI parsing, file names, raw arrays and mode orders
(modal-cmb_gb300/modal_files.py), against the conventions of parameter.c,
arrays.c, io.c and set_terms_late; the GPU driver end to end is in
test_gpu_files.py."""
import os

import numpy as np
import pytest

import modal_files as mf

INI = """
; comment line
[model]
directory = "{d}"   ; trailing comment
T_lmin = 2
T_lmax = 2000
E_lmin = 3
E_lmax = 1500
do_polarisation = 0
[basis]
terms = 4960
order_prim = 3
order_late = 2
orthol_file = orthol
# another comment
gamma_file = gamma
[old]
gflag_pca = 1
"""


def _ini(tmp_path):
    p = tmp_path / "run.ini"
    p.write_text(INI.format(d=str(tmp_path) + "/"))
    return os.fspath(p)


def test_read_ini_keys(tmp_path):
    ini = mf.read_ini(_ini(tmp_path))
    assert ini["model:directory"] == str(tmp_path) + "/"
    assert mf.getint(ini, "model:T_lmax", 0) == 2000
    assert mf.getint(ini, "basis:terms", 0) == 4960
    assert mf.getint(ini, "model:missing", 7) == 7
    assert mf.getstring(ini, "basis:orthol_file", "") == "orthol"


def test_output_names_follow_parameter_c(tmp_path):
    d = str(tmp_path) + "/"
    names = mf.output_names(mf.read_ini(_ini(tmp_path)))
    # parameter.c: directory + name + _XXX_ + T range [+ _ + E range] + _order_late + _terms
    assert names["orthol_TTT"] == d + "orthol_TTT_2-2000_2_4960"
    assert names["orthol_TTE"] == d + "orthol_TTE_2-2000_3-1500_2_4960"
    assert names["orthol_TEE"] == d + "orthol_TEE_2-2000_3-1500_2_4960"
    assert names["orthol_EEE"] == d + "orthol_EEE_3-1500_2_4960"
    assert names["lambdal_TTT"] == d + "lambdal_TTT_2-2000_2_4960"
    assert names["modes_EEE"] == d + "modes_EEE_3-1500_2_4960"
    # gamma carries the primordial order too
    assert names["gamma_TTT"] == d + "gamma_TTT_2-2000_3_2_4960"
    assert names["gamma_TTE"] == d + "gamma_TTE_2-2000_3-1500_3_2_4960"


def test_raw_arrays_and_triples(tmp_path):
    a = np.random.default_rng(1).standard_normal((7, 5))
    p = os.fspath(tmp_path / "a.unf")
    mf.array_write(p, a)
    assert os.path.getsize(p) == 7 * 5 * 8
    assert np.array_equal(mf.array_read(p, 35).reshape(7, 5), a)
    with pytest.raises(ValueError):
        mf.array_read(p, 36)
    t = tmp_path / "order.txt"
    t.write_text("0 0 0\n0 0 1\n0 1 1\n")
    assert mf.load_three_int(os.fspath(t)).tolist() == [[0, 0, 0], [0, 0, 1], [0, 1, 1]]


def test_mode_orders(mg):
    c2 = mf._order_case2(200)
    assert c2[:7].tolist() == [[0, 0, 0], [0, 0, 1], [0, 1, 1], [0, 0, 2], [1, 1, 1], [0, 1, 2], [0, 0, 3]]
    s = c2.sum(1)
    assert np.all(np.diff(s) >= 0) and len({tuple(r) for r in c2.tolist()}) == 200
    assert np.all(c2[:, 0] <= c2[:, 1]) and np.all(c2[:, 1] <= c2[:, 2])
    for P in (4, 6):  # the benchmark's lists are case 2 restricted to indices < P
        want = mg.mode_triples(P)
        got = np.array([r for r in mf._order_case2(400).tolist() if max(r) < P][:len(want)])
        assert np.array_equal(got, want)
    c1 = mf._order_case1(12)
    assert len({tuple(r) for r in c1.tolist()}) == 12
