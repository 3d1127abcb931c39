"""The library's own reader of FLINT's input files (flint_tables_read, the C
counterpart of read_idealgas_thermo / read_idealgas_transport / read_chemistry,
Load_ThermoTransport.f90:7-174, Load_Chemistry.f90:7-164) against the Python
reader on the same folders, and its error returns.  Host only: no GPU."""
import copy
import json
import os

import numpy as np
import pytest

from flint_gb300 import mechgen, native, tables
from flint_gb300.mech import Mechanism

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _same(a, b):
    assert a["ns"] == b["ns"] and a["names"] == b["names"]
    for k in ("tmin", "tmax", "ti1", "ti2", "nr_arrh", "nr_troe", "nr_lind"):
        assert a[k] == b[k], k
    for k in tables.ARRAYS:
        if b.get(k) is None or np.asarray(b[k]).size == 0:
            assert a.get(k) is None or np.asarray(a[k]).size == 0, k
            continue
        np.testing.assert_array_equal(a[k], np.asarray(b[k]).reshape(a[k].shape), err_msg=k)


@pytest.fixture(scope="module")
def pel_folder(tmp_path_factory):
    m = Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json"))
    t = tables.generate(m, 1, 3000)
    d = tmp_path_factory.mktemp("pel")
    tables.write_folder(t, str(d))
    return t, str(d)


def test_native_reader_matches_python_reader(pel_folder):
    t, d = pel_folder
    a, b = tables.read_folder_native(d), tables.read_folder(d)
    _same(a, b)
    assert a["tmin"] == 0 and np.all(a["h_tab"][:, 0] == 0.0)   # row 0 cloned, h(0) = 0
    assert a["nr_troe"] == 2 and a["nr_lind"] == 4
    assert a["runiv"] == 8314.51


def test_native_reader_transport_and_prefix(tmp_path):
    m = copy.deepcopy(mechgen.load("c1"))
    t = tables.generate(m, 200, 4000)
    T = np.arange(t["tmin"], t["tmax"] + 1, dtype=np.float64)
    t["mi_tab"] = np.array([(1.0 + 0.1 * k) * 1.8e-5 * (T / 300.0) ** 0.7 for k in range(m.ns)])
    t["k_tab"] = np.array([(1.0 + 0.1 * k) * 0.025 * (T / 300.0) ** 0.8 for k in range(m.ns)])
    tables.write_folder(t, str(tmp_path))
    for f in os.listdir(tmp_path):                      # same files under a prefix
        os.link(tmp_path / f, tmp_path / ("case_" + f))
    a, b = tables.read_folder_native(str(tmp_path), "case_"), tables.read_folder(str(tmp_path), "case_")
    _same(a, b)
    assert a["tmin"] == 200 and a["mi_tab"].shape == (m.ns, 3801)


def test_native_reader_reference_chemistry_info(tmp_path):
    """The reference's WD chemistry-info.txt and phase.txt, as in the Python reader's test."""
    g = json.load(open(os.path.join(GOLD, "wd_info.json")))
    (tmp_path / "chemistry-info.txt").write_text("\n".join(g["info_lines"]) + "\n")
    (tmp_path / "phase.txt").write_text("ideal-gas phase\n" + "".join(f"{k} {v}\n" for k, v in g["phase"].items()))
    T = np.arange(1.0, 11.0)
    names = list(g["phase"])
    tables._write_zones(str(tmp_path / "thermo.dat"), "t", ["Temperature", "Cp", "Enthalpy", "Entropy", "dCp"],
                        [(n, [np.full(10, 1000.0 + i), np.arange(10.0) * (i + 1), np.ones(10), np.zeros(10)])
                         for i, n in enumerate(names)], T)
    tables._write_zones(str(tmp_path / "chemistry-Arrhenius.dat"), "a", ["Temperature", "kf", "kb"],
                        [(f"Reaction {j + 1}", [np.arange(10.0) + j, np.zeros(10)]) for j in range(3)], T)
    a, b = tables.read_folder_native(str(tmp_path)), tables.read_folder(str(tmp_path))
    _same(a, b)
    assert a["ni1_arrh"][0, names.index("O2")] == 1.5 and a["ni2_arrh"][0, names.index("H2O")] == 2.0


def test_native_reader_fortran_exponents(tmp_path):
    """Tecplot rows written with Fortran D exponents parse like E exponents."""
    m = copy.deepcopy(mechgen.load("c1"))
    t = tables.generate(m, 300, 400)
    tables.write_folder(t, str(tmp_path))
    for f in ("thermo.dat", "chemistry-Arrhenius.dat"):
        p = tmp_path / f
        p.write_text(p.read_text().replace("E+", "D+").replace("E-", "D-"))
    _same(tables.read_folder_native(str(tmp_path)), tables.read_folder(str(tmp_path)))


@pytest.mark.parametrize("missing", ["phase.txt", "thermo.dat", "chemistry-info.txt", "chemistry-Arrhenius.dat",
                                     "chemistry-Troe.dat"])
def test_native_reader_missing_file_is_an_io_error(pel_folder, tmp_path, missing):
    _, d = pel_folder
    for f in os.listdir(d):
        if f != missing:
            os.link(os.path.join(d, f), tmp_path / f)
    with pytest.raises(RuntimeError, match=r"status 4\).*" + missing.split(".")[0]):
        tables.read_folder_native(str(tmp_path))


def test_native_reader_ragged_zone_is_an_io_error(pel_folder, tmp_path):
    _, d = pel_folder
    for f in os.listdir(d):
        os.link(os.path.join(d, f), tmp_path / f)
    p = tmp_path / "chemistry-Arrhenius.dat"
    lines = open(os.path.join(d, "chemistry-Arrhenius.dat")).read().splitlines()
    del lines[10]                                          # one row short in zone 1
    os.unlink(p)
    p.write_text("\n".join(lines) + "\n")
    with pytest.raises(RuntimeError, match="ragged"):
        tables.read_folder_native(str(tmp_path))


def test_from_files_null_arguments():
    L = native.lib()
    assert L.flint_tables_read(None, None, None) == 1
    assert L.flint_mech_create_from_files(b"/nonexistent-folder", None, None) == 1


def test_native_reader_on_reference_wd_files(tmp_path):
    """FLINT's own WD input, rebuilt in the reference's exact text formats from
    the committed fixtures (phase.txt and chemistry-info.txt verbatim; the rows
    T = 999-1001 K of each chemistry-Arrhenius.dat zone as the file prints
    them): the library's reader returns the reference's rate constants, kf at
    1000 K = 1.798555407738E+01 and 2.851560446681E+03 for reactions 1 and 2.
    thermo.dat is missing from the reference tree, so a flat one stands in."""
    info = json.load(open(os.path.join(GOLD, "wd_info.json")))
    arr = json.load(open(os.path.join(GOLD, "wd_arrhenius.json")))
    (tmp_path / "phase.txt").write_text(
        "ideal-gas phase\n" + "".join(f"{k} {v:.6f}\n" for k, v in info["phase"].items()))
    (tmp_path / "chemistry-info.txt").write_text("\n".join(info["info_lines"]) + "\n")
    lines = ['TITLE = "Arrhenius data"', 'VARIABLES = "Temperature", "kf", "kb"']
    for z in arr["zones"]:
        rows = [r for r in z["rows"] if 999.0 <= r[0] <= 1001.0]
        assert [r[0] for r in rows] == [999.0, 1000.0, 1001.0]
        lines += [f'ZONE T="{z["zone"]}"', f"I={len(rows)}, F=POINT"]
        lines += [f"{r[0]:12.3f}   {r[1]:.12E}   {r[2]:.12E}" for r in rows]
    (tmp_path / "chemistry-Arrhenius.dat").write_text("\n".join(lines) + "\n")
    names = list(info["phase"])
    T = np.array([999.0, 1000.0, 1001.0])
    tables._write_zones(str(tmp_path / "thermo.dat"), "t", ["Temperature", "Cp", "Enthalpy", "Entropy", "dCp"],
                        [(n, [np.full(3, 1000.0), np.zeros(3), np.ones(3), np.zeros(3)]) for n in names], T)
    t = tables.read_folder_native(str(tmp_path))
    assert t["ns"] == 5 and t["names"] == names and t["nr_arrh"] == 3
    np.testing.assert_array_equal(t["wm"], list(info["phase"].values()))
    assert (t["ti1"], t["ti2"]) == (999, 1001)
    assert t["kf_tab"][0, 1] == 1.798555407738E+01 and t["kf_tab"][1, 1] == 2.851560446681E+03
    assert t["ni1_arrh"][0, names.index("CH4")] == 1.0 and t["ni1_arrh"][0, names.index("O2")] == 1.5
    _same(t, tables.read_folder(str(tmp_path)))


def test_native_reader_on_reference_pelucchi_files(tmp_path):
    """The reference's Pelucchi falloff and thermo files in their exact text
    formats (rows T = 999-1001 K of chemistry-Troe.dat, chemistry-Lindemann.dat
    and thermo.dat from the committed fixtures, headers as the files print
    them; phase.txt, chemistry-info.txt and the Arrhenius table written by this
    package for the same mechanism): the library's reader returns the
    reference's numbers, digit for digit."""
    m = Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json"))
    tables.write_folder(tables.generate(m, 999, 1001), str(tmp_path))

    def zones(fname):
        return [(z["zone"], [r for r in z["rows"] if 999.0 <= r[0] <= 1001.0])
                for z in json.load(open(os.path.join(GOLD, fname)))["zones"]]

    def rate_file(path, title, cols, zs):
        out = [f'TITLE = "{title}"', "VARIABLES = " + ", ".join(f'"{c}"' for c in cols)]
        for name, rows in zs:
            out += [f'ZONE T="{name}"', f"I={len(rows)}, F=POINT"]
            out += [f"{r[0]:12.3f}" + "".join(f"{v:21.12E}" for v in r[1:]) for r in rows]
        path.write_text("\n".join(out) + "\n")
    troe, lind, thermo = zones("pelucchi_troe.json"), zones("pelucchi_lind.json"), zones("pelucchi_thermo.json")
    rate_file(tmp_path / "chemistry-Troe.dat", "Fall-off Troe data",
              ["Temperature", "k_inf", "k_0", "k_c", "F_cent"], troe)
    rate_file(tmp_path / "chemistry-Lindemann.dat", "Fall-off Lindemann data",
              ["Temperature", "k_inf", "k_0", "k_c"], lind)
    out = ['TITLE = "Mass Thermodynamic Properties"',
           'VARIABLES = "Temperature", "Cp", "Enthalpy", "Entropy", "dCp"']
    for name, rows in thermo:
        out += [f'ZONE T="{name}"', f"I={len(rows)}, F=POINT"]
        out += [f"{r[0]:.1f} " + " ".join(f"{v:.6f}" for v in r[1:]) for r in rows]
    (tmp_path / "thermo.dat").write_text("\n".join(out) + "\n")
    t = tables.read_folder_native(str(tmp_path))
    assert (t["nr_troe"], t["nr_lind"], t["tmin"], t["tmax"]) == (2, 4, 999, 1001)
    for j, (_, rows) in enumerate(troe):
        for c, key in enumerate(("kinf_troe", "k0_troe", "kc_troe", "fcent_troe")):
            assert list(t[key][j]) == [r[1 + c] for r in rows], key
    for j, (_, rows) in enumerate(lind):
        for c, key in enumerate(("kinf_lind", "k0_lind", "kc_lind")):
            assert list(t[key][j]) == [r[1 + c] for r in rows], key
    for k, (_, rows) in enumerate(thermo):
        assert list(t["cp_tab"][k]) == [r[1] for r in rows] and list(t["h_tab"][k]) == [r[2] for r in rows]
    _same(t, tables.read_folder(str(tmp_path)))
