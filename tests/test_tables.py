"""FLINT's tabulated input: generator pinned to the reference tables, file
round trip, chemistry-info parsing, and the table path against the analytic one."""
import json
import os

import numpy as np
import pytest

from flint_gb300 import mechgen, tables
from flint_gb300.mech import Mechanism
from oracle.oracle import Oracle, TableOracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def pel():
    m = Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json"))
    return m, tables.generate(m, 1, 3000)


def test_generator_matches_reference_falloff_tables(pel):
    m, t = pel
    for fname, kind, cols in (("pelucchi_troe.json", "troe", ("kinf_troe", "k0_troe", "kc_troe", "fcent_troe")),
                              ("pelucchi_lind.json", "lind", ("kinf_lind", "k0_lind", "kc_lind"))):
        g = json.load(open(os.path.join(GOLD, fname)))
        for i, z in enumerate(g["zones"]):
            rows = np.array(z["rows"])
            ti = rows[:, 0].astype(int) - t["ti1"]
            for c, nm in enumerate(cols):
                ref, mine = rows[:, 1 + c], t[nm][i][ti]
                np.testing.assert_allclose(mine, ref, rtol=2e-12, atol=0)


def test_generator_matches_reference_thermo_table(pel):
    m, t = pel
    g = json.load(open(os.path.join(GOLD, "pelucchi_thermo.json")))
    for k, z in enumerate(g["zones"]):
        sp = m.species[k]
        rows = np.array([r for r in z["rows"] if sp.tlow <= r[0] <= sp.thigh])
        ti = rows[:, 0].astype(int) - t["tmin"]
        np.testing.assert_allclose(t["cp_tab"][k][ti], rows[:, 1], rtol=1e-8)
        np.testing.assert_allclose(t["h_tab"][k][ti], rows[:, 2], rtol=0, atol=1e-8 * np.abs(rows[:, 1] * rows[:, 0]).max())


def test_write_read_roundtrip(pel, tmp_path):
    m, t = pel
    tables.write_folder(t, str(tmp_path))
    t2 = tables.read_folder(str(tmp_path))
    assert t2["ns"] == t["ns"] and t2["nr_arrh"] == t["nr_arrh"] and t2["nr_troe"] == 2 and t2["nr_lind"] == 4
    assert t2["tmin"] == 0 and t2["tmax"] == 3000       # row 0 cloned (Tmin = 1)
    np.testing.assert_allclose(t2["cp_tab"][:, 1:], t["cp_tab"], rtol=1e-12)
    assert np.all(t2["h_tab"][:, 0] == 0.0)
    for k in ("kf_tab", "kb_tab", "kinf_troe", "kc_lind"):
        np.testing.assert_allclose(t2[k], t[k], rtol=1e-12, atol=1e-300)
    for k in ("ni1_arrh", "ni2_arrh", "ni1_troe", "eps_lind"):
        np.testing.assert_array_equal(t2[k], t[k])


def test_parse_reference_chemistry_info(tmp_path):
    """The reference's own WD chemistry-info.txt and phase.txt parse as read_chemistry does."""
    g = json.load(open(os.path.join(GOLD, "wd_info.json")))
    (tmp_path / "chemistry-info.txt").write_text("\n".join(g["info_lines"]) + "\n")
    (tmp_path / "phase.txt").write_text("ideal-gas phase\n" + "".join(f"{k} {v}\n" for k, v in g["phase"].items()))
    # minimal thermo / rate files so the reader runs end to end
    T = np.arange(1.0, 11.0)
    t0 = {"ns": 5, "names": list(g["phase"]), "wm": np.array(list(g["phase"].values())), "T": T,
          "cp_tab": np.ones((5, 10)), "h_tab": np.zeros((5, 10)), "s_tab": np.ones((5, 10)),
          "dcp_tab": np.zeros((5, 10)), "nr_arrh": 3, "nr_troe": 0, "nr_lind": 0,
          "kf_tab": np.ones((3, 10)), "kb_tab": np.zeros((3, 10)), "mech_name": "WD"}
    tables._write_zones(str(tmp_path / "thermo.dat"), "t", ["Temperature", "Cp", "Enthalpy", "Entropy", "dCp"],
                        [(n, [np.ones(10), np.zeros(10), np.ones(10), np.zeros(10)]) for n in t0["names"]], T)
    tables._write_zones(str(tmp_path / "chemistry-Arrhenius.dat"), "a", ["Temperature", "kf", "kb"],
                        [(f"Reaction {j + 1}", [np.ones(10), np.zeros(10)]) for j in range(3)], T)
    t = tables.read_folder(str(tmp_path))
    assert t["mech_name"] == "WD" and t["ns"] == 5 and t["nr_arrh"] == 3
    names = t["names"]
    # reaction 1: CH4 + 1.5 O2 -> CO + 2 H2O
    assert t["ni1_arrh"][0, names.index("CH4")] == 1.0 and t["ni1_arrh"][0, names.index("O2")] == 1.5
    assert t["ni2_arrh"][0, names.index("H2O")] == 2.0 and t["ni1_arrh"][0, 5] == 0.0
    assert t["ti1"] == 1 and t["ti2"] == 10


def test_table_path_consistent_with_analytic(pel):
    """general on the generated 1-K tables vs the analytic source terms: the
    difference is the linear-interpolation error (~1e-8 median)."""
    m, t = pel
    T, p, Y = mechgen.c2_states(2000, m, seed=5)
    W = np.array([s.mw for s in m.species])
    rho = p / (m.r_eos * T * (Y / W).sum(1))
    wg = TableOracle(t).general(rho[:, None] * Y, T)
    w, ws, _, _ = Oracle(m).wdot_batch(T, p, Y)
    err = np.abs(wg.ravel() - w) / (ws + 1e-300)
    assert np.median(err) < 1e-6 and err.max() < 1e-3
