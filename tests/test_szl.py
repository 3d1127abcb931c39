"""FLINT's SZL binary tables (.szplt): the readers and the oracle pins they give.

The reference ships its Troyes, TSR-Rich-31 and TSR-GP-24 tables only as SZL
binaries, which FLINT's loaders read when the ASCII .dat is absent
(src/lib/Load_Chemistry.f90:95-96, src/lib/Load_ThermoTransport.f90:57-60).
The values in them are float32, so the pins below hold to float32 rounding:
|oracle / table - 1| <= 1.2e-7 (two half-units of float32's last place).

* the Python reader (tables.read_szplt) and the library's native reader
  (flint_tables_read) return the same arrays, bit for bit, on files written by
  tables.write_szplt in float32 and float64, and refuse truncated files;
* Troyes chemistry-Arrhenius.szplt: kf of its 17 elementary and three-body
  reactions and kb = kf / Kc of the reversible ones -- a pin of the Gibbs ->
  Kc path on elementary reactions;
* TSR-Rich-31 and TSR-GP-24 chemistry-Troe.szplt: k_inf, k_0, k_c and F_cent;
* Troyes and TSR-Rich-31 thermo.szplt: mass-specific cp, h, s.
The sampled rows in tests/golden/*_szl.json come from
tests/golden/make_golden.py (its own decode of the files, checked there
against tables.read_szplt).
"""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

from flint_gb300 import mechgen, tables
from flint_gb300.mech import Mechanism
from oracle.oracle import Oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")
F32_BAR = 1.2e-7


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def _mech(name):
    return Mechanism.load(os.path.join(GOLD, name))


# ------------------------------------------------------------------ readers
def _szl_folder(tmp_path, dtype):
    """A complete table folder with every table as .szplt (no .dat)."""
    mech = mechgen.load("c2")
    tables.write_folder(tables.generate(mech, 300, 1200), str(tmp_path))
    t = tables.read_folder(str(tmp_path))   # the ASCII tables as printed
    for base in ("thermo", "chemistry-Arrhenius", "chemistry-Troe", "chemistry-Lindemann"):
        p = os.path.join(str(tmp_path), base + ".dat")
        if not os.path.exists(p):
            continue
        zones = tables.read_tecplot_points(p)
        with open(p) as f:
            names = re.findall(r'"([^"]*)"', [ln for ln in f if ln.startswith("VARIABLES")][0])
        tables.write_szplt(os.path.join(str(tmp_path), base + ".szplt"), base, names, zones, dtype=dtype)
        os.remove(p)
    return t


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_python_and_native_readers_agree(tmp_path, dtype):
    t_src = _szl_folder(tmp_path, dtype)
    a = tables.read_folder(str(tmp_path))
    b = tables.read_folder_native(str(tmp_path))
    assert a["nr_troe"] == t_src["nr_troe"] and a["nr_arrh"] == t_src["nr_arrh"]
    for k in ("tmin", "tmax", "ti1", "ti2", "ns", "nr_arrh", "nr_troe", "nr_lind"):
        assert a[k] == b[k], k
    for k in tables.ARRAYS:
        x = a.get(k)
        if x is None or np.asarray(x).size == 0:
            continue
        assert np.array_equal(np.asarray(x, dtype=np.float64), np.asarray(b[k], dtype=np.float64)), k
    # the values are those written (exactly, in float64; rounded once, in float32)
    cast = ((lambda v: np.asarray(np.clip(v, -1e36, 1e36), dtype=np.float32).astype(np.float64))
            if dtype == np.float32 else np.asarray)
    assert np.array_equal(a["kf_tab"], cast(t_src["kf_tab"]))
    assert np.array_equal(a["kc_troe"], cast(t_src["kc_troe"]))


def test_truncated_file_is_refused(tmp_path):
    _szl_folder(tmp_path, np.float32)
    p = os.path.join(str(tmp_path), "chemistry-Arrhenius.szplt")
    data = open(p, "rb").read()
    with open(p, "wb") as f:
        f.write(data[: len(data) // 2])
    with pytest.raises(ValueError):
        tables.read_szplt(p)
    from flint_gb300 import native
    L = native.lib()
    h = C.c_void_p()
    rc = L.flint_tables_read(os.fsencode(str(tmp_path)), b"", C.byref(h))
    assert rc != 0
    assert b"SZL" in L.flint_last_error()


# ------------------------------------------------------------- oracle pins
def test_troyes_arrhenius_kf_and_kb():
    """Troyes kf and kb = kf / Kc (NASA-7 Gibbs energies) against chemistry-Arrhenius.szplt."""
    mech = _mech("mech_troyes.json")
    orc = Oracle(mech)
    g = _load("troyes_arrhenius_szl.json")
    idx = [i for i, r in enumerate(mech.reactions) if r.rtype in (0, 1)]
    assert len(idx) == len(g["zones"]) == 17
    wf = wb = 0.0
    nkb = 0
    for z, r in zip(g["zones"], idx):
        for T, kf_ref, kb_ref in z["rows"]:
            kf, Kc, _, _ = (a[r] for a in orc.rate_constants(T))
            wf = max(wf, abs(kf / kf_ref - 1.0))
            if kb_ref > 0.0:
                wb = max(wb, abs(kf / Kc / kb_ref - 1.0))
                nkb += 1
    assert nkb > 100
    assert wf < F32_BAR and wb < F32_BAR, (wf, wb)


@pytest.mark.parametrize("mname,fname", [("mech_tsr_rich_31.json", "tsr_rich_31_troe_szl.json"),
                                         ("mech_tsr_gp_24.json", "tsr_gp_24_troe_szl.json")])
def test_troe_tables(mname, fname):
    """k_inf, k_0, Kc and F_cent of the Troe reactions (zone "ReactionN" = reaction N)."""
    mech = _mech(mname)
    orc = Oracle(mech)
    g = _load(fname)
    worst = np.zeros(4)
    for z in g["zones"]:
        r = int(re.findall(r"\d+", z["zone"])[0]) - 1
        assert mech.reactions[r].rtype == 3
        for T, ki, k0r, kc, fc in z["rows"]:
            kf, Kc, k0, fcent = (a[r] for a in orc.rate_constants(T))
            tiny = np.finfo(np.float32).tiny   # the file's float32 underflows below this
            e = [abs(kf / ki - 1.0) if ki > tiny else 0.0, abs(k0 / k0r - 1.0) if k0r > tiny else 0.0,
                 abs(Kc / kc - 1.0) if tiny < kc < 1e35 else 0.0,   # the generator caps k_c at 1e36
                 abs(fcent - fc) / abs(fc)]
            worst = np.maximum(worst, e)
    assert worst.max() < F32_BAR, worst


@pytest.mark.parametrize("mname,fname", [("mech_troyes.json", "troyes_thermo_szl.json"),
                                         ("mech_tsr_rich_31.json", "tsr_rich_31_thermo_szl.json")])
def test_thermo_tables(mname, fname):
    """Mass-specific cp, h, s from NASA-7 inside each species' range."""
    mech = _mech(mname)
    orc = Oracle(mech)
    g = _load(fname)
    R = mech.r_thermo
    names = [s.name for s in mech.species]
    worst = np.zeros(3)
    n = 0
    for z in g["zones"]:
        k = names.index(z["zone"])
        sp = mech.species[k]
        for row in z["rows"]:
            T = row[0]
            if not (sp.tlow <= T <= sp.thigh):
                continue
            cpR, hRT, sR, _ = orc.species_thermo(T)
            cp, h, s = cpR[k] * R / sp.mw, hRT[k] * R * T / sp.mw, sR[k] * R / sp.mw
            worst = np.maximum(worst, [abs(cp / row[1] - 1.0), abs(h - row[2]) / max(abs(row[2]), cp * T),
                                       abs(s / row[3] - 1.0)])
            n += 1
    assert n > 200
    assert worst.max() < F32_BAR, worst


def test_troyes_table_set_runs_the_general_loop():
    """The Troyes tables (read from the reference's .szplt files) drive the
    oracle's general loop: finite rates that conserve mass per cell."""
    from oracle.oracle import TableOracle
    t = troyes_tables()
    rng = np.random.default_rng(3)
    n = 64
    T = rng.uniform(300.0, 2900.0, n)
    Y = rng.dirichlet(np.full(t["ns"], 0.5), n)
    rho = rng.uniform(0.1, 5.0, n)
    w = TableOracle(t).general(rho[:, None] * Y, T)
    assert np.isfinite(w).all()
    assert np.abs(w.sum(1)).max() <= 1e-9 * np.abs(w).sum(1).max()


def troyes_tables():
    """The Troyes table set of tests/golden/troyes_tables_szl.npz as a table dict."""
    z = np.load(os.path.join(GOLD, "troyes_tables_szl.npz"))
    t = {k: z[k] for k in z.files}
    for k in ("ns", "tmin", "tmax", "ti1", "ti2"):
        t[k] = int(t[k])
    for k in ("cp_tab", "h_tab", "kf_tab", "kb_tab"):
        t[k] = t[k].astype(np.float64)
    t["names"] = [str(x) for x in t["names"]]
    t["nr_arrh"], t["nr_troe"], t["nr_lind"] = t["kf_tab"].shape[0], 0, 0
    for key in ("troe", "lind"):
        t[f"ni1_{key}"] = t[f"ni2_{key}"] = t[f"eps_{key}"] = np.zeros((0, t["ns"] + 1))
    t["runiv"] = tables.RUNIV_FLINT
    return t
