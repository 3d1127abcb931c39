"""Pin the FP64 oracle against the reference's own tables (tests/golden/).

The rate and thermo tables FLINT loads (chemistry-*.dat, thermo.dat) were
generated from the YAML mechanisms; the oracle recomputes them from the same
YAML parameters and must reproduce the printed digits.
"""
import json
import os

import numpy as np
import pytest

from flint_gb300.mech import Mechanism
from flint_gb300 import data_path
from oracle.oracle import Oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def pelucchi():
    return Oracle(Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json")))


def test_wd_arrhenius_table():
    """kf(T) of WD reactions 1-2: A T^b exp(-Ea/RT) with cm/mol -> m/kmol scaling."""
    orc = Oracle(Mechanism.load(data_path("mech_c1.json")))
    g = _load("wd_arrhenius.json")
    worst = 0.0
    for r in range(2):
        for row in g["zones"][r]["rows"]:
            T, kf_ref, kb_ref = row
            kf = orc.rate_constants(T)[0][r]
            assert kb_ref == 0.0  # irreversible
            if kf_ref == 0.0:
                assert kf < 1e-300 or T < 50
                continue
            worst = max(worst, abs(kf / kf_ref - 1.0))
    assert worst < 2e-12, worst


def _falloff_rows(pelucchi, fname, rtype):
    g = _load(fname)
    mech = pelucchi.mech
    idx = [i for i, r in enumerate(mech.reactions) if r.rtype == rtype]
    assert len(idx) == len(g["zones"])
    return g, idx


@pytest.mark.parametrize("fname,rtype", [("pelucchi_troe.json", 3), ("pelucchi_lind.json", 2)])
def test_pelucchi_falloff_tables(pelucchi, fname, rtype):
    """k_inf, k_0, Kc (Gibbs, NASA-7) and Troe F_cent against chemistry-{Troe,Lindemann}.dat."""
    g, idx = _falloff_rows(pelucchi, fname, rtype)
    worst = np.zeros(4)
    for z, r in zip(g["zones"], idx):
        for row in z["rows"]:
            T = row[0]
            kf, Kc, k0, fc = (a[r] for a in pelucchi.rate_constants(T))
            errs = [abs(kf / row[1] - 1), abs(k0 / row[2] - 1)]
            if row[3] < 1e299:  # the generator caps Kc at 1e300
                errs.append(abs(Kc / row[3] - 1))
            else:
                errs.append(0.0)
            if len(row) > 4:
                errs.append(abs(fc - row[4]) / max(abs(row[4]), 1e-300))
            else:
                errs.append(0.0)
            worst = np.maximum(worst, errs)
    assert worst.max() < 5e-12, worst


def test_pelucchi_thermo_table(pelucchi):
    """Mass-specific cp, h, s from NASA-7 against thermo.dat (10 printed digits)."""
    g = _load("pelucchi_thermo.json")
    mech = pelucchi.mech
    R = mech.r_thermo
    worst = np.zeros(3)
    for k, z in enumerate(g["zones"]):
        sp = mech.species[k]
        assert z["zone"] == sp.name
        for row in z["rows"]:
            T = row[0]
            if not (sp.tlow <= T <= sp.thigh):
                continue
            cpR, hRT, sR, _ = pelucchi.species_thermo(T)
            cp = cpR[k] * R / sp.mw
            h = hRT[k] * R * T / sp.mw
            s = sR[k] * R / sp.mw
            worst = np.maximum(worst, [abs(cp / row[1] - 1), abs(h - row[2]) / (cp * T), abs(s / row[3] - 1)])
    assert worst.max() < 1e-8, worst
