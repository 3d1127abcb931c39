"""Generate the committed golden fixtures and mechanism data from the FLINT tree.

Run once in a container where the reference tree is mounted:

    python tests/golden/make_golden.py <path of the FLINT source tree>

It writes, from the reference's own input files only (nothing is computed here
except unit conversion of YAML rate parameters into the IR):

* tests/golden/wd_arrhenius.json   sampled rows of test/WD/INPUT/chemistry-Arrhenius.dat
* tests/golden/pelucchi_troe.json  sampled rows of test/Pelucchi/INPUT/chemistry-Troe.dat
* tests/golden/pelucchi_lind.json  sampled rows of test/Pelucchi/INPUT/chemistry-Lindemann.dat
* tests/golden/pelucchi_thermo.json sampled rows of test/Pelucchi/INPUT/thermo.dat
* tests/golden/mech_pelucchi.json  the Pelucchi YAML as a mechanism IR
* tests/golden/*_szl.json          sampled rows of the SZL binary tables (float32 values):
                                   Troyes chemistry-Arrhenius.szplt (kf, kb) and thermo.szplt,
                                   TSR-Rich-31 chemistry-Troe.szplt and thermo.szplt,
                                   TSR-GP-24 chemistry-Troe.szplt
* tests/golden/fortran_forms.json  the generated Fortran mechanism routines
                                   (src/lib/Lib_ChemMech/*.f90) parsed into their rate
                                   sources, concentration factors, third bodies and
                                   omegadot terms
* tests/golden/troyes_tables_szl.npz  the whole Troyes table set (phase.txt,
                                   chemistry-info.txt and the two .szplt tables, read by
                                   the library's reader), rows 280-3000 K
* tests/golden/wd_info.json        WD chemistry-info.txt stoichiometry + phase.txt
* tests/golden/mech_<name>.json    the other in-tree mechanisms (Ecker, Smooke, TSR-CDF-13,
                                   TSR-GP-24, TSR-Rich-31, Troyes, ZK, CORIA; WD and Cross
                                   with NASA-9 thermo) as IR
* flint_gb300/data/mech_c1.json    the 2-step CH4/air mechanism: WD reactions 1-2
                                   (test/WD/INPUT/WD.yaml) with NASA-7 data of CH4, O2,
                                   CO, CO2, H2O (TSR-Rich-31.yaml) and N2 (troyes.yaml),
                                   molar masses from the phase.txt files
* flint_gb300/data/chon_species.json  names + compositions of the C/H/O/N species in
                                   the in-tree YAML files (species pool of the
                                   synthetic mechanisms)

The GPU machine never reads the reference tree; it reads these files.
"""
from __future__ import annotations

import glob
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from flint_gb300 import mech as M  # noqa: E402
from flint_gb300 import yamlsub  # noqa: E402


def read_tecplot_points(path):
    """Tecplot ASCII POINT zones -> list of (zone title, rows ndarray)."""
    zones, cur = [], None
    with open(path) as f:
        for ln in f:
            s = ln.strip()
            if s.startswith("ZONE"):
                cur = [s.split('"')[1], []]
                zones.append(cur)
            elif s and cur is not None and (s[0].isdigit() or s[0] in "+-."):
                cur[1].append([float(x) for x in s.split()])
    return [(z, np.array(r)) for z, r in zones]


def szl_zones(path):
    """Ordered 1-D zones of an SZL binary (.szplt) -> list of (title, rows).

    A decode of its own, independent of flint_gb300.tables.read_szplt: the file
    header's tag table (offset at byte 42) gives the zone count (tag 1), the
    variable count (2), zone titles (0x100), zone-header offsets (0x102), the
    I extent per zone (0x107) and the data type per zone and variable (0x302,
    1 = float32, 2 = float64); each zone header's tag 0x600 points at the
    offsets of its variables' contiguous value arrays."""
    import struct
    d = open(path, "rb").read()
    assert d[:7] == b"#!SZPLT" and d[34:42] == bytes([8, 7, 6, 5, 4, 3, 2, 1])

    def table(o):
        n = struct.unpack_from("<H", d, o)[0]
        return dict(zip(struct.unpack_from(f"<{n}H", d, o + 2), struct.unpack_from(f"<{n}Q", d, o + 2 + 2 * n)))

    H = table(struct.unpack_from("<Q", d, 42)[0])
    nz, nv = H[1], H[2]
    ln = struct.unpack_from("<Q", d, H[0x100])[0]
    titles = d[H[0x100] + 8:H[0x100] + 8 + ln].decode().split("\r")[:nz]
    out = []
    for z in range(nz):
        I = struct.unpack_from("<Q", d, H[0x107] + 8 * z)[0]
        Z = table(struct.unpack_from("<Q", d, H[0x102] + 8 * z)[0])
        cols = []
        for v in range(nv):
            off = struct.unpack_from("<Q", d, Z[0x600] + 8 * v)[0]
            dt = {1: "<f4", 2: "<f8"}[d[H[0x302] + z * nv + v]]
            cols.append(np.frombuffer(d, dtype=dt, count=I, offset=off).astype(np.float64))
        out.append((titles[z], np.stack(cols, axis=1)))
    return out


# the generated Fortran mechanism routines (utils/YTF.py's output form) and the
# IR fixture of the same mechanism
FORTRAN_FORMS = [("TSR-CDF-13.f90", "mech_tsr_cdf_13.json"), ("TSR-GP-24.f90", "mech_tsr_gp_24.json"),
                 ("TSR-Rich-31.f90", "mech_tsr_rich_31.json"), ("ZK.f90", "mech_zk.json"),
                 ("coria.f90", "mech_coria.json"), ("cross.f90", "mech_cross.json"),
                 ("ecker.f90", "mech_ecker.json"), ("pelucchi.f90", "mech_pelucchi.json"),
                 ("smooke.f90", "mech_smooke.json"), ("troyes.f90", "mech_troyes.json")]


def parse_fortran_form(path):
    """One generated mechanism routine (src/lib/Lib_ChemMech/*.f90) as data.

    Per reaction, in the routine's order: the rate source ("arrh" f_kf/f_kb
    row a, "troe" / "lind" f_k_troe / f_k_lindemann row a, 1-based), the
    species of each concentration factor of prodf and prodb (0-based, repeated
    for powers), whether prodf/prodb carry the third body M, and M itself as
    {species: efficiency} ("sum" = every species with 1); per species the
    omegadot terms [reaction, nu_product, nu_reactant].  The concentration
    clamp of the routine's first loop, if any, is recorded as written."""
    import re
    lines = open(path).read().splitlines()
    rx, cur_M, cur_k = {}, None, None
    omega = {}
    clamp = None
    for ln in lines:
        s = ln.split("!")[0].strip().replace(" ", "")
        if not s:
            continue
        if s.startswith("roi(is)=max(roi(is),0"):
            clamp = "roi = max(roi, 0)"
        m = re.match(r"M=(.*)$", s)
        if m:
            e = m.group(1)
            if e.startswith("sum("):
                cur_M = "sum"
            else:
                cur_M = {}
                for term in e.split("+"):
                    t = re.match(r"coi\((\d+)\)(?:\*([0-9.eEdD+-]+))?$", term)
                    assert t, (path, term)
                    cur_M[int(t.group(1)) - 1] = float((t.group(2) or "1").replace("d", "e").replace("D", "e"))
            continue
        m = re.match(r"k=f_k_(troe|lindemann)\((\d+),", s)
        if m:
            cur_k = ("troe" if m.group(1) == "troe" else "lind", int(m.group(2)))
            continue
        m = re.match(r"prod([fb])\((\d+)\)=(.*)$", s)
        if m:
            side, r, e = m.group(1), int(m.group(2)) - 1, m.group(3)
            d = rx.setdefault(r, {})
            src = re.match(r"f_k([fb])\((\d+),", e)
            if src:
                d["kind"], d["table_index"] = "arrh", int(src.group(2))
            else:
                assert e.startswith(f"k({1 if side == 'f' else 2})"), (path, e)
                d["kind"], d["table_index"] = cur_k
            d["fwd" if side == "f" else "bwd"] = sorted(int(x) - 1 for x in re.findall(r"coi\((\d+)\)", e))
            d["M" + side] = e.endswith("*M")
            if e.endswith("*M") or d["kind"] != "arrh":
                d["M"] = cur_M
            continue
        m = re.match(r"omegadot\((\d+)\)=(.*)$", s)
        if m:
            k, e = int(m.group(1)) - 1, m.group(2)
            omega[k] = [[int(r) - 1, float(a), float(b)] for a, b, r in
                        re.findall(r"\(([0-9.]+)-([0-9.]+)\)\*\(prodf\((\d+)\)", e)]
    n = max(rx) + 1
    assert sorted(rx) == list(range(n)), path
    return {"reactions": [rx[r] for r in range(n)], "omegadot": [omega.get(k, []) for k in range(max(omega) + 1)],
            "clamp": clamp}


def sample_rows(rows, temps):
    out = []
    for T in temps:
        i = int(round(T - rows[0, 0]))
        assert rows[i, 0] == T, (T, rows[i, 0])
        out.append(rows[i].tolist())
    return out


# the reference's in-tree mechanisms (WD and Cross with NASA-9 thermo)
INTREE = [("Ecker", "ecker.yaml"), ("Smooke", "smooke.yaml"), ("TSR-CDF-13", "TSR-CDF-13.yaml"),
          ("TSR-GP-24", "TSR-GP-24.yaml"), ("TSR-Rich-31", "TSR-Rich-31.yaml"), ("Troyes", "troyes.yaml"),
          ("ZK", "ZK.yaml"), ("CORIA", "coria.yaml"), ("WD", "WD.yaml"), ("Cross", "cross.yaml")]


def main(ref):
    test = os.path.join(ref, "test")
    gold = HERE
    data = os.path.join(REPO, "flint_gb300", "data")
    os.makedirs(data, exist_ok=True)

    # ---- WD rate table (kf, kb per reaction; T = 1..15000) -------------------
    wd = read_tecplot_points(os.path.join(test, "WD/INPUT/chemistry-Arrhenius.dat"))
    temps = sorted(set([300.0, 500.0, 999.0, 1000.0, 1001.0, 1500.0, 2000.0, 2500.0, 3000.0, 5000.0]
                       + [float(t) for t in range(250, 3001, 125)]))
    json.dump({"source": "test/WD/INPUT/chemistry-Arrhenius.dat",
               "columns": ["T", "kf", "kb"],
               "zones": [{"zone": z, "rows": sample_rows(r, temps)} for z, r in wd]},
              open(os.path.join(gold, "wd_arrhenius.json"), "w"), indent=0)

    # ---- Pelucchi falloff + thermo tables ------------------------------------
    P = os.path.join(test, "Pelucchi/INPUT")
    temps_p = sorted(set([float(t) for t in range(300, 3000, 97)] + [999.0, 1000.0, 1001.0, 2999.0]))
    for fname, key, cols in (("chemistry-Troe.dat", "pelucchi_troe", ["T", "k_inf", "k_0", "k_c", "F_cent"]),
                             ("chemistry-Lindemann.dat", "pelucchi_lind", ["T", "k_inf", "k_0", "k_c"])):
        zs = read_tecplot_points(os.path.join(P, fname))
        json.dump({"source": "test/Pelucchi/INPUT/" + fname, "columns": cols,
                   "zones": [{"zone": z, "rows": sample_rows(r, temps_p)} for z, r in zs]},
                  open(os.path.join(gold, key + ".json"), "w"), indent=0)
    zs = read_tecplot_points(os.path.join(P, "thermo.dat"))
    json.dump({"source": "test/Pelucchi/INPUT/thermo.dat", "columns": ["T", "Cp", "Enthalpy", "Entropy", "dCp"],
               "zones": [{"zone": z, "rows": sample_rows(r, temps_p)} for z, r in zs]},
              open(os.path.join(gold, "pelucchi_thermo.json"), "w"), indent=0)
    mp = M.from_yaml(os.path.join(P, "pelucchi.yaml"), phase_mw=M.read_phase_txt(os.path.join(P, "phase.txt")))
    with open(os.path.join(gold, "mech_pelucchi.json"), "w") as f:
        f.write(mp.to_json())

    # ---- WD chemistry-info (general-loop stoichiometry) ----------------------
    info = open(os.path.join(test, "WD/INPUT/chemistry-info.txt")).read().splitlines()
    json.dump({"source": "test/WD/INPUT/chemistry-info.txt + phase.txt",
               "info_lines": info,
               "phase": M.read_phase_txt(os.path.join(test, "WD/INPUT/phase.txt"))},
              open(os.path.join(gold, "wd_info.json"), "w"), indent=0)

    # ---- SZL binary tables (Troyes, TSR-Rich-31, TSR-GP-24) --------------------
    # sampled rows for the oracle pins, checked against the library's reader
    from flint_gb300 import tables as TB
    temps_s = sorted(set([float(t) for t in range(300, 3501, 89)] + [500.0, 999.0, 1000.0, 1001.0, 2500.0]))
    szl = [("Troyes/INPUT/chemistry-Arrhenius.szplt", "troyes_arrhenius_szl", ["T", "kf", "kb"]),
           ("Troyes/INPUT/thermo.szplt", "troyes_thermo_szl", ["T", "Cp", "Enthalpy", "Entropy", "dCp"]),
           ("TSR-Rich-31/INPUT/chemistry-Troe.szplt", "tsr_rich_31_troe_szl", ["T", "k_inf", "k_0", "k_c", "F_cent"]),
           ("TSR-Rich-31/INPUT/thermo.szplt", "tsr_rich_31_thermo_szl", ["T", "Cp", "Enthalpy", "Entropy", "dCp"]),
           ("TSR-GP-24/INPUT/chemistry-Troe.szplt", "tsr_gp_24_troe_szl", ["T", "k_inf", "k_0", "k_c", "F_cent"])]
    for rel, key, cols in szl:
        zs = szl_zones(os.path.join(test, rel))
        mine = TB.read_szplt(os.path.join(test, rel))
        assert [z for z, _ in zs] == [z for z, _ in mine]
        assert all(np.array_equal(a, b) for (_, a), (_, b) in zip(zs, mine)), rel
        json.dump({"source": "test/" + rel + " (float32 values)", "columns": cols, "rows_per_zone": int(zs[0][1].shape[0]),
                   "first_T": zs[0][1][0, 0],
                   "zones": [{"zone": z, "rows": sample_rows(r, [t for t in temps_s if r[0, 0] <= t <= r[-1, 0]])}
                             for z, r in zs]},
                  open(os.path.join(gold, key + ".json"), "w"), indent=0)
    # the complete Troyes table set, read from the reference's own files
    # (phase.txt, chemistry-info.txt, chemistry-Arrhenius.szplt, thermo.szplt)
    # by the library's reader, rows 280-3000 K, for the GPU general-loop test
    t = TB.read_folder(os.path.join(test, "Troyes/INPUT"))
    lo, hi = 280, 3000
    keep = {"ns": t["ns"], "names": np.array(t["names"]), "wm": t["wm"], "tmin": lo, "tmax": hi, "ti1": lo, "ti2": hi,
            "cp_tab": t["cp_tab"][:, lo - t["tmin"]:hi - t["tmin"] + 1].astype(np.float32),
            "h_tab": t["h_tab"][:, lo - t["tmin"]:hi - t["tmin"] + 1].astype(np.float32),
            "kf_tab": t["kf_tab"][:, lo - t["ti1"]:hi - t["ti1"] + 1].astype(np.float32),
            "kb_tab": t["kb_tab"][:, lo - t["ti1"]:hi - t["ti1"] + 1].astype(np.float32),
            "ni1_arrh": t["ni1_arrh"], "ni2_arrh": t["ni2_arrh"], "eps_arrh": t["eps_arrh"]}
    for k in ("cp_tab", "h_tab", "kf_tab", "kb_tab"):   # float32 in the files: the cast is exact
        src = t[k][:, lo - (t["tmin"] if k in ("cp_tab", "h_tab") else t["ti1"]):][:, :hi - lo + 1]
        assert np.array_equal(keep[k].astype(np.float64), src), k
    np.savez_compressed(os.path.join(gold, "troyes_tables_szl.npz"), **keep)

    # ---- the generated Fortran mechanism routines ------------------------------
    forms = {}
    for fname, mname in FORTRAN_FORMS:
        f = parse_fortran_form(os.path.join(ref, "src/lib/Lib_ChemMech", fname))
        f.update({"source": "src/lib/Lib_ChemMech/" + fname, "mechanism": mname})
        forms[os.path.splitext(fname)[0]] = f
    json.dump(forms, open(os.path.join(gold, "fortran_forms.json"), "w"), indent=0)

    # ---- C1 mechanism ---------------------------------------------------------
    rich = yamlsub.load(os.path.join(test, "TSR-Rich-31/INPUT/TSR-Rich-31.yaml"))
    troy = yamlsub.load(os.path.join(test, "Troyes/INPUT/troyes.yaml"))
    wdy = yamlsub.load(os.path.join(test, "WD/INPUT/WD.yaml"))
    mw = M.read_phase_txt(os.path.join(test, "WD/INPUT/phase.txt"))
    mw.update({"N2": M.read_phase_txt(os.path.join(P, "phase.txt"))["N2"]})
    spd = {s["name"]: s for s in rich["species"]}
    spd["N2"] = [s for s in troy["species"] if s["name"] == "N2"][0]
    names = ["CH4", "O2", "CO", "CO2", "H2O", "N2"]
    species = []
    for n in names:
        th = spd[n]["thermo"]
        tr = th["temperature-ranges"]
        species.append(M.Species(n, mw[n], dict(spd[n]["composition"]), float(tr[0]), float(tr[1]),
                                 float(tr[2]), [float(x) for x in th["data"][0]],
                                 [float(x) for x in th["data"][1]]))
    # WD reactions 1-2 with the IR unit conversion of from_yaml
    conc_f, eaf = M._unit_factors(wdy["units"])
    reactions = []
    for r in wdy["reactions"][:2]:
        eq = r["equation"]
        lhs, arrow, rhs = M._ARROW_RE.split(eq)
        reac, _, _ = M._parse_side(lhs)
        prod, _, _ = M._parse_side(rhs)
        orders = {k: float(v) for k, v in r["orders"].items()}
        forder = sum(orders.get(k, v) for k, v in reac.items())
        A, b, E = M._rate(r["rate-constant"], conc_f, eaf, forder)
        # WD.f90:31-34 writes the orders as default-real (single precision)
        # literals, coi(1)**0.70: the compiled exponent is float32(0.70).
        orders = {k: float(np.float32(v)) for k, v in orders.items()}
        reactions.append(M.Reaction(eq, M.TYPE_ELEMENTARY, reac, prod, orders, arrow != "=>", A, b, E))
    c1 = M.Mechanism("CH4-air-2step", species, reactions, ["C", "H", "O", "N"])
    with open(os.path.join(data, "mech_c1.json"), "w") as f:
        f.write(c1.to_json())

    # ---- C/H/O/N species pool -------------------------------------------------
    pool = {}
    for fy in sorted(glob.glob(os.path.join(test, "*/INPUT/*.yaml"))):
        d = yamlsub.load(fy)
        for s in d["species"]:
            comp = s["composition"]
            if set(comp) <= {"C", "H", "O", "N"} and s["name"] not in pool:
                pool[s["name"]] = {k: int(v) for k, v in comp.items()}
    order = [s for s in rich["phases"][0]["species"]] + sorted(k for k in pool if k not in rich["phases"][0]["species"])
    json.dump({"source": "C/H/O/N species of test/*/INPUT/*.yaml (TSR-Rich-31 order first)",
               "species": [{"name": n, "composition": pool[n]} for n in order]},
              open(os.path.join(data, "chon_species.json"), "w"), indent=1)
    # ---- in-tree mechanisms with NASA-7 thermo, as IR -------------------------
    for sub, yname in INTREE:
        d = os.path.join(test, sub, "INPUT")
        mi = M.from_yaml(os.path.join(d, yname), phase_mw=M.read_phase_txt(os.path.join(d, "phase.txt")))
        with open(os.path.join(gold, "mech_" + os.path.splitext(yname)[0].lower().replace("-", "_") + ".json"),
                  "w") as f:
            f.write(mi.to_json())
    print("wrote fixtures")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the FLINT source tree>")
    main(sys.argv[1])
