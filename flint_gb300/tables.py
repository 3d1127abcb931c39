"""FLINT's tabulated mechanism files: reader, generator and the GPU handle.

FLINT's loaders fill module arrays from plain-text files (paths within the
FLINT project):

* ``phase.txt``  header line, then ``NAME MW`` per species
  (read_idealgas_thermo, src/lib/Load_ThermoTransport.f90:37-54);
* ``thermo.dat`` Tecplot ASCII POINT zones, one per species, columns
  T, Cp, Enthalpy, Entropy, dCp in mass units (:57-85; row 0 cloned when Tmin=1);
* ``chemistry-info.txt`` name, reaction count, one type line per reaction and
  ``ns+1`` stoichiometry rows ``idx name ni1 ni2 eps`` per reaction, the last
  row being the third body "M" (read_chemistry, src/lib/Load_Chemistry.f90:26-91);
* ``chemistry-Arrhenius.dat`` zones of (T, kf, kb), ``chemistry-Troe.dat``
  zones of (T, k_inf, k_0, k_c, F_cent), ``chemistry-Lindemann.dat`` zones of
  (T, k_inf, k_0, k_c) (:93-162).

``read_folder`` parses these files into the arrays ``flint_table_desc``
points at; ``write_folder`` is the table generator FLINT's input.ini refers to
(tables on a 1-K grid from a NASA-7 / Arrhenius mechanism); ``Tables`` is the
GPU handle running FLINT's ``general`` loop and ``rhs_native`` on them.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import native
from .native import TableDesc
from .mech import Mechanism, TYPE_ELEMENTARY, TYPE_THREEBODY, TYPE_LINDEMANN, TYPE_TROE

RUNIV_FLINT = 8314.51
KC_CAP = 1e300   # the reference tables cap k_c at 1e300 (test/Pelucchi/INPUT/chemistry-Troe.dat)

_dp = C.POINTER(C.c_double)


ARRAYS = ("wm", "cp_tab", "h_tab", "kf_tab", "kb_tab", "kinf_troe", "k0_troe", "kc_troe", "fcent_troe",
          "kinf_lind", "k0_lind", "kc_lind", "ni1_arrh", "ni2_arrh", "eps_arrh", "ni1_troe", "ni2_troe",
          "eps_troe", "ni1_lind", "ni2_lind", "eps_lind", "mi_tab", "k_tab")


def table_desc(t):
    """ctypes TableDesc over a table dict (arrays (ncol, nrow) C-contiguous = Fortran (nrow, ncol))."""
    keep = {}
    d = TableDesc()
    d.ns, d.nr_arrh, d.nr_troe, d.nr_lind = t["ns"], t["nr_arrh"], t["nr_troe"], t["nr_lind"]
    d.tmin, d.tmax, d.ti1, d.ti2 = t["tmin"], t["tmax"], t["ti1"], t["ti2"]
    for name in ARRAYS:
        a = t.get(name)
        if a is None or a.size == 0:
            setattr(d, name, None)
            continue
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep[name] = a
        setattr(d, name, a.ctypes.data_as(_dp))
    d.runiv = float(t.get("runiv", RUNIV_FLINT))
    return d, keep


# ---------------------------------------------------------------- generator
def _nasa(sp, T):
    if sp.nasa9:
        rng = sp.nasa9
        idx = np.zeros(T.size, dtype=int)
        for i, r in enumerate(rng[:-1]):
            idx += (T > r[1]).astype(int)
        a = np.array([r[2:11] for r in rng])[idx]
        iT = 1.0 / T
        cpR = a[:, 0] * iT ** 2 + a[:, 1] * iT + a[:, 2] + a[:, 3] * T + a[:, 4] * T ** 2 + a[:, 5] * T ** 3 + a[:, 6] * T ** 4
        hRT = (-a[:, 0] * iT ** 2 + a[:, 1] * np.log(T) * iT + a[:, 2] + a[:, 3] * T / 2 + a[:, 4] * T ** 2 / 3
               + a[:, 5] * T ** 3 / 4 + a[:, 6] * T ** 4 / 5 + a[:, 7] * iT)
        sR = (-a[:, 0] * iT ** 2 / 2 - a[:, 1] * iT + a[:, 2] * np.log(T) + a[:, 3] * T + a[:, 4] * T ** 2 / 2
              + a[:, 5] * T ** 3 / 3 + a[:, 6] * T ** 4 / 4 + a[:, 8])
        dcpR = (-2 * a[:, 0] * iT ** 3 - a[:, 1] * iT ** 2 + a[:, 3] + 2 * a[:, 4] * T + 3 * a[:, 5] * T ** 2
                + 4 * a[:, 6] * T ** 3)
        return cpR, hRT, sR, dcpR
    a = np.where((T <= sp.tmid)[:, None], np.array(sp.low)[None, :], np.array(sp.high)[None, :])
    cpR = a[:, 0] + a[:, 1] * T + a[:, 2] * T ** 2 + a[:, 3] * T ** 3 + a[:, 4] * T ** 4
    hRT = a[:, 0] + a[:, 1] * T / 2 + a[:, 2] * T ** 2 / 3 + a[:, 3] * T ** 3 / 4 + a[:, 4] * T ** 4 / 5 + a[:, 5] / T
    sR = a[:, 0] * np.log(T) + a[:, 1] * T + a[:, 2] * T ** 2 / 2 + a[:, 3] * T ** 3 / 3 + a[:, 4] * T ** 4 / 4 + a[:, 6]
    dcpR = a[:, 1] + 2 * a[:, 2] * T + 3 * a[:, 3] * T ** 2 + 4 * a[:, 4] * T ** 3
    return cpR, hRT, sR, dcpR


def generate(mech: Mechanism, tmin=1, tmax=3000):
    """Tabulate a NASA-7 / Arrhenius mechanism on FLINT's 1-K grid (rows tmin..tmax).

    Arrhenius zones hold elementary and three-body reactions (kf includes the
    third-body units, kb = kf / Kc or 0), falloff reactions go to the Troe or
    Lindemann zones; k_c is capped at 1e300 as the reference tables are.
    """
    ns = mech.ns
    T = np.arange(tmin, tmax + 1, dtype=np.float64)
    R = mech.r_thermo
    cp = np.zeros((ns, T.size)); h = np.zeros((ns, T.size)); s = np.zeros((ns, T.size)); dcp = np.zeros((ns, T.size))
    gRT = np.zeros((ns, T.size))
    for k, sp in enumerate(mech.species):
        cpR, hRT, sR, dcpR = _nasa(sp, T)
        cp[k] = cpR * R / sp.mw
        h[k] = hRT * R * T / sp.mw
        s[k] = sR * R / sp.mw
        dcp[k] = dcpR * R / sp.mw
        gRT[k] = hRT - sR
    lnT = np.log(T)
    idx = {sp.name: i for i, sp in enumerate(mech.species)}

    def kc_of(r):
        dG = np.zeros_like(T); dn = 0.0
        for n_, nu in r.products.items():
            dG += nu * gRT[idx[n_]]; dn += nu
        for n_, nu in r.reactants.items():
            dG -= nu * gRT[idx[n_]]; dn -= nu
        with np.errstate(over="ignore"):
            kc = np.exp(-dG + dn * np.log(mech.p_ref / (R * T)))
        return np.minimum(kc, KC_CAP)

    def stoich(r, tb):
        n1 = np.zeros(ns + 1); n2 = np.zeros(ns + 1); ep = np.zeros(ns + 1)
        for n_, nu in r.reactants.items():
            n1[idx[n_]] = nu
        for n_, nu in r.products.items():
            n2[idx[n_]] = nu
        if tb:
            n1[ns] = 1.0
            n2[ns] = 1.0
            if r.collider is not None:
                ep[idx[r.collider]] = 1.0
            else:
                ep[:ns] = r.default_eff
                for n_, e in (r.efficiencies or {}).items():
                    ep[idx[n_]] = e
        return n1, n2, ep

    def cap(x):   # the generator's tables hold finite numbers only (|x| <= 1e300)
        return np.clip(np.nan_to_num(x, nan=0.0, posinf=KC_CAP, neginf=-KC_CAP), -KC_CAP, KC_CAP)

    arr, troe, lind = [], [], []
    old = np.seterr(over="ignore", divide="ignore", invalid="ignore")
    for r in mech.reactions:
        kf = cap(r.A * np.exp(r.b * lnT - r.EaR / T))
        if r.rtype in (TYPE_ELEMENTARY, TYPE_THREEBODY):
            kb = cap(kf / kc_of(r)) if r.reversible else np.zeros_like(T)
            arr.append((r, kf, kb))
        else:
            k0 = cap(r.A0 * np.exp(r.b0 * lnT - r.EaR0 / T))
            kc = kc_of(r) if r.reversible else np.full_like(T, KC_CAP)
            if r.rtype == TYPE_TROE:
                a, T3, T1, T2 = (list(r.troe) + [0.0] * 4)[:4]
                fc = (1 - a) * np.exp(-T / T3) + a * np.exp(-T / T1) + (np.exp(-T2 / T) if T2 else 0.0)
                troe.append((r, kf, k0, kc, fc))
            else:
                lind.append((r, kf, k0, kc))
    np.seterr(**old)
    out = {"ns": ns, "tmin": int(tmin), "tmax": int(tmax), "ti1": int(tmin), "ti2": int(tmax),
           "names": [sp.name for sp in mech.species], "wm": np.array([sp.mw for sp in mech.species]),
           "cp_tab": cp, "h_tab": h, "s_tab": s, "dcp_tab": dcp, "T": T, "runiv": RUNIV_FLINT,
           "nr_arrh": len(arr), "nr_troe": len(troe), "nr_lind": len(lind), "mech_name": mech.name,
           "rxn_kinds": []}
    for key, lst, cols in (("arrh", arr, 2), ("troe", troe, 4), ("lind", lind, 3)):
        st = [stoich(x[0], x[0].rtype != TYPE_ELEMENTARY) for x in lst]
        out[f"ni1_{key}"] = np.array([a for a, _, _ in st]).reshape(len(lst), ns + 1)
        out[f"ni2_{key}"] = np.array([b for _, b, _ in st]).reshape(len(lst), ns + 1)
        out[f"eps_{key}"] = np.array([c for _, _, c in st]).reshape(len(lst), ns + 1)
    out["kf_tab"] = np.array([x[1] for x in arr]).reshape(len(arr), T.size)
    out["kb_tab"] = np.array([x[2] for x in arr]).reshape(len(arr), T.size)
    for i, nm in enumerate(("kinf_troe", "k0_troe", "kc_troe", "fcent_troe")):
        out[nm] = np.array([x[1 + i] for x in troe]).reshape(len(troe), T.size)
    for i, nm in enumerate(("kinf_lind", "k0_lind", "kc_lind")):
        out[nm] = np.array([x[1 + i] for x in lind]).reshape(len(lind), T.size)
    kinds = []
    for r in mech.reactions:
        kinds.append("falloff-Troe" if r.rtype == TYPE_TROE else "falloff-Lindemann" if r.rtype == TYPE_LINDEMANN
                     else ("three-body-Arrhenius" if r.rtype == TYPE_THREEBODY else "Arrhenius"))
    out["rxn_kinds"] = kinds
    return out


# ------------------------------------------------------------- file formats
def _write_zones(path, title, variables, zones, T):
    with open(path, "w") as f:
        f.write(f'TITLE = "{title}"\n')
        f.write("VARIABLES = " + ", ".join(f'"{v}"' for v in variables) + "\n")
        for name, cols in zones:
            f.write(f'ZONE T="{name}"\nI={T.size}, F=POINT\n')
            for i in range(T.size):
                f.write(f"{T[i]:12.3f}" + "".join(f" {c[i]: .12E}" for c in cols) + "\n")


def write_folder(t, folder):
    """Write a table dict in FLINT's input formats (see module docstring)."""
    os.makedirs(folder, exist_ok=True)
    ns, names, T = t["ns"], t["names"], t["T"]
    with open(os.path.join(folder, "phase.txt"), "w") as f:
        f.write("ideal-gas phase\n")
        for n_, w in zip(names, t["wm"]):
            f.write(f"{n_} {w:.6f}\n")
    _write_zones(os.path.join(folder, "thermo.dat"), "Mass Thermodynamic Properties",
                 ["Temperature", "Cp", "Enthalpy", "Entropy", "dCp"],
                 [(names[k], [t["cp_tab"][k], t["h_tab"][k], t["s_tab"][k], t["dcp_tab"][k]]) for k in range(ns)], T)
    nr = t["nr_arrh"] + t["nr_troe"] + t["nr_lind"]
    kinds = t["rxn_kinds"]
    with open(os.path.join(folder, "chemistry-info.txt"), "w") as f:
        f.write(f"{t['mech_name']}\nN.ro species = {ns}\nN.ro reactions = {nr:4d}\n\n"
                "General loop info. They are not used if the mechanism is exlplicitly defined\n\nReaction type\n")
        for j, k in enumerate(kinds):
            f.write(f"{j + 1} {k}\n")
        f.write("\nReaction definition\n")
        counters = {"arrh": 0, "troe": 0, "lind": 0}
        for j, k in enumerate(kinds):
            key = "troe" if "Troe" in k else ("lind" if "Lindemann" in k else "arrh")
            i = counters[key]; counters[key] += 1
            for s in range(ns + 1):
                nm = names[s] if s < ns else "M"
                f.write(f"{j + 1} {nm} {t['ni1_' + key][i, s]:.1f} {t['ni2_' + key][i, s]:.1f} "
                        f"{t['eps_' + key][i, s]:.4f}\n")
    if t["nr_arrh"]:
        _write_zones(os.path.join(folder, "chemistry-Arrhenius.dat"), "Arrhenius data", ["Temperature", "kf", "kb"],
                     [(f"Reaction {j + 1}", [t["kf_tab"][j], t["kb_tab"][j]]) for j in range(t["nr_arrh"])], T)
    if t["nr_troe"]:
        _write_zones(os.path.join(folder, "chemistry-Troe.dat"), "Fall-off Troe data",
                     ["Temperature", "k_inf", "k_0", "k_c", "F_cent"],
                     [(f"Reaction {j + 1}", [t[n_][j] for n_ in ("kinf_troe", "k0_troe", "kc_troe", "fcent_troe")])
                      for j in range(t["nr_troe"])], T)
    if t["nr_lind"]:
        _write_zones(os.path.join(folder, "chemistry-Lindemann.dat"), "Fall-off Lindemann data",
                     ["Temperature", "k_inf", "k_0", "k_c"],
                     [(f"Reaction {j + 1}", [t[n_][j] for n_ in ("kinf_lind", "k0_lind", "kc_lind")])
                      for j in range(t["nr_lind"])], T)
    if t.get("mi_tab") is not None:
        _write_zones(os.path.join(folder, "transport.dat"), "Transport Properties",
                     ["Temperature", "Viscosity", "Conductivity"],
                     [(names[k], [t["mi_tab"][k], t["k_tab"][k]]) for k in range(ns)], T)


def read_tecplot_points(path):
    """Tecplot ASCII POINT file -> list of (zone title, rows (n, nvar))."""
    zones, cur = [], None
    with open(path) as f:
        for ln in f:
            s = ln.strip()
            if s.startswith("ZONE"):
                cur = [s.split('"')[1] if '"' in s else s, []]
                zones.append(cur)
            elif s and cur is not None and (s[0].isdigit() or s[0] in "+-."):
                cur[1].append([float(x.replace("D", "E")) for x in s.split()])
    return [(z, np.array(r, dtype=np.float64)) for z, r in zones]


# ------------------------------------------------------------ SZL binary
# Tecplot's SZL binary (.szplt), the format FLINT's loaders fall back to when
# the ASCII file is absent (Load_Chemistry.f90:95-96,
# Load_ThermoTransport.f90:57-60), for the ordered one-dimensional zones FLINT's
# tables are.  Layout, as the reference's own .szplt tables hold it:
#   bytes 0-33   the text line "#!SZPLT 105BF $Revision: ... $\r\n"
#   bytes 34-41  byte-order mark 08 07 06 05 04 03 02 01 (little-endian)
#   bytes 42-49  uint64 offset of the file header
#   file header  uint16 n, n uint16 tags, n uint64 values; a value is a count
#                or the offset of a record:
#                0x001 zones, 0x002 variables, 0x100 zone titles, 0x200
#                variable names (uint64 byte length, then names each ended by
#                '\r'), 0x101 zone type per zone ('o' ordered), 0x102 offset of
#                each zone's header (uint64 per zone), 0x107/0x108/0x109 I, J, K
#                per zone (uint64), 0x301 value location per zone and variable
#                (1 nodal), 0x302 data type per zone and variable (1 float32,
#                2 float64), 0x304 zone a variable is shared from (int32,
#                -1 none)
#   zone header  uint16 m, m tags, m values; tag 0x600 = offset of the
#                variables' data offsets (uint64 per variable); each variable
#                is then I*J*K contiguous values of its data type.
SZL_MAGIC = b"#!SZPLT 105BF $Revision: 00000 $\r\n"
SZL_BOM = bytes([8, 7, 6, 5, 4, 3, 2, 1])


def read_szplt(path):
    """SZL binary file -> list of (zone title, rows (n, nvar) float64), like read_tecplot_points."""
    import struct
    with open(path, "rb") as f:
        d = f.read()
    if d[:7] != b"#!SZPLT" or len(d) < 50 or d[34:42] != SZL_BOM:
        raise ValueError(f"{path}: not a little-endian SZL file")

    def u(fmt, o, n=1):
        sz = struct.calcsize("<" + fmt) * n
        if o < 0 or o + sz > len(d):
            raise ValueError(f"{path}: record at {o} runs past the end of the file")
        return struct.unpack_from(f"<{n}{fmt}", d, o)

    def tags(o):
        (n,) = u("H", o)
        return dict(zip(u("H", o + 2, n), u("Q", o + 2 + 2 * n, n)))

    H = tags(u("Q", 42)[0])
    for t in (0x1, 0x2, 0x100, 0x101, 0x102, 0x107, 0x108, 0x109, 0x200, 0x301, 0x302, 0x304):
        if t not in H:
            raise ValueError(f"{path}: file header lacks tag {t:#x}")
    nz, nv = H[0x1], H[0x2]

    def names(o, count):
        (ln,) = u("Q", o)
        out = d[o + 8:o + 8 + ln].decode("latin-1").split("\r")[:count]
        if len(out) != count:
            raise ValueError(f"{path}: {len(out)} names where {count} are expected")
        return out

    ztitle, vname = names(H[0x100], nz), names(H[0x200], nv)
    ztype = u("B", H[0x101], nz)
    zhead = u("Q", H[0x102], nz)
    I, J, K = u("Q", H[0x107], nz), u("Q", H[0x108], nz), u("Q", H[0x109], nz)
    loc, dtyp, share = u("B", H[0x301], nz * nv), u("B", H[0x302], nz * nv), u("i", H[0x304], nz * nv)
    zones = []
    for z in range(nz):
        if ztype[z] != ord("o"):
            raise ValueError(f"{path}: zone {z + 1} is not an ordered zone")
        Z = tags(zhead[z])
        if 0x600 not in Z:
            raise ValueError(f"{path}: zone {z + 1} header lacks its variable offsets")
        voff = u("Q", Z[0x600], nv)
        cnt = I[z] * J[z] * K[z]
        cols = []
        for v in range(nv):
            k = z * nv + v
            if loc[k] != 1 or share[k] != -1 or dtyp[k] not in (1, 2):
                raise ValueError(f"{path}: zone {z + 1} variable {vname[v]}: only unshared nodal float32/float64 "
                                 "data is supported")
            dt = np.dtype("<f4" if dtyp[k] == 1 else "<f8")
            if voff[v] + cnt * dt.itemsize > len(d):
                raise ValueError(f"{path}: zone {z + 1} variable {vname[v]} runs past the end of the file")
            cols.append(np.frombuffer(d, dtype=dt, count=cnt, offset=voff[v]).astype(np.float64))
        zones.append((ztitle[z], np.stack(cols, axis=1)))
    return zones


def write_szplt(path, title, variables, zones, dtype=np.float32):
    """Write ordered 1-D zones [(title, rows (n, nvar))] in the layout read_szplt reads.

    In float32, values are first clipped to +-1e36, the cap of the reference's
    float32 tables (their k_c at low T), so that nothing overflows."""
    import struct
    nz, nv = len(zones), len(variables)
    code = 1 if np.dtype(dtype) == np.float32 else 2
    body = bytearray(SZL_MAGIC + SZL_BOM + bytes(8) + bytes(24))
    zhead = []
    for _, rows in zones:
        rows = np.asarray(rows)
        offs = []
        if np.dtype(dtype) == np.float32:
            rows = np.clip(rows, -1e36, 1e36)
        for v in range(nv):
            offs.append(len(body))
            body += np.ascontiguousarray(rows[:, v], dtype=np.dtype(dtype).newbyteorder("<")).tobytes()
        zhead.append(len(body))
        body += struct.pack("<H", 1) + struct.pack("<H", 0x600) + struct.pack("<Q", len(body) + 12)
        body += struct.pack(f"<{nv}Q", *offs)

    def names(lst):
        s = "".join(x + "\r" for x in lst).encode("latin-1")
        return struct.pack("<Q", len(s)) + s

    recs = {0x100: names([z for z, _ in zones]), 0x101: b"o" * nz, 0x102: struct.pack(f"<{nz}Q", *zhead),
            0x107: struct.pack(f"<{nz}Q", *[np.asarray(r).shape[0] for _, r in zones]),
            0x108: struct.pack(f"<{nz}Q", *[1] * nz), 0x109: struct.pack(f"<{nz}Q", *[1] * nz),
            0x200: names(list(variables)), 0x301: b"\x01" * (nz * nv), 0x302: bytes([code]) * (nz * nv),
            0x304: struct.pack(f"<{nz * nv}i", *[-1] * (nz * nv))}
    vals = {0x1: nz, 0x2: nv}
    for t, r in recs.items():
        vals[t] = len(body)
        body += r
    hdr = len(body)
    keys = sorted(vals)
    body += struct.pack("<H", len(keys)) + struct.pack(f"<{len(keys)}H", *keys)
    body += struct.pack(f"<{len(keys)}Q", *[vals[k] for k in keys])
    struct.pack_into("<Q", body, 42, hdr)
    with open(path, "wb") as f:
        f.write(bytes(body))


def read_table_file(folder_prefix, base):
    """The ASCII file base.dat, else the SZL binary base.szplt (the reference's order)."""
    if os.path.exists(folder_prefix + base + ".dat"):
        return read_tecplot_points(folder_prefix + base + ".dat")
    if os.path.exists(folder_prefix + base + ".szplt"):
        return read_szplt(folder_prefix + base + ".szplt")
    raise FileNotFoundError(f"{folder_prefix}{base}.dat / .szplt")


def read_folder(folder, prefix=""):
    """Parse FLINT's input files into a table dict (read_idealgas_thermo + read_chemistry).

    Each table is read from its ASCII .dat file or, when that is absent, from
    its SZL binary .szplt (the loaders' fallback).  Raises FileNotFoundError
    where the reference prints [ERROR] and returns or stops (phase.txt, thermo,
    chemistry-Arrhenius)."""
    P = lambda n: os.path.join(folder, prefix + n)  # noqa: E731
    with open(P("phase.txt")) as f:
        lines = [ln for ln in f.read().splitlines()[1:] if ln.strip()]
    names = [ln.split()[0] for ln in lines]
    wm = np.array([float(ln.split()[1]) for ln in lines])
    ns = len(names)
    th = read_table_file(P(""), "thermo")
    T0 = int(round(th[0][1][0, 0]))
    rows = th[0][1].shape[0]
    tmin, tmax = T0, T0 + rows - 1
    cp = np.array([z[1][:, 1] for z in th[:ns]])
    h = np.array([z[1][:, 2] for z in th[:ns]])
    if tmin == 1:   # Load_ThermoTransport.f90:70,80-85: row 0 cloned (h(0) = 0)
        cp = np.hstack([cp[:, :1], cp]); h = np.hstack([np.zeros((ns, 1)), h]); tmin = 0
    t = {"ns": ns, "names": names, "wm": wm, "tmin": tmin, "tmax": tmax, "cp_tab": cp, "h_tab": h,
         "runiv": RUNIV_FLINT}
    with open(P("chemistry-info.txt")) as f:
        info = f.read().splitlines()
    t["mech_name"] = info[0].strip()
    nrc = int(info[2][17:21])
    kinds = [info[7 + j].split()[1] for j in range(nrc)]
    t["rxn_kinds"] = kinds
    body = info[7 + nrc + 2:]
    st = {"arrh": [], "troe": [], "lind": []}
    for j, k in enumerate(kinds):
        key = "troe" if "Troe" in k else ("lind" if "Lindemann" in k else "arrh")
        blk = body[j * (ns + 1):(j + 1) * (ns + 1)]
        st[key].append(np.array([[float(x) for x in ln.split()[2:5]] for ln in blk]))
    for key in st:
        a = np.array(st[key]).reshape(len(st[key]), ns + 1, 3)
        t[f"ni1_{key}"], t[f"ni2_{key}"], t[f"eps_{key}"] = (np.ascontiguousarray(a[:, :, i]) for i in range(3))
        t[f"nr_{key}"] = len(st[key])
    arr = read_table_file(P(""), "chemistry-Arrhenius")
    ti1 = int(round(arr[0][1][0, 0]))
    t["ti1"], t["ti2"] = ti1, ti1 + arr[0][1].shape[0] - 1
    t["kf_tab"] = np.array([z[1][:, 1] for z in arr[:t["nr_arrh"]]]).reshape(t["nr_arrh"], -1)
    t["kb_tab"] = np.array([z[1][:, 2] for z in arr[:t["nr_arrh"]]]).reshape(t["nr_arrh"], -1)
    if t["nr_troe"]:
        z = read_table_file(P(""), "chemistry-Troe")
        for i, nm in enumerate(("kinf_troe", "k0_troe", "kc_troe", "fcent_troe")):
            t[nm] = np.array([zz[1][:, 1 + i] for zz in z[:t["nr_troe"]]])
    if t["nr_lind"]:
        z = read_table_file(P(""), "chemistry-Lindemann")
        for i, nm in enumerate(("kinf_lind", "k0_lind", "kc_lind")):
            t[nm] = np.array([zz[1][:, 1 + i] for zz in z[:t["nr_lind"]]])
    # transport.dat (read_idealgas_transport, Load_ThermoTransport.f90:129-174):
    # optional; mu and k per species on the thermo rows (row 0 cloned likewise)
    if os.path.exists(P("transport.dat")):
        tr = read_tecplot_points(P("transport.dat"))
        mu = np.array([z[1][:, 1] for z in tr[:ns]])
        kt = np.array([z[1][:, 2] for z in tr[:ns]])
        if mu.shape[1] == t["tmax"] - t["tmin"]:
            mu = np.hstack([mu[:, :1], mu]); kt = np.hstack([kt[:, :1], kt])
        t["mi_tab"], t["k_tab"] = mu, kt
    return t


def read_folder_native(folder, prefix=""):
    """The same files through the library's own reader (flint_tables_read):
    a table dict of copies of its arrays, for callers and tests that want the
    parse a Fortran-free host would do."""
    L = native.lib()
    h = C.c_void_p()
    native.check(L.flint_tables_read(os.fsencode(folder), prefix.encode(), C.byref(h)), "flint_tables_read")
    try:
        d = native.TableDesc()
        native.check(L.flint_tables_desc(h, C.byref(d)), "flint_tables_desc")
        ns, nrow, nti = d.ns, d.tmax - d.tmin + 1, d.ti2 - d.ti1 + 1
        t = {"ns": ns, "tmin": d.tmin, "tmax": d.tmax, "ti1": d.ti1, "ti2": d.ti2, "runiv": d.runiv,
             "nr_arrh": d.nr_arrh, "nr_troe": d.nr_troe, "nr_lind": d.nr_lind,
             "names": [L.flint_tables_species_name(h, k).decode() for k in range(ns)]}
        nr = {"arrh": d.nr_arrh, "troe": d.nr_troe, "lind": d.nr_lind}
        shape = {"wm": (ns,), "cp_tab": (ns, nrow), "h_tab": (ns, nrow), "mi_tab": (ns, nrow), "k_tab": (ns, nrow)}
        for name in ARRAYS:
            key = name.rsplit("_", 1)[-1]
            shp = shape.get(name) or ((nr[key], ns + 1) if name[:3] in ("ni1", "ni2", "eps")
                                      else (nr["arrh" if name in ("kf_tab", "kb_tab") else key], nti))
            ptr = getattr(d, name)
            t[name] = (np.ctypeslib.as_array(ptr, shape=shp).copy() if ptr and all(shp)
                       else np.zeros(shp) if name not in ("mi_tab", "k_tab") else None)
        if t["mi_tab"] is None:
            del t["mi_tab"], t["k_tab"]
        return t
    finally:
        L.flint_tables_free(h)


# ----------------------------------------------------------------- handle
class Tables:
    """A tabulated mechanism on the GPU: FLINT's general loop and rhs_native."""

    def __init__(self, t):
        self.t = t
        self.L = native.lib()
        desc, self._keep = table_desc(t)
        h = C.c_void_p()
        native.check(self.L.flint_mech_create_tables(C.byref(desc), C.byref(h)), "flint_mech_create_tables")
        self.h = h
        self.ns = t["ns"]

    @classmethod
    def from_files(cls, folder, prefix=""):
        """A handle straight from FLINT's input files (flint_mech_create_from_files)."""
        obj = cls.__new__(cls)
        obj.L = native.lib()
        h = C.c_void_p()
        native.check(obj.L.flint_mech_create_from_files(os.fsencode(folder), prefix.encode(), C.byref(h)),
                     "flint_mech_create_from_files")
        obj.h, obj.t, obj._keep = h, None, {}
        ns = C.c_int()
        native.check(obj.L.flint_mech_sizes(h, C.byref(ns), None), "flint_mech_sizes")
        obj.ns = ns.value
        return obj

    def close(self):
        if self.h:
            self.L.flint_mech_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def chemistry_source(self, roi, T, omegadot=None):
        """general(roi, temp, omegadot) over N cells (device tensors, roi (N, ns))."""
        import torch
        if omegadot is None:
            omegadot = torch.empty_like(roi)
        s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        native.check(self.L.flint_chemistry_source_batch(self.h, T.shape[0], C.c_void_p(roi.data_ptr()),
                                                         C.c_void_p(T.data_ptr()), C.c_void_p(omegadot.data_ptr()),
                                                         s), "flint_chemistry_source_batch")
        return omegadot

    def rhs_native(self, Z, F=None):
        """rhs_native over N cells: Z (N, ns+1) = (rho_i, T) -> F (N, ns+1)."""
        import torch
        if F is None:
            F = torch.empty_like(Z)
        s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        native.check(self.L.flint_rhs_native_batch(self.h, Z.shape[0], C.c_void_p(Z.data_ptr()),
                                                   C.c_void_p(F.data_ptr()), s), "flint_rhs_native_batch")
        return F

    def transport(self, rhoi, T, mu=None, lam=None):
        """Wilke mixture viscosity and conductivity over N cells: rhoi (N, ns), T (N,)."""
        import torch
        if mu is None:
            mu = torch.empty_like(T)
        if lam is None:
            lam = torch.empty_like(T)
        s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        native.check(self.L.flint_transport_batch(self.h, rhoi.shape[0], C.c_void_p(rhoi.data_ptr()),
                                                  C.c_void_p(T.data_ptr()), C.c_void_p(mu.data_ptr()),
                                                  C.c_void_p(lam.data_ptr()), s), "flint_transport_batch")
        return mu, lam

    def cons2prim(self, cons, T, prim=None, T_out=None):
        """cons2prim over N cells: cons (N, ns+ndim+1) = (rho_i, rho u, rho E0) and
        the Newton start T (N,) -> prim (N, ns+ndim+1) = (rho_i, u, p), last T."""
        import torch
        ndim = cons.shape[1] - self.ns - 1
        if prim is None:
            prim = torch.empty_like(cons)
        if T_out is None:
            T_out = torch.empty_like(T)
        s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        native.check(self.L.flint_cons2prim_batch(self.h, cons.shape[0], ndim, C.c_void_p(cons.data_ptr()),
                                                  C.c_void_p(T.data_ptr()), C.c_void_p(prim.data_ptr()),
                                                  C.c_void_p(T_out.data_ptr()), s), "flint_cons2prim_batch")
        return prim, T_out
