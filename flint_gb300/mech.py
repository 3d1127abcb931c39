"""Mechanism intermediate representation (IR) for the GB300 chemistry path.

The IR carries exactly what FLINT's chemistry path needs:

* species: molar mass (kg/kmol, as ``phase.txt`` gives it and as
  ``read_idealgas_thermo`` stores it in ``wm_tab``, Load_ThermoTransport.f90:50-54),
  element composition (``composition.txt``, Load_ThermoTransport.f90:113-124) and
  NASA 7-coefficient polynomials (the YAML ``thermo`` block the table generator
  consumed, docs/input_yaml.md:176-209);
* reactions: the forms FLINT's general loop and the YTF generator handle
  (Lib_Chemistry_wdot.f90:96-220, utils/YTF.py:96-232): elementary Arrhenius
  with optional custom (non-integer) orders, third-body, Lindemann and Troe
  falloff, reversible or irreversible.

Units inside the IR are SI with kmol: A in (m^3/kmol)^(order-1)/s, Ea stored as
Ea/R in kelvin.  ``from_yaml`` converts Cantera-style YAML units the way the
reference's rate tables were produced (A scaled by (1e-3)^(order-1) for
cm/mol input, Ea divided by Cantera's gas constant 1.98720425864083 cal/mol/K).

``to_arrays`` flattens the IR into the plain arrays that the C-ABI
``flint_mech_desc`` struct points at (include/flint_gpu.h).
"""
from __future__ import annotations

import json
import math
import re
from dataclasses import dataclass, field, asdict

import numpy as np

from . import yamlsub

# FLINT's universal gas constant, used for R_i = Runiv / W_i and the energy
# equation (Lib_ThermoTransport.f90:13).
RUNIV_FLINT = 8314.51
# Cantera's gas constant: the reference's rate and thermo tables were made with it.
RUNIV_CANTERA = 6.02214076e26 * 1.380649e-23  # N_A * k_B = 8314.46261815324
R_CAL = 1.98720425864083  # cal/(mol K) = RUNIV_CANTERA / 4184
P_ATM = 101325.0

MAXSP_PER_SIDE = 3   # distinct species per reaction side
TYPE_ELEMENTARY, TYPE_THREEBODY, TYPE_LINDEMANN, TYPE_TROE = 0, 1, 2, 3

ATOMIC_WEIGHTS = {  # Cantera's values (kg/kmol)
    "H": 1.008, "C": 12.011, "O": 15.999, "N": 14.007, "Ar": 39.95, "He": 4.002602,
    "Cl": 35.45,
}


@dataclass
class Species:
    name: str
    mw: float
    composition: dict
    tlow: float
    tmid: float
    thigh: float
    low: list   # 7 NASA coefficients valid in [tlow, tmid]
    high: list  # 7 NASA coefficients valid in [tmid, thigh]
    # NASA-9 polynomials instead (1-3 ranges): [[T_lo, T_hi, a1..a7, b1, b2], ...];
    # low/high are then unused
    nasa9: list = None


@dataclass
class Reaction:
    equation: str
    rtype: int
    reactants: dict          # species -> stoichiometric coefficient
    products: dict
    orders: dict             # species -> forward order (defaults to reactant coefficient)
    reversible: bool
    A: float                 # SI kmol units (high-pressure limit for falloff)
    b: float
    EaR: float               # Ea / R  [K]
    A0: float = 0.0          # low-pressure limit (falloff)
    b0: float = 0.0
    EaR0: float = 0.0
    troe: list = None        # [a, T3, T1, T2] ; T2 = 0 means absent
    efficiencies: dict = None  # species -> efficiency (third-body / falloff)
    default_eff: float = 1.0
    collider: str = None     # explicit collider species "(+AR)"


def _orders_custom(self):
    """True when the reaction's forward orders differ from its reactant coefficients."""
    return any(self.orders.get(nm, nu) != nu for nm, nu in self.reactants.items()) or \
        any(nm not in self.reactants for nm in self.orders)


Reaction.orders_custom = _orders_custom


@dataclass
class Mechanism:
    name: str
    species: list
    reactions: list
    elements: list = field(default_factory=list)
    r_eos: float = RUNIV_FLINT        # EOS and energy-equation gas constant
    r_thermo: float = RUNIV_CANTERA   # NASA7 -> mass-specific cp/h/s and Kc
    p_ref: float = P_ATM              # standard-state pressure for Kc

    # ------------------------------------------------------------------ basic
    @property
    def ns(self):
        return len(self.species)

    @property
    def nr(self):
        return len(self.reactions)

    def index(self, name):
        for i, s in enumerate(self.species):
            if s.name == name:
                return i
        raise KeyError(name)

    # ------------------------------------------------------------------ arrays
    def to_arrays(self):
        """Flatten to the arrays of the C-ABI mechanism descriptor.

        Reactant / product sides hold up to MAXSP_PER_SIDE distinct species each;
        unused slots have index -1 and coefficient 0.
        """
        ns, nr = self.ns, self.nr
        a = {}
        a["mw"] = np.array([s.mw for s in self.species], dtype=np.float64)
        nasa = np.zeros((ns, 17), dtype=np.float64)
        for i, s in enumerate(self.species):
            nasa[i, 0], nasa[i, 1], nasa[i, 2] = s.tlow, s.tmid, s.thigh
            nasa[i, 3:10] = s.low
            nasa[i, 10:17] = s.high
        a["nasa7"] = nasa
        a["rtype"] = np.array([r.rtype for r in self.reactions], dtype=np.int32)
        a["reversible"] = np.array([1 if r.reversible else 0 for r in self.reactions], dtype=np.int32)
        arr = np.zeros((nr, 3)); arr0 = np.zeros((nr, 3)); troe = np.zeros((nr, 4))
        rsp = -np.ones((nr, MAXSP_PER_SIDE), dtype=np.int32)
        rnu = np.zeros((nr, MAXSP_PER_SIDE)); rord = np.zeros((nr, MAXSP_PER_SIDE))
        psp = -np.ones((nr, MAXSP_PER_SIDE), dtype=np.int32)
        pnu = np.zeros((nr, MAXSP_PER_SIDE))
        eff = np.zeros((nr, ns))
        for j, r in enumerate(self.reactions):
            arr[j] = (r.A, r.b, r.EaR)
            arr0[j] = (r.A0, r.b0, r.EaR0)
            if r.troe is not None:
                t = list(r.troe) + [0.0] * (4 - len(r.troe))
                troe[j] = t[:4]
            # reactant side: union of species with stoichiometry and species with orders
            rnames = list(r.reactants.keys()) + [k for k in r.orders if k not in r.reactants]
            if len(rnames) > MAXSP_PER_SIDE or len(r.products) > MAXSP_PER_SIDE:
                raise ValueError(f"reaction {r.equation!r} has more than {MAXSP_PER_SIDE} species on a side")
            for m, name in enumerate(rnames):
                rsp[j, m] = self.index(name)
                rnu[j, m] = r.reactants.get(name, 0.0)
                rord[j, m] = r.orders.get(name, r.reactants.get(name, 0.0))
            for m, (name, nu) in enumerate(r.products.items()):
                psp[j, m] = self.index(name)
                pnu[j, m] = nu
            if r.rtype != TYPE_ELEMENTARY:
                if r.collider is not None:
                    eff[j, self.index(r.collider)] = 1.0
                else:
                    eff[j, :] = r.default_eff
                    for name, e in (r.efficiencies or {}).items():
                        eff[j, self.index(name)] = e
        a.update(arrh=arr, arrh0=arr0, troe=troe, rsp=rsp, rnu=rnu, rord=rord,
                 psp=psp, pnu=pnu, eff=eff)
        a["consts"] = np.array([self.r_eos, self.r_thermo, self.p_ref], dtype=np.float64)
        if any(sp.nasa9 for sp in self.species):
            a["nasa9"] = self.nasa9_array()
        return a

    # Field order of the IR blob after its header (flint_mech_create_from_ir)
    IR_FIELDS = (("mw", "<f8"), ("nasa7", "<f8"), ("rtype", "<i4"), ("reversible", "<i4"), ("arrh", "<f8"),
                 ("arrh0", "<f8"), ("troe", "<f8"), ("rsp", "<i4"), ("rnu", "<f8"), ("rord", "<f8"),
                 ("psp", "<i4"), ("pnu", "<f8"), ("eff", "<f8"))

    def to_ir(self):
        """The mechanism as one IR blob (bytes): the 48-byte header "FLIR",
        version 1, ns, nr, flags (bit 0: NASA-9), 0, r_eos, r_thermo, p_ref, then
        the arrays of to_arrays() little-endian in IR_FIELDS order (+ nasa9)."""
        a = self.to_arrays()
        n9 = "nasa9" in a
        head = (np.array([0x52494C46, 1, self.ns, self.nr, 1 if n9 else 0, 0], dtype="<u4").tobytes()
                + np.asarray(a["consts"], dtype="<f8").tobytes())
        body = [np.ascontiguousarray(a[k], dtype=t).tobytes() for k, t in self.IR_FIELDS]
        if n9:
            body.append(np.ascontiguousarray(a["nasa9"], dtype="<f8").tobytes())
        return head + b"".join(body)

    def nasa9_array(self):
        """(ns, 32) NASA-9 rows: [nranges, T0, T1, T2, T3, 3 x (a1..a7, b1, b2)];
        NASA-7 species in their exact NASA-9 form (a1 = a2 = 0)."""
        out = np.zeros((self.ns, 32))
        for k, sp in enumerate(self.species):
            if sp.nasa9:
                rng = [list(r) for r in sp.nasa9]
            else:
                lo, hi = list(sp.low), list(sp.high)
                rng = [[sp.tlow, sp.tmid, 0.0, 0.0] + lo[:5] + [lo[5], lo[6]],
                       [sp.tmid, sp.thigh, 0.0, 0.0] + hi[:5] + [hi[5], hi[6]]]
            if not 1 <= len(rng) <= 3:
                raise ValueError(f"species {sp.name}: 1-3 NASA-9 ranges supported")
            out[k, 0] = len(rng)
            bps = [rng[0][0]] + [r[1] for r in rng]
            for i in range(4):
                out[k, 1 + i] = bps[i] if i < len(bps) else np.inf
            for i, r in enumerate(rng):
                out[k, 5 + 9 * i:14 + 9 * i] = r[2:11]
        return out

    def element_matrix(self):
        """(ne, ns) element counts; row order = self.elements."""
        E = np.zeros((len(self.elements), self.ns))
        for k, s in enumerate(self.species):
            for e, n in s.composition.items():
                E[self.elements.index(e), k] = n
        return E

    # ------------------------------------------------------------------ YTF
    def ytf_form(self):
        """This mechanism as FLINT's generator writes it into a Fortran routine
        (utils/YTF.py:96-232, the Lib_ChemMech/*.f90 family), so that the
        kernels compute what such a routine computes:

        * the concentration factors of the forward and reverse rates are the
          stoichiometric coefficients truncated to integers (stoich_to_mult,
          YTF.py:20-27, int(n) repetitions); custom orders are not used
          ("no custom orders are implemented", YTF.py:2); the net coefficients
          of the species sums keep their full values (YTF.py:246-249) -- where
          truncation changes a product's power the reverse rate differs, so
          such mechanisms (none among the generated routines) are refused;
        * third-body efficiencies as the routine prints them, '%.8g'
          (format_eff, YTF.py:29-34); zero efficiencies of three-body
          reactions are dropped (YTF.py:140), which changes no value;
        * falloff reactions take the efficiencies listed in the YAML and 1.0
          for every other species (efficiencies.get(sp, 1.0), YTF.py:156-158
          and :191-193): a reaction's default efficiency is not used;
        * an elementary termolecular reaction in which one species appears on
          both sides ("H + 2 O2 <=> HO2 + O2", "2 H + H2 <=> 2 H2") is the
          three-body reaction with that species as the third body, as Cantera
          reads it for the generator: one unit of it leaves both sides and
          becomes M (the routine's "M=coi(k)"); the rates of progress are the
          same products.  Bimolecular ones ("CH2(S) + H2O <=> CH2 + H2O")
          stay elementary, as in the routines.
        """
        import copy
        out = copy.deepcopy(self)
        out.name = self.name + " (YTF form)"
        names = [sp.name for sp in self.species]
        for r in out.reactions:
            both = [nm for nm in r.reactants if nm in r.products]
            termolecular = max(sum(r.reactants.values()), sum(r.products.values())) == 3.0
            if r.rtype == TYPE_ELEMENTARY and len(both) == 1 and termolecular and not r.orders_custom():
                x = both[0]
                r.rtype, r.collider, r.default_eff, r.efficiencies = TYPE_THREEBODY, x, 0.0, None
                r.reactants = {nm: (nu - 1.0 if nm == x else nu) for nm, nu in r.reactants.items()}
                r.reactants = {nm: nu for nm, nu in r.reactants.items() if nu > 0.0}
                r.products = {nm: (nu - 1.0 if nm == x else nu) for nm, nu in r.products.items()}
                r.products = {nm: nu for nm, nu in r.products.items() if nu > 0.0}
        for r in out.reactions:
            for nm, nu in r.products.items():
                if nu != int(nu):
                    raise ValueError(f"{r.equation}: non-integer product coefficient {nu} "
                                     "(the routine's reverse power would differ from Kc's)")
            r.orders = {nm: float(int(nu)) for nm, nu in r.reactants.items() if int(nu) > 0}
            if r.rtype == TYPE_ELEMENTARY:
                continue
            if r.rtype == TYPE_THREEBODY:
                if r.collider is not None:
                    continue
                effs = {nm: float(f"{(r.efficiencies or {}).get(nm, r.default_eff):.8g}") for nm in names}
            else:
                effs = {nm: float(f"{(r.efficiencies or {}).get(nm, 1.0):.8g}") for nm in names}
                if r.collider is not None:
                    effs = {nm: 1.0 for nm in names}
                r.collider = None
            r.default_eff = 1.0
            r.efficiencies = {nm: e for nm, e in effs.items() if e != 1.0}
        return out

    # ------------------------------------------------------------------ json
    def to_json(self):
        d = {"name": self.name, "elements": self.elements, "r_eos": self.r_eos,
             "r_thermo": self.r_thermo, "p_ref": self.p_ref,
             "species": [asdict(s) for s in self.species],
             "reactions": [asdict(r) for r in self.reactions]}
        return json.dumps(d, indent=1)

    @staticmethod
    def from_json(text):
        d = json.loads(text)
        sp = [Species(**s) for s in d["species"]]
        rx = [Reaction(**r) for r in d["reactions"]]
        return Mechanism(d["name"], sp, rx, d.get("elements", []), d["r_eos"], d["r_thermo"], d["p_ref"])

    @staticmethod
    def load(path):
        with open(path) as f:
            return Mechanism.from_json(f.read())


# ---------------------------------------------------------------------- YAML
_ARROW_RE = re.compile(r"\s*(<=>|=>|=)\s*")


def _parse_side(side: str):
    """Parse one side of an equation into ({species: coeff}, has_M, falloff_collider)."""
    falloff = None
    m = re.search(r"\(\+\s*([^)]+?)\s*\)", side)
    if m:
        falloff = m.group(1)
        side = side[:m.start()] + side[m.end():]
    terms = [t.strip() for t in re.split(r"\s\+\s", " " + side.strip() + " ") if t.strip()]
    out, has_m = {}, False
    for t in terms:
        if t == "M":
            has_m = True
            continue
        mm = re.match(r"^(\d+(?:\.\d*)?|\.\d+)\s+(\S+)$", t)
        if mm:
            coef, name = float(mm.group(1)), mm.group(2)
        else:
            mm = re.match(r"^(\d+)([A-Za-z].*)$", t)
            if mm and False:
                coef, name = float(mm.group(1)), mm.group(2)
            else:
                coef, name = 1.0, t
        out[name] = out.get(name, 0.0) + coef
    return out, has_m, falloff


def _unit_factors(units: dict):
    length = (units or {}).get("length", "m")
    quantity = (units or {}).get("quantity", "kmol")
    ea = (units or {}).get("activation-energy", "J/kmol")
    lf = {"cm": 1e-2, "m": 1.0, "mm": 1e-3}[length]
    qf = {"mol": 1e-3, "kmol": 1.0, "molec": 1.0 / 6.02214076e26}[quantity]
    conc = lf ** 3 / qf  # factor turning (length^3/quantity) into m^3/kmol
    eaf = {"cal/mol": 1.0 / R_CAL, "kcal/mol": 1000.0 / R_CAL,
           "J/mol": 1.0 / (RUNIV_CANTERA / 1000.0), "kJ/mol": 1000.0 / (RUNIV_CANTERA / 1000.0),
           "J/kmol": 1.0 / RUNIV_CANTERA, "K": 1.0}[ea]
    return conc, eaf


def _rate(rc, conc_f, eaf, order):
    A = float(rc["A"]) * conc_f ** (order - 1.0)
    return A, float(rc.get("b", 0.0)), float(rc.get("Ea", 0.0)) * eaf


def _mw(comp):
    return sum(ATOMIC_WEIGHTS[e] * n for e, n in comp.items())


def from_yaml(path, phase_mw=None, name=None):
    """Build a Mechanism from a Cantera-style YAML file (NASA-7 or NASA-9 species).

    ``phase_mw`` optionally maps species -> molar mass as read from FLINT's
    ``phase.txt`` (the loader takes molar masses from there, not from the YAML).
    """
    d = yamlsub.load(path)
    phase = d["phases"][0]
    conc_f, eaf = _unit_factors(d.get("units"))
    names = phase["species"]
    if names == "all":   # Cantera's shorthand: every species of the file, in order
        names = [s["name"] for s in d["species"]]
    spd = {s["name"]: s for s in d["species"]}
    species = []
    for n in names:
        s = spd[n]
        th = s["thermo"]
        mw = phase_mw[n] if phase_mw and n in phase_mw else _mw(s["composition"])
        tr = [float(x) for x in th["temperature-ranges"]]
        if th["model"] == "NASA9":
            rng = [[tr[i], tr[i + 1]] + [float(x) for x in th["data"][i]] for i in range(len(tr) - 1)]
            species.append(Species(n, float(mw), dict(s["composition"]), tr[0], tr[1], tr[-1], [0.0] * 7,
                                   [0.0] * 7, nasa9=rng))
            continue
        if th["model"] != "NASA7":
            raise ValueError(f"species {n}: thermo model {th['model']} is neither NASA7 nor NASA9")
        low, high = th["data"][0], th["data"][-1]
        if len(tr) == 2:
            tr = [tr[0], tr[1], tr[1]]
        species.append(Species(n, float(mw), dict(s["composition"]), float(tr[0]), float(tr[1]),
                               float(tr[2]), [float(x) for x in low], [float(x) for x in high]))
    reactions = []
    for r in d.get("reactions", []):
        eq = r["equation"]
        parts = _ARROW_RE.split(eq)
        lhs, arrow, rhs = parts[0], parts[1], parts[2]
        reac, m1, f1 = _parse_side(lhs)
        prod, m2, f2 = _parse_side(rhs)
        rtype_s = r.get("type", "three-body" if m1 else ("falloff" if f1 else "elementary"))
        orders = {k: float(v) for k, v in (r.get("orders") or {}).items()}
        forder = sum(orders.get(k, v) for k, v in reac.items()) + sum(
            v for k, v in orders.items() if k not in reac)
        rev = arrow != "=>"
        effs = {k: float(v) for k, v in (r.get("efficiencies") or {}).items()}
        deff = float(r.get("default-efficiency", 1.0))
        if rtype_s == "three-body":
            A, b, E = _rate(r["rate-constant"], conc_f, eaf, forder + 1.0)
            rx = Reaction(eq, TYPE_THREEBODY, reac, prod, orders, rev, A, b, E,
                          efficiencies=effs, default_eff=deff)
        elif rtype_s == "falloff":
            A, b, E = _rate(r["high-P-rate-constant"], conc_f, eaf, forder)
            A0, b0, E0 = _rate(r["low-P-rate-constant"], conc_f, eaf, forder + 1.0)
            troe = None
            rt = TYPE_LINDEMANN
            if "Troe" in r:
                t = r["Troe"]
                troe = [float(t["A"]), float(t["T3"]), float(t["T1"]), float(t.get("T2", 0.0))]
                rt = TYPE_TROE
            coll = f1 if (f1 and f1 != "M") else None
            rx = Reaction(eq, rt, reac, prod, orders, rev, A, b, E, A0, b0, E0, troe,
                          efficiencies=effs, default_eff=deff, collider=coll)
        else:
            A, b, E = _rate(r["rate-constant"], conc_f, eaf, forder)
            rx = Reaction(eq, TYPE_ELEMENTARY, reac, prod, orders, rev, A, b, E)
        reactions.append(rx)
    return Mechanism(name or phase["name"], species, reactions, list(phase.get("elements", [])))


def read_phase_txt(path):
    """FLINT phase.txt: header line, then 'NAME MW' per species (Load_ThermoTransport.f90:37-51)."""
    out = {}
    with open(path) as f:
        lines = f.read().splitlines()[1:]
    for ln in lines:
        t = ln.split()
        if len(t) >= 2:
            out[t[0]] = float(t[1])
    return out
