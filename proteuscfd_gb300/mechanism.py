"""Reading a reaction mechanism and its species data the way the reference
does, into the mechanism description ``chem.model_struct`` and
``chem.ChemModel`` take: {"species": [{"name", "MW" (kg/mol), "lo", "hi"
(NASA-7 below and above 1000 K), "hf298", "mu", "k" (McBride-Gordon fits,
rows T_lo, T_hi, A, B, C, D)}], "reactions": [{"type", "A", "EA", "n",
"third_bodies", "species", "global", "nup", "nupp", "tbeff"}]}.

* The reaction file (``.rxn``): ChemModel::ReadReactionsFile and
  Reaction::ReadReactionFromFile / ParseReactionBlockLine / ParseReaction /
  ParseThirdBodies (ucs/chem.tcc:9-100, ucs/reaction.tcc:100-540), with the
  units tag of ChemModel::CheckReactionFileUnits (CGS when there is none)
  and Reaction::ConvertArrheniusCGSToSI (ucs/reaction.tcc:924).  The
  model's species are the reactions' species (third bodies included) in
  order of first appearance (ChemModel::BuildGlobalSpeciesList,
  ucs/chem.tcc:163).
* The species data: the reference reads them from the HDF5 database its
  builder writes (Species::GetDBInfo, ucs/species.tcc:140); here they are
  read from the builder's own text sources with its rules - the Burcat
  thermodynamic file (chemdata/chemDB.py process_burcat: the last four
  80-column lines of each record, the first record of a species kept) and
  the McBride-Gordon transport file (process_mcbride: V and C fits, the
  first record of a species kept, the listed ions sharing their neutral's
  fits).  A species without transport fits takes N2's, as GetDBInfo does.

Backward rates given in the file (rxnTypeBackward, Ab, EAb, nb) are not
supported: the library forms backward rates from equilibrium constants."""
from __future__ import annotations

import re
from pathlib import Path

CAL_TO_JOULE = 4184.0  # ucs/chem_constants.h (applied to EA in calories per mole)


def _num(text):
    """The leading number of text, as a C++ stream reads it (0 when none)."""
    m = re.match(r"\s*([-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?)", text)
    return float(m.group(1)) if m else 0.0


def _int(text):
    m = re.match(r"\s*([-+]?\d+)", text)
    return int(m.group(1)) if m else 0


def _after_eq(line):
    return line[line.index("=") + 1:] if "=" in line else ""


def _species_symbol(token):
    """Stoichiometric prefix and species name of one equation token; the
    ion marks (+) and (-) become + and - suffixes, E- becomes e-."""
    i = 0
    while i < len(token) and not token[i].isalpha():
        i += 1
    stoich = _num(token[:i]) if i else 1.0
    name = token[i:]
    for mark, sign in (("(+)", "+"), ("(-)", "-")):
        if mark in name:
            name = name.replace(mark, "") + sign
    return stoich, name


def _parse_equation(eq):
    """Reaction::ParseReaction: reactants then products, 'M' and '+' tokens
    dropped, repeated species merged at their first appearance with their
    coefficients summed."""
    lhs, rhs = eq.split("<==>", 1)
    names, nup, nupp = [], [], []
    for side, text in ((0, lhs), (1, rhs)):
        for tok in text.split():
            if tok in ("+", "M"):
                continue
            stoich, name = _species_symbol(tok)
            if name in names:
                k = names.index(name)
            else:
                names.append(name)
                nup.append(0.0)
                nupp.append(0.0)
                k = len(names) - 1
            if side == 0:
                nup[k] += stoich
            else:
                nupp[k] += stoich
    names = ["e-" if n == "E-" else n for n in names]
    return names, nup, nupp


def _parse_third_bodies(line, rx):
    """Reaction::ParseThirdBodies: 'M = SYM[eff], ...'; efficiencies of
    species not in the equation extend the reaction's species list."""
    text = _after_eq(line)
    rx["tbeff"] = [1.0] * len(rx["species"])
    for sym, val in re.findall(r"([A-Z][^\[\s,]*)\s*\[([^\]]*)\]", text):
        for mark, sign in (("(+)", "+"), ("(-)", "-")):
            if mark in sym:
                sym = sym.replace(mark, "") + sign
        if sym == "E-":
            sym = "e-"
        eff = _num(val)
        if sym in rx["species"]:
            rx["tbeff"][rx["species"].index(sym)] = eff
        else:
            rx["species"].append(sym)
            rx["nup"].append(0.0)
            rx["nupp"].append(0.0)
            rx["tbeff"].append(eff)


def read_rxn(path):
    """The reactions of a .rxn file -> (reactions, model species order)."""
    lines = Path(path).read_text().splitlines()
    units = None
    nrx = None
    for ln in lines:
        if ln[:1] in ("#", " ", ""):
            continue
        # the first line naming the units decides (CheckReactionFileUnits)
        if units is None and "units" in ln and "=" in ln:
            u = _after_eq(ln)
            units = "SI" if "SI" in u else ("CGS" if "CGS" in u else None)
        if nrx is None and "rxnInModel" in ln:
            nrx = _int(_after_eq(ln))
    units = units or "CGS"
    if nrx is None:
        raise ValueError("%s: no rxnInModel line" % path)
    reactions = []
    for r in range(1, nrx + 1):
        try:
            start = next(i for i, ln in enumerate(lines) if ln[:1] not in ("#", " ")
                         and ln.strip() == "REACTION %d" % r)
        except StopIteration:
            raise ValueError("%s: reaction %d not found" % (path, r)) from None
        rx = {"type": 0, "A": 0.0, "EA": 0.0, "n": 0.0, "third_bodies": 0, "species": [], "nup": [], "nupp": [],
              "tbeff": None}
        for ln in lines[start + 1:]:
            if ln[:1] in ("#", " ", ""):
                continue
            if ln.startswith("REACTION"):
                break
            # the keyword tests of ParseReactionBlockLine, in its order
            if "<==>" in ln:
                rx["species"], rx["nup"], rx["nupp"] = _parse_equation(ln)
            elif "rxnTypeBackward" in ln or ln.startswith(("Ab", "nb", "EAb")):
                raise ValueError("%s: reaction %d gives a backward rate, which is not supported" % (path, r))
            elif "rxnType" in ln:
                rx["type"] = _int(_after_eq(ln))
            elif "thirdBodiesPresent" in ln:
                rx["third_bodies"] = _int(_after_eq(ln))
            elif ln.startswith("A"):
                rx["A"] = _num(_after_eq(ln))
            elif ln.startswith("EA"):
                rx["EA"] = _num(_after_eq(ln))
            elif "n" in ln:
                rx["n"] = _num(_after_eq(ln))
            elif "M" in ln:
                _parse_third_bodies(ln, rx)
            else:
                raise ValueError("%s: cannot parse line %r" % (path, ln))
        if rx["tbeff"] is None:
            rx["tbeff"] = [1.0] * len(rx["species"])
        if units == "CGS":
            # Reaction::ConvertArrheniusCGSToSI
            zp = 0.0
            for v in rx["nup"]:
                zp += v
            rx["EA"] = rx["EA"] * CAL_TO_JOULE
            factor = 1.0e-3 * 1.0e-6
            rx["A"] = rx["A"] * factor ** (1.0 - zp)
        reactions.append(rx)
    order = []
    for rx in reactions:
        for s in rx["species"]:
            if s not in order:
                order.append(s)
    for rx in reactions:
        rx["global"] = [order.index(s) for s in rx["species"]]
    return reactions, order


def _coeff(line, pos, nchar=15):
    """chemDB.py read_coeff: a fixed-width field with the Burcat file's
    missing exponent signs repaired; 'N/A' reads as 0."""
    c = line[pos:pos + nchar]
    if nchar == 15:
        if c[11:13] == "E ":
            c = c[0:12] + "+" + c[13:15]
        if c[10:12] == " E":
            c = c[0:10] + "0" + c[11:15]
    if "N/A" in c:
        return 0.0
    return float(c)


def read_burcat(path, names):
    """NASA-7 fits and molecular weights of the named species from the
    Burcat thermodynamic file -> {name: {"MW" (g/mol), "lo", "hi", "hf298"}}."""
    text = "".join(Path(path).read_text(errors="replace").splitlines(keepends=True)[88:])
    pat = re.compile(r"[0-9]+\-[0-9]*\-[0-9].+?\n[ \t\n]*?\n", re.DOTALL)
    out = {}
    for match in pat.findall(text):
        rec = match.strip().split("\n")[-4:]
        if len(rec) != 4:
            continue
        name = rec[0].split()[0]
        rec = [r.expandtabs().rstrip() for r in rec]
        if any(len(r) != 80 or r[79] != str(i + 1) for i, r in enumerate(rec)):
            continue
        if name not in names or name in out:
            continue
        hi = [_coeff(rec[1], p) for p in (0, 15, 30, 45, 60)] + [_coeff(rec[2], p) for p in (0, 15)]
        lo = [_coeff(rec[2], p) for p in (30, 45, 60)] + [_coeff(rec[3], p) for p in (0, 15, 30, 45)]
        out[name] = {"MW": float(rec[0][69:78]), "lo": lo, "hi": hi, "hf298": _coeff(rec[3], 60)}
    return out


# ions that share the transport fits of their neutral (chemDB.py process_mcbride)
_ION_COPIES = {"O2": "+-", "O": "+-", "N2": "-+", "N": "+", "NO": "+", "CO": "+", "OH": "+-", "H2": "+-",
               "H2O": "+"}


def read_mcbride(path):
    """Viscosity and conductivity fits of every species in the McBride-Gordon
    transport file -> {name: {"mu": rows, "k": rows}}."""
    lines = Path(path).read_text(errors="replace").splitlines()[1:]
    out = {}
    i = 0
    while i < len(lines):
        header = lines[i]
        if header.strip() == "end":
            break
        name = header.split()[0]
        nv, nc = int(header[35]), int(header[37])
        visc = lines[i + 1:i + 1 + nv]
        cond = lines[i + 1 + nv:i + 1 + nv + nc]
        i += 1 + nv + nc

        def rows(block):
            return [[_coeff(ln, 3, 6), _coeff(ln, 11, 7), _coeff(ln, 20), _coeff(ln, 35), _coeff(ln, 50),
                     _coeff(ln, 65)] for ln in block]

        d = {}
        if nv > 0:
            d["mu"] = rows(visc)
        if nc > 0:
            d["k"] = rows(cond)
        for nm in [name] + [name + s for s in _ION_COPIES.get(name, "")]:
            got = out.setdefault(nm, {})
            for key, v in d.items():
                got.setdefault(key, v)
    return out


def load_rxn(rxn_path, thermo_path, transport_path):
    """The mechanism of a .rxn file with its species' data, as ChemModel
    builds it (the model's species in first-appearance order)."""
    reactions, order = read_rxn(rxn_path)
    thermo = read_burcat(thermo_path, set(order))
    trans = read_mcbride(transport_path)
    species = []
    for s in order:
        if s not in thermo:
            raise ValueError("species %s has no record in %s" % (s, thermo_path))
        t = thermo[s]
        tr = trans.get(s, {})
        # a fit the transport file lacks is N2's (Species::GetDBInfo, ucs/species.tcc:234-290)
        species.append({"name": s, "MW": t["MW"] / 1000.0, "lo": t["lo"], "hi": t["hi"], "hf298": t["hf298"],
                        "mu": tr.get("mu", trans["N2"]["mu"]), "k": tr.get("k", trans["N2"]["k"])})
    return {"source": "%s + %s and %s" % (Path(rxn_path).name, Path(thermo_path).name, Path(transport_path).name),
            "species": species, "reactions": reactions}
