"""Writes tests/golden/chem_5species_air.json: the 5-species air model of
the reference's 6-reaction mechanism file chemModels/5speciesAir.rxn, with
each species' molecular weight and NASA-7 polynomials as the reference's own
database builder (chemdata/chemDB.py, process_burcat) extracts them from
chemdata/BURCAT_FIXED.THR, and its viscosity and conductivity curve fits as
the builder's process_mcbride extracts them from chemdata/trans.inp.

The builder is imported from the reference tree with an in-memory stand-in
for the HDF5 file (h5py is not installed); the reaction file is parsed by the
rules of Reaction<T>::ParseReactionBlockLine / ParseReaction /
ParseThirdBodies (ucs/reaction.tcc:185,315,494), and the global species
order is ChemModel<T>::BuildGlobalSpeciesList's (ucs/chem.tcc:167): first
appearance over the reactions' species lists.

Run from the repository root with the reference tree present:
    python tests/golden/make_chem_fixture.py [reference_root]
"""
import importlib.util
import json
import os
import re
import sys
import tempfile
import types
from pathlib import Path

_REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PCFD_REFERENCE_SRC")
if not _REF:
    sys.exit("usage: make_chem_fixture.py <reference checkout> (or set PCFD_REFERENCE_SRC)")
REF = Path(_REF)
OUT = Path(__file__).resolve().parent / "chem_5species_air.json"


class _Group(dict):
    def require_group(self, name):
        return self.setdefault(name, _Group())

    def create_dataset(self, name, data):
        self[name] = data


def burcat_species():
    """The species groups the database builder writes from the Burcat thermo
    file and then from the McBride-Gordon transport file (its own order:
    Burcat, CEA, McBride-Gordon; only the last writes transport fits, and
    the first fit written for a species stays)."""
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    spec = importlib.util.spec_from_file_location("chemDB", REF / "chemdata" / "chemDB.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    h5 = _Group()
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)  # the builder writes a scratch file into the working directory
        try:
            import contextlib, io
            with contextlib.redirect_stdout(io.StringIO()):
                mod.process_burcat(h5, str(REF / "chemdata" / "BURCAT_FIXED.THR"))
                mod.process_mcbride(h5, str(REF / "chemdata" / "trans.inp"))
        finally:
            os.chdir(cwd)
    return h5["/species"]


def parse_equation(eq):
    lhs, rhs = eq.split("<==>")
    out = []
    for side, text in ((0, lhs), (1, rhs)):
        for tok in text.split():
            if tok in ("+", "M"):
                continue
            m = re.match(r"^([^A-Za-z]*)(.*)$", tok)
            stoich = float(m.group(1)) if m.group(1) else 1.0
            out.append((m.group(2), stoich if side == 0 else 0.0, stoich if side == 1 else 0.0))
    # merge duplicates in order of first appearance
    names, nup, nupp = [], [], []
    for name, a, b in out:
        if name in names:
            k = names.index(name)
            nup[k] += a
            nupp[k] += b
        else:
            names.append(name)
            nup.append(a)
            nupp.append(b)
    return names, nup, nupp


def parse_rxn(path):
    lines = Path(path).read_text().splitlines()
    nrx = None
    for ln in lines:
        if ln.startswith("rxnInModel"):
            nrx = int(ln.split("=")[1])
    reactions = []
    for r in range(1, nrx + 1):
        start = next(i for i, ln in enumerate(lines) if ln.startswith("REACTION %d" % r) and
                     ln.strip() == "REACTION %d" % r)
        rx = {"type": 0, "A": 0.0, "EA": 0.0, "n": 0.0, "third_bodies": 0}
        names = nup = nupp = None
        tbeff = None
        for ln in lines[start + 1:]:
            if ln[:1] in ("#", " ", ""):
                continue
            if ln.startswith("REACTION"):
                break
            key = ln.split("=")[0].strip()
            val = ln.split("=", 1)[1].strip() if "=" in ln else ""
            if "<==>" in ln:
                names, nup, nupp = parse_equation(ln)
            elif key == "rxnType":
                rx["type"] = int(val)
            elif key == "thirdBodiesPresent":
                rx["third_bodies"] = int(val)
            elif key == "A":
                rx["A"] = float(val)
            elif key == "EA":
                rx["EA"] = float(val)
            elif key == "n":
                rx["n"] = float(val)
            elif key == "M":
                tbeff = [1.0] * len(names)
                for name, v in re.findall(r"([A-Z][A-Za-z0-9]*)\[([^\]]+)\]", val):
                    if name in names:
                        tbeff[names.index(name)] = float(v)
                    else:
                        names.append(name)
                        nup.append(0.0)
                        nupp.append(0.0)
                        tbeff.append(float(v))
        if tbeff is None:
            tbeff = [1.0] * len(names)
        rx["species"] = names
        rx["nup"] = nup
        rx["nupp"] = nupp
        rx["tbeff"] = tbeff
        reactions.append(rx)
    return reactions


def main():
    reactions = parse_rxn(REF / "chemModels" / "5speciesAir.rxn")
    order = []
    for rx in reactions:
        for s in rx["species"]:
            if s not in order:
                order.append(s)
    db = burcat_species()
    species = []
    for s in order:
        d = db[s]
        # a species without transport fits takes N2's (Species::Init,
        # ucs/species.tcc:241-246,281-286)
        tr = d if "mu" in d and "k" in d else db["N2"]
        species.append({"name": s, "MW": float(d["MW"]) / 1000.0,
                        "lo": [float(v) for v in d["NASA7_burcat1"]],
                        "hi": [float(v) for v in d["NASA7_burcat2"]],
                        "hf298": float(d["NASA7_burcat_coeff15"]),
                        "mu": [[float(v) for v in row] for row in tr["mu"]],
                        "k": [[float(v) for v in row] for row in tr["k"]]})
    for rx in reactions:
        rx["global"] = [order.index(s) for s in rx["species"]]
    fixture = {"source": "chemModels/5speciesAir.rxn + chemdata/BURCAT_FIXED.THR and chemdata/trans.inp via "
                         "chemdata/chemDB.py",
               "univ_r": 8.31447215, "pref": 101325.0, "species": species, "reactions": reactions}
    OUT.write_text(json.dumps(fixture, indent=1) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
