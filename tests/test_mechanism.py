"""The product's mechanism reader (proteuscfd_gb300/mechanism.py): the
reference's .rxn rules and its database builder's text-file rules on small
synthetic files, and, with the reference checkout, the 5-species air model
read from the reference's own files equal to the fixture its database builder
produced (tests/golden/make_chem_fixture.py)."""
import json
import os
from pathlib import Path

import pytest

from proteuscfd_gb300.mechanism import CAL_TO_JOULE, load_rxn, read_burcat, read_mcbride, read_rxn

REF = os.environ.get("PCFD_REFERENCE_SRC")
FIXTURE = Path(__file__).resolve().parent / "golden" / "chem_5species_air.json"

RXN_CGS = """# no units tag: CGS, as the reference defaults
rxnInModel = 3

REACTION 1
rxnType = 1
thirdBodiesPresent = 1
O2 + M <==> 2O + M
A = 2.0E18
EA = 1.0E5
n = -1.5
M = O[5.0], N2[2.0]

REACTION 2
rxnType = 2
thirdBodiesPresent = 0
N2 + N <==> 2N + N
A = 4.0E16
EA = 2.0E4
n = -0.5

REACTION 3
rxnType = 0
thirdBodiesPresent = 0
NO(+) + E(-) <==> N + O
A = 1.0E12
EA = 0.0
n = 0.0
"""


def test_rxn_rules(tmp_path):
    p = tmp_path / "m.rxn"
    p.write_text(RXN_CGS)
    rx, order = read_rxn(p)
    # third bodies outside the equation extend the reaction's species list
    assert rx[0]["species"] == ["O2", "O", "N2"]
    assert rx[0]["nup"] == [1.0, 0.0, 0.0] and rx[0]["nupp"] == [0.0, 2.0, 0.0]
    assert rx[0]["tbeff"] == [1.0, 5.0, 2.0] and rx[0]["third_bodies"] == 1 and rx[0]["type"] == 1
    # a species on both sides is merged at its first appearance
    assert rx[1]["species"] == ["N2", "N"] and rx[1]["nup"] == [1.0, 1.0] and rx[1]["nupp"] == [0.0, 3.0]
    assert rx[1]["tbeff"] == [1.0, 1.0]
    # ion marks become suffixes, E- becomes e-
    assert rx[2]["species"] == ["NO+", "e-", "N", "O"]
    # the model's species in order of first appearance, third bodies included
    assert order == ["O2", "O", "N2", "N", "NO+", "e-"]
    assert rx[2]["global"] == [4, 5, 3, 1]
    # CGS: EA times 4184 and A times (1e-9)^(1 - sum of reactant coefficients)
    assert rx[0]["EA"] == 1.0e5 * CAL_TO_JOULE and rx[0]["n"] == -1.5
    assert rx[0]["A"] == 2.0e18 * (1.0e-3 * 1.0e-6) ** (1.0 - 1.0)
    assert rx[1]["A"] == 4.0e16 * (1.0e-3 * 1.0e-6) ** (1.0 - 2.0)


def test_rxn_si_and_refusals(tmp_path):
    p = tmp_path / "si.rxn"
    p.write_text("units = SI\n" + RXN_CGS)
    rx, _ = read_rxn(p)
    assert rx[0]["A"] == 2.0e18 and rx[0]["EA"] == 1.0e5
    q = tmp_path / "back.rxn"
    q.write_text(RXN_CGS.replace("n = -0.5\n", "n = -0.5\nrxnTypeBackward = 1\nAb = 1.0\n"))
    with pytest.raises(ValueError, match="backward"):
        read_rxn(q)


def burcat_record(name, mw, lo, hi, c15):
    """One record in the Burcat file's layout: a CAS line, a title, then four
    80-column lines numbered 1..4 in column 80, and a blank line."""
    def f(v):
        return "%15.8E" % v
    l1 = list(("%s test" % name).ljust(80))
    l1[47:55] = "%8.3f" % 200.0      # T1
    l1[56:65] = "%9.3f" % 6000.0     # T3
    l1[69:78] = "%9.5f" % mw         # molecular weight
    l1[79] = "1"
    l1 = "".join(l1)
    l2 = ("".join(f(v) for v in hi[:5])).ljust(79) + "2"
    l3 = ("".join(f(v) for v in hi[5:7] + lo[:3])).ljust(79) + "3"
    l4 = ("".join(f(v) for v in lo[3:7] + [c15])).ljust(79) + "4"
    return "1-23-4\n%s title line\n%s\n%s\n%s\n%s\n\n" % (name, l1, l2, l3, l4)


def test_burcat_and_mcbride_rules(tmp_path):
    lo = [3.5, -1.0e-4, 2.0e-6, -3.0e-9, 1.0e-12, -1.0e3, 3.0]
    hi = [3.6, 6.0e-4, -2.0e-7, 3.0e-11, -1.0e-15, -1.2e3, 3.2]
    lo2 = [v * 2.0 for v in lo]
    body = ("\n" * 88 + burcat_record("XY", 28.01348, lo, hi, -100.5) + burcat_record("XY", 30.0, lo2, hi, 1.0)
            + burcat_record("ZW", 32.0, hi, lo, 7.25))
    # the Burcat file's missing exponent sign: 'E 02' reads as E+02
    body = body.replace(" 3.20000000E+00", " 3.20000000E 00", 1)
    th = tmp_path / "t.thr"
    th.write_text(body)
    got = read_burcat(th, {"XY", "ZW"})
    assert got["XY"]["MW"] == 28.01348 and got["XY"]["lo"] == lo and got["XY"]["hi"] == hi
    assert got["XY"]["hf298"] == -100.5  # the first record of a species is kept
    assert got["ZW"]["lo"] == hi and got["ZW"]["hi"] == lo
    tr = tmp_path / "trans.inp"
    head = "header line\n"
    rec = ("O2                                V2C1  test\n"
           " V  200.0   1000.0   0.61205763E 00-0.67714354E 02 0.19040660E 03 0.21588272E 01\n"
           " V 1000.0   5000.0   0.69357334E 00 0.70953943E 02-0.28386007E 05 0.14856447E 01\n"
           " C  200.0   1000.0   0.60968928E 00-0.70892249E 02 0.58420624E 03 0.19337152E 01\n")
    tr.write_text(head + rec + "end\n")
    m = read_mcbride(tr)
    assert m["O2"]["mu"][0] == [200.0, 1000.0, 0.61205763, -67.714354, 190.4066, 2.1588272]
    assert len(m["O2"]["mu"]) == 2 and len(m["O2"]["k"]) == 1
    # the listed ions share their neutral's fits
    assert m["O2+"] == m["O2"] and m["O2-"] == m["O2"]


@pytest.mark.skipif(not (REF and (Path(REF) / "chemdata" / "trans.inp").exists()),
                    reason="PCFD_REFERENCE_SRC names no reference checkout")
def test_reference_air_model_equals_fixture():
    r = Path(REF)
    m = load_rxn(r / "chemModels" / "5speciesAir.rxn", r / "chemdata" / "BURCAT_FIXED.THR",
                 r / "chemdata" / "trans.inp")
    f = json.loads(FIXTURE.read_text())
    assert [s["name"] for s in m["species"]] == [s["name"] for s in f["species"]]
    for a, b in zip(m["species"], f["species"]):
        for k in ("MW", "lo", "hi", "hf298", "mu", "k"):
            assert a[k] == b[k], (a["name"], k)
    assert len(m["reactions"]) == len(f["reactions"])
    for a, b in zip(m["reactions"], f["reactions"]):
        for k in ("type", "A", "EA", "n", "third_bodies", "species", "nup", "nupp", "tbeff", "global"):
            assert a[k] == b[k], k
