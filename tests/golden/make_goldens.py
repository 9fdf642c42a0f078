"""Extract the golden values of Quiqbox.jl's own test-suite into JSON fixtures.

The reference is a Julia package and Julia is not available, so the golden
vectors are read as TEXT out of the reference's test files and written to
``tests/golden/goldens.json``.  Every value carries the reference file:line it
came from.  Run once (needs the reference checkout; the JSON is committed):

    python tests/golden/make_goldens.py /path/to/Quiqbox.jl

Nothing at test time reads the reference checkout.
"""
import json
import re
import sys
from pathlib import Path

NUM = r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?"


def _lines(root, rel):
    return (Path(root) / rel).read_text().splitlines()


def _find(lines, pattern, start=0):
    rx = re.compile(pattern)
    for i in range(start, len(lines)):
        if rx.search(lines[i]):
            return i
    raise KeyError(pattern)


def _nums(text):
    return [float(x) for x in re.findall(NUM, text)]


def _block(lines, begin_pat, end_pat, start=0):
    """Text of the lines from the first match of begin_pat to end_pat (inclusive)."""
    b = _find(lines, begin_pat, start)
    e = _find(lines, end_pat, b)
    return b, e, "\n".join(lines[b:e + 1])


def boys(root):
    rel = "test/unit-tests/Integration/BoysFunction-test.jl"
    L = _lines(root, rel)
    b, e, txt = _block(L, r"refPoints = \[", r"^\]")
    pts = []
    for m in re.finditer(r"\(\s*(" + NUM + r"),\s*(\d+),\s*(" + NUM + r")\)", txt):
        pts.append({"x": float(m.group(1)), "n": int(m.group(2)), "F": float(m.group(3))})
    return {"source": f"{rel}:{b + 1}-{e + 1}", "rtol": "sqrt(eps(Float64))", "points": pts}


def _prim_defs(txt):
    """name -> (center, exponent, ijk) from `PrimGaussTypeOrbInfo(...)` lines."""
    out = {}
    rx = re.compile(r"(\w+)\s*=\s*PrimGaussTypeOrbInfo\(\(([^)]*)\),\s*(" + NUM + r"),\s*\(([^)]*)\)\)")
    for m in rx.finditer(txt):
        out[m.group(1)] = {"center": _nums(m.group(2)), "alpha": float(m.group(3)),
                           "ijk": [int(v) for v in m.group(4).split(",")]}
    return out


def coulomb(root):
    rel = "test/unit-tests/Integration/Coulomb-test.jl"
    L = _lines(root, rel)
    txt = "\n".join(L)
    prims = _prim_defs(txt)
    prods = {}
    for m in re.finditer(r"(gtoProd\w+)\s*=\s*GaussProductInfo\(\((\w+),\s*(\w+)\)\)", txt):
        prods[m.group(1)] = [m.group(2), m.group(3)]
    one_body = []
    i = 0
    while True:
        try:
            i = _find(L, r"computePGTOrbOneBodyRepulsion!\(emptyCache, coord, gtoProd\d\d\) ==", i)
        except KeyError:
            break
        j = i
        while "≈" not in L[j]:
            j += 1
        prod = re.search(r"(gtoProd\d\d)", L[i]).group(1)
        val = float(re.findall(NUM, L[j].split("≈")[1])[0])
        one_body.append({"pair": prods[prod], "point": [0.0, 0.0, 0.0], "value": val,
                         "source": f"{rel}:{i + 1}"})
        i = j + 1
    two_body = []
    i = 0
    while True:
        try:
            i = _find(L, r"@test computePGTOrbTwoBodyRepulsion!\(sizedCache, gtoProd", i)
        except KeyError:
            break
        m = re.search(r"\(sizedCache, (gtoProd\d\d), (gtoProd\d\d)\)", L[i])
        j = i
        while not re.search(r"^\s*" + NUM + r"\s*$", L[j]):
            j += 1
        two_body.append({"bra": prods[m.group(1)], "ket": prods[m.group(2)],
                         "value": float(L[j].strip()), "source": f"{rel}:{i + 1}-{j + 1}"})
        i = j + 1
    # LiH basis (inner-renormalised primitives) and its nuclear-attraction matrix
    lih = _lih_basis(L, rel, "consH = ")
    b, e, vtxt = _block(L, r"@test all\(vec\(V2\) \.≈", r"\]\)")
    v2 = _nums(vtxt.split("≈", 1)[1])
    return {"prims": prims, "one_body": one_body, "two_body": two_body,
            "lih_basis": lih,
            "lih_nuclei": {"Z": [1, 3], "coords": [[0.0, 0.0, 0.0], [1.4, 0.0, 0.0]],
                           "source": f"{rel}:{_find(L, r'coords2 = ') + 1}"},
            "lih_V_colmajor": {"values": v2, "source": f"{rel}:{b + 1}-{e + 1}"}}


def _lih_basis(L, rel, anchor):
    """The six contracted functions bfH, bfLi1..bfLi5 of the LiH tests."""
    i0 = _find(L, anchor)
    txt = "\n".join(L[i0:i0 + 24])
    funcs = []
    rx = re.compile(r"(bf\w+)\s*=\s*genGaussTypeOrb\(\(([^)]*)\),\s*\[([^\]]*)\],\s*"
                    r"(\[[^\]]*\]|consH)(?:,\s*\(([^)]*)\))?,\s*\n?\s*innerRenormalize=true\)",
                    re.S)
    consH = _nums(re.search(r"consH = \[([^\]]*)\]", txt).group(1))
    for m in rx.finditer(txt):
        cons = consH if m.group(4) == "consH" else _nums(m.group(4))
        ijk = [int(v) for v in m.group(5).split(",")] if m.group(5) else [0, 0, 0]
        funcs.append({"name": m.group(1), "center": _nums(m.group(2)),
                      "alphas": _nums(m.group(3)), "coeffs": cons, "ijk": ijk,
                      "inner_renormalize": True, "outer_renormalize": False})
    assert [f["name"] for f in funcs] == ["bfH", "bfLi1", "bfLi2", "bfLi3", "bfLi4", "bfLi5"], funcs
    return {"functions": funcs, "source": f"{rel}:{i0 + 1}-{i0 + 24}"}


def overlap(root):
    rel = "test/unit-tests/Integration/Overlap-test.jl"
    L = _lines(root, rel)
    lih = _lih_basis(L, rel, "consH = ")
    b, e, txt = _block(L, r"@test overlaps\(bsLiH\) ≈", r"0\.0 0\.0 0\.0 0\.0 0\.0 1\.0+\d*\]")
    S = _nums(txt.split("≈", 1)[1])
    b2, e2, t2 = _block(L, r"s_gfHs = \[", r"\]$", b)
    sH = _nums(t2.split("=", 1)[1])
    h = re.search(r"bfH_t = genGaussTypeOrb\(\(([^)]*)\), \[([^\]]*)\]", "\n".join(L))
    return {"lih_basis": lih,
            "lih_S_rowmajor": {"values": S, "source": f"{rel}:{b + 1}-{e + 1}"},
            "h_prims": {"center": _nums(h.group(1)), "alphas": _nums(h.group(2)),
                        "S_rowmajor": sH, "note": "unnormalised primitives (weights 1)",
                        "source": f"{rel}:{b2 + 1}-{e2 + 1}"}}


def kinetic(root):
    rel = "test/unit-tests/Integration/Kinetic-test.jl"
    L = _lines(root, rel)
    i = _find(L, r"pgf1 = genGaussTypeOrb\(\(0\.1, 0\.2, 0\.3\), 2\.0, \(1, 0, 0\)\)")
    j = _find(L, r"0\.4350256247524772", i)
    k = _find(L, r"cgf1 = genGaussTypeOrb\(", j)
    m = _find(L, r"0\.06737210531634309", k)
    cg = re.search(r"genGaussTypeOrb\(\(([^)]*)\), \[([^\]]*)\], \[([^\]]*)\], \(([^)]*)\)\)", L[k])
    return {"pgto": {"center": [0.1, 0.2, 0.3], "alpha": 2.0, "ijk": [1, 0, 0],
                     "T": float(re.findall(NUM, L[j].split("≈")[-1])[0]),
                     "source": f"{rel}:{i + 1}-{j + 1}"},
            "cgto": {"center": _nums(cg.group(1)), "alphas": _nums(cg.group(2)),
                     "coeffs": _nums(cg.group(3)), "ijk": [int(v) for v in cg.group(4).split(",")],
                     "T": 0.06737210531634309, "source": f"{rel}:{k + 1}-{m + 1}"}}


def interface(root):
    rel = "test/unit-tests/Integration/Interface-test.jl"
    L = _lines(root, rel)
    txt = "\n".join(L)
    g = lambda name: _nums(re.search(name + r" = [\(\[]([^\)\]]*)[\)\]]", txt).group(1))
    i = _find(L, r"s2 = \[0\.28")
    return {"cgf1": {"center": g("cen1"), "alphas": g("xpns1"), "coeffs": g("cons1"), "ijk": [1, 0, 0]},
            "cgf2": {"center": g("cen2"), "alphas": g("xpns2"), "coeffs": g("cons2"), "ijk": [1, 0, 0]},
            "S_rowmajor": _nums(L[i].split("=", 1)[1]),
            "source": f"{rel}:{i + 1}"}


def hartree_fock(root):
    rel = "test/unit-tests/HartreeFock-test.jl"
    L = _lines(root, rel)
    out = {}
    i = _find(L, r"nucCoords = \[\(-0\.7")
    out["h2o"] = {"atoms": ["H", "H", "O"],
                  "coords": [[-0.7, 0.0, 0.0], [0.7, 0.0, 0.0], [0.0, 0.0, 0.0]],
                  "basis": "STO-3G", "source": f"{rel}:{i + 1}-{i + 2}"}
    i = _find(L, r"first\(res1\.energy\), -93\.")
    out["h2o"]["rhf_E_elec"] = float(re.findall(NUM, L[i])[-2])
    out["h2o"]["rhf_E_source"] = f"{rel}:{i + 1}"
    out["h2o"]["tol"] = 7.5e-8
    b, e, t = _block(L, r"@test isapprox\(res1\.fock\[1\],", r"atol=errorThreshold1\)")
    out["h2o"]["rhf_fock_rowmajor"] = _nums(t.split("[", 2)[2].rsplit("]", 1)[0])
    out["h2o"]["rhf_fock_source"] = f"{rel}:{b + 1}-{e + 1}"
    b, e, t = _block(L, r"@test isapprox\(res1\.occu\[begin\]\.left,", r"atol=errorThreshold1\)")
    out["h2o"]["rhf_orbital_energies"] = _nums(t.split("[", 1)[1].rsplit("]", 1)[0])
    out["h2o"]["rhf_orbital_energies_source"] = f"{rel}:{b + 1}-{e + 1}"
    i = _find(L, r"first\(res2\.energy\), -93\.")
    out["h2o"]["uhf_E_elec"] = float(re.findall(NUM, L[i])[-2])
    out["h2o"]["uhf_E_source"] = f"{rel}:{i + 1}"
    for key in ("rhfs", "uhfs"):
        b, e, t = _block(L, key + r" = \[", r"\]$")
        out["h2_" + key] = {"values": _nums(t.split("=", 1)[1]), "source": f"{rel}:{b + 1}-{e + 1}"}
    i = _find(L, r"bondLenRange = ")
    out["h2_curve"] = {"bond_lengths": {"start": 0.1, "step": 0.2, "stop": 19.9},
                       "basis": "3-21G", "tol": 7.5e-7, "quantity": "E_elec + E_nn",
                       "source": f"{rel}:{i + 1}"}
    i = _find(L, r"AtoBr = ")
    j = _find(L, r"Ehf_H2O2 = ", i)
    k = _find(L, r"coords_H2O2 = ", i)
    ctext = L[k] + L[k + 1]
    coords = [_nums(c) for c in re.findall(r"\[([^\[\]]+)\]", ctext.split("=", 1)[1])]
    out["h2o2"] = {"atoms": ["O", "O", "H", "H"], "coords_angstrom": coords,
                   "angstrom_to_bohr": float(re.findall(NUM, L[i])[0]),
                   "E_elec": float(re.findall(NUM, L[j].split("=", 1)[1])[0]), "tol": 5 * 5e-10,
                   "basis": "6-31G", "threshold": 5e-10, "secondary_conv_ratio": [5, 5],
                   "source": f"{rel}:{i + 1}-{j + 1}"}
    return out


def main(root):
    data = {"reference": "Quiqbox.jl v0.6.3 test-suite (values read as text)",
            "boys": boys(root), "coulomb": coulomb(root), "overlap": overlap(root),
            "kinetic": kinetic(root), "interface": interface(root),
            "hartree_fock": hartree_fock(root)}
    out = Path(__file__).with_name("goldens.json")
    out.write_text(json.dumps(data, indent=1))
    print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <path of the Quiqbox.jl source tree>")
    main(sys.argv[1])
