"""Build ``basis_sets.json`` from Quiqbox.jl's basis-set library text.

Quiqbox ships its atomic basis sets (collected from basissetexchange.org) as
Gaussian-format text blocks inside ``lib/BasisSets/BasisSets.jl``: one block per
(family, element), ``nothing`` where a family has no entry for an element.
This script reads that file once and writes the blocks as structured data:

    {family: {element: [{"shell": "S"|"SP"|"P"|"D"|..., "exponents": [...],
                         "coefficients": [[...], ...]}, ...]}}

where ``coefficients`` has one row per angular momentum of the subshell (two
rows for "SP").  The parse follows ``genGaussTypeOrbSeq``
(src/OrbitalBases.jl:502-542): ``D`` exponents are rewritten as ``E``, a header
line is one whose first token is a subshell label and which has >2 tokens.

    python quiqbox.jl_gb300/data/make_basis_sets.py /path/to/Quiqbox.jl
"""
import json
import re
import sys
from pathlib import Path

ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne",
            "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar", "K", "Ca"]   # src/Lexicons.jl:10-11


def parse_block(text):
    lines = [ln.split() for ln in text.replace("D+", "E+").replace("D-", "E-").splitlines()]
    shells = []
    i = 0
    while i < len(lines):
        tok = lines[i]
        if len(tok) > 2 and re.fullmatch(r"[A-Z]+", tok[0]):
            nprim = int(tok[1])
            rows = [[float(v) for v in lines[i + 1 + k]] for k in range(nprim)]
            shells.append({"shell": tok[0], "exponents": [r[0] for r in rows],
                           "coefficients": [[r[c] for r in rows] for c in range(1, len(rows[0]))]})
            i += 1 + nprim
        else:
            i += 1
    return shells


def main(root):
    src = (Path(root) / "lib/BasisSets/BasisSets.jl").read_text()
    names = re.findall(r'^"([^"\n]+)",?\s*$', src.split("const AtomicGTOrbSetTexts")[0], re.M)
    body = src.split("const AtomicGTOrbSetTexts", 1)[1]
    fams = re.split(r"^#[^\n]*\nMemory\{NothingOr\{String\}\}\(\[", body, flags=re.M)[1:]
    assert len(fams) == len(names), (names, len(fams))
    out = {}
    for name, fam in zip(names, fams):
        entries = re.findall(r'"""(.*?)"""|^(nothing),?\s*$', fam, re.S | re.M)
        table = {}
        for el, (text, nothing) in zip(ELEMENTS, entries):
            if not nothing:
                table[el] = parse_block(text)
        out[name] = table
    dst = Path(__file__).with_name("basis_sets.json")
    dst.write_text(json.dumps(out, separators=(",", ":")))
    print("wrote", dst, {k: len(v) for k, v in out.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <path of the Quiqbox.jl source tree>")
    main(sys.argv[1])
