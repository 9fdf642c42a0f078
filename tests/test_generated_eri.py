"""The generated ERI class code itself, run on the CPU: for every angular-momentum class
the emitted VRR (`prim`) and HRR (`hrr`) statements of csrc/gen_eri.py are evaluated in
Python on one primitive quartet and compared with the oracle's primitive ERI, the
restatement of computePGTOrbTwoBodyRepulsion! (src/Integration/Engines/GaussianOrbitals.jl:
594-663).  This checks the generator's recursion choices (axis per node, shared brackets,
dependency pruning) without a GPU."""
import importlib.util
import math
import re
from pathlib import Path

import numpy as np
import pytest

GEN = Path(__file__).resolve().parents[1] / "quiqbox.jl_gb300" / "csrc" / "gen_eri.py"


def _gen():
    spec = importlib.util.spec_from_file_location("gen_eri_cpu", GEN)
    g = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(g)
    return g


def _body(code, start_marker):
    lines = code.splitlines()
    i = next(k for k, l in enumerate(lines) if start_marker in l) + 1
    out = []
    while lines[i] != "  }":
        out.append(lines[i].strip())
        i += 1
    return out


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def _python(lines):
    """The generated C statements as Python statements."""
    py = []
    for l in lines:
        if not l or l.startswith("//") or l.startswith("#"):
            continue
        l = l.rstrip(";")
        m = re.match(r"double F\[(\d+)\]$", l)
        if m:
            continue
        m = re.match(r"qb_boys_scaled<(\d+)>\(T, pre, boys_tab, F\)$", l)
        if m:
            py.append(f"F = boys_scaled({m.group(1)}, T, pre)")
            continue
        if l.startswith("const double "):
            for decl in _split_top(l[len("const double "):]):
                py.append(decl)
            continue
        py.append(l)
    return "\n".join(py)


class _Pair:
    def __init__(self, A, a, B, b):
        p = a + b
        P = (a * A + b * B) / p
        self.p, self.Px, self.Py, self.Pz = p, *P
        self.PAx, self.PAy, self.PAz = P - A
        self.K = math.sqrt(2.0) * math.pi ** 1.25 * math.exp(-a * b / p * float(np.dot(A - B, A - B))) / p
        self.oo2p = 0.5 / p


@pytest.mark.parametrize("cls", [(2, 2, 2, 2), (2, 2, 2, 1), (2, 1, 2, 1), (2, 1, 1, 1), (1, 1, 1, 1),
                                 (1, 1, 1, 0), (2, 2, 1, 1), (2, 0, 2, 0), (1, 0, 0, 0), (0, 0, 0, 0),
                                 (2, 2, 0, 0), (2, 1, 2, 0), (2, 0, 1, 1), (2, 2, 2, 0)])
def test_generated_class_code_vs_oracle(oracle, cls):
    g = _gen()
    cg = g.ClassGen(*cls)
    code = cg.generate()
    prim = _python(_body(code, "Sink&& sink) {"))
    hrr = _python(_body(code, "double (&I)[NINT]) {"))
    la, lb, lc, ld = cls
    rng = np.random.default_rng(sum(v * 10 ** k for k, v in enumerate(cls)))
    for trial in range(3):
        A, B, C, D = (rng.uniform(-1.2, 1.2, 3) for _ in range(4))
        a, b, c, d = rng.uniform(0.4, 3.0, 4)
        targets = [0.0] * (len(cg.esets) * len(cg.fsets))

        def sink(k, v):
            targets[k] += v

        def boys_scaled(M, T, pre):
            return [pre * v for v in oracle.boys_sequence(T, int(M))]

        ns = {"B": _Pair(A, a, B, b), "Kt": _Pair(C, c, D, d), "sink": sink, "boys_scaled": boys_scaled,
              "fma": lambda x, y, z: x * y + z, "rsqrt": lambda x: 1.0 / math.sqrt(x)}
        exec(prim, ns)
        I = [0.0] * (g.ncart(la) * g.ncart(lb) * g.ncart(lc) * g.ncart(ld))
        ABx, ABy, ABz = A - B
        CDx, CDy, CDz = C - D
        hs = {"A": targets, "ABx": ABx, "ABy": ABy, "ABz": ABz, "CDx": CDx, "CDy": CDy, "CDz": CDz, "I": I,
              "fma": lambda x, y, z: x * y + z}
        exec(hrr, hs)
        ref = [oracle.prim_eri((A, a, ia), (B, b, ib), (C, c, ic), (D, d, id_))
               for ia in g.comps(la) for ib in g.comps(lb) for ic in g.comps(lc) for id_ in g.comps(ld)]
        ref = np.array(ref)
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(np.array(I) - ref).max() < 1e-11 * scale, (cls, trial)
