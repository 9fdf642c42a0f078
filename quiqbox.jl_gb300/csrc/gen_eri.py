"""Generator of the shell-quartet ERI class kernels (HGP scheme) for sm_103a.

For every angular-momentum class (la lb | lc ld) of contracted Cartesian shells
(la >= lb, lc >= ld, bra pair class >= ket pair class, l <= LMAX) it emits a
straight-line CUDA device function that

  1. loops over the primitive pairs of the bra and ket shell pairs,
  2. evaluates the Boys function F_m(T), m <= la+lb+lc+ld, from a Taylor table,
  3. runs the Obara–Saika vertical recursion (bra, then ket with the
     electron-transfer cross term) only for the intermediates [e0|f0]^(m) that
     the targets actually need (backward dependency pruning),
  4. accumulates the contracted [e0|f0]^(0), e = la..la+lb, f = lc..lc+ld,
  5. applies the horizontal recursion (bra, then ket) once per contracted
     quartet to produce the (ab|cd) block in SubshellXYZs component order.

This is the algorithm of Head-Gordon & Pople (J. Chem. Phys. 89, 5777 (1988))
with the Obara–Saika VRR (J. Chem. Phys. 84, 3963 (1986)); the reference
evaluates the same integrals one Cartesian component at a time with an
axis-by-axis OS/electron-transfer scheme
(src/Integration/Engines/GaussianOrbitals.jl:529-663).

The generator also counts the FP64 operations it emits (add/mul = 1 flop,
fma = 2 flops) per primitive quartet and per contracted quartet and writes
them to ``flops_table.json``; that table is the algorithmic-work figure of the
FP64 roofline.

    python gen_eri.py OUTDIR [--lmax 2]
"""
import json
import sys
from pathlib import Path

LMAX_DEFAULT = 2
BOYS_TAYLOR = 8          # Taylor terms j = 0..7 of the Boys table
AXES = "xyz"


def comps(L):
    """SubshellXYZs[L] (src/Lexicons.jl:17-36)."""
    return [(i, j, L - i - j) for i in range(L, -1, -1) for j in range(L - i, -1, -1)]


def ncart(L):
    return (L + 1) * (L + 2) // 2


def pair_classes(lmax):
    return [(a, b) for a in range(lmax + 1) for b in range(a + 1)]


def quartet_classes(lmax):
    pcs = pair_classes(lmax)
    out = []
    for i, bra in enumerate(pcs):
        for ket in pcs[:i + 1]:
            out.append(bra + ket)
    return out


def sub(t, i, k=1):
    return tuple(v - (k if a == i else 0) for a, v in enumerate(t))


def add(t, i, k=1):
    return tuple(v + (k if a == i else 0) for a, v in enumerate(t))


def vrr_axis(node):
    """VRR recursion direction of node (e, f, m): the ket side while f has angular momentum,
    else the bra side; among the axes with a nonzero power there, the one whose node costs
    the fewest FP64 operations (a power of 1 has no two-down term; on the ket side an axis
    with e_i = 0 has no cross term), then the smallest power, then x, y, z.  Against
    recursing along the largest power this needs 5-20 % fewer VRR operations in the d
    classes ((dp|pp) 4.8 %, (dp|dp) 12.9 %, (dd|dp) 13.4 %)."""
    e, f, m = node
    if sum(f) > 0:
        return min((i for i in range(3) if f[i] > 0),
                   key=lambda i: (2 + (2 if f[i] > 1 else 0) + (1 if e[i] > 0 else 0), f[i], i))
    return min((i for i in range(3) if e[i] > 0), key=lambda i: (2 + (2 if e[i] > 1 else 0), e[i], i))


def pick_axis(t):
    """HRR recursion direction: the axis with the largest power (first on ties)."""
    best = 0
    for a in range(3):
        if t[a] > t[best]:
            best = a
    return best


class Counter:
    def __init__(self):
        self.add = 0
        self.mul = 0
        self.fma = 0

    def flops(self):
        return self.add + self.mul + 2 * self.fma


def tname(e):
    return "".join(str(v) for v in e)


class ClassGen:
    def __init__(self, la, lb, lc, ld):
        self.la, self.lb, self.lc, self.ld = la, lb, lc, ld
        self.L = la + lb + lc + ld
        self.name = f"{la}{lb}{lc}{ld}"
        self.prim = Counter()     # per primitive quartet
        self.contr = Counter()    # per contracted quartet (HRR)
        self.esets = [e for L in range(la, la + lb + 1) for e in comps(L)]
        self.fsets = [f for L in range(lc, lc + ld + 1) for f in comps(L)]
        self.seg = len(self.esets) * len(self.fsets) >= SEG_MIN_NT

    # -- VRR dependency analysis ------------------------------------------------
    def vrr_children(self, node):
        e, f, m = node
        if sum(f) > 0:
            i = vrr_axis(node)
            f1 = sub(f, i)
            ch = [(e, f1, m), (e, f1, m + 1)]
            if f1[i] > 0:
                f2 = sub(f1, i)
                ch += [(e, f2, m), (e, f2, m + 1)]
            if e[i] > 0:
                ch.append((sub(e, i), f1, m + 1))
            return ch
        if sum(e) > 0:
            i = vrr_axis(node)
            e1 = sub(e, i)
            ch = [(e1, f, m), (e1, f, m + 1)]
            if e1[i] > 0:
                e2 = sub(e1, i)
                ch += [(e2, f, m), (e2, f, m + 1)]
            return ch
        return []

    def vrr_nodes(self):
        targets = [(e, f, 0) for e in self.esets for f in self.fsets]
        need = set()
        stack = list(targets)
        while stack:
            n = stack.pop()
            if n in need:
                continue
            need.add(n)
            stack.extend(self.vrr_children(n))
        order = sorted(need, key=lambda n: (sum(n[0]) + sum(n[1]), sum(n[1]), -n[2], n))
        return self.schedule(order), targets

    def schedule(self, nodes):
        """Emission order of the VRR nodes: greedy list scheduling that, among the nodes whose
        inputs are ready, takes the one that frees the most live values (ties: lower angular
        momentum first).  Keeps the live set ~35% below a level-by-level order, which is
        what decides register spilling in the larger classes."""
        ch = {n: sorted(set(self.vrr_children(n))) for n in nodes}
        parents = {n: [] for n in nodes}
        for n in nodes:
            for c in ch[n]:
                parents[c].append(n)
        uses = {n: len(parents[n]) for n in nodes}
        ndeps = {n: len(ch[n]) for n in nodes}
        ready = [n for n in nodes if ndeps[n] == 0]
        out = []
        while ready:
            best = min(ready, key=lambda n: ((1 if parents[n] else 0) - sum(1 for c in ch[n] if uses[c] == 1),
                                             sum(n[0]) + sum(n[1]), n))
            ready.remove(best)
            out.append(best)
            for c in ch[best]:
                uses[c] -= 1
            for par in parents[best]:
                ndeps[par] -= 1
                if ndeps[par] == 0:
                    ready.append(par)
        assert len(out) == len(nodes)
        return out

    @staticmethod
    def vname(n):
        e, f, m = n
        if sum(e) == 0 and sum(f) == 0:
            return f"F{m}"
        return f"v{tname(e)}_{tname(f)}_{m}"

    def emit_vrr(self, out, ind, seg=False):
        """The VRR body.  seg=False: sink(k, value) per target as soon as it is final.
        seg=True: targets are gathered in emission order into batches of SEG_W values and
        each full batch goes to red(b, v0, ..., v7) (the last one padded with zeros);
        self.seg_pos[k] is then the emission slot of target k."""
        order, targets = self.vrr_nodes()
        tindex = {t: k for k, t in enumerate(targets)}
        c = self.prim if not seg else Counter()
        pending = []
        self.seg_pos = [None] * len(targets)
        nbatch = [0]

        def emit_target(k, name):
            if not seg:
                out.append(f"{ind}sink({k}, {name});")
                return
            self.seg_pos[k] = nbatch[0] * SEG_W + len(pending)
            pending.append(name)
            if len(pending) == SEG_W:
                out.append(f"{ind}red({nbatch[0]}, {', '.join(pending)});")
                pending.clear()
                nbatch[0] += 1
        # The "two-down" term of a node, (1/2p)([e2]^(m) - (rho/p) [e2]^(m+1)) on the bra side and
        # its ket analogue, depends on (e2, f, m) only, not on the recursion axis: the bracket
        # is computed once where several nodes use it (same operations, same results).
        cuse = {}
        for n in order:
            e, f, m = n
            if sum(f) > 0:
                i = vrr_axis(n)
                f1 = sub(f, i)
                if f1[i] > 0:
                    key = ("k", e, sub(f1, i), m)
                    cuse[key] = cuse.get(key, 0) + 1
            elif sum(e) > 0:
                i = vrr_axis(n)
                e1 = sub(e, i)
                if e1[i] > 0:
                    key = ("b", sub(e1, i), f, m)
                    cuse[key] = cuse.get(key, 0) + 1
        cdone = set()

        def bracket(key, coef, b0, b1):
            if cuse[key] < 2:
                return f"fma({coef}, {b1}, {b0})", 1
            kind, e_, f_, m_ = key
            cn = f"c{kind}{tname(e_)}_{tname(f_)}_{m_}"
            if key in cdone:
                return cn, 0
            cdone.add(key)
            out.append(f"{ind}const double {cn} = fma({coef}, {b1}, {b0});")
            return cn, 1

        for n in order:
            e, f, m = n
            if sum(e) == 0 and sum(f) == 0:
                continue
            nm = self.vname(n)
            if sum(f) > 0:
                i = vrr_axis(n)
                ax = AXES[i]
                f1 = sub(f, i)
                a0, a1 = self.vname((e, f1, m)), self.vname((e, f1, m + 1))
                expr = f"fma(QC{ax}, {a0}, WQ{ax} * {a1})"
                c.mul += 1
                c.fma += 1
                if f1[i] > 0:
                    f2 = sub(f1, i)
                    b0, b1 = self.vname((e, f2, m)), self.vname((e, f2, m + 1))
                    cb, nf = bracket(("k", e, f2, m), "-ppq", b0, b1)
                    expr = f"fma(oo2q_{f1[i]}, {cb}, {expr})"
                    c.fma += 1 + nf
                if e[i] > 0:
                    d1 = self.vname((sub(e, i), f1, m + 1))
                    expr = f"fma(oo2pq_{e[i]}, {d1}, {expr})"
                    c.fma += 1
            else:
                i = vrr_axis(n)
                ax = AXES[i]
                e1 = sub(e, i)
                a0, a1 = self.vname((e1, f, m)), self.vname((e1, f, m + 1))
                expr = f"fma(PA{ax}, {a0}, WP{ax} * {a1})"
                c.mul += 1
                c.fma += 1
                if e1[i] > 0:
                    e2 = sub(e1, i)
                    b0, b1 = self.vname((e2, f, m)), self.vname((e2, f, m + 1))
                    cb, nf = bracket(("b", e2, f, m), "-qpq", b0, b1)
                    expr = f"fma(oo2p_{e1[i]}, {cb}, {expr})"
                    c.fma += 1 + nf
            out.append(f"{ind}const double {nm} = {expr};")
            if n in tindex:
                emit_target(tindex[n], nm)
        for k, t in enumerate(targets):
            if sum(t[0]) == 0 and sum(t[1]) == 0:
                emit_target(k, self.vname(t))
        if seg and pending:
            out.append(f"{ind}red({nbatch[0]}, {', '.join(pending + ['0.0'] * (SEG_W - len(pending)))});")
            nbatch[0] += 1
        self.seg_nbatch = nbatch[0]
        c.add += len(targets)   # the accumulation of every target into its contracted sum
        used_m = sorted({n[2] for n in order if sum(n[0]) == 0 and sum(n[1]) == 0})
        maxo2p = max([n[0][vrr_axis(n)] - 1 for n in order if sum(n[1]) == 0 and sum(n[0]) > 0] + [0])
        maxo2q = max([n[1][vrr_axis(n)] - 1 for n in order if sum(n[1]) > 0] + [0])
        maxo2pq = max([n[0][vrr_axis(n)] for n in order if sum(n[1]) > 0] + [0])
        return used_m, maxo2p, maxo2q, maxo2pq

    # -- HRR ---------------------------------------------------------------------
    def emit_hrr(self, out, ind):
        c = self.contr
        la, lb, lc, ld = self.la, self.lb, self.lc, self.ld
        # bra HRR for every ket target f: (a,b|f) from (e,0|f)
        def bra_nodes(a_list):
            need = set()
            stack = list(a_list)
            while stack:
                n = stack.pop()
                if n in need:
                    continue
                need.add(n)
                a, b = n
                if sum(b) > 0:
                    i = pick_axis(b)
                    stack += [(add(a, i), sub(b, i)), (a, sub(b, i))]
            return sorted(need, key=lambda n: (sum(n[1]), n))

        bra_t = [(a, b) for a in comps(la) for b in comps(lb)]
        bnodes = bra_nodes(bra_t)

        def hname(a, b, f):
            if sum(b) == 0:
                return f"acc_{tname(a)}_{tname(f)}"
            return f"h{tname(a)}{tname(b)}_{tname(f)}"

        for f in self.fsets:
            for (a, b) in bnodes:
                if sum(b) == 0:
                    continue
                i = pick_axis(b)
                b1 = sub(b, i)
                out.append(f"{ind}const double {hname(a, b, f)} = fma(AB{AXES[i]}, {hname(a, b1, f)}, "
                           f"{hname(add(a, i), b1, f)});")
                c.fma += 1

        # ket HRR for every bra function pair (a,b): (ab|c,d) from (ab|e,0)
        knodes = bra_nodes([(cc, dd) for cc in comps(lc) for dd in comps(ld)])

        def kname(a, b, cc, dd):
            if sum(dd) == 0:
                return hname(a, b, cc)
            return f"k{tname(a)}{tname(b)}_{tname(cc)}{tname(dd)}"

        for a, b in bra_t:
            for (cc, dd) in knodes:
                if sum(dd) == 0:
                    continue
                i = pick_axis(dd)
                d1 = sub(dd, i)
                out.append(f"{ind}const double {kname(a, b, cc, dd)} = fma(CD{AXES[i]}, "
                           f"{kname(a, b, cc, d1)}, {kname(a, b, add(cc, i), d1)});")
                c.fma += 1
        k = 0
        for a in comps(la):
            for b in comps(lb):
                for cc in comps(lc):
                    for dd in comps(ld):
                        out.append(f"{ind}I[{k}] = {kname(a, b, cc, dd)};")
                        k += 1

    def emit_hrr_split(self, o):
        """The HRR as two one-dimensional transforms for the warp-cooperative epilogue:
        hrr_bra maps one ket component's column of contracted targets (e0|f) (e in esets
        order) to (ab|f); hrr_ket maps one bra function pair's row (ab|f0) (f in fsets
        order) to (ab|cd).  Same recursions and operation order as emit_hrr."""
        la, lb, lc, ld = self.la, self.lb, self.lc, self.ld

        def nodes(pairs):
            need = set()
            stack = list(pairs)
            while stack:
                n = stack.pop()
                if n in need:
                    continue
                need.add(n)
                a, b = n
                if sum(b) > 0:
                    i = pick_axis(b)
                    stack += [(add(a, i), sub(b, i)), (a, sub(b, i))]
            return sorted(need, key=lambda n: (sum(n[1]), n))

        for side, (l1, l2, src, D) in (("bra", (la, lb, self.esets, "AB")), ("ket", (lc, ld, self.fsets, "CD"))):
            outs = [(x, y) for x in comps(l1) for y in comps(l2)]
            nd = nodes(outs)

            def nm(x, y):
                return f"v{tname(x)}" if sum(y) == 0 else f"h{tname(x)}{tname(y)}"
            used = {x for (x, y) in nd if sum(y) == 0}
            o.append(f"  template <class In, class Out>")
            o.append(f"  static __device__ __forceinline__ void hrr_{side}(const In& in, double {D}x, double {D}y, "
                     f"double {D}z, Out&& out) {{")
            for k, e in enumerate(src):
                if e in used:
                    o.append(f"    const double {nm(e, (0, 0, 0))} = in[{k}];")
            for (x, y) in nd:
                if sum(y) == 0:
                    continue
                i = pick_axis(y)
                y1 = sub(y, i)
                o.append(f"    const double {nm(x, y)} = fma({D}{AXES[i]}, {nm(x, y1)}, {nm(add(x, i), y1)});")
            for k, (x, y) in enumerate(outs):
                o.append(f"    out({k}, {nm(x, y)});")
            o.append("  }")

    # -- Boys / quartet setup ----------------------------------------------------
    def emit_quartet_setup(self, out, ind, used_m, o2q, o2pq):
        c = self.prim
        M = self.L
        L = out.append
        L(f"{ind}const double pq = p + q;")
        L(f"{ind}const double rs = rsqrt(pq);")
        L(f"{ind}const double ipq = rs * rs;")
        L(f"{ind}const double PQx = Px - Qx, PQy = Py - Qy, PQz = Pz - Qz;")
        L(f"{ind}const double R2 = fma(PQz, PQz, fma(PQy, PQy, PQx * PQx));")
        L(f"{ind}const double qpq = q * ipq;")
        L(f"{ind}const double T = (p * qpq) * R2;")
        L(f"{ind}const double pre = (Kab * Kcd) * rs;")
        c.add += 4          # pq, PQ
        c.mul += 2 + 1 + 1 + 2 + 2   # ipq, PQx^2, qpq, T (2), pre (2)
        c.fma += 2
        c.add += 8          # rsqrt ~ (counted as 8 flops: approximation + Newton step)
        if M > 0:
            L(f"{ind}const double ppq = p * ipq;")
            L(f"{ind}const double WPx = -qpq * PQx, WPy = -qpq * PQy, WPz = -qpq * PQz;")
            L(f"{ind}const double WQx = ppq * PQx, WQy = ppq * PQy, WQz = ppq * PQz;")
            c.mul += 7
        for k in range(1, o2q + 1):
            L(f"{ind}const double oo2q_{k} = {float(k)} * oo2q;")
            c.mul += 1
        if o2pq:
            L(f"{ind}const double oo2pq_1 = 0.5 * ipq;")
            c.mul += 1
            for k in range(2, o2pq + 1):
                L(f"{ind}const double oo2pq_{k} = {float(k)} * oo2pq_1;")
                c.mul += 1
        # Boys F_0..F_M scaled by the prefactor
        L(f"{ind}double F[{M + 1}];")
        L(f"{ind}qb_boys_scaled<{M}>(T, pre, boys_tab, F);")
        for m in used_m:
            L(f"{ind}const double F{m} = F[{m}];")
        # Boys cost as emitted by qb_boys_scaled (qb_common.cuh), table branch: Taylor on
        # the Horner form (7 fma per order evaluated) and the prefactor scaling; for M > 2
        # one Horner evaluation, e^{-T} from the table (degree-8 Taylor, 2 mul) and the
        # downward recursion (fma + mul per order).
        if M <= 2:
            c.fma += 7 * (M + 1)
            c.mul += M + 1
        else:
            c.fma += 7 + 8 + M
            c.mul += 1 + 2 + M

    def generate(self):
        la, lb, lc, ld = self.la, self.lb, self.lc, self.ld
        na, nb, nc, nd = ncart(la), ncart(lb), ncart(lc), ncart(ld)
        nint = na * nb * nc * nd
        nt = len(self.esets) * len(self.fsets)
        body = []
        ind = "    "
        used_m, o2p, o2q, o2pq = self.emit_vrr(body, ind)
        setup = []
        self.emit_quartet_setup(setup, ind, used_m, o2q, o2pq)
        hrr = []
        self.emit_hrr(hrr, "    ")
        o = []
        o.append(f"// class ({la}{lb}|{lc}{ld}): {len(self.esets)}x{len(self.fsets)} contracted "
                 f"[e0|f0], {nint} integrals")
        o.append(f"template <> struct EriClass<{la}, {lb}, {lc}, {ld}> {{")
        o.append(f"  static constexpr int NA = {na}, NB = {nb}, NC = {nc}, ND = {nd}, NINT = {nint}, NT = {nt}, "
                 f"NE = {len(self.esets)}, NF = {len(self.fsets)};")
        o.append("  // VRR targets [e0|f0]^(0) of one primitive quartet (bra pair B, ket pair Kt), prefactor")
        o.append("  // included: sink(k, value) receives target k (in (e, f) order) as soon as it is final.")
        o.append("  template <class Sink>")
        o.append("  static __device__ __forceinline__ void prim(const PrimPair& B, const PrimPair& Kt,")
        o.append("                                              const double* __restrict__ boys_tab, Sink&& sink) {")
        o.append("    const double p = B.p, Px = B.Px, Py = B.Py, Pz = B.Pz, Kab = B.K;")
        if la + lb > 0:
            o.append("    const double PAx = B.PAx, PAy = B.PAy, PAz = B.PAz;")
        if o2p:
            o.append("    const double oo2p = B.oo2p;")
            for k in range(1, o2p + 1):
                o.append(f"    const double oo2p_{k} = {float(k)} * oo2p;")
        o.append("    const double q = Kt.p, Qx = Kt.Px, Qy = Kt.Py, Qz = Kt.Pz, Kcd = Kt.K;")
        if lc + ld > 0:
            o.append("    const double QCx = Kt.PAx, QCy = Kt.PAy, QCz = Kt.PAz;")
        if o2q:
            o.append("    const double oo2q = Kt.oo2p;")
        o += setup
        o += body
        o.append("  }")
        if self.seg:
            prim_head = o[o.index("  template <class Sink>") + 3: o.index(setup[0])]
            seg_body = []
            self.emit_vrr(seg_body, ind, seg=True)
            o.append(f"  // The same VRR for the segmented kernel: targets in emission order, {SEG_W} at a time,")
            o.append(f"  // go to red(batch, v0..v{SEG_W - 1}) ({self.seg_nbatch} batches; the slot of target k is")
            o.append("  // seg_pos()[k]).")
            o.append(f"  static constexpr int NSEGB = {self.seg_nbatch};")
            o.append(f"  static __device__ __forceinline__ const unsigned short* seg_pos() {{ return qb_seg_pos_{self.name}; }}")
            o.append("  template <class Red>")
            o.append("  static __device__ __forceinline__ void prim_seg(const PrimPair& B, const PrimPair& Kt,")
            o.append("                                                  const double* __restrict__ boys_tab, Red&& red) {")
            o += prim_head
            o += setup
            o += seg_body
            o.append("  }")
            table = (f"static __device__ const unsigned short qb_seg_pos_{self.name}[{len(self.seg_pos)}] = {{" +
                     ", ".join(str(v) for v in self.seg_pos) + "};")
            o.insert(o.index(f"template <> struct EriClass<{la}, {lb}, {lc}, {ld}> {{"), table)
        o.append("  // Contracted targets -> (ab|cd) block by the horizontal recursion.")
        o.append("  // A[k] is the contracted target k: a register array or a shared-memory row.")
        o.append("  template <class Acc>")
        o.append("  static __device__ __forceinline__ void hrr(const Acc& A, double ABx, double ABy, double ABz,")
        o.append("                                             double CDx, double CDy, double CDz, double (&I)[NINT]) {")
        k = 0
        for e in self.esets:
            for f in self.fsets:
                o.append(f"    const double acc_{tname(e)}_{tname(f)} = A[{k}];")
                k += 1
        o += hrr
        o.append("  }")
        o.append("  // The same HRR as two one-dimensional transforms (warp-cooperative epilogue).")
        self.emit_hrr_split(o)
        o.append("  // One contracted quartet in one thread: a flattened loop over the primitive quartets")
        o.append("  // whose screening keys (qb_kabs: |K|, or the primitive Schwarz factor; pairs sorted by")
        o.append("  // descending key) multiply to >= eps (eps = 0 evaluates all of them, as the Schwarz")
        o.append("  // factors need), then the HRR.")
        o.append("  static __device__ __forceinline__ void block(")
        o.append("      const PrimPair* __restrict__ bp, int nbp, const PrimPair* __restrict__ kp, int nkp,")
        o.append("      double ABx, double ABy, double ABz, double CDx, double CDy, double CDz,")
        o.append("      const double* __restrict__ boys_tab, double (&I)[NINT], unsigned& nprimq,")
        o.append("      const float eps = (float)QB_PRIM_EPS) {")
        o.append("    double A[NT];")
        o.append("#pragma unroll")
        o.append("    for (int t = 0; t < NT; ++t) A[t] = 0.0;")
        o.append("    const float kmax_ket = nkp > 0 ? qb_kabs(kp) : 0.f;")
        o.append("    int ib = 0, ik = 0;")
        o.append("    float kb = nbp > 0 ? qb_kabs(bp) : 0.f;")
        o.append("    bool active = nbp > 0 && nkp > 0 && kb * kmax_ket >= eps;")
        o.append("    PrimPair B;")
        o.append("    if (active) B = qb_load_pair(bp);")
        o.append("    while (active) {")
        o.append("      const PrimPair Kt = qb_load_pair(kp + ik);")
        o.append("      ++nprimq;")
        o.append("      prim(B, Kt, boys_tab, [&](int t, double v) { A[t] += v; });")
        o.append("      ++ik;")
        o.append("      if (ik >= nkp || kb * qb_kabs(kp + ik) < eps) {")
        o.append("        ++ib;")
        o.append("        ik = 0;")
        o.append("        if (ib >= nbp) {")
        o.append("          active = false;")
        o.append("        } else {")
        o.append("          kb = qb_kabs(bp + ib);")
        o.append("          if (kb * kmax_ket < eps) active = false;")
        o.append("          else B = qb_load_pair(bp + ib);")
        o.append("        }")
        o.append("      }")
        o.append("    }")
        o.append("    hrr(A, ABx, ABy, ABz, CDx, CDy, CDz, I);")
        o.append("  }")
        o.append("};")
        return "\n".join(o)


# Warp-cooperative kernel: 4 warps per block; each warp holds S rows of accumulators
# ((NT | 1) doubles each) for G <= 32 owner quartets in shared memory, within 50 KiB per
# warp (the rest of the 227 KiB is the kernel's static tables).  Configurations, as
# (S, regroup by Boys branch, plain adds for ranks < S-1):
#   1: S = 1, no regrouping (every add atomic; G = 32 where one row per owner fits)
#   2: S = 4 rows where they fit (else 3, 2), regrouping, plain adds
#   3: S = 2, regrouping, every add atomic
WARPS_PER_BLOCK = 4
SMEM_PER_WARP = 50 * 1024

# Default variant per class (0: per-thread kernel), measured on GB300 with the J/K build
# of 64 H + 16 C/N/O, 3-primitive s/p/d shells.  Classes not listed use variant 1.
PREFERRED = {"2211": 5, "2221": 5, "2111": 5, "2121": 5, "2220": 4, "2222": 4,
             "0000": 2, "1000": 2, "1010": 2, "1100": 2, "2000": 2, "2010": 2, "2100": 2,
             "1110": 3, "2020": 3}


# Segmented kernel (variant 5, classes with >= SEG_MIN_NT contracted targets): four lane
# segments of SEG_W lanes per warp, one contracted quartet per segment; the segment's
# lanes evaluate SEG_W of its primitive quartets at a time and reduce-scatter the targets
# over the segment (shuffles, no atomics) into the quartet's shared-memory row.
SEG_W = 8
SEG_MIN_NT = 90
SEG_STATIC_PER_WARP = 2560     # bytes of static shared memory per warp (tables) in qb_jk_seg_kernel
SEG_STAGE = 2 * 32 * 9         # doubles per warp of the reduce-scatter staging areas
SMEM_LIMIT = 227 * 1024


def seg_warps(nsegb, nab, nf, nint, nt):
    """Warps per block of the segmented kernel: as many as shared memory allows, at most 8,
    and 4 for the classes of >= 400 targets (at 8 warps ptxas gives their VRR 32 registers
    and keeps everything else in local memory; at 4 it uses 255)."""
    per_warp = 8 * (4 * nsegb * SEG_W + max(nab * nf + max(nint, nt), SEG_STAGE)) + SEG_STATIC_PER_WARP
    return max(1, min(8 if nt < 400 else 4, SMEM_LIMIT // per_warp))


COOP_MIN_NINT = 324   # classes with at least this many integrals get the cooperative epilogue
BIG_NT = 90           # classes with at least this many contracted targets get variant 4
SMEM_PER_WARP_8 = 24 * 1024   # variant 4 with 8 warps per block (two per SM sub-partition)


def warp_configs(nt, nint=0, nab=0, nf=0):
    """{variant: (G, S, regroup, plain, coop, warps per block)} of the warp kernel for a
    class with NT targets.  Variant 4, for the classes whose accumulators fill shared
    memory at four warps per block: eight warps per block with half the shared memory per
    warp (more warps to hide the FP64 and shared-memory latencies), four where that
    leaves fewer than two owners; coop (classes of >= 324 integrals): the whole warp runs
    each owner's HRR and J/K digestion from shared memory."""
    rows = SMEM_PER_WARP // ((nt | 1) * 8)
    cfg = {}
    if rows >= 1:
        if rows < 32:
            cfg[1] = (rows, 1, False, False, False, WARPS_PER_BLOCK)
        else:
            cfg[1] = (32, 1, False, False, False, WARPS_PER_BLOCK)
            s_max = min(4, rows // 32)
            if s_max >= 2:
                cfg[2] = (32, s_max, True, True, False, WARPS_PER_BLOCK)
                cfg[3] = (32, 2, True, False, False, WARPS_PER_BLOCK)
    if nt >= BIG_NT:
        coop = nint >= COOP_MIN_NINT
        extra = nab * nf + nint if coop else 0
        for per_warp, wpb in ((SMEM_PER_WARP_8, 8), (SMEM_PER_WARP, WARPS_PER_BLOCK)):
            g = (per_warp // 8 - extra) // (nt | 1)
            if g >= 2 or (wpb == WARPS_PER_BLOCK and g >= 1):
                cfg[4] = (min(32, g), 1, False, False, coop, wpb)
                break
    return cfg


HEADER = """// GENERATED by gen_eri.py -- do not edit.
#pragma once
#include "qb_common.cuh"
"""


def main(outdir, lmax=LMAX_DEFAULT):
    outdir = Path(outdir)
    outdir.mkdir(parents=True, exist_ok=True)
    table = {}
    files = []
    for cls in quartet_classes(lmax):
        g = ClassGen(*cls)
        code = g.generate()
        name = g.name
        (outdir / f"eri_class_{name}.cuh").write_text(HEADER + code + "\n")
        la, lb, lc, ld = cls
        nt = len(g.esets) * len(g.fsets)
        nint_c = ncart(la) * ncart(lb) * ncart(lc) * ncart(ld)
        cfgs = warp_configs(nt, nint_c, ncart(la) * ncart(lb), len(g.fsets))
        cu = [f'// GENERATED by gen_eri.py -- do not edit.',
              f'#include "eri_class_{name}.cuh"', '#include "eri_kernels.cuh"',
              f'QB_DEFINE_LAUNCHERS({la}, {lb}, {lc}, {ld})']
        jk, occ = [f"qb_jk_launch_{name}"], [f"qb_occ_{name}"]
        if g.seg:
            cfgs[5] = seg_warps(g.seg_nbatch, ncart(la) * ncart(lb), len(g.fsets), nint_c, nt)
        for v in (1, 2, 3, 4, 5):
            if v == 5 and v in cfgs:
                cu.append(f"QB_DEFINE_SEG_LAUNCHERS({v}, {la}, {lb}, {lc}, {ld}, {cfgs[5]})")
                jk.append(f"qb_jkw{v}_launch_{name}")
                occ.append(f"qb_occw{v}_{name}")
            elif v in cfgs:
                G_, S_, rg, pl, co, wpb = cfgs[v]
                cu.append(f"QB_DEFINE_WARP_LAUNCHERS({v}, {la}, {lb}, {lc}, {ld}, {wpb}, {G_}, {S_}, "
                          f"{'true' if rg else 'false'}, {'true' if pl else 'false'}, "
                          f"{'true' if co else 'false'})")
                jk.append(f"qb_jkw{v}_launch_{name}")
                occ.append(f"qb_occw{v}_{name}")
            else:
                jk.append("nullptr")
                occ.append("nullptr")
        pref = PREFERRED.get(name, 1 if 1 in cfgs else 0)
        schwarz, primkey = "nullptr", "nullptr"
        if (la, lb) == (lc, ld):
            cu.append(f"QB_DEFINE_SCHWARZ_LAUNCHER({la}, {lb})")
            schwarz, primkey = f"qb_schwarz_launch_{name}", f"qb_primkey_launch_{name}"
        cu.append(f"ClassLaunchers qb_class_{name}() {{ return {{{{{', '.join(jk)}}}, {{{', '.join(occ)}}}, "
                  f"{la}, {lb}, {lc}, {ld}, {pref}, {schwarz}, {primkey}}}; }}")
        (outdir / f"eri_class_{name}.cu").write_text("\n".join(cu) + "\n")
        files.append(name)
        table[name] = {"prim_flops": g.prim.flops(), "contr_flops": g.contr.flops(),
                       "nint": ncart(cls[0]) * ncart(cls[1]) * ncart(cls[2]) * ncart(cls[3]),
                       "jk_flops_per_int": 12, "vrr_nodes": len(g.vrr_nodes()[0])}
    disp = ['// GENERATED by gen_eri.py -- do not edit.', '#include "eri_kernels.cuh"']
    disp += [f"ClassLaunchers qb_class_{n}();" for n in files]
    disp.append(f"extern const int QB_NCLASS = {len(files)};")
    disp.append(f"extern const int QB_LMAX_SHELL = {lmax};")
    disp.append("extern const double QB_CLASS_PRIM_FLOPS[] = {" +
                ", ".join(f"{table[n]['prim_flops']}.0" for n in files) + "};")
    disp.append("extern const double QB_CLASS_CONTR_FLOPS[] = {" +
                ", ".join(f"{table[n]['contr_flops'] + 12 * table[n]['nint']}.0" for n in files) + "};")
    disp.append("extern const int QB_CLASS_NINT[] = {" + ", ".join(str(table[n]['nint']) for n in files) + "};")
    disp.append("void qb_get_class_launchers(ClassLaunchers* out) {")
    disp += [f"  out[{k}] = qb_class_{n}();" for k, n in enumerate(files)]
    disp.append("}")
    (outdir / "eri_dispatch.cu").write_text("\n".join(disp) + "\n")
    (outdir / "eri_classes.json").write_text(json.dumps({"lmax": lmax, "classes": files}, indent=1))
    return table


if __name__ == "__main__":
    args = sys.argv[1:]
    lmax = LMAX_DEFAULT
    if "--lmax" in args:
        k = args.index("--lmax")
        lmax = int(args[k + 1])
        del args[k:k + 2]
    tab = main(args[0] if args else "gen", lmax)
    flops_out = Path(__file__).with_name("flops_table.json")
    if "--write-flops" in sys.argv:
        flops_out.write_text(json.dumps({"unit": "FP64 flops (add/mul 1, fma 2)", "lmax": lmax,
                                         "classes": tab}, indent=1))
    for k, v in tab.items():
        print(k, v)
