"""Recipe: derive the Shan-Chen psi-gradient stencils from the reference source.

The wall-aware isotropic gradient of the reference (lbm_forcing.F90,
LBMAddFluidFluidForcesD3 :51-958 and LBMAddFluidFluidForcesD2 :960-1299) is a
long hand-unrolled list of ``if (walls(...).eq.0 ...) then`` blocks.  Parity
at the level of rounding needs the SAME term order, the same multipliers and
the same wall-path conditions, so this recipe reads that file and emits:

* ``oracle/ff_stencil_oracle.h``  - one explicit C block per reference term,
  used by the CPU oracle (a literal restatement of each block);
* ``taxila-lbm_gb300/csrc/tx_ff_stencil.cuh`` - a compact term table (offset,
  weight index, auxiliary path cells and a truth table over them) used by the
  CUDA kernels.

Both files are committed; ``tests/test_stencil_pin.py`` re-parses the
reference (when it is present) and checks the committed table term by term.

Usage:  python oracle/ff_stencil_parse.py [path/to/lbm_forcing.F90]
"""
import os
import re
import sys

# the reference checkout (TAXILA_REFERENCE overrides the default location)
DEFAULT_SRC = os.path.join(os.environ.get("TAXILA_REFERENCE", "/root/reference"), "src/lbm/lbm_forcing.F90")
AXIS = {"X_DIRECTION": 0, "Y_DIRECTION": 1, "Z_DIRECTION": 2}


def _logical_lines(path, sub):
    """Join Fortran continuation lines of subroutine ``sub``; keep line numbers."""
    raw = open(path).read().split("\n")
    out, buf, first = [], "", None
    for no, ln in enumerate(raw, 1):
        st = ln.strip()
        if st.startswith("!"):
            out.append((no, st))
            continue
        code = ln.split("!")[0].rstrip()
        if first is None:
            first = no
        if code.endswith("&"):
            buf += code[:-1] + " "
            continue
        out.append((first, (buf + code).strip()))
        buf, first = "", None
    start = next(i for i, (_, l) in enumerate(out) if l.startswith("subroutine " + sub + "("))
    end = next(i for i, (_, l) in enumerate(out) if i > start and l.startswith("end subroutine " + sub))
    return out[start:end]


def _offset(text, nd):
    parts = [p.replace(" ", "") for p in text.split(",")]
    res = []
    for p, v in zip(parts, "ijk"[:nd]):
        assert p.startswith(v), (p, v)
        res.append(int(p[1:]) if len(p) > 1 else 0)
    return tuple(res)


def parse(sub, nd, path=DEFAULT_SRC):
    """Return the ordered list of gradient terms of one reference subroutine."""
    terms, level, cur = [], 4, None
    for lineno, l in _logical_lines(path, sub):
        if "order isotropy" in l:
            level = int(re.search(r"(\d+)th order", l).group(1))
            continue
        if l.startswith("!"):
            continue
        m = re.match(r"if\s*\((.*)\)\s*then$", l)
        if m and "walls(" in m.group(1):
            cells = []

            def rep(mm):
                o = _offset(mm.group(1), nd)
                if o not in cells:
                    cells.append(o)
                return "F[%d]" % cells.index(o)

            expr = re.sub(r"walls\(([^)]*)\)\s*\.eq\.\s*0(\.d0|\.(?![a-z]))?(?![0-9])", rep, m.group(1))
            expr = expr.replace(".and.", " and ").replace(".or.", " or ")
            cur = dict(line=lineno, cells=cells, expr=expr, level=level, grad={}, ws={})
            terms.append(cur)
            continue
        if cur is None:
            continue
        s = l.replace(" ", "")
        m = re.match(r"gradrho\(:,(\w+),[ijk,]+\)=gradrho\(:,\w+,[ijk,]+\)([+-])(?:(\d)\.\*)?"
                     r"dist%disc%ffw\((\d+)\)\*\(rho\(:,([^)]*)\)-rho\(:,[ijk,]+\)\)$", s)
        if m:
            ax = AXIS[m.group(1)]
            sign = 1 if m.group(2) == "+" else -1
            mult = int(m.group(3) or 1)
            assert _offset(m.group(5), nd) == cur["cells"][0], (lineno, l)
            assert ax not in cur["grad"]
            cur["grad"][ax] = (sign, mult, int(m.group(4)))
            continue
        m = re.match(r"weightsum\((\w+)\)=weightsum\(\w+\)\+dist%disc%ffw\((\d+)\)(?:\*(\d)\.)?$", s)
        if m:
            ax = AXIS[m.group(1)]
            assert ax not in cur["ws"]
            cur["ws"][ax] = (int(m.group(3) or 1), int(m.group(2)))
            continue
        assert not (s.startswith("gradrho") or s.startswith("weightsum(")), ("unparsed", lineno, l)
    return [t for t in terms if t["grad"]]


def truth_table(t):
    """Bit b set <=> the term is taken when aux cell q is fluid iff bit q of b."""
    aux = t["cells"][1:]
    tt = 0
    for bits in range(1 << len(aux)):
        F = [True] + [bool((bits >> q) & 1) for q in range(len(aux))]
        if eval(t["expr"], {"F": F}):
            tt |= 1 << bits
        F[0] = False
        assert not eval(t["expr"], {"F": F})
    return tt


def check_geometry(t, nd):
    e = t["cells"][0]
    for ax in range(nd):
        g, w = t["grad"].get(ax), t["ws"].get(ax)
        if e[ax] == 0:
            assert g is None and w is None, t
        else:
            assert g[0] * g[1] == e[ax] and w[0] == e[ax] ** 2 and g[2] == w[1], t


def emit_oracle(terms, nd, name):
    """Explicit C statements, one block per reference term, same expression shapes."""
    out = ["/* %s: %d terms, reference order */" % (name, len(terms)),
           "#define %s(WALL, RHO, GR, WS, FFW, NS) do { \\" % name]
    for t in terms:
        e = t["cells"][0]
        cond = t["expr"]
        for q, c in enumerate(t["cells"]):
            cond = cond.replace("F[%d]" % q, "WALL(%s)" % ",".join(str(v) for v in (list(c) + [0] * (3 - nd))))
        cond = cond.replace(" and ", " && ").replace(" or ", " || ")
        body = []
        off = ",".join(str(v) for v in (list(e) + [0] * (3 - nd)))
        for ax in range(nd):
            if ax in t["grad"]:
                sign, mult, w = t["grad"][ax]
                coef = ("%d.0*FFW[%d]" % (mult, w)) if mult != 1 else ("FFW[%d]" % w)
                body.append("for (int mm_ = 0; mm_ < NS; ++mm_) GR(mm_,%d) = GR(mm_,%d) %s %s*(RHO(mm_,%s) - RHO(mm_,0,0,0));"
                            % (ax, ax, "+" if sign > 0 else "-", coef, off))
        for ax in range(nd):
            if ax in t["ws"]:
                mult, w = t["ws"][ax]
                body.append("WS[%d] = WS[%d] + FFW[%d]%s;" % (ax, ax, w, ("*%d.0" % mult) if mult != 1 else ""))
        guard = "" if t["level"] == 4 else ("if (ISO > %d) " % (4 if t["level"] == 8 else 8))
        out.append("  /* lbm_forcing.F90:%d */ %sif (%s) { %s } \\" % (t["line"], guard, cond, " ".join(body)))
    out.append("} while (0)")
    return "\n".join(out) + "\n"


def emit_table(terms, nd, name):
    """constexpr accessor ``name(t)`` returning term t as a tx::FFTerm."""
    rows = []
    for idx, t in enumerate(terms):
        e = list(t["cells"][0]) + [0] * (3 - nd)
        aux = [list(c) + [0] * (3 - nd) for c in t["cells"][1:]]
        aux += [[0, 0, 0]] * (4 - len(aux))
        w = next(iter(t["grad"].values()))[2]
        auxs = ", ".join("{%d, %d, %d}" % tuple(a) for a in aux)
        rows.append("    case %d: return FFTerm{{%d, %d, %d}, %d, %d, %d, {%s}, 0x%xu};  // lbm_forcing.F90:%d"
                    % (idx, e[0], e[1], e[2], w, t["level"], len(t["cells"]) - 1, auxs, truth_table(t), t["line"]))
    return ("constexpr int %s_COUNT = %d;\n__host__ __device__ constexpr FFTerm %s(int t) {\n  switch (t) {\n%s\n"
            "    default: return FFTerm{{0, 0, 0}, 0, 0, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0u};\n  }\n}\n"
            % (name.upper(), len(terms), name, "\n".join(rows)))


def main(path=DEFAULT_SRC):
    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(here)
    d3 = parse("LBMAddFluidFluidForcesD3", 3, path)
    d2 = parse("LBMAddFluidFluidForcesD2", 2, path)
    for t in d3:
        check_geometry(t, 3)
    for t in d2:
        check_geometry(t, 2)
    hdr = ("/* Generated by oracle/ff_stencil_parse.py from the reference's lbm_forcing.F90.\n"
           " * Oracle-only: explicit restatement of the wall-aware psi-gradient blocks.\n"
           " * WALL(dx,dy,dz) is true when the neighbour is pore space; RHO(m,dx,dy,dz) is psi;\n"
           " * GR(m,axis) and WS[axis] are the per-cell accumulators; ISO is the isotropy order. */\n")
    with open(os.path.join(here, "ff_stencil_oracle.h"), "w") as f:
        f.write(hdr + emit_oracle(d3, 3, "ORC_FF_GRADIENT_D3") + emit_oracle(d2, 2, "ORC_FF_GRADIENT_D2"))
    thdr = ("/* Generated by oracle/ff_stencil_parse.py from the reference's lbm_forcing.F90\n"
            " * (LBMAddFluidFluidForcesD3 :51-958, LBMAddFluidFluidForcesD2 :960-1299).\n"
            " * One row per gradient term in the reference's accumulation order:\n"
            " *   e      neighbour offset; the term adds (e_d * w) * (psi(x+e) - psi(x)) to\n"
            " *          grad_d and (e_d^2 * w) to weightsum_d for every axis with e_d != 0;\n"
            " *   w      index into the isotropy weight vector ffw (1-based);\n"
            " *   level  4, 8 or 10: the term is used when isotropy_order >= level;\n"
            " *   naux/aux  path cells between x and x+e; bit b of truth is set when the\n"
            " *          term is taken with aux cell q pore space iff bit q of b is set\n"
            " *          (x+e itself must always be pore space). */\n"
            "#pragma once\nnamespace tx {\n"
            "struct FFTerm { int e[3]; int w; int level; int naux; int aux[4][3]; unsigned truth; };\n")
    with open(os.path.join(repo, "taxila-lbm_gb300", "csrc", "tx_ff_stencil.cuh"), "w") as f:
        f.write(thdr + emit_table(d3, 3, "ff_d3") + emit_table(d2, 2, "ff_d2") + "}  // namespace tx\n")
    print("D3 terms", len(d3), "D2 terms", len(d2))


if __name__ == "__main__":
    main(*(sys.argv[1:2]))
