"""Generate ``quad_tables.inc``: the quadrature rules the DG space uses.

The triangle rules are tabulated data (Intrepid2 / Dunavant rules on the reference
triangle (0,0),(1,0),(0,1), weights summing to 1/2) and the 1D Gauss-Legendre rules
on [-1, 1].  FP64 parity with dgfem needs bit-identical rules, so the numbers are
read from dgfem's own table (``dgfem/src/quadrature/factory.cpp``:
``get_dunavant_rule`` lines 238-717 and ``compute_gauss_legendre`` lines 75-236)
and re-emitted as shortest round-trip decimal literals.  Every literal or constant
expression in that file is evaluated here in IEEE double arithmetic, which is what
a C++ compiler does for the same ``constexpr`` expressions.

Usage:  python gen_quad_tables.py <path to dgfem/src/quadrature/factory.cpp> [out]

The generated file is committed; this script only needs re-running if the rules
change.  It is not used at build or run time.
"""

import math
import re
import sys
from pathlib import Path

ONE_THIRD = 1.0 / 3.0
ONE_HALF = 0.5
ONE_SIXTH = 1.0 / 6.0


def _eval(expr: str, env: dict) -> float:
    expr = expr.strip()
    if not re.fullmatch(r"[0-9eE+\-*/(). _a-z]+", expr):
        raise ValueError(f"unexpected expression {expr!r}")
    return float(eval(expr, {"__builtins__": {}}, dict(env)))


def parse_dunavant(src: str) -> dict:
    body = src[src.index("void QuadratureFactory::get_dunavant_rule"):]
    # split on "case N:" labels; consecutive labels share one block
    parts = re.split(r"\n\s*case (\d+):", body)
    env = {"one_third": ONE_THIRD, "one_half": ONE_HALF, "one_sixth": ONE_SIXTH}
    rules, pending = {}, []
    for i in range(1, len(parts), 2):
        order = int(parts[i])
        block = parts[i + 1]
        pending.append(order)
        if "resize(" not in block and "get_dunavant_rule(" not in block:
            continue  # label without its own block (fall-through)
        m = re.search(r"get_dunavant_rule\((\d+)", block)
        if m:
            rule = rules[int(m.group(1))]
        else:
            n = int(re.search(r"points\.resize\((\d+), 2\)", block).group(1))
            pts = [[None, None] for _ in range(n)]
            wts = [None] * n
            for q, c, e in re.findall(r"points\((\d+), (\d)\) = ([^;]+);", block):
                pts[int(q)][int(c)] = _eval(e, env)
            # chained assignments: "weights[0] = weights[1] = weights[2] = one_sixth;"
            for stmt in re.findall(r"((?:weights\[\d+\] = )+[^;]+);", block):
                lhs = re.findall(r"weights\[(\d+)\] =", stmt)
                val = _eval(stmt.split("=")[-1], env)
                for q in lhs:
                    wts[int(q)] = val
            if any(v is None for row in pts for v in row) or any(w is None for w in wts):
                raise ValueError(f"incomplete rule for order {order}")
            rule = (pts, wts)
        for o in pending:
            rules[o] = rule
        pending = []
    return rules


def gauss_legendre() -> dict:
    """The 1-8 point rules exactly as dgfem's compute_gauss_legendre builds them."""
    sqrt_3_inv = 1.0 / 1.732050807568877293527446341505872366942805253810380628055
    sqrt_3_5 = 0.774596669241483377035853079956479922166584341058318165320
    w_5_9 = 5.0 / 9.0
    w_8_9 = 8.0 / 9.0
    r = {1: ([0.0], [2.0]),
         2: ([-sqrt_3_inv, sqrt_3_inv], [1.0, 1.0]),
         3: ([-sqrt_3_5, 0.0, sqrt_3_5], [w_5_9, w_8_9, w_5_9])}
    sqrt_6_5 = 1.095445115010332226913939565601604642850062938142840310385
    a = math.sqrt(3.0 / 7.0 - 2.0 / 7.0 * sqrt_6_5)
    b = math.sqrt(3.0 / 7.0 + 2.0 / 7.0 * sqrt_6_5)
    sqrt_30 = 5.477225575051661134569697828008021321125314690714201551925
    w1 = (18.0 + sqrt_30) / 36.0
    w2 = (18.0 - sqrt_30) / 36.0
    r[4] = ([-b, -a, a, b], [w2, w1, w1, w2])
    return r


def parse_gl_tabulated(src: str, rules: dict) -> dict:
    """Cases 5-8 of compute_gauss_legendre are literal tables."""
    body = src[src.index("void QuadratureFactory::compute_gauss_legendre"):
               src.index("void QuadratureFactory::get_dunavant_rule")]
    for n in (5, 6, 7, 8):
        blk = body[body.index(f"case {n}: {{"):]
        blk = blk[:blk.index("break;")]
        env = dict(re.findall(r"constexpr double (\w+) = ([0-9.eE+\-]+);", blk))
        env = {k: float(v) for k, v in env.items()}
        pts = [None] * n
        wts = [None] * n
        for q, e in re.findall(r"points\[(\d+)\] = ([^;]+);", blk):
            pts[int(q)] = _eval(e, env)
        for q, e in re.findall(r"weights\[(\d+)\] = ([^;]+);", blk):
            wts[int(q)] = _eval(e, env)
        rules[n] = (pts, wts)
    return rules


def emit(dun: dict, gl: dict) -> str:
    out = ["// Generated by gen_quad_tables.py from dgfem/src/quadrature/factory.cpp",
           "// (get_dunavant_rule lines 238-717, compute_gauss_legendre lines 75-236).",
           "// Do not edit: values are shortest round-trip decimal forms of the doubles.",
           ""]
    orders = sorted(dun)
    out.append(f"#define DGX_TRI_MAX_ORDER {max(orders)}")
    out.append("static const int dgx_tri_rule_npts[] = {" +
               ", ".join(str(len(dun[o][1])) for o in orders) + "};")
    flat_p, flat_w, offs = [], [], []
    for o in orders:
        offs.append(len(flat_w))
        pts, wts = dun[o]
        for p in pts:
            flat_p += p
        flat_w += wts
    out.append("static const int dgx_tri_rule_offset[] = {" + ", ".join(map(str, offs)) + "};")
    out.append("static const double dgx_tri_rule_points[] = {")
    out += [f"    {repr(a)}, {repr(b)}," for a, b in zip(flat_p[0::2], flat_p[1::2])]
    out.append("};")
    out.append("static const double dgx_tri_rule_weights[] = {")
    out += [f"    {repr(w)}," for w in flat_w]
    out.append("};")
    out.append(f"#define DGX_GL_MAX_POINTS {max(gl)}")
    out.append("static const double dgx_gl_points[][8] = {")
    for n in range(1, max(gl) + 1):
        out.append("    {" + ", ".join(repr(x) for x in gl[n][0]) + "},")
    out.append("};")
    out.append("static const double dgx_gl_weights[][8] = {")
    for n in range(1, max(gl) + 1):
        out.append("    {" + ", ".join(repr(x) for x in gl[n][1]) + "},")
    out.append("};")
    return "\n".join(out) + "\n"


def main(argv):
    src = Path(argv[1]).read_text()
    out = Path(argv[2]) if len(argv) > 2 else Path(__file__).with_name("quad_tables.inc")
    dun = parse_dunavant(src)
    gl = parse_gl_tabulated(src, gauss_legendre())
    out.write_text(emit(dun, gl))
    print(f"wrote {out}: triangle orders {sorted(dun)}, GL points 1..{max(gl)}")


if __name__ == "__main__":
    main(sys.argv)
