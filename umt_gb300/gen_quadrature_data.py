"""Regenerate umt_gb300/quadrature_data.py from the UMT source tree.

The product-quadrature ordinates and weights of Teton are tabulated numbers
(mods/QuadratureData_mod.F90:1144-2839: first/last offsets per order, and
cosTheta / weightTheta / cosPhiXYZ / weightPhiXYZ, and cosPhiRZ / weightPhiRZ
for the 2-D RZ product set).  Directions must be
identical to the reference's for parity, so the tables are extracted
verbatim as data by this script (run on a machine that has the source tree):

    python -m umt_gb300.gen_quadrature_data PATH_TO_UMT_SOURCE_TREE
"""
import re
import sys

NAMES = ["first", "last", "cosTheta", "weightTheta", "cosPhiXYZ", "weightPhiXYZ", "cosPhiRZ", "weightPhiRZ"]


def parse(path):
    text = open(path).read()
    out = {}
    for name in NAMES:
        m = re.search(r"data\s+%s\s*/(.*?)/" % name, text, re.S)
        body = m.group(1)
        body = "\n".join(l.split("!")[0] for l in body.splitlines())
        toks = [t.strip() for t in body.replace("&", " ").split(",") if t.strip()]
        if name in ("first", "last"):
            out[name] = [int(t) for t in toks]
        else:
            out[name] = [float(t.replace("_adqt", "").replace("d", "e")) for t in toks]
    return out


def main(root):
    d = parse(root.rstrip("/") + "/src/teton/mods/QuadratureData_mod.F90")
    assert len(d["first"]) == 32 and all(len(d[n]) == 528 for n in NAMES[2:])
    lines = ['"""Product-quadrature tables (generated by gen_quadrature_data.py; data only).',
             "",
             "Extracted from the Teton source tree, mods/QuadratureData_mod.F90:1144-2839.",
             "Entries for order n occupy [first[n-1]-1, last[n-1]) of each list.",
             '"""', ""]
    for n in NAMES:
        vals = d[n]
        fmt = (lambda v: "%d" % v) if n in ("first", "last") else (lambda v: repr(v))
        lines.append("%s = [" % n)
        for i in range(0, len(vals), 4):
            lines.append("    " + ", ".join(fmt(v) for v in vals[i:i + 4]) + ",")
        lines.append("]")
        lines.append("")
    open(__file__.replace("gen_quadrature_data.py", "quadrature_data.py"), "w").write("\n".join(lines))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python -m umt_gb300.gen_quadrature_data PATH_TO_UMT_SOURCE_TREE")
    main(sys.argv[1])
