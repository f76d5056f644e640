"""Generate ``hermite_table.h``: Gauss-Hermite nodes and weights for n = 1..11 nodes.

INCA integrates the per-dimension Cioslowski-Liu polynomial with an n-point Gauss-Hermite
rule, n = floor(L/2) + 1 for a total power L (src/mod_intrastuff.f90:198-341, ``gauherm``),
and screens with the largest root of the Hermite polynomial with t_i + t_k + 1 roots
(src/mod_intrastuff.f90:43-113, ``JA8``). This script computes the roots of the physicists'
Hermite polynomials H_n to 30 significant digits with SymPy and the weights with the
classical formula w_i = 2^(n-1) n! sqrt(pi) / (n^2 H_(n-1)(x_i)^2), then writes them as
double literals (ascending node order). Run from the repository root:

    python inca_parallel_gb300/csrc/gen_hermite.py
"""
import os

import sympy as sp

NMAX = 11


def main():
    x = sp.Symbol("x")
    rows = []
    for n in range(1, NMAX + 1):
        Hn = sp.hermite(n, x)
        Hm = sp.hermite(n - 1, x)
        roots = sorted(sp.Poly(Hn, x).nroots(n=40, maxsteps=200), key=lambda r: float(sp.re(r)))
        nodes = []
        for r in roots:
            r = sp.re(r)
            w = (sp.Integer(2) ** (n - 1) * sp.factorial(n) * sp.sqrt(sp.pi)) / (n * n * Hm.subs(x, r) ** 2)
            nodes.append((sp.N(r, 30), sp.N(w, 30)))
        rows.append(nodes)
    out = ["// Generated by gen_hermite.py (SymPy, 30 digits). Do not edit.",
           "// Gauss-Hermite rule with n nodes (weight exp(-x^2)), ascending nodes.",
           "#pragma once",
           "namespace inca_gh {",
           f"static const int kMaxNodes = {NMAX};",
           f"static const double kNode[{NMAX + 1}][{NMAX}] = {{",
           "  {" + ", ".join(["0.0"] * NMAX) + "},"]
    for nodes in rows:
        vals = [f"{float(r):.17e}" if False else sp.sstr(r) for r, _ in nodes] + ["0.0"] * (NMAX - len(nodes))
        out.append("  {" + ", ".join(vals) + "},")
    out.append("};")
    out.append(f"static const double kWeight[{NMAX + 1}][{NMAX}] = {{")
    out.append("  {" + ", ".join(["0.0"] * NMAX) + "},")
    for nodes in rows:
        vals = [sp.sstr(w) for _, w in nodes] + ["0.0"] * (NMAX - len(nodes))
        out.append("  {" + ", ".join(vals) + "},")
    out.append("};")
    out.append("}  // namespace inca_gh")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hermite_table.h")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
