"""Generate ``lebedev_table.h``: the Lebedev-Laikov orbit generators for the 32 rules.

The Lebedev-Laikov rules (V.I. Lebedev and D.N. Laikov, Doklady Mathematics 59 (1999)
477-481) are published as a list of octahedral orbit generators per rule: an orbit type
(1..6), its free coordinates ``a`` (and ``b``) and the weight ``v`` (weights sum to 1).
INCA uses them through ``LD0006`` ... ``LD5810`` (src/lebedev.f, ``gen_oh`` at lines 1-588).

This script reads the same published literals from SciPy's independent distribution of the
rules (``scipy.integrate._lebedev.get_lebedev_sphere``) and writes them as a C table. The
orbit expansion itself is written in ``host_tables.cpp``. Run it from the repository root:

    python inca_parallel_gb300/csrc/gen_lebedev.py

The output is committed; the GPU build does not need SciPy.
"""
import inspect
import os
import re

import scipy.integrate._lebedev as _leb

RULES = [6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194, 230, 266, 302, 350, 434, 590, 770,
         974, 1202, 1454, 1730, 2030, 2354, 2702, 3074, 3470, 3890, 4334, 4802, 5294, 5810]
ORBIT_SIZE = {1: 6, 2: 12, 3: 8, 4: 24, 5: 24, 6: 48}


def extract():
    src = inspect.getsource(_leb.get_lebedev_sphere)
    rules = {}
    cur = None
    vals = {}
    for line in src.splitlines():
        s = line.strip()
        m = re.match(r"case (\d+):", s)
        if m:
            cur = int(m.group(1))
            rules[cur] = []
            vals = {}
            continue
        m = re.match(r"([abv]) = ([-+0-9.Ee]+)$", s)
        if m and cur is not None:
            vals[m.group(1)] = m.group(2)
            continue
        m = re.match(r"leb_tmp, start = get_lebedev_recurrence_points\((\d), start, a, b, v, leb_tmp\)", s)
        if m and cur is not None:
            code = int(m.group(1))
            a = vals.get("a", "0.0") if code in (4, 5, 6) else "0.0"
            b = vals.get("b", "0.0") if code == 6 else "0.0"
            rules[cur].append((code, a, b, vals["v"]))
    return rules


def main():
    rules = extract()
    out = []
    out.append("// Generated by gen_lebedev.py from the published Lebedev-Laikov generator literals.")
    out.append("// Do not edit. Each row: orbit type (1..6), a, b, v; weights of a rule sum to 1.")
    out.append("#pragma once")
    out.append("namespace inca_leb {")
    out.append("struct Orbit { int code; double a, b, v; };")
    offs = [0]
    rows = []
    for n in RULES:
        orb = rules[n]
        tot = sum(ORBIT_SIZE[o[0]] for o in orb)
        assert tot == n, (n, tot)
        rows.extend(orb)
        offs.append(len(rows))
    out.append(f"static const int kNumRules = {len(RULES)};")
    out.append("static const int kRulePoints[kNumRules] = {" + ", ".join(map(str, RULES)) + "};")
    out.append("static const int kRuleOffset[kNumRules + 1] = {" + ", ".join(map(str, offs)) + "};")
    out.append(f"static const Orbit kOrbits[{len(rows)}] = {{")
    for (c, a, b, v) in rows:
        out.append(f"  {{{c}, {a}, {b}, {v}}},")
    out.append("};")
    out.append("}  // namespace inca_leb")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lebedev_table.h")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", path, len(rows), "orbits")


if __name__ == "__main__":
    main()
