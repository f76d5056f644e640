"""Copy the reference's CH4 test fixtures and golden outputs into tests/golden/.

Source: the reference repository's own test suite (tests/data/ch4.{fchk,dm2p},
tests/data/ch4_ops.bas, tests/refs/ch4_ref.{rad,cube}, tests/inputs/test_*.inp and the
scalar goldens of tests/run_tests.py:24-28). Large files are gzip-compressed. Run once,
where the reference tree is mounted:

    python tests/golden/make_fixtures.py /path/to/reference
"""
import gzip
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    data = os.path.join(ref, "tests", "data")
    refs = os.path.join(ref, "tests", "refs")
    inputs = os.path.join(ref, "tests", "inputs")
    shutil.copy(os.path.join(data, "ch4.fchk"), os.path.join(HERE, "ch4.fchk"))
    shutil.copy(os.path.join(data, "ch4_ops.bas"), os.path.join(HERE, "ch4_ops.bas"))
    for src, dst in [(os.path.join(data, "ch4.dm2p"), "ch4.dm2p.gz"),
                     (os.path.join(refs, "ch4_ref.cube"), "ch4_ref.cube.gz")]:
        with open(src, "rb") as f, gzip.GzipFile(os.path.join(HERE, dst), "wb", mtime=0) as g:
            g.write(f.read())
    shutil.copy(os.path.join(refs, "ch4_ref.rad"), os.path.join(HERE, "ch4_ref.rad"))
    os.makedirs(os.path.join(HERE, "inputs"), exist_ok=True)
    for name in sorted(os.listdir(inputs)):
        if name.endswith(".inp"):
            shutil.copy(os.path.join(inputs, name), os.path.join(HERE, "inputs", name))
    # scalar goldens of the Methane system (tests/run_tests.py:19-28)
    text = open(os.path.join(ref, "tests", "run_tests.py")).read()
    block = text[text.index('"name": "Methane"'):]
    block = block[:block.index("}")]
    val = float(re.search(r'"val":\s*([-0-9.eE+]+)', block).group(1))
    err = float(re.search(r'"err":\s*([-0-9.eE+]+)', block).group(1))
    zero = float(re.search(r'"zero":\s*([-0-9.eE+]+)', block).group(1))
    tp = re.search(r'"two_points":\s*\(([-0-9.eE+]+),\s*([-0-9.eE+]+)\)', block)
    tol = float(re.search(r"TOLERANCE\s*=\s*([-0-9.eE+]+)", text).group(1))
    gold = {"radial_integral": val, "radial_integral_error": err, "intracule_at_zero": zero,
            "two_points": [float(tp.group(1)), float(tp.group(2))], "reference_tolerance": tol,
            "source": "tests/run_tests.py:14,24-28 of the reference"}
    with open(os.path.join(HERE, "ch4_goldens.json"), "w") as f:
        json.dump(gold, f, indent=1)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <reference checkout>")
    main(sys.argv[1])
