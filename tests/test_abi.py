"""The C-ABI library builds, loads and exports every entry point of include/inca_gpu.h (CPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from inca_parallel_gb300 import build
    build.build()
    from inca_parallel_gb300 import _lib
    return _lib.load()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "inca_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(inca_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    from inca_parallel_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_abi_version(lib):
    assert lib.inca_abi_version() == 2


def test_struct_layouts_match_header(tmp_path):
    # the ctypes mirrors of the header's structs: same fields at the same offsets, same size
    # (compiled against include/inca_gpu.h with the host C compiler)
    import ctypes
    import shutil
    import subprocess
    from inca_parallel_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = {"inca_tuning": _lib.Tuning, "inca_counts": _lib.Counts}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "inca_gpu.h"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append(f'printf("{name} . %zu\\n", sizeof({name}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        name, field, val = ln.split()
        got[(name, field)] = int(val)
    for name, cls in structs.items():
        assert got[(name, ".")] == ctypes.sizeof(cls), name
        for f, _ in cls._fields_:
            assert got[(name, f)] == getattr(cls, f).offset, (name, f)


def test_centercalc_matches_oracle(lib):
    import numpy as np
    import oracle_lib as O
    from inca_parallel_gb300 import centercalc
    rng = np.random.default_rng(7)
    an = np.array([6, 8, 1, 7, 1, 6])
    cart = rng.uniform(-3, 3, size=(6, 3))
    for nohydro in (True, False):
        a = centercalc(an, cart, nohydro=nohydro)
        b = O.centercalc(an, cart, nohydro=nohydro)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)


def test_context_without_gpu_fails_loudly(lib):
    # in a container without a GPU the context must not silently fall back to the CPU
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from inca_parallel_gb300 import Context, IncaError
    with pytest.raises(IncaError):
        Context(0)


def test_driver_built():
    from inca_parallel_gb300 import build
    build.build()
    assert os.access(build.DRIVER, os.X_OK)
