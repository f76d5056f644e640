"""ctypes access to the CPU oracle (oracle/inca_oracle.cpp) and fixture parsers for tests.

Test infrastructure only: used by tests/, __graft_entry__.smoke() and the CPU-baseline leg
of bench.py as the checker. The parsers here follow the reference's readers
(src/mod_read_files.f90:432-726 for .fchk/.bas, src/mod_intracule.f90:164-262 for .dm2p).
"""
import ctypes
import gzip
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "oracle"))

_lib = None
DP = ctypes.POINTER(ctypes.c_double)
IP = ctypes.POINTER(ctypes.c_int)
LP = ctypes.POINTER(ctypes.c_long)
U8P = ctypes.POINTER(ctypes.c_ubyte)
MAXCOEF = 17


def lib():
    global _lib
    if _lib is None:
        import build as obuild  # oracle/build.py
        path = obuild.build()
        _lib = ctypes.CDLL(path)
        L = _lib
        L.orc_lebedev.argtypes = [ctypes.c_int, DP, DP, DP, DP]
        L.orc_gauleg.argtypes = [ctypes.c_int, DP, DP]
        L.orc_normprim.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_normprim.restype = ctypes.c_double
        L.orc_lu_solve.argtypes = [ctypes.c_int, DP, DP]
        L.orc_centercalc.argtypes = [ctypes.c_int, IP, DP, ctypes.c_int, ctypes.c_int, IP, DP, DP, DP]
        L.orc_gridpoints.argtypes = [ctypes.c_int, IP, IP, DP, DP, DP, ctypes.c_int, DP, DP, DP, IP, LP, LP]
        L.orc_gridpoints.restype = ctypes.c_long
        L.orc_gridpoints2.argtypes = [ctypes.c_int, DP, DP, DP, IP, ctypes.c_int, DP, DP, IP, DP, IP]
        L.orc_gridpoints2.restype = ctypes.c_long
        L.orc_gridpoints3.argtypes = [DP, DP, IP, DP]
        L.orc_gridpoints3.restype = ctypes.c_long
        L.orc_prepare.argtypes = [ctypes.c_int, DP, IP, DP, ctypes.c_int, ctypes.c_double, ctypes.c_long,
                                  IP, DP, U8P, DP, DP, DP, DP, DP, IP, DP, LP]
        L.orc_prepare.restype = ctypes.c_long
        L.orc_intracule.argtypes = [ctypes.c_int, DP, IP, DP, ctypes.c_int, ctypes.c_double, ctypes.c_long,
                                    IP, DP, ctypes.c_long, DP, DP, LP, ctypes.c_int]
        L.orc_eval_records.argtypes = [ctypes.c_long, DP, DP, DP, IP, DP, ctypes.c_long, DP, DP]
        L.orc_intracule_closed_shell.argtypes = [ctypes.c_int, DP, IP, DP, ctypes.c_int, ctypes.c_double, DP,
                                                 ctypes.c_int, ctypes.c_long, DP, DP, LP, ctypes.c_int]
        L.orc_radial_smearing.argtypes = [ctypes.c_long, DP, DP, DP, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_double, DP, DP, DP]
    return _lib


def _d(a):
    return a.ctypes.data_as(DP)


def _i(a):
    return a.ctypes.data_as(IP)


# ---------------------------------------------------------------- fixtures / parsers
def read_fchk(path):
    """natoms, atomic numbers, cartesian coordinates, nelec (mod_read_files.f90:432-520)."""
    lines = open(path).read().splitlines()

    def scalar(key):
        for ln in lines:
            if ln.startswith(key):
                return ln.split()[-1]
        raise KeyError(key)

    def array(key, n, conv):
        for idx, ln in enumerate(lines):
            if ln.startswith(key):
                vals = []
                j = idx + 1
                while len(vals) < n:
                    vals.extend(lines[j].split())
                    j += 1
                return [conv(v) for v in vals[:n]]
        raise KeyError(key)

    natoms = int(scalar("Number of atoms"))
    na = int(scalar("Number of alpha electrons"))
    nb = int(scalar("Number of beta electrons"))
    an = array("Atomic numbers", natoms, int)
    xyz = array("Current cartesian coordinates", 3 * natoms, float)
    return {"natoms": natoms, "an": np.array(an, dtype=np.int32),
            "cartes": np.array(xyz).reshape(natoms, 3), "nelec": na + nb}


def read_bas(path):
    """Primitive centres, exponents and Cartesian powers in .dm2p order
    (mod_read_files.f90:695-726)."""
    rows = []
    started = False
    for ln in open(path):
        if not started:
            if "#" in ln:
                started = True
            continue
        if ln.strip():
            rows.append(ln.split())
    xyz = np.array([[float(r[1]), float(r[2]), float(r[3])] for r in rows])
    alpha = np.array([float(r[4]) for r in rows])
    tmn = np.array([[int(r[5]), int(r[6]), int(r[7])] for r in rows], dtype=np.int32)
    return {"nprim": len(rows), "xyz": xyz, "alpha": alpha, "tmn": tmn}


DM2P_DTYPE = np.dtype([("i", "<i4"), ("j", "<i4"), ("k", "<i4"), ("l", "<i4"), ("v", "<f8")])


def parse_dm2p_bytes(raw, nprim):
    """Format sniffing and record reading (mod_intracule.f90:164-195, 229-262): flat stream or
    4-byte-marker sequential records of <i4 i,j,k,l; f8 v>; reading stops at EOF or at the
    first record with an index out of range."""
    if len(raw) < 8:
        return np.zeros((0, 4), np.int32), np.zeros(0)
    rec_len, rec_tail = np.frombuffer(raw[:8], "<i4")
    if rec_len == 24 and rec_tail == 0:
        raise ValueError("unsupported .dm2p format (8-byte markers)")
    if rec_len == 0:
        raise ValueError("unsupported .dm2p format (zero markers)")
    if rec_len == 24:
        n = len(raw) // 32
        rec = np.frombuffer(raw[:n * 32], dtype=np.dtype([("h", "<i4"), ("i", "<i4"), ("j", "<i4"), ("k", "<i4"),
                                                          ("l", "<i4"), ("v", "<f8"), ("t", "<i4")]))
    else:
        n = len(raw) // 24
        rec = np.frombuffer(raw[:n * 24], dtype=DM2P_DTYPE)
    ijkl = np.stack([rec["i"], rec["j"], rec["k"], rec["l"]], axis=1).astype(np.int32)
    bad = (ijkl[:, 0] < 1) | (ijkl[:, 0] > nprim) | (ijkl[:, 1:] < 1).any(axis=1)
    if bad.any():
        n = int(np.argmax(bad))
        ijkl = ijkl[:n]
        rec = rec[:n]
    return np.ascontiguousarray(ijkl), np.ascontiguousarray(rec["v"].astype(np.float64))


def ch4():
    """The reference's CH4/STO-3G fixture: primitives, geometry, DM2 records, goldens."""
    bas = read_bas(os.path.join(GOLDEN, "ch4_ops.bas"))
    fchk = read_fchk(os.path.join(GOLDEN, "ch4.fchk"))
    raw = gzip.open(os.path.join(GOLDEN, "ch4.dm2p.gz")).read()
    ijkl, v = parse_dm2p_bytes(raw, bas["nprim"])
    gold = json.load(open(os.path.join(GOLDEN, "ch4_goldens.json")))
    return {**bas, **fchk, "ijkl": ijkl, "v": v, "gold": gold, "raw": raw}


def ref_rad():
    vals = []
    for ln in open(os.path.join(GOLDEN, "ch4_ref.rad")):
        if ln.strip() and not ln.strip().startswith("#"):
            vals.append([float(x) for x in ln.split()])
    return np.array(vals)


def ref_cube():
    lines = gzip.open(os.path.join(GOLDEN, "ch4_ref.cube.gz")).read().decode().splitlines()
    return np.array([float(x) for x in lines[11:]]), lines[:11]


# ---------------------------------------------------------------- oracle wrappers
def lebedev(nang):
    x, y, z, w = (np.zeros(nang) for _ in range(4))
    if lib().orc_lebedev(nang, _d(x), _d(y), _d(z), _d(w)):
        raise ValueError(nang)
    return x, y, z, w


def gauleg(n):
    t, w = np.zeros(n), np.zeros(n)
    lib().orc_gauleg(n, _d(t), _d(w))
    return t, w


def centercalc(an, cartes, nohydro=True, betaone=False):
    natoms = len(an)
    cap = natoms * (natoms - 1) + 1
    an = np.ascontiguousarray(an, dtype=np.int32)
    cart = np.ascontiguousarray(cartes, dtype=np.float64)
    nq = ctypes.c_int()
    cent, Ps, alf = np.zeros(3 * cap), np.zeros(cap), np.zeros(cap)
    lib().orc_centercalc(natoms, _i(an), _d(cart), int(nohydro), int(betaone), ctypes.byref(nq), _d(cent), _d(Ps), _d(alf))
    n = nq.value
    return cent[:3 * n].reshape(n, 3), Ps[:n], alf[:n]


def gridpoints(nradc, nangc, sfalpha, cent, Ps, nosym=False):
    nq = len(nradc)
    nradc = np.ascontiguousarray(nradc, dtype=np.int32)
    nangc = np.ascontiguousarray(nangc, dtype=np.int32)
    cap = int((nradc.astype(np.int64) * nangc).sum())
    r, w, wv = np.zeros(3 * cap), np.zeros(cap), np.zeros(cap)
    cm = np.zeros(cap, dtype=np.int32)
    mg, rg = ctypes.c_long(), ctypes.c_long()
    n = lib().orc_gridpoints(nq, _i(nradc), _i(nangc), _d(np.ascontiguousarray(sfalpha, dtype=np.float64)),
                             _d(np.ascontiguousarray(cent, dtype=np.float64).reshape(-1)),
                             _d(np.ascontiguousarray(Ps, dtype=np.float64)), int(nosym), _d(r), _d(w), _d(wv),
                             _i(cm), ctypes.byref(mg), ctypes.byref(rg))
    if n < 0:
        raise ValueError("bad grid")
    return {"r": r[:3 * n].reshape(n, 3), "w": w[:n], "wvee": wv[:n], "cmap": cm[:n],
            "maxgrid": mg.value, "rgrid": rg.value}


def gridpoints2(start, end, step, nang, nosym=False):
    nb = len(start)
    start = np.ascontiguousarray(start, dtype=np.float64)
    end = np.ascontiguousarray(end, dtype=np.float64)
    step = np.ascontiguousarray(step, dtype=np.float64)
    nang = np.ascontiguousarray(nang, dtype=np.int32)
    npb = [int((end[b] - start[b]) / step[b]) + 1 for b in range(nb)]
    cap = sum(npb[b] * int(nang[b]) for b in range(nb))
    nr = sum(npb)
    r, wa = np.zeros(3 * cap), np.zeros(cap)
    smn, radi = np.zeros(nr, dtype=np.int32), np.zeros(nr)
    nradi = ctypes.c_int()
    n = lib().orc_gridpoints2(nb, _d(start), _d(end), _d(step), _i(nang), int(nosym), _d(r), _d(wa), _i(smn), _d(radi),
                              ctypes.byref(nradi))
    return {"r": r[:3 * n].reshape(n, 3), "w_ang": wa[:n], "smn": smn, "radi": radi}


def gridpoints3(center, step, npts):
    center = np.ascontiguousarray(center, dtype=np.float64)
    step = np.ascontiguousarray(step, dtype=np.float64)
    npts = np.ascontiguousarray(npts, dtype=np.int32)
    n = int(np.prod(npts))
    r = np.zeros(3 * n)
    lib().orc_gridpoints3(_d(center), _d(step), _i(npts), _d(r))
    return r.reshape(n, 3)


def prepare(sys_, thresh, normalize=True, records=False):
    nq = len(sys_["v"])
    flags = np.zeros(nq, dtype=np.uint8)
    s1, s2 = np.zeros(nq), np.zeros(nq)
    counts = np.zeros(3, dtype=np.int64)
    alpha = np.ascontiguousarray(sys_["alpha"], dtype=np.float64)
    tmn = np.ascontiguousarray(sys_["tmn"], dtype=np.int32)
    xyz = np.ascontiguousarray(sys_["xyz"], dtype=np.float64)
    ijkl = np.ascontiguousarray(sys_["ijkl"], dtype=np.int32)
    v = np.ascontiguousarray(sys_["v"], dtype=np.float64)
    if records:
        A, S = np.zeros(nq), np.zeros(nq)
        D, L = np.zeros(3 * nq), np.zeros(3 * nq, dtype=np.int32)
        C = np.zeros(nq * 3 * MAXCOEF)
        args = (_d(A), _d(S), _d(D), _i(L), _d(C))
    else:
        args = (None, None, None, None, None)
    ns = lib().orc_prepare(len(alpha), _d(alpha), _i(tmn), _d(xyz), int(normalize), thresh, nq, _i(ijkl), _d(v),
                           flags.ctypes.data_as(U8P), _d(s1), _d(s2), *args, counts.ctypes.data_as(LP))
    out = {"flags": flags, "s1": s1, "s2": s2, "counts": counts}
    if records:
        out.update({"A": A[:ns], "sqe": S[:ns], "d": D[:3 * ns].reshape(ns, 3), "L": L[:3 * ns].reshape(ns, 3),
                    "C": C[:ns * 3 * MAXCOEF].reshape(ns, 3, MAXCOEF)})
    return out


def intracule(sys_, thresh, r, normalize=True, nthreads=0):
    r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
    ng = len(r)
    Iv = np.zeros(ng)
    counts = np.zeros(3, dtype=np.int64)
    alpha = np.ascontiguousarray(sys_["alpha"], dtype=np.float64)
    tmn = np.ascontiguousarray(sys_["tmn"], dtype=np.int32)
    xyz = np.ascontiguousarray(sys_["xyz"], dtype=np.float64)
    ijkl = np.ascontiguousarray(sys_["ijkl"], dtype=np.int32)
    v = np.ascontiguousarray(sys_["v"], dtype=np.float64)
    lib().orc_intracule(len(alpha), _d(alpha), _i(tmn), _d(xyz), int(normalize), thresh, len(v), _i(ijkl), _d(v), ng,
                        _d(r), _d(Iv), counts.ctypes.data_as(LP), nthreads)
    return Iv, counts


def intracule_closed_shell(basis, D, thresh, r, unique=False, normalize=True, nthreads=0):
    """The oracle over the closed-shell DM2 of the 1-RDM D, generated as the library's device
    generator does (inca_gen_closed_shell_dm2), in batches; returns I at r and the counts."""
    r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
    Iv = np.zeros(len(r))
    counts = np.zeros(3, dtype=np.int64)
    alpha = np.ascontiguousarray(basis["alpha"], dtype=np.float64)
    tmn = np.ascontiguousarray(basis["tmn"], dtype=np.int32)
    xyz = np.ascontiguousarray(basis["xyz"], dtype=np.float64)
    Dc = np.ascontiguousarray(np.asarray(D, dtype=np.float64).T)  # column-major D(nprim, nprim)
    lib().orc_intracule_closed_shell(len(alpha), _d(alpha), _i(tmn), _d(xyz), int(normalize), thresh, _d(Dc),
                                     int(unique), len(r), _d(r), _d(Iv), counts.ctypes.data_as(LP), nthreads)
    return Iv, counts


def eval_records(rec, r):
    r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
    Iv = np.zeros(len(r))
    A = np.ascontiguousarray(rec["A"]); S = np.ascontiguousarray(rec["sqe"])
    D = np.ascontiguousarray(rec["d"]).reshape(-1); L = np.ascontiguousarray(rec["L"], dtype=np.int32).reshape(-1)
    C = np.ascontiguousarray(rec["C"]).reshape(-1)
    lib().orc_eval_records(len(A), _d(A), _d(S), _d(D), _i(L), _d(C), len(r), _d(r), _d(Iv))
    return Iv


def radial_smearing(r, w, dens, u_max, n_bins=1000, sigma=0.15):
    r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
    u, P, I = np.zeros(n_bins), np.zeros(n_bins), np.zeros(n_bins)
    lib().orc_radial_smearing(len(r), _d(r), _d(np.ascontiguousarray(w)), _d(np.ascontiguousarray(dens)), u_max, n_bins,
                              sigma, _d(u), _d(P), _d(I))
    return u, P, I
