"""ctypes binding of libinca_gpu.so (include/inca_gpu.h).

The library is built in-tree by inca_parallel_gb300.build. There is no CPU fallback: if the
shared object is missing or no sm_103 device is present, calls raise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libinca_gpu.so")

INCA_OK = 0
INCA_FP64 = 0
INCA_MIXED = 1
INCA_FP64_SCREENED = 2
MAX_COEF = 17
STATUS = {0: "INCA_OK", 1: "INCA_E_ARG", 2: "INCA_E_CUDA", 3: "INCA_E_IO", 4: "INCA_E_FORMAT",
          5: "INCA_E_STATE", 6: "INCA_E_NOMEM", 7: "INCA_E_LIMIT", 8: "INCA_E_TIMEOUT"}

DP = ctypes.POINTER(ctypes.c_double)
FP = ctypes.POINTER(ctypes.c_float)
IP = ctypes.POINTER(ctypes.c_int32)
I64P = ctypes.POINTER(ctypes.c_int64)
U8P = ctypes.POINTER(ctypes.c_uint8)
VP = ctypes.c_void_p


class Tuning(ctypes.Structure):
    _fields_ = [("items_per_cta", ctypes.c_int32), ("sample_stride", ctypes.c_int32),
                ("estimate_safety", ctypes.c_double), ("best_ms", ctypes.c_double), ("default_ms", ctypes.c_double),
                ("drop_fraction", ctypes.c_double), ("ctas_per_sm", ctypes.c_int32), ("cheap_slack", ctypes.c_int32),
                ("points_per_lane", ctypes.c_int32)]


class Counts(ctypes.Structure):
    _fields_ = [("read", ctypes.c_int64), ("after_screen1", ctypes.c_int64), ("after_screen2", ctypes.c_int64)]


# name -> (restype, argtypes): every entry point declared in include/inca_gpu.h
SIGNATURES = {
    "inca_abi_version": (ctypes.c_int, []),
    "inca_ctx_create": (ctypes.c_int, [ctypes.POINTER(VP), ctypes.c_int]),
    "inca_ctx_destroy": (ctypes.c_int, [VP]),
    "inca_last_error": (ctypes.c_char_p, [VP]),
    "inca_set_primitives": (ctypes.c_int, [VP, ctypes.c_int32, DP, IP, DP, DP, DP]),
    "inca_load_dm2p": (ctypes.c_int, [VP, ctypes.c_char_p, I64P]),
    "inca_set_quartets": (ctypes.c_int, [VP, ctypes.c_int64, IP, DP]),
    "inca_read_dm2p": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int64, IP, DP, I64P, ctypes.c_char_p,
                                      ctypes.c_int32]),
    "inca_gen_closed_shell_dm2": (ctypes.c_int, [VP, DP, ctypes.c_int, I64P]),
    "inca_prepare": (ctypes.c_int, [VP, ctypes.c_double, ctypes.c_int, ctypes.POINTER(Counts)]),
    "inca_get_screening": (ctypes.c_int, [VP, U8P, DP, DP]),
    "inca_get_records": (ctypes.c_int, [VP, DP, DP, DP, IP, DP]),
    "inca_grid_radial": (ctypes.c_int, [VP, ctypes.c_int32, IP, IP, DP, DP, DP, ctypes.c_int, I64P, I64P, I64P]),
    "inca_grid_scan": (ctypes.c_int, [VP, ctypes.c_int32, DP, DP, DP, IP, ctypes.c_int, IP, I64P]),
    "inca_grid_cube": (ctypes.c_int, [VP, DP, DP, IP, I64P]),
    "inca_grid_points": (ctypes.c_int, [VP, ctypes.c_int64, DP]),
    "inca_grid_copy": (ctypes.c_int, [VP, DP, DP, DP, IP]),
    "inca_eval": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_double, DP]),
    "inca_radial_integral": (ctypes.c_int, [VP, DP, DP, DP, DP]),
    "inca_radial_plot": (ctypes.c_int, [VP, DP, DP]),
    "inca_radial_smearing": (ctypes.c_int, [VP, ctypes.c_double, ctypes.c_int32, ctypes.c_double, DP, DP, DP]),
    "inca_centercalc": (ctypes.c_int, [ctypes.c_int32, IP, DP, ctypes.c_int, ctypes.c_int, IP, DP, DP, DP]),
    "inca_last_eval_timing": (ctypes.c_int, [VP, DP, DP, IP, IP]),
    "inca_last_eval_stats": (ctypes.c_int, [VP, I64P, I64P, I64P, I64P]),
    "inca_get_stream": (ctypes.c_int, [VP, ctypes.POINTER(VP)]),
    "inca_last_eval_phases": (ctypes.c_int, [VP, DP, DP]),
    "inca_last_eval_cheap_pairs": (ctypes.c_int, [VP, I64P]),
    "inca_kernel_launches": (ctypes.c_int, [VP, I64P]),
    "inca_fp32_fma_peak": (ctypes.c_int, [VP, DP]),
    "inca_mlp_create": (ctypes.c_int, [ctypes.POINTER(VP), ctypes.c_int, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_int32, ctypes.c_uint64]),
    "inca_mlp_destroy": (ctypes.c_int, [VP]),
    "inca_mlp_param_count": (ctypes.c_int, [VP, I64P]),
    "inca_mlp_get_params": (ctypes.c_int, [VP, FP]),
    "inca_mlp_set_params": (ctypes.c_int, [VP, FP]),
    "inca_mlp_forward": (ctypes.c_int, [VP, ctypes.c_int64, FP, FP]),
    "inca_mlp_gradient": (ctypes.c_int, [VP, ctypes.c_int64, FP, FP, FP, FP]),
    "inca_mlp_train": (ctypes.c_int, [VP, ctypes.c_int64, FP, FP, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                      ctypes.c_uint64, FP]),
    "inca_eval_graph": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_double, DP]),
    "inca_autotune": (ctypes.c_int, [VP, ctypes.c_double, ctypes.c_int32, ctypes.POINTER(Tuning)]),
    "inca_set_tuning": (ctypes.c_int, [VP, ctypes.POINTER(Tuning)]),
    "inca_batch_clear": (ctypes.c_int, [VP]),
    "inca_batch_add_closed_shell": (ctypes.c_int, [VP, ctypes.c_int32, DP, IP, DP, DP, DP, DP, ctypes.c_int,
                                                   ctypes.c_int32, DP, DP, DP, IP, ctypes.c_int, IP]),
    "inca_batch_prepare": (ctypes.c_int, [VP, ctypes.c_double, ctypes.POINTER(Counts), I64P]),
    "inca_batch_eval": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_double, DP]),
    "inca_eval_records_noalloc": (ctypes.c_int, [ctypes.c_int64, VP, VP, VP, VP, VP, ctypes.c_int64, VP, VP, VP]),
}

_lib = None


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built: run inca_parallel_gb300.build.build() first")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class IncaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def _d(a):
    return None if a is None else a.ctypes.data_as(DP)


def _i(a):
    return None if a is None else a.ctypes.data_as(IP)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Context:
    """One inca_ctx on a CUDA device; methods mirror the C entry points."""

    def __init__(self, device=0):
        self.lib = load()
        h = VP()
        st = self.lib.inca_ctx_create(ctypes.byref(h), device)
        if st != INCA_OK:
            raise IncaError(st, "inca_ctx_create failed (no usable sm_103 device?)")
        self.h = h
        self.ngrid = 0
        self.nquad = 0
        self.nradi = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.inca_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        if st != INCA_OK:
            raise IncaError(st, self.lib.inca_last_error(self.h).decode())

    # ---- inputs
    def set_primitives(self, alpha, tmn, xyz):
        alpha = f64(alpha)
        n = len(alpha)
        tmn_cm = i32(np.asarray(tmn, dtype=np.int32).reshape(n, 3).T.reshape(-1))  # TMN(nprim,3)
        xyz = np.asarray(xyz, dtype=np.float64).reshape(n, 3)
        xs, ys, zs = f64(xyz[:, 0]), f64(xyz[:, 1]), f64(xyz[:, 2])
        self._check(self.lib.inca_set_primitives(self.h, n, _d(alpha), _i(tmn_cm), _d(xs), _d(ys), _d(zs)))
        self.nprim = n

    def load_dm2p(self, path):
        n = ctypes.c_int64()
        self._check(self.lib.inca_load_dm2p(self.h, os.fsencode(path), ctypes.byref(n)))
        return n.value

    def set_quartets(self, ijkl, v):
        ijkl = i32(ijkl).reshape(-1)
        v = f64(v)
        self._check(self.lib.inca_set_quartets(self.h, len(v), _i(ijkl), _d(v)))

    def gen_closed_shell_dm2(self, D, unique=False):
        D = f64(np.asarray(D, dtype=np.float64).T.reshape(-1))  # column-major
        n = ctypes.c_int64()
        self._check(self.lib.inca_gen_closed_shell_dm2(self.h, _d(D), int(unique), ctypes.byref(n)))
        return n.value

    # ---- batches of molecules (radial-scan I(s) for each, evaluated together)
    def batch_clear(self):
        self._check(self.lib.inca_batch_clear(self.h))
        self.batch_nradi = []

    def batch_add_closed_shell(self, alpha, tmn, xyz, D, start, end, step, nang, unique=False, nosym=False):
        alpha = f64(alpha)
        n = len(alpha)
        tmn_cm = i32(np.asarray(tmn, dtype=np.int32).reshape(n, 3).T.reshape(-1))
        xyz = np.asarray(xyz, dtype=np.float64).reshape(n, 3)
        xs, ys, zs = f64(xyz[:, 0]), f64(xyz[:, 1]), f64(xyz[:, 2])
        Dc = f64(np.asarray(D, dtype=np.float64).T.reshape(-1))
        start, end, step, nang = f64(start), f64(end), f64(step), i32(nang)
        nr = ctypes.c_int32()
        self._check(self.lib.inca_batch_add_closed_shell(self.h, n, _d(alpha), _i(tmn_cm), _d(xs), _d(ys), _d(zs),
                                                         _d(Dc), int(unique), len(start), _d(start), _d(end),
                                                         _d(step), _i(nang), int(nosym), ctypes.byref(nr)))
        if not hasattr(self, "batch_nradi"):
            self.batch_nradi = []
        self.batch_nradi.append(nr.value)
        return nr.value

    def batch_prepare(self, thresh):
        c = Counts()
        ng = ctypes.c_int64()
        self._check(self.lib.inca_batch_prepare(self.h, thresh, ctypes.byref(c), ctypes.byref(ng)))
        self.counts = (c.read, c.after_screen1, c.after_screen2)
        self.nradi = int(sum(self.batch_nradi))
        self.ngrid = ng.value
        return self.counts

    def batch_eval(self, mode=INCA_MIXED, tol=1e-8):
        """I(s) of every molecule of the batch, as a list of arrays (one per molecule)."""
        out = np.zeros(int(sum(self.batch_nradi)))
        self._check(self.lib.inca_batch_eval(self.h, mode, tol, _d(out)))
        parts, k = [], 0
        for nr in self.batch_nradi:
            parts.append(out[k:k + nr])
            k += nr
        return parts

    def prepare(self, thresh, normalize=True):
        c = Counts()
        self._check(self.lib.inca_prepare(self.h, thresh, int(normalize), ctypes.byref(c)))
        self.counts = (c.read, c.after_screen1, c.after_screen2)
        return self.counts

    def screening(self):
        n = self.counts[0]
        flags = np.zeros(n, dtype=np.uint8)
        s1, s2 = np.zeros(n), np.zeros(n)
        self._check(self.lib.inca_get_screening(self.h, flags.ctypes.data_as(U8P), _d(s1), _d(s2)))
        return flags, s1, s2

    def records(self):
        ns = self.counts[2]
        A, S = np.zeros(ns), np.zeros(ns)
        D, L = np.zeros(3 * ns), np.zeros(3 * ns, dtype=np.int32)
        C = np.zeros(ns * 3 * MAX_COEF)
        self._check(self.lib.inca_get_records(self.h, _d(A), _d(S), _d(D), _i(L), _d(C)))
        return {"A": A, "sqe": S, "d": D.reshape(ns, 3), "L": L.reshape(ns, 3), "C": C.reshape(ns, 3, MAX_COEF)}

    # ---- grids
    def grid_radial(self, nradc, nangc, sfalpha, cent, Ps, nosym=False):
        nq = len(Ps)
        nradc, nangc = i32(nradc), i32(nangc)
        sf, ps = f64(sfalpha), f64(Ps)
        ce = f64(np.asarray(cent, dtype=np.float64).reshape(nq, 3).reshape(-1))  # cent(3,nquad)
        mg, rg, ng = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.inca_grid_radial(self.h, nq, _i(nradc), _i(nangc), _d(sf), _d(ce), _d(ps), int(nosym),
                                              ctypes.byref(mg), ctypes.byref(rg), ctypes.byref(ng)))
        self.ngrid, self.nquad = ng.value, nq
        return mg.value, rg.value, ng.value

    def grid_scan(self, start, end, step, nang, nosym=False):
        start, end, step, nang = f64(start), f64(end), f64(step), i32(nang)
        nr, ng = ctypes.c_int32(), ctypes.c_int64()
        self._check(self.lib.inca_grid_scan(self.h, len(start), _d(start), _d(end), _d(step), _i(nang), int(nosym),
                                            ctypes.byref(nr), ctypes.byref(ng)))
        self.ngrid, self.nradi = ng.value, nr.value
        return nr.value, ng.value

    def grid_cube(self, center, step, npts):
        c, s, n = f64(center), f64(step), i32(npts)
        ng = ctypes.c_int64()
        self._check(self.lib.inca_grid_cube(self.h, _d(c), _d(s), _i(n), ctypes.byref(ng)))
        self.ngrid = ng.value
        return ng.value

    def grid_points(self, r):
        r = f64(np.asarray(r, dtype=np.float64).reshape(-1, 3).reshape(-1))
        self._check(self.lib.inca_grid_points(self.h, len(r) // 3, _d(r)))
        self.ngrid = len(r) // 3

    def grid_copy(self, weights=True, vee=False, cmap=False):
        n = self.ngrid
        r = np.zeros(3 * n)
        w = np.zeros(n) if weights else None
        wv = np.zeros(n) if vee else None
        cm = np.zeros(n, dtype=np.int32) if cmap else None
        self._check(self.lib.inca_grid_copy(self.h, _d(r), _d(w), _d(wv), _i(cm)))
        out = {"r": r.reshape(n, 3)}
        if weights:
            out["w"] = w
        if vee:
            out["wvee"] = wv
        if cmap:
            out["cmap"] = cm
        return out

    # ---- evaluation / reductions
    def eval(self, mode=INCA_FP64, tol=1e-10, copy=True, out=None):
        """I at every grid point (a new array, or `out`: contiguous float64 of ngrid values, e.g.
        pinned host memory); copy=False leaves the result on the device only."""
        if out is not None:
            if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous
                    and out.size == self.ngrid):
                raise ValueError("out must be a contiguous float64 array of ngrid values")
            iv = out
        else:
            iv = np.zeros(self.ngrid) if copy else None
        self._check(self.lib.inca_eval(self.h, mode, tol, _d(iv)))
        return iv

    def autotune(self, tol=1e-10, reps=3):
        """Tune the mixed evaluation's schedule on the current grid and records (see inca_autotune)."""
        t = Tuning()
        self._check(self.lib.inca_autotune(self.h, tol, reps, ctypes.byref(t)))
        return {f: getattr(t, f) for f, _ in Tuning._fields_}

    def set_tuning(self, items_per_cta=None, sample_stride=None, estimate_safety=None, drop_fraction=-1.0,
                   ctas_per_sm=0, cheap_slack=0, points_per_lane=0):
        if items_per_cta is None:
            self._check(self.lib.inca_set_tuning(self.h, None))
            return
        t = Tuning(items_per_cta, sample_stride, estimate_safety, 0.0, 0.0, drop_fraction, ctas_per_sm, cheap_slack,
                   points_per_lane)
        self._check(self.lib.inca_set_tuning(self.h, ctypes.byref(t)))

    def eval_graph(self, mode=INCA_MIXED, tol=1e-10, copy=True):
        """inca_eval through a captured CUDA graph (the first call per grid/records/tol captures)."""
        iv = np.zeros(self.ngrid) if copy else None
        self._check(self.lib.inca_eval_graph(self.h, mode, tol, _d(iv)))
        return iv

    def radial_integral(self):
        t, v = ctypes.c_double(), ctypes.c_double()
        pc, vc = np.zeros(self.nquad), np.zeros(self.nquad)
        self._check(self.lib.inca_radial_integral(self.h, ctypes.byref(t), ctypes.byref(v), _d(pc), _d(vc)))
        return t.value, v.value, pc, vc

    def radial_plot(self):
        radi, ri = np.zeros(self.nradi), np.zeros(self.nradi)
        self._check(self.lib.inca_radial_plot(self.h, _d(radi), _d(ri)))
        return radi, ri

    def radial_smearing(self, u_max, n_bins=1000, sigma=0.15):
        u, P, I = np.zeros(n_bins), np.zeros(n_bins), np.zeros(n_bins)
        self._check(self.lib.inca_radial_smearing(self.h, u_max, n_bins, sigma, _d(u), _d(P), _d(I)))
        return u, P, I

    def timing(self):
        t, k = ctypes.c_double(), ctypes.c_double()
        kl, l = ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.inca_last_eval_timing(self.h, ctypes.byref(t), ctypes.byref(k), ctypes.byref(kl),
                                                   ctypes.byref(l)))
        return {"total_ms": t.value, "kernel_ms": k.value, "kernel_launches": kl.value, "launches": l.value}

    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        p = VP()
        self._check(self.lib.inca_get_stream(self.h, ctypes.byref(p)))
        return p.value or 0

    def kernel_launches(self):
        n = ctypes.c_int64()
        self._check(self.lib.inca_kernel_launches(self.h, ctypes.byref(n)))
        return n.value

    def stats(self):
        a, b, c, d = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.inca_last_eval_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                                  ctypes.byref(d)))
        e = ctypes.c_int64()
        self._check(self.lib.inca_last_eval_cheap_pairs(self.h, ctypes.byref(e)))
        return {"fp32_pairs": a.value, "precise_pairs": b.value, "skipped_pairs": c.value, "corrected_terms": d.value,
                "cheap_pairs": e.value}

    def fp32_peak_tflops(self):
        """Measured FP32 FMA throughput of the context's GPU (TFLOP/s)."""
        t = ctypes.c_double()
        self._check(self.lib.inca_fp32_fma_peak(self.h, ctypes.byref(t)))
        return t.value

    def phases(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.inca_last_eval_phases(self.h, ctypes.byref(a), ctypes.byref(b)))
        return {"pass1_ms": a.value, "pass2_ms": b.value}


def read_dm2p(path, nprim):
    """The library's .dm2p reader on the host (no device): (ijkl (n,4) int32 1-based, v (n,)).
    Raises IncaError with the library's status and message."""
    lib = load()
    n = ctypes.c_int64()
    err = ctypes.create_string_buffer(512)
    st = lib.inca_read_dm2p(os.fsencode(path), int(nprim), 0, None, None, ctypes.byref(n), err, 512)
    if st:
        raise IncaError(st, err.value.decode(errors="replace"))
    ijkl = np.zeros((n.value, 4), dtype=np.int32)
    v = np.zeros(n.value)
    st = lib.inca_read_dm2p(os.fsencode(path), int(nprim), n.value, _i(ijkl), _d(v), ctypes.byref(n), err, 512)
    if st:
        raise IncaError(st, err.value.decode(errors="replace"))
    return ijkl, v


def centercalc(an, cartes, nohydro=True, betaone=False):
    """Automatic centres (host side of the library): returns cent (nquad,3), Ps, sfalpha."""
    lib = load()
    an = i32(an)
    natoms = len(an)
    cart_cm = f64(np.asarray(cartes, dtype=np.float64).reshape(natoms, 3).T.reshape(-1))  # cartes(natoms,3)
    cap = natoms * (natoms - 1) + 1
    nq = ctypes.c_int32()
    cent, Ps, sf = np.zeros(3 * cap), np.zeros(cap), np.zeros(cap)
    st = lib.inca_centercalc(natoms, _i(an), _d(cart_cm), int(nohydro), int(betaone), ctypes.byref(nq), _d(cent),
                             _d(Ps), _d(sf))
    if st != INCA_OK:
        raise IncaError(st, "inca_centercalc failed")
    n = nq.value
    return cent[:3 * n].reshape(n, 3), Ps[:n], sf[:n]


class MLP:
    """The library's multilayer perceptron (nin -> nhidden -> nhidden -> nout, tanh), trained
    and evaluated on the GPU by its own kernels (include/inca_gpu.h, inca_mlp_*)."""

    def __init__(self, nin, nhidden, nout, seed=1, device=0):
        self.lib = load()
        self.h = VP()
        st = self.lib.inca_mlp_create(ctypes.byref(self.h), device, nin, nhidden, nout, seed)
        if st:
            raise IncaError(st, "inca_mlp_create")
        self.nin, self.nh, self.nout = nin, nhidden, nout
        n = ctypes.c_int64()
        self.lib.inca_mlp_param_count(self.h, ctypes.byref(n))
        self.nparam = n.value

    def _check(self, st, what):
        if st:
            raise IncaError(st, what)

    def close(self):
        if self.h:
            self.lib.inca_mlp_destroy(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.zeros(self.nparam, dtype=np.float32)
        self._check(self.lib.inca_mlp_get_params(self.h, p.ctypes.data_as(FP)), "inca_mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparam
        self._check(self.lib.inca_mlp_set_params(self.h, p.ctypes.data_as(FP)), "inca_mlp_set_params")

    def forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, self.nin)
        Y = np.zeros((len(X), self.nout), dtype=np.float32)
        self._check(self.lib.inca_mlp_forward(self.h, len(X), X.ctypes.data_as(FP), Y.ctypes.data_as(FP)),
                    "inca_mlp_forward")
        return Y

    def gradient(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, self.nin)
        T = np.ascontiguousarray(T, dtype=np.float32).reshape(-1, self.nout)
        loss = ctypes.c_float()
        g = np.zeros(self.nparam, dtype=np.float32)
        self._check(self.lib.inca_mlp_gradient(self.h, len(X), X.ctypes.data_as(FP), T.ctypes.data_as(FP),
                                               ctypes.byref(loss), g.ctypes.data_as(FP)), "inca_mlp_gradient")
        return loss.value, g

    def train(self, X, T, epochs, batch=256, lr=1e-3, seed=7):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, self.nin)
        T = np.ascontiguousarray(T, dtype=np.float32).reshape(-1, self.nout)
        loss = ctypes.c_float()
        self._check(self.lib.inca_mlp_train(self.h, len(X), X.ctypes.data_as(FP), T.ctypes.data_as(FP), epochs, batch,
                                            lr, seed, ctypes.byref(loss)), "inca_mlp_train")
        return loss.value
