"""ctypes wrapper of the CPU oracle (oracle/_build/libft_oracle.so).

Test infrastructure: used only by the tests, the smoke check and the CPU-baseline
leg of bench.py, always as the checker, never as the thing measured or shipped.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
_libs = {}
_lock = threading.Lock()


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "oracle"], check=True)


def lib(fast=False):
    name = "libft_oracle_fast.so" if fast else "libft_oracle.so"
    with _lock:
        if name not in _libs:
            path = os.path.join(ORACLE_DIR, "_build", name)
            if not os.path.exists(path):
                build()
            L = ctypes.CDLL(path)
            L.fto_prepare.restype = ctypes.c_void_p
            L.fto_prepare.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_double]
            L.fto_last_error.restype = ctypes.c_char_p
            L.fto_free.argtypes = [ctypes.c_void_p]
            L.fto_info.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            L.fto_table.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 4
            L.fto_samples.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64] + [
                ctypes.c_void_p] * 6
            L.fto_integrate.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p]
            L.fto_skip.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p]
            L.fto_count_ops.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                        ctypes.c_void_p, ctypes.c_void_p]
            _libs[name] = L
        return _libs[name]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleError(Exception):
    pass


class Prepared:
    """An input dict in the reference's JSON schema, preprocessed by the oracle."""

    def __init__(self, inp, fast=False):
        self.L = lib(fast)
        edges = np.array([[e[0][0], e[0][1]] for e in inp["graph"]], dtype=np.int32).reshape(-1)
        nu = np.array([float(e[1]) for e in inp["graph"]], dtype=np.float64)
        self.E = len(nu)
        self.V = int(edges.max()) + 1 if self.E else 0
        P = np.array(inp["scalarproducts"], dtype=np.float64).reshape(-1)
        m2 = np.array(inp["masses_sqr"], dtype=np.float64)
        self.K = int(inp["num_eps_terms"])
        self._keep = (edges, nu, P, m2)
        h = self.L.fto_prepare(self.E, self.V, _ptr(edges), _ptr(nu), _ptr(P), _ptr(m2), float(inp["dimension"]),
                               self.K, float(inp["lambda"]))
        if not h:
            raise OracleError(self.L.fto_last_error().decode())
        self.h = ctypes.c_void_p(h)
        info = np.zeros(10)
        self.L.fto_info(self.h, _ptr(info))
        (self.W, self.W_ref, self.IGtr, loops, eu, pe, ge, gp, wz, self.def_ref) = info
        self.loops = int(loops)
        self.euclidean, self.pseudo_euclidean, self.generic, self.gp, self.W_zero = map(bool, (eu, pe, ge, gp, wz))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.fto_free(self.h)

    def table(self):
        n = 1 << self.E
        Jr, r = np.zeros(n), np.zeros(n)
        mm, L = np.zeros(n, np.uint8), np.zeros(n, np.uint8)
        self.L.fto_table(self.h, _ptr(Jr), _ptr(r), _ptr(mm), _ptr(L))
        return Jr, r, mm, L

    def samples(self, seed, first, count):
        E, K = self.E, self.K
        order = np.zeros((count, E), np.int32)
        X = np.zeros((count, E))
        psi, xi = np.zeros(count), np.zeros(count)
        R = np.zeros((count, K, 2))
        dropped = np.zeros(count, np.uint8)
        rc = self.L.fto_samples(self.h, seed, first, count, _ptr(order), _ptr(X), _ptr(psi), _ptr(xi), _ptr(R),
                                _ptr(dropped))
        if rc:
            raise OracleError(self.L.fto_last_error().decode())
        return {"order": order, "X": X, "psi_tr": psi, "xi_tr": xi, "R": R[..., 0] + 1j * R[..., 1],
                "dropped": dropped.astype(bool)}

    def count_ops(self, seed, first, count, values=False):
        """Floating-point operations of samples first..first+count-1, counted by running
        the restatement with the counting scalar (oracle/opcount.hpp).  Returns a dict of
        totals (add, mul, div, sqrt, trans, cmp, dropped) and, with values=True, the
        counted run's per-sample values (count x K complex)."""
        out = np.zeros(7)
        R = np.zeros((count, self.K, 2)) if values else None
        rc = self.L.fto_count_ops(self.h, seed, first, count, _ptr(out), _ptr(R) if values else None)
        if rc:
            raise OracleError(self.L.fto_last_error().decode())
        d = dict(zip(("add", "mul", "div", "sqrt", "trans", "cmp", "dropped"), out.tolist()))
        if values:
            d["R"] = R[..., 0] + 1j * R[..., 1]
        return d

    def integrate(self, N, seed=0, threads=1):
        out = np.zeros((self.K, 4))
        counts = np.zeros(2, np.uint64)
        rc = self.L.fto_integrate(self.h, N, seed, threads, _ptr(out), _ptr(counts))
        if rc:
            raise OracleError(self.L.fto_last_error().decode())
        return out, int(counts[0]), int(counts[1])


def skip_state(seed, steps):
    st = np.zeros(4, np.uint64)
    lib().fto_skip(seed, steps, _ptr(st))
    return st
