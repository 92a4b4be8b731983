"""feyntrop_gb300: feyntrop's tropical sampling + integrand evaluation loop on GB300.

Python side of the C ABI in include/feyntrop_gb300.h (ctypes, no torch types).
The sampling runs only on the GPU: without the native library or without a
CUDA device every entry point raises instead of falling back to anything else.

    from feyntrop_gb300 import Plan, run_json
    plan = Plan(input_dict)                  # the reference's JSON schema
    out = plan.integrate(N=10**7, seed=0)    # {"integral": [[[re, dre], [im, dim]], ...], ...}
    out = run_json(input_dict)               # the CLI contract, in process

py_feyntrop (the reference's Python front end) is mirrored in
feyntrop_gb300.py_feyntrop.
"""
import ctypes
import math
import json
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfeyntrop_gb300.so")
CLI_PATH = os.path.join(HERE, "_build", "feyntrop")

FT_OK = 0
FT_ERR_INVALID_ARGUMENT = 1
FT_ERR_DOMAIN = 2
FT_ERR_RUNTIME = 3
FT_ERR_CUDA = 4
FT_ERR_NO_DEVICE = 5
FP64 = 0
MIXED = 1

EXPORTED = ["ft_plan_create", "ft_plan_destroy", "ft_plan_get_info", "ft_plan_log_line", "ft_integrate",
            "ft_integrate_batch", "ft_finalize_moments", "ft_sample_records", "ft_run_json", "ft_free",
            "ft_precompile", "ft_last_error", "ft_version", "ft_subgraph_table", "ft_device_peaks", "ft_integrate_noalloc",
            "ft_batch_create", "ft_batch_destroy", "ft_batch_run", "ft_batch_get_info", "ft_plans_create",
            "ft_autotune"]
PRECOMPILE_BATCH = 0x100


class FeyntropError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


class Problem(ctypes.Structure):
    _fields_ = [("num_edges", ctypes.c_int32), ("edges", ctypes.c_void_p), ("nu", ctypes.c_void_p),
                ("num_vertices", ctypes.c_int32), ("scalarproducts", ctypes.c_void_p),
                ("masses_sqr", ctypes.c_void_p), ("dimension", ctypes.c_double), ("num_eps_terms", ctypes.c_int32),
                ("lambda_", ctypes.c_double)]


class PlanInfo(ctypes.Structure):
    _fields_ = [("W", ctypes.c_double), ("IGtr", ctypes.c_double), ("loops", ctypes.c_int32),
                ("euclidean", ctypes.c_int32), ("pseudo_euclidean", ctypes.c_int32), ("generic", ctypes.c_int32),
                ("gp_property", ctypes.c_int32), ("deformed", ctypes.c_int32), ("lambda_used", ctypes.c_double),
                ("seconds_preprocessing", ctypes.c_double), ("table_bytes", ctypes.c_uint64),
                ("num_log_lines", ctypes.c_int32)]


class RunOptions(ctypes.Structure):
    _fields_ = [("num_samples", ctypes.c_uint64), ("seed", ctypes.c_uint64), ("first_sample", ctypes.c_uint64),
                ("precision", ctypes.c_int32), ("stream", ctypes.c_void_p)]


class Moments(ctypes.Structure):
    _fields_ = [("n", ctypes.c_double), ("s1_hi", ctypes.c_double), ("s1_lo", ctypes.c_double),
                ("s2_hi", ctypes.c_double), ("s2_lo", ctypes.c_double)]


class Result(ctypes.Structure):
    _fields_ = [("num_eps_terms", ctypes.c_int32), ("re_avg", ctypes.c_void_p), ("re_acc", ctypes.c_void_p),
                ("im_avg", ctypes.c_void_p), ("im_acc", ctypes.c_void_p), ("moments", ctypes.c_void_p),
                ("kept", ctypes.c_uint64), ("dropped", ctypes.c_uint64), ("fp64_fallback", ctypes.c_uint64),
                ("exact_steps", ctypes.c_uint64), ("robust", ctypes.c_uint64), ("kernel_ms", ctypes.c_double),
                ("seconds_sampling", ctypes.c_double), ("kernel_launches", ctypes.c_int32)]


class TuneResult(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("min_blocks_per_sm", ctypes.c_int32), ("variant", ctypes.c_int32),
                ("samples_per_second", ctypes.c_double), ("default_samples_per_second", ctypes.c_double),
                ("candidates", ctypes.c_int32), ("batch_chunk", ctypes.c_uint64),
                ("batch_samples_per_second", ctypes.c_double)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("num_integrals", ctypes.c_int32), ("num_classes", ctypes.c_int32),
                ("graph_captures", ctypes.c_int32), ("kernel_launches", ctypes.c_int32),
                ("work_items", ctypes.c_uint64), ("fp64_queue_capacity", ctypes.c_uint64),
                ("kernel_ms", ctypes.c_double)]


_lib = None
_lock = threading.Lock()


def lib():
    """The native library; raises if it has not been built (no fallback path exists)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError("feyntrop_gb300 native library missing (%s): build it with "
                                  "`python -m feyntrop_gb300.build`" % LIB_PATH)
            L = ctypes.CDLL(LIB_PATH)
            L.ft_last_error.restype = ctypes.c_char_p
            L.ft_version.restype = ctypes.c_char_p
            L.ft_plan_log_line.restype = ctypes.c_char_p
            L.ft_plan_create.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(ctypes.c_void_p)]
            L.ft_plan_destroy.argtypes = [ctypes.c_void_p]
            L.ft_plan_get_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(PlanInfo)]
            L.ft_plan_log_line.argtypes = [ctypes.c_void_p, ctypes.c_int32]
            L.ft_integrate.argtypes = [ctypes.c_void_p, ctypes.POINTER(RunOptions), ctypes.POINTER(Result)]
            L.ft_integrate_batch.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
            L.ft_finalize_moments.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                              ctypes.POINTER(Result)]
            L.ft_sample_records.argtypes = [ctypes.c_void_p, ctypes.POINTER(RunOptions)] + [ctypes.c_void_p] * 4
            L.ft_run_json.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p),
                                      ctypes.POINTER(ctypes.c_void_p)]
            L.ft_free.argtypes = [ctypes.c_void_p]
            L.ft_precompile.argtypes = [ctypes.POINTER(Problem), ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
            L.ft_integrate_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(RunOptions), ctypes.c_void_p]
            L.ft_device_peaks.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
            L.ft_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(TuneResult)]
            L.ft_plans_create.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
            L.ft_batch_create.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.POINTER(ctypes.c_void_p)]
            L.ft_batch_destroy.argtypes = [ctypes.c_void_p]
            L.ft_batch_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            L.ft_batch_get_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(BatchInfo)]
            L.ft_subgraph_table.argtypes = [ctypes.POINTER(Problem)] + [ctypes.c_void_p] * 4 + [
                ctypes.POINTER(PlanInfo)]
            _lib = L
        return _lib


def _check(rc):
    if rc != FT_OK:
        raise FeyntropError(rc, lib().ft_last_error().decode(errors="replace"))


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class _ProblemArrays:
    """Keeps the numpy arrays behind an ft_problem alive."""

    def __init__(self, inp):
        if isinstance(inp, str):
            inp = json.loads(inp)
        self.inp = inp
        self.edges = np.ascontiguousarray([[int(e[0][0]), int(e[0][1])] for e in inp["graph"]],
                                          dtype=np.int32).reshape(-1)
        self.nu = np.ascontiguousarray([float(e[1]) for e in inp["graph"]], dtype=np.float64)
        self.P = np.ascontiguousarray(np.array(inp["scalarproducts"], dtype=np.float64).reshape(-1))
        self.m2 = np.ascontiguousarray(inp["masses_sqr"], dtype=np.float64)
        self.V = int(self.edges.max()) + 1 if len(self.edges) else 0
        self.E = len(self.nu)
        self.K = int(inp["num_eps_terms"])
        self.struct = Problem(self.E, _ptr(self.edges).value, _ptr(self.nu).value, self.V, _ptr(self.P).value,
                              _ptr(self.m2).value, float(inp["dimension"]), self.K, float(inp["lambda"]))


def subgraph_table(inp):
    """Host preprocessing only: (Jr, r, mm, loops, info) of the J(gamma) table."""
    a = _ProblemArrays(inp)
    n = 1 << a.E
    Jr, r = np.zeros(n), np.zeros(n)
    mm, L = np.zeros(n, np.uint8), np.zeros(n, np.uint8)
    info = PlanInfo()
    _check(lib().ft_subgraph_table(ctypes.byref(a.struct), _ptr(Jr), _ptr(r), _ptr(mm), _ptr(L), ctypes.byref(info)))
    return Jr, r, mm, L, {f: getattr(info, f) for f, _ in PlanInfo._fields_}


def device_peaks():
    """Measured (FP32, FP64) FMA issue rates of the current device in TFLOP/s."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(lib().ft_device_peaks(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def precompile(inp, precision=MIXED):
    """Compile the kernels of this input's topology into the cache; returns seconds."""
    a = _ProblemArrays(inp)
    s = ctypes.c_double()
    _check(lib().ft_precompile(ctypes.byref(a.struct), precision, ctypes.byref(s)))
    return s.value


class Plan:
    """One integral on the GPU (host preprocessing + device tables)."""

    def __init__(self, inp, _handle=None):
        self.arrays = inp if isinstance(inp, _ProblemArrays) else _ProblemArrays(inp)
        self.E, self.V, self.K = self.arrays.E, self.arrays.V, self.arrays.K
        if _handle is None:
            h = ctypes.c_void_p()
            _check(lib().ft_plan_create(ctypes.byref(self.arrays.struct), ctypes.byref(h)))
        else:
            h = _handle
        self.h = h
        info = PlanInfo()
        _check(lib().ft_plan_get_info(self.h, ctypes.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in PlanInfo._fields_}
        self.log = [lib().ft_plan_log_line(self.h, i).decode() for i in range(info.num_log_lines)]

    def close(self):
        if getattr(self, "h", None):
            lib().ft_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def integrate(self, N, seed=0, precision=FP64, first_sample=0, stream=None):
        K = self.K
        arr = np.zeros((4, K))
        mom = (Moments * (2 * K))()
        res = Result(K, _ptr(arr[0]).value, _ptr(arr[1]).value, _ptr(arr[2]).value, _ptr(arr[3]).value,
                     ctypes.cast(mom, ctypes.c_void_p).value)
        opts = RunOptions(int(N), int(seed), int(first_sample), int(precision), stream)
        _check(lib().ft_integrate(self.h, ctypes.byref(opts), ctypes.byref(res)))
        return {
            "integral": [[[arr[0, j], arr[1, j]], [arr[2, j], arr[3, j]]] for j in range(K)],
            "IGtr": self.info["IGtr"],
            "moments": [[m.n, m.s1_hi, m.s1_lo, m.s2_hi, m.s2_lo] for m in mom],
            "kept": res.kept, "dropped": res.dropped, "fp64_fallback": res.fp64_fallback,
            "exact_steps": res.exact_steps, "robust": res.robust, "kernel_ms": res.kernel_ms,
            "seconds_sampling": res.seconds_sampling, "kernel_launches": res.kernel_launches,
        }

    def autotune(self, precision=MIXED, samples=2_000_000):
        """Time this plan's kernel class under candidate launch shapes and record the
        fastest in the tuning table (used by every later plan and batch of the class)."""
        t = TuneResult()
        _check(lib().ft_autotune(self.h, int(precision), int(samples), ctypes.byref(t)))
        return {f: getattr(t, f) for f, _ in TuneResult._fields_}

    def records(self, count, seed=0, first_sample=0, precision=FP64):
        """Per-sample records of samples first_sample .. first_sample+count-1."""
        E, K = self.E, self.K
        order = np.zeros((count, E), np.uint8)
        X = np.zeros((count, E))
        R = np.zeros((count, K, 2))
        flags = np.zeros(count, np.uint8)
        opts = RunOptions(int(count), int(seed), int(first_sample), int(precision), None)
        _check(lib().ft_sample_records(self.h, ctypes.byref(opts), _ptr(order), _ptr(X), _ptr(R), _ptr(flags)))
        return {"order": order.astype(np.int32), "X": X, "R": R[..., 0] + 1j * R[..., 1], "flags": flags}


def create_plans(inputs, skip_failed=False):
    """Plans for many inputs at once (ft_plans_create: host preprocessing on all host
    threads).  A failing input raises FeyntropError, or gives None with skip_failed."""
    arrays = [_ProblemArrays(x) for x in inputs]
    n = len(arrays)
    probs = (Problem * n)(*[a.struct for a in arrays])
    hs = (ctypes.c_void_p * n)()
    st = (ctypes.c_int32 * n)()
    rc = lib().ft_plans_create(ctypes.cast(probs, ctypes.c_void_p), n, ctypes.cast(hs, ctypes.c_void_p),
                               ctypes.cast(st, ctypes.c_void_p))
    if rc != FT_OK and not skip_failed:
        msg = lib().ft_last_error().decode(errors="replace")
        for h in hs:
            if h:
                lib().ft_plan_destroy(ctypes.c_void_p(h))
        raise FeyntropError(rc, msg)
    return [Plan(a, _handle=ctypes.c_void_p(h)) if h else None for a, h in zip(arrays, hs)]


class _ResultArrays:
    """Caller-owned result buffers of one integral."""

    def __init__(self, K):
        self.K = K
        self.arr = np.zeros((4, K))
        self.mom = (Moments * (2 * K))()
        self.res = Result(K, _ptr(self.arr[0]).value, _ptr(self.arr[1]).value, _ptr(self.arr[2]).value,
                          _ptr(self.arr[3]).value, ctypes.cast(self.mom, ctypes.c_void_p).value)

    def as_dict(self, IGtr):
        arr, res, K = self.arr, self.res, self.K
        return {
            "integral": [[[arr[0, j], arr[1, j]], [arr[2, j], arr[3, j]]] for j in range(K)],
            "IGtr": IGtr,
            "moments": [[m.n, m.s1_hi, m.s1_lo, m.s2_hi, m.s2_lo] for m in self.mom],
            "kept": res.kept, "dropped": res.dropped, "fp64_fallback": res.fp64_fallback,
            "exact_steps": res.exact_steps, "robust": res.robust, "kernel_ms": res.kernel_ms,
            "seconds_sampling": res.seconds_sampling, "kernel_launches": res.kernel_launches,
        }


class Batch:
    """Many integrals in one CUDA graph launch (ft_batch_*): one persistent sampling
    launch per kernel class (topology, eps orders, regime), classes side by side.
    The plans must stay open while the batch is used."""

    def __init__(self, plans, precision=MIXED):
        self.plans = list(plans)
        arr = (ctypes.c_void_p * len(self.plans))(*[p.h.value for p in self.plans])
        h = ctypes.c_void_p()
        _check(lib().ft_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(self.plans), int(precision),
                                     ctypes.byref(h)))
        self.h = h
        self.precision = precision

    def run(self, N, seeds=0, first_samples=0, stream=None):
        """N, seeds, first_samples: scalars or one per integral; returns one result
        dict per integral (as Plan.integrate)."""
        n = len(self.plans)
        Ns = list(N) if hasattr(N, "__len__") else [N] * n
        ss = list(seeds) if hasattr(seeds, "__len__") else [seeds] * n
        fs = list(first_samples) if hasattr(first_samples, "__len__") else [first_samples] * n
        opts = (RunOptions * n)(*[RunOptions(int(Ns[i]), int(ss[i]), int(fs[i]), int(self.precision),
                                             stream if i == 0 else None) for i in range(n)])
        ras = [_ResultArrays(p.K) for p in self.plans]
        res = (Result * n)(*[r.res for r in ras])
        _check(lib().ft_batch_run(self.h, ctypes.cast(opts, ctypes.c_void_p), ctypes.cast(res, ctypes.c_void_p)))
        out = []
        for i, r in enumerate(ras):
            r.res = res[i]
            out.append(r.as_dict(self.plans[i].info["IGtr"]))
        return out

    def run_sharded(self, N, rank, world, seeds=0, first_samples=0, mode="samples", group=None, stream=None):
        """The batch over `world` processes, one per GPU, every rank holding the same
        batch (torch.distributed initialised, any backend): mode "samples" runs rank's
        contiguous block of every integral's samples, mode "integrals" every world-th
        integral whole (feyntrop_gb300.shard.batch_sharded).  The per-integral moments
        of all ranks are gathered and merged; every rank returns, per integral,
        {"integral", "moments", "samples"} of the whole batch."""
        from . import shard
        n = len(self.plans)
        Ns = [int(x) for x in N] if hasattr(N, "__len__") else [int(N)] * n

        def run(mine, seeds_, firsts):
            return self.run([m or 0 for m in mine], seeds=seeds_, first_samples=firsts, stream=stream)

        integrals, moments = shard.batch_sharded(run, Ns, [p.K for p in self.plans],
                                                 [not p.info["deformed"] for p in self.plans], rank, world,
                                                 seeds=seeds, first_samples=first_samples, mode=mode, group=group)
        return [{"integral": i, "moments": m, "samples": Ns[k]} for k, (i, m) in enumerate(zip(integrals, moments))]

    def run_to_accuracy(self, rel_target, pilot=100_000, max_samples=10**10, seeds=0, eps_order=0, stream=None):
        """Variance-adaptive sample counts: a pilot run of `pilot` samples per integral
        estimates each integral's per-sample spread; a second run continues every
        integral's stream (first sample = pilot) with the samples that bring its
        standard error at eps order `eps_order` to rel_target times |value| (at most
        max_samples in total). The moments of both runs are merged, so each result is
        that of one run over all its samples. Returns the result dicts, each with
        "samples" (the total used)."""
        from . import shard
        n = len(self.plans)
        first = self.run(pilot, seeds=seeds, stream=stream)
        extra = []
        for r in first:
            (re, dre), (im, dim) = r["integral"][eps_order]
            scale = max(abs(re), abs(im))
            spread = max(dre, dim) * math.sqrt(pilot)       # per-sample standard deviation
            if scale == 0 or not math.isfinite(spread):
                need = pilot
            else:
                need = (spread / (rel_target * scale)) ** 2
            extra.append(int(min(max_samples, max(pilot, math.ceil(need)))) - pilot)
        out = []
        if any(e > 0 for e in extra):
            second = self.run([max(e, 1) for e in extra], seeds=seeds, first_samples=pilot, stream=stream)
        else:
            second = [None] * n
        for i, (a, b, e) in enumerate(zip(first, second, extra)):
            moments = a["moments"] if e <= 0 else shard.merge_moments([a["moments"], b["moments"]])
            res = dict(a if e <= 0 else b)
            res["moments"] = moments
            res["integral"] = finalize_moments(moments, self.plans[i].K, not self.plans[i].info["deformed"])
            res["samples"] = pilot + max(e, 0)
            if e > 0:
                for k in ("kept", "dropped", "fp64_fallback", "exact_steps", "robust"):
                    res[k] = a[k] + b[k]
            out.append(res)
        return out

    def info(self):
        bi = BatchInfo()
        _check(lib().ft_batch_get_info(self.h, ctypes.byref(bi)))
        return {f: getattr(bi, f) for f, _ in BatchInfo._fields_}

    def close(self):
        if getattr(self, "h", None):
            lib().ft_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def choose_lambda(inputs, candidates=(0.05, 0.1, 0.2, 0.3, 0.5, 0.8), pilot=200_000, precision=MIXED, seed=0,
                  eps_order=0):
    """Deformation parameter per integral from pilot runs: for every candidate lambda,
    all inputs (the low-level JSON dicts) at that lambda integrated as one batch with
    `pilot` samples; per input the lambda with the smallest relative standard error of
    its eps order `eps_order` (max over Re and Im, relative to the larger of |Re|, |Im|).
    The contour deformation does not change the integral, only the spread of the
    integrand (srcs/feynman_integral.hpp:288-291), so the best lambda shortens the time
    to a target error by the square of the error ratio.  Inputs whose plan the checks
    reject at some lambda skip it.  Returns [(lambda, relative error, {lambda: relative
    error})] per input."""
    table = [dict() for _ in inputs]
    for lam in candidates:
        plans = create_plans([dict(x, **{"lambda": lam}) for x in inputs], skip_failed=True)
        idx = [i for i, p in enumerate(plans) if p is not None]
        if not idx:
            continue
        b = Batch([plans[i] for i in idx], precision)
        out = b.run(pilot, seeds=seed)
        b.close()
        for k, i in enumerate(idx):
            (re, dre), (im, dim) = out[k]["integral"][eps_order]
            scale = max(abs(re), abs(im))
            rel = max(dre, dim) / scale if scale > 0 else math.inf
            table[i][lam] = rel if math.isfinite(rel) else math.inf
        for p in plans:
            if p is not None:
                p.close()
    best = []
    for t in table:
        if not t:
            best.append((None, math.inf, t))
            continue
        lam = min(t, key=lambda l: (t[l], l))
        best.append((lam, t[lam], t))
    return best


def integrate_batch(plans, N, seeds=0, precision=MIXED, first_samples=0):
    """ft_integrate_batch: a transient batch over the plans (same precision for all)."""
    n = len(plans)
    Ns = list(N) if hasattr(N, "__len__") else [N] * n
    ss = list(seeds) if hasattr(seeds, "__len__") else [seeds] * n
    fs = list(first_samples) if hasattr(first_samples, "__len__") else [first_samples] * n
    arr = (ctypes.c_void_p * n)(*[p.h.value for p in plans])
    opts = (RunOptions * n)(*[RunOptions(int(Ns[i]), int(ss[i]), int(fs[i]), int(precision), None)
                               for i in range(n)])
    ras = [_ResultArrays(p.K) for p in plans]
    res = (Result * n)(*[r.res for r in ras])
    _check(lib().ft_integrate_batch(ctypes.cast(arr, ctypes.c_void_p), n, ctypes.cast(opts, ctypes.c_void_p),
                                    ctypes.cast(res, ctypes.c_void_p)))
    out = []
    for i, r in enumerate(ras):
        r.res = res[i]
        out.append(r.as_dict(plans[i].info["IGtr"]))
    return out


def finalize_moments(moments, K, real_only):
    """avg/acc from merged moments (list of 2K [n, s1_hi, s1_lo, s2_hi, s2_lo])."""
    m = (Moments * (2 * K))(*[Moments(*x) for x in moments])
    arr = np.zeros((4, K))
    res = Result(K, _ptr(arr[0]).value, _ptr(arr[1]).value, _ptr(arr[2]).value, _ptr(arr[3]).value, None)
    _check(lib().ft_finalize_moments(ctypes.cast(m, ctypes.c_void_p), K, 1 if real_only else 0, ctypes.byref(res)))
    return [[[arr[0, j], arr[1, j]], [arr[2, j], arr[3, j]]] for j in range(K)]


def run_json(inp, with_log=False):
    """The reference's CLI contract in process: input (dict or JSON text) -> output dict."""
    text = inp if isinstance(inp, str) else json.dumps(inp)
    out = ctypes.c_void_p()
    log = ctypes.c_void_p()
    L = lib()
    rc = L.ft_run_json(text.encode(), ctypes.byref(out), ctypes.byref(log))
    log_text = ctypes.string_at(log.value).decode() if log.value else ""
    if log.value:
        L.ft_free(log)
    if rc != FT_OK:
        if out.value:
            L.ft_free(out)
        raise FeyntropError(rc, log_text.strip())
    res = json.loads(ctypes.string_at(out.value).decode().replace("NaN", "null"))
    L.ft_free(out)
    return (res, log_text) if with_log else res
