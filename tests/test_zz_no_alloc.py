"""ft_integrate_noalloc: the integration entry point for callers that must not
allocate device memory while they integrate (for instance an application that owns
all device memory itself, or a serving loop in which allocation is not allowed).
It runs the same launches as ft_integrate on the same samples, with its scratch in a
static device array instead of cudaMalloc'd buffers, and writes the final sums into
a device buffer the caller owns.

Called through the C ABI twice in a row (the scratch keeps the previous call's
contents), in both precisions, and compared with ft_integrate on the same samples;
also with a launch of several waves of blocks, past the FP64 hand-off queue's
capacity, and with the inputs it must reject.  This file is collected last on purpose.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import feyntrop_gb300 as ft

pytestmark = pytest.mark.gpu

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))
N = 2_000_000
# identical samples and identical launch shape: the sums agree to rounding of the
# block reduction order (which is the same), so the integrals agree to 1e-12
RTOL = 1e-12


def slots_to_integral(slots, K, real_only):
    moments = []
    kept = slots[8 * K]
    for j in range(K):
        for part in range(2):
            b = 8 * j + 4 * part
            moments.append([kept, slots[b], slots[b + 1], slots[b + 2], slots[b + 3]])
    return ft.finalize_moments(moments, K, real_only), int(slots[8 * K]), int(slots[8 * K + 1])


@pytest.mark.parametrize("name", ["C2_double_box", "C1_K4"])
@pytest.mark.parametrize("precision", [ft.FP64, ft.MIXED])
def test_noalloc_matches_integrate_on_two_calls(name, precision):
    torch = pytest.importorskip("torch")
    inp = PINS["cases"][name]["input"]
    plan = ft.Plan(inp)
    K = plan.K
    real_only = not plan.info["deformed"]
    # the regular entry point: reference result, and it loads the plan's kernels
    ref = plan.integrate(N, seed=7, precision=precision)
    out = torch.full((8 * K + 8,), float("nan"), dtype=torch.float64, device="cuda")
    lib = ft.lib()
    opts = ft.RunOptions(N, 7, 0, precision, None)
    for call in range(2):
        rc = lib.ft_integrate_noalloc(plan.h, ctypes.byref(opts), ctypes.c_void_p(out.data_ptr()))
        assert rc == ft.FT_OK, lib.ft_last_error().decode()
        torch.cuda.synchronize()
        slots = out.cpu().numpy()
        integral, kept, dropped = slots_to_integral(slots, K, real_only)
        assert kept + dropped == N
        assert kept == ref["kept"]
        for j in range(K):
            for part in range(2):
                a, da = integral[j][part]
                b, db = ref["integral"][j][part]
                assert abs(a - b) <= RTOL * max(abs(b), 1e-300) or a == b, (call, j, part, a, b)
                assert abs(da - db) <= RTOL * max(abs(db), 1e-300) or da == db, (call, j, part, da, db)
        out.fill_(float("nan"))
    plan.close()


def test_noalloc_rejects_what_the_scratch_cannot_hold():
    torch = pytest.importorskip("torch")
    # 17 eps orders need 144 slots per block, more than the static scratch holds
    inp = dict(PINS["cases"]["K4_masses_1to6"]["input"], num_eps_terms=17)
    plan = ft.Plan(inp)
    plan.integrate(1000, precision=ft.FP64)   # loads the kernels
    out = torch.zeros(8 * plan.K + 8, dtype=torch.float64, device="cuda")
    lib = ft.lib()
    opts = ft.RunOptions(1000, 0, 0, ft.FP64, None)
    rc = lib.ft_integrate_noalloc(plan.h, ctypes.byref(opts), ctypes.c_void_p(out.data_ptr()))
    assert rc == ft.FT_ERR_INVALID_ARGUMENT
    assert "16 eps orders" in lib.ft_last_error().decode()
    plan.close()


def _noalloc(plan, N, precision, seed=7):
    torch = pytest.importorskip("torch")
    out = torch.full((8 * plan.K + 8,), float("nan"), dtype=torch.float64, device="cuda")
    opts = ft.RunOptions(N, seed, 0, precision, None)
    rc = ft.lib().ft_integrate_noalloc(plan.h, ctypes.byref(opts), ctypes.c_void_p(out.data_ptr()))
    torch.cuda.synchronize()
    return rc, out.cpu().numpy()


def test_noalloc_rejects_unloaded_kernels_and_zero_samples():
    plan = ft.Plan(PINS["cases"]["C1_K4"]["input"])
    rc, _ = _noalloc(plan, 1000, ft.FP64)   # nothing loaded yet: loading would allocate
    assert rc == ft.FT_ERR_INVALID_ARGUMENT
    assert "not loaded" in ft.lib().ft_last_error().decode()
    plan.integrate(1000, precision=ft.FP64)
    rc, _ = _noalloc(plan, 0, ft.FP64)
    assert rc == ft.FT_ERR_INVALID_ARGUMENT
    assert "num_samples" in ft.lib().ft_last_error().decode()
    plan.close()


def test_noalloc_several_waves_match_integrate():
    """An FP64 kernel without the per-sample barrier runs waves of at most 128 samples
    per thread; the no-allocation path keeps them (here two waves of one block per SM)."""
    os.environ["FEYNTROP_GB300_VARIANT"] = "0"
    try:
        plan = ft.Plan(PINS["cases"]["C2_double_box"]["input"])
        n = 6_000_000
        ref = plan.integrate(n, seed=3, precision=ft.FP64)
        for call in range(2):
            rc, slots = _noalloc(plan, n, ft.FP64, seed=3)
            assert rc == ft.FT_OK, ft.lib().ft_last_error().decode()
            integral, kept, dropped = slots_to_integral(slots, plan.K, False)
            assert kept == ref["kept"] and kept + dropped == n
            for j in range(plan.K):
                for part in range(2):
                    a, da = integral[j][part]
                    b, db = ref["integral"][j][part]
                    assert abs(a - b) <= RTOL * abs(b) and abs(da - db) <= RTOL * db, (call, j, part, a, b)
        plan.close()
    finally:
        del os.environ["FEYNTROP_GB300_VARIANT"]


def test_noalloc_reports_fp64_queue_overflow():
    """More samples handed to the FP64 pass than its 65536 queue entries: the ones
    beyond are not evaluated, and slot 8K+2 (every hand-off) and kept + dropped < N
    say so.  The double box at its Minkowski point without the deformation (lambda = 0,
    one eps order): V changes sign inside the domain, and every sample with V near or
    below zero goes to the FP64 pass."""
    from feyntrop_gb300 import workloads
    plan = ft.Plan(dict(workloads.double_box(N=1000, lam=0.0), num_eps_terms=1))
    probe = plan.integrate(200_000, seed=1, precision=ft.MIXED)
    rate = probe["fp64_fallback"] / 200_000
    assert rate > 0.01, rate
    n = int(min(2e9, 3 * 65536 / rate))
    rc, slots = _noalloc(plan, n, ft.MIXED, seed=1)
    assert rc == ft.FT_OK, ft.lib().ft_last_error().decode()
    K = plan.K
    handed = slots[8 * K + 2]
    kept, dropped = slots[8 * K], slots[8 * K + 1]
    assert handed > 65536
    assert kept + dropped == n - (handed - 65536)
    plan.close()
