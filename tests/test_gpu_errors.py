"""Error paths of the step, provoked without faulting the GPU
(gbodeTestInject), through the C ABI.

* A grid barrier whose counter starts one arrival short (and, under the
  two-level sweep's neighbour waits, every block's step counter one step
  short): every block's bounded wait runs out (2^22 polls, a second or two), the solver kernel
  returns, gbodeWorldSynchronize reports ERR_BARRIER_TIMEOUT (0x1), and the
  next step runs normally on the same context.
* A staging wait that names a copy never issued: ERR_STAGE_TIMEOUT (0x100),
  the blocks leave together, the next step runs normally.
* Capacities the kernels see lowered below what is allocated: contacts
  (ERR_CONTACT_OVERFLOW, 0x4; the step keeps the first contacts), contact
  rows (ERR_ROW_OVERFLOW, 0x8; the step keeps the first contacts whose rows
  fit), colours (ERR_COLOUR_OVERFLOW, 0x10).
* A device allocation that fails, at every allocation a first step makes in
  turn: dWorldQuickStep (or the collision before it) returns 0 with a
  message, the world's state is unchanged, and the step then succeeds with
  the same result as a world that never failed (the reference's allocation
  failure contract, ode.cpp:1852-1863, util.cpp:1162-1217).
Nothing here traps, faults or hangs: every wait is bounded.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_BARRIER_TIMEOUT, ERR_CONTACT_OVERFLOW, ERR_ROW_OVERFLOW = 0x1, 0x4, 0x8
ERR_COLOUR_OVERFLOW, ERR_STAGE_TIMEOUT = 0x10, 0x100


def _sync_bits(w):
    """gbodeWorldSynchronize: (ok, error bits named in the message)."""
    L = w.L
    if L.gbodeWorldSynchronize(w.w):
        return True, 0
    msg = L.gbodeGetLastError().decode()
    assert "device error bits" in msg, msg
    return False, int(msg.split("0x")[1].split()[0], 16)


def _settled_pile(two_level=0, n=2048, steps=40, classes=0):
    from ode_gb300 import scenes, sim
    w = sim.GBWorld(scenes.pile(n, seed=11))
    w.L.dWorldSetQuickStepNumIterations(w.w, 30)
    w.L.gbodeWorldSetTwoLevelSweep(w.w, two_level)
    w.L.gbodeWorldSetCrossClasses(w.w, classes)
    for _ in range(steps):
        w.step_fused()
    assert _sync_bits(w) == (True, 0)
    return w


@pytest.fixture(autouse=True)
def _injection_off(gblib):
    from ode_gb300 import ode
    gblib.gbodeTestInject(ode.GBODE_TEST_OFF, 0, 0)
    yield
    gblib.gbodeTestInject(ode.GBODE_TEST_OFF, 0, 0)


@pytest.mark.parametrize("two_level,classes", [(0, 0), (2, 0), (2, 4)])
@pytest.mark.parametrize("kind,bit", [("barrier", ERR_BARRIER_TIMEOUT), ("stage", ERR_STAGE_TIMEOUT)])
def test_bounded_waits_run_out_and_report(gblib, two_level, classes, kind, bit):
    from ode_gb300 import ode
    L = gblib
    w = _settled_pile(two_level, classes=classes)
    before = w.stats().iterations
    L.gbodeTestInject(ode.GBODE_TEST_BARRIER if kind == "barrier" else ode.GBODE_TEST_STAGE, 1, 0)
    t0 = time.perf_counter()
    w.step_fused()
    ok, bits = _sync_bits(w)
    dt = time.perf_counter() - t0
    print(f"{kind} ({'two-level' if two_level else 'one-level'} sweep): error bits {bits:#x} after {dt:.2f} s "
          f"(sweeps of the last good step {before})")
    assert not ok and bits & bit
    assert dt < 60.0
    # the context is usable: the next step runs and reports nothing
    for _ in range(3):
        w.step_fused()
    assert _sync_bits(w) == (True, 0)
    assert w.stats().iterations > 0 and np.isfinite(w.state()).all()
    w.close()


def test_capacity_overflows_are_reported(gblib):
    from ode_gb300 import ode
    L = gblib
    w = _settled_pile(steps=150)
    s = w.stats()
    nc = s.contacts
    assert nc > 400 and s.colours > 2
    # contacts: the narrow phase keeps the first half
    L.gbodeTestInject(ode.GBODE_TEST_CONTACT_CAP, nc // 2, 0)
    w.step_fused()
    ok, bits = _sync_bits(w)
    assert not ok and bits & ERR_CONTACT_OVERFLOW
    assert w.stats().contacts == nc // 2
    L.gbodeTestInject(ode.GBODE_TEST_CONTACT_CAP, 0, 0)
    # rows: the assembly keeps the first contacts whose rows (3 each) fit in 301
    L.gbodeTestInject(ode.GBODE_TEST_ROW_CAP, 301, 0)
    w.step_fused()
    ok, bits = _sync_bits(w)
    assert not ok and bits & ERR_ROW_OVERFLOW
    s = w.stats()
    assert s.rows == 300 and s.contacts == 100, (s.rows, s.contacts)
    L.gbodeTestInject(ode.GBODE_TEST_ROW_CAP, 0, 0)
    # colours: two colours cannot separate the pile's manifolds
    L.gbodeTestInject(ode.GBODE_TEST_COLOUR_CAP, 2, 0)
    w.step_fused()
    ok, bits = _sync_bits(w)
    assert not ok and bits & ERR_COLOUR_OVERFLOW
    L.gbodeTestInject(ode.GBODE_TEST_COLOUR_CAP, 0, 0)
    for _ in range(3):
        w.step_fused()
    assert _sync_bits(w) == (True, 0)
    assert np.isfinite(w.state()).all()
    w.close()


@pytest.mark.parametrize("two_level,classes", [(0, 0), (2, 0), (2, 4)])
def test_failed_allocation_leaves_state_unchanged(gblib, two_level, classes):
    from ode_gb300 import ode, scenes, sim
    L = gblib
    sc = scenes.pile(512, seed=13)

    def world():
        w = sim.GBWorld(sc)
        L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        L.gbodeWorldSetTwoLevelSweep(w.w, two_level)
        L.gbodeWorldSetCrossClasses(w.w, classes)
        return w

    def fused(w):
        ok = L.gbodeSpaceCollideContacts(w.space, w.w, w.group, ctypes.byref(w.surface), sc.maxc)
        if ok:
            ok = L.dWorldQuickStep(w.w, sc.dt)
        L.dJointGroupEmpty(w.group)
        return ok

    ref = world()
    assert fused(ref) == 1
    assert _sync_bits(ref) == (True, 0)
    expect = ref.state()
    ref.close()
    failed = tolerated = 0
    for k in range(1000):
        w = world()
        start = w.state()
        L.gbodeTestInject(ode.GBODE_TEST_ALLOC, k, 1)
        ok = fused(w)
        pending = L.gbodeTestInject(ode.GBODE_TEST_ALLOC_PENDING, 0, 0)
        L.gbodeTestInject(ode.GBODE_TEST_ALLOC, -1, 0)
        if ok:
            assert _sync_bits(w) == (True, 0)
            if pending:  # the step made fewer than k + 1 allocations: every one has failed in turn
                w.close()
                break
            # a failure the library works around (the scan's scratch-free path): same result
            tolerated += 1
            np.testing.assert_array_equal(w.state(), expect, err_msg=f"allocation {k} worked around")
            w.close()
            continue
        failed += 1
        assert L.gbodeGetLastError().decode() != "", f"allocation {k}: no message"
        np.testing.assert_array_equal(w.state(), start, err_msg=f"allocation {k}")
        assert fused(w) == 1, L.gbodeGetLastError()
        assert _sync_bits(w) == (True, 0)
        np.testing.assert_array_equal(w.state(), expect, err_msg=f"after allocation {k} failed")
        w.close()
    else:
        pytest.fail("the step kept allocating")
    print(f"{'two-level' if two_level else 'one-level'} sweep{' in split classes' if classes else ''}: "
          f"{failed} allocation points of a first step "
          f"failed in turn, each leaving the state unchanged; {tolerated} worked around with the same result")
    assert failed > 20
