"""Serving: requests submitted while others run are admitted by memory budget,
batched together, and each result equals the same solve run alone (bitwise);
failures stay isolated; a stalled worker is detected on the host."""
import time

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import periodic_square
from dgcuda_gb300.serve import Server, request
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

VORTEX = (5.0, 5.0, 3.0, 1.0, 0.5, 10.0, 10.0)
GAUSS = (0.3, 0.6, 0.02, 1.0, 1.0)


def specs():
    out = []
    for i in range(12):
        euler = i % 2 == 0
        out.append(dict(n=[6, 9, 12, 16][i % 4], order=1 + i % 4,
                        equation=_ffi.EULER if euler else _ffi.ADVECTION,
                        ic=_ffi.IC_VORTEX if euler else _ffi.IC_GAUSSIAN,
                        params=VORTEX if euler else GAUSS, t_end=0.05 + 0.01 * i,
                        lx=10.0 if euler else 1.0, ly=10.0 if euler else 1.0,
                        jitter=0.15, seed=100 + i, a=(1.0, 0.6)))
    return out


def run_alone(sp):
    m = periodic_square(sp["n"], lx=sp["lx"], ly=sp["ly"], jitter=sp["jitter"], seed=sp["seed"])
    sv = Solver(m, sp["order"], sp["equation"], _ffi.FLUX_LLF, _ffi.FP32, a=sp["a"])
    sv.project(sp["ic"], sp["params"])
    sv.set_dt(None, cfl=0.7)
    n, t = sv.run(t_end=sp["t_end"])
    return sv.get_state(), n, t


def test_results_equal_alone_and_in_mix(gpu):
    srv = Server(budget_bytes=1 << 30, max_active=64)
    srv.set_steps_per_check(4)
    ids = []
    for k, sp in enumerate(specs()):
        ids.append(srv.submit(request(keep_state=True, **sp)))
        if k % 3 == 2:
            time.sleep(0.01)          # later requests arrive while earlier ones run
    assert srv.wait_idle(120.0) == _ffi.OK
    st = srv.stats()
    assert st["completed"] == 12 and st["failed"] == 0 and st["repacks"] >= 1
    assert st["p99_latency_s"] >= st["p50_latency_s"] > 0
    for rid, sp in zip(ids, specs()):
        ref, nref, tref = run_alone(sp)
        state, tot, steps, tfin = srv.result(rid, ref.size)
        assert steps == nref and tfin == tref
        np.testing.assert_array_equal(state.reshape(ref.shape), ref)
    srv.close()


def test_budget_admission_serialises_but_completes(gpu):
    sp = dict(specs()[0], n=6, order=1)
    # a budget (64 KiB) that holds one of these solves (mesh and solver blocks,
    # 48 KiB) at a time
    srv = Server(budget_bytes=64 << 10, max_active=64)
    ids = [srv.submit(request(**dict(sp, seed=sp["seed"] + i))) for i in range(4)]
    assert srv.wait_idle(120.0) == _ffi.OK
    st = srv.stats()
    assert st["completed"] == 4
    # each admission had to evict the previous request's idle mesh to fit
    assert st["cached_meshes"] == 1
    for rid in ids:
        assert srv.status(rid)[0] == _ffi.REQ_DONE
    srv.close()


def test_pool_reuse_and_mesh_cache(gpu):
    sp = specs()
    srv = Server(budget_bytes=1 << 30, max_active=64)
    first = [srv.submit(request(**dict(s, keep_state=1))) for s in sp]
    assert srv.wait_idle(120.0) == _ffi.OK
    st1 = srv.stats()
    assert st1["completed"] == len(sp) and st1["pool_misses"] > 0
    assert st1["cached_meshes"] == len({(s["n"], s["lx"], s["seed"]) for s in sp})
    # the same requests again: their meshes come from the cache, their solver
    # blocks from the pool (nothing is allocated), and the results repeat
    second = [srv.submit(request(**dict(s, keep_state=1))) for s in sp]
    assert srv.wait_idle(120.0) == _ffi.OK
    st2 = srv.stats()
    assert st2["completed"] == 2 * len(sp)
    assert st2["pool_misses"] == st1["pool_misses"] and st2["pool_hits"] >= st1["pool_hits"] + len(sp)
    assert st2["cached_meshes"] == st1["cached_meshes"]
    for s, a, b in zip(sp, first, second):
        size = (4 if s["equation"] == _ffi.EULER else 1) * (s["order"] + 1) * (s["order"] + 2) // 2 * 2 * s["n"] ** 2
        ra, rb = srv.result(a, size), srv.result(b, size)
        np.testing.assert_array_equal(ra[0], rb[0])
        np.testing.assert_array_equal(ra[1], rb[1])
        assert ra[2] == rb[2] and ra[3] == rb[3]
    srv.close()


def test_failed_request_is_isolated(gpu):
    srv = Server(budget_bytes=1 << 30, max_active=64)
    good = srv.submit(request(**specs()[0]))
    # negative density: the device status word flags it, the solve fails alone
    bad = srv.submit(request(n=8, order=2, equation=_ffi.EULER, ic=_ffi.IC_CONSTANT,
                             params=(-1.0, 0.0, 0.0, 1.0), t_end=0.1, lx=10, ly=10))
    assert srv.wait_idle(120.0) == _ffi.OK
    assert srv.status(good)[0] == _ffi.REQ_DONE
    state, _, rc = srv.status(bad)
    assert state == _ffi.REQ_FAILED and rc == _ffi.ERR_NONFINITE
    srv.close()


def test_cancel_and_stall_detection(gpu):
    srv = Server(budget_bytes=1 << 30, max_active=64)
    srv.inject_stall(0.5)             # the worker sleeps after every check
    ids = [srv.submit(request(**dict(specs()[1], t_end=0.5))) for _ in range(3)]
    srv.cancel(ids[2])
    # a stalled worker shows up as a timeout on the host, not as a hung GPU
    assert srv.wait_idle(0.2) == _ffi.ERR_TIMEOUT
    srv.inject_stall(0.0)
    assert srv.wait_idle(120.0) == _ffi.OK
    assert srv.status(ids[2])[0] == _ffi.REQ_CANCELLED
    assert srv.status(ids[0])[0] == _ffi.REQ_DONE
    srv.close()
