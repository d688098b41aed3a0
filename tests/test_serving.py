"""Serving (sstmc_server_*): continuous batching of renders over resident
scenes.  A request's result depends only on (scene, seed), so every request
gives the same result alone and in the mix: identical iteration counts and
statistics, and fields equal up to the order of the FP64 accumulation."""
import ctypes as C

import numpy as np
import pytest

from temporalspecklescode_gb300 import workloads as wl
from tests.scenes import small_scenes

SCENES = small_scenes()
TIMEOUT = 101
CANCELLED = 102


def rel_fro(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def api():
    from temporalspecklescode_gb300 import api as A
    A.load_library()
    return A


def test_server_rejects_null_handles():
    from temporalspecklescode_gb300 import _build
    import os
    if not os.path.exists(_build.lib_path()):
        _build.build_library()
    lib = C.CDLL(_build.lib_path())
    assert lib.sstmc_server_destroy(None) == 103
    assert lib.sstmc_submit(None, None, C.c_uint64(0), None, None, None) == 103
    assert lib.sstmc_poll(None, C.c_uint64(1), None, None) == 103


@pytest.mark.gpu
def test_same_result_alone_and_in_the_mix(api):
    names = ["speckle_2d", "correlation_3d", "transmission_matrix_3d", "corr_far_2d_drift", "field_point_3d", "mcx_3d",
             "vmf_transmission_3d", "forced_bin_2d_cbs", "tabular_corr_2d"]
    scenes = {n: api.Scene(*SCENES[n]) for n in names}
    big = api.Scene(*wl.correlation_3d(batch_size=8192, full_iteration=2, n_side=8, n_lags=8))
    try:
        alone = {}
        for n, s in scenes.items():
            u, it = s.render(seed=17)
            alone[n] = (u, it, s.stats())
        ub, itb = big.render(seed=3)
        with api.Server(slots=4) as srv:
            reqs = [srv.submit(big, 3)]
            for rep in range(2):
                for n in names:
                    reqs.append(srv.submit(scenes[n], 17))
            outs = [r.result() for r in reqs]
            st = srv.stats()
        u, it = outs[0]
        assert np.array_equal(it, itb)
        assert rel_fro(u, ub) <= 1e-12
        for k, r in enumerate(reqs[1:]):
            n = names[k % len(names)]
            u, it = outs[k + 1]
            assert np.array_equal(it, alone[n][1]), n
            assert rel_fro(u, alone[n][0]) <= 1e-12, (n, rel_fro(u, alone[n][0]))
        assert st["completed"] == len(reqs)
        assert st["p99_ms"] >= st["p50_ms"] > 0 and st["contributions_per_s"] > 0
    finally:
        big.close()
        for s in scenes.values():
            s.close()


@pytest.mark.gpu
def test_budget_admission_and_cancel(api):
    # a budget smaller than one request: requests run one at a time, all complete
    cfg, dims = wl.correlation_3d(batch_size=4096, full_iteration=2, n_side=8, n_lags=8)
    scenes = [api.Scene(cfg, dims) for _ in range(3)]
    try:
        ref, itr = scenes[0].render(seed=9)
        with api.Server(hbm_budget_bytes=1 << 20, slots=3) as srv:
            reqs = [srv.submit(s, 9) for s in scenes]
            late = srv.submit(scenes[0], 9)
            late.cancel()
            outs = [r.result() for r in reqs]
            st_late = late.wait()
        # the small reservation gives smaller chunks than the direct render: the
        # paths are the same, the compensated FP32 windows of the contraction
        # fall elsewhere (FP32-level differences, far inside the 1e-5 budget)
        for u, it in outs:
            assert np.array_equal(it, itr)
            assert rel_fro(u, ref) <= 1e-6
        assert st_late in (0, CANCELLED)
    finally:
        for s in scenes:
            s.close()


@pytest.mark.gpu
def test_wait_times_out_on_an_open_request(api):
    cfg, dims = wl.correlation_3d(batch_size=1 << 16, full_iteration=4, n_side=8, n_lags=8)
    with api.Scene(cfg, dims) as s, api.Server(slots=1) as srv:
        r = srv.submit(s, 1)
        with pytest.raises(api.SstmcError) as ex:
            r.wait(timeout=0.0)
        assert ex.value.code == TIMEOUT
        assert r.wait() == 0


@pytest.mark.gpu
def test_busy_scene_does_not_block_other_scenes(api):
    """Two requests on one scene, then requests on two other scenes, on a
    two-slot server: the second request on the busy scene is passed over, so
    the other scenes' requests start on the free slot and complete while the
    first long render is still running, instead of waiting behind it."""
    import time
    big = api.Scene(*wl.correlation_3d(batch_size=1 << 20, full_iteration=2, n_side=8, n_lags=8))
    small = [api.Scene(*SCENES[n]) for n in ("speckle_2d", "corr_far_2d_drift")]
    try:
        big.render(seed=1)                       # warm-up: kernels loaded, pool grown
        for s in small:
            s.render(seed=1)
        with api.Server(slots=2) as srv:
            reqs = [srv.submit(big, 5), srv.submit(big, 6)] + [srv.submit(s, 7) for s in small]
            order = []
            t0 = time.perf_counter()
            while len(order) < len(reqs) and time.perf_counter() - t0 < 300:
                for i, r in enumerate(reqs):
                    if i not in order and r.done():
                        order.append(i)
                time.sleep(1e-4)
            outs = [r.result() for r in reqs]
            st = srv.stats()
        assert len(order) == len(reqs)
        # both small requests finish before the first render of the busy scene
        assert order.index(2) < order.index(0) and order.index(3) < order.index(0), order
        assert order.index(0) < order.index(1), order
        for s, (u, it) in zip(small, outs[2:]):
            ua, ita = s.render(seed=7)
            assert np.array_equal(ita, it) and rel_fro(u, ua) <= 1e-6
        assert st["completed"] == 4
    finally:
        big.close()
        for s in small:
            s.close()
