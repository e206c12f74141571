"""Server scheduling on the host executor (no GPU): admission by slots and HBM budget, pass slicing,
cancellation, back-pressure, malformed jobs, concurrent submitters and an injected device failure.
Failures are made on the host (a simulated device error, an over-budget job), never on a GPU."""
import threading
import time

import numpy as np
import pytest

from ataraxia_gb300 import AtxError, Camera, Server, Settings, scenes
from tests.helpers import job_bytes_bound


def job_scene(w=32, h=16, n=20, seed=0):
    sc = scenes.config1()
    return scenes.SyntheticScene(**{**sc.__dict__, "spheres": sc.spheres[seed:seed + n], "width": w, "height": h,
                                    "max_bounces": 4})


def test_jobs_complete_with_all_frames():
    with Server(host_executor=True, pass_spp=4) as s:
        ids = [s.submit(job_scene(seed=i), target) for i, target in enumerate([1, 4, 9, 16])]
        for j, target in zip(ids, [1, 4, 9, 16]):
            s.wait(j, 10000)
            info = s.poll(j)
            assert info["state"] == "done" and info["frames_done"] == target
            assert info["submit_s"] <= info["admit_s"] <= info["done_s"]
            assert np.all(s.image(j) == target)
            assert np.all(s.accumulation(j)[:, 3] == target)
        st = s.stats()
        assert st["completed"] == 4 and st["active"] == 0 and st["queued"] == 0
        assert st["passes"] >= 4           # the 16-spp job needs four 4-spp passes


def test_admission_respects_hbm_budget():
    sc = job_scene(64, 64)
    from ataraxia_gb300 import _native as N
    import ctypes as C

    per_job = job_bytes_bound(sc)
    budget = int(2.5 * per_job)
    peak = {"bytes": 0, "active": 0}
    with Server(host_executor=True, hbm_budget_bytes=budget, pass_spp=2) as s:
        ids = [s.submit(sc, 8) for _ in range(6)]
        done = False
        while not done:
            st = s.stats()
            peak["bytes"] = max(peak["bytes"], st["device_bytes"])
            peak["active"] = max(peak["active"], st["active"])
            done = st["completed"] == 6
            time.sleep(0.0005)
        assert peak["bytes"] <= budget
        assert 1 <= peak["active"] <= 2
        assert all(s.poll(j)["state"] == "done" for j in ids)


def test_over_budget_job_rejected_and_backpressure():
    with Server(host_executor=True, hbm_budget_bytes=10000, max_pending=2) as s:
        with pytest.raises(AtxError) as e:
            s.submit(job_scene(256, 256), 4)
        assert e.value.status == 2
        assert s.stats()["rejected"] == 1
    # a worker that cannot keep up: the third queued job is refused with BUSY
    with Server(host_executor=True, max_active_jobs=1, max_pending=2, pass_spp=1) as s:
        big = job_scene(512, 512)
        s.submit(big, 1000)                       # occupies the only slot for a while
        time.sleep(0.05)
        s.submit(big, 1)
        s.submit(big, 1)
        with pytest.raises(AtxError) as e:
            s.submit(big, 1)
        assert e.value.status == 5


def test_malformed_jobs_rejected():
    sc = job_scene()
    with Server(host_executor=True) as s:
        bad = sc.spheres.copy()
        bad["radius"][3] = np.nan
        cam = Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction)
        st = Settings(True, False, 4)
        for args in [(bad, sc.materials, sc.lights, cam, sc.width, sc.height, st, 4),
                     (sc.spheres, sc.materials, sc.lights, cam, 0, 10, st, 4),
                     (sc.spheres, sc.materials, sc.lights, cam, 8, 8, st, 0),
                     (sc.spheres, sc.materials[:0], sc.lights, cam, 8, 8, st, 4)]:
            with pytest.raises(AtxError) as e:
                s.submit_scene(*args)
            assert e.value.status == 1
        with pytest.raises(AtxError) as e:
            s.poll(12345)
        assert e.value.status == 6


def test_cancel_queued_and_active():
    with Server(host_executor=True, max_active_jobs=1, pass_spp=1) as s:
        a = s.submit(job_scene(512, 512), 200)
        b = s.submit(job_scene(), 4)
        time.sleep(0.01)
        s.cancel(b)
        assert s.poll(b)["state"] == "cancelled"
        s.cancel(a)
        with pytest.raises(AtxError) as e:
            s.wait(a, 10000)
        assert e.value.status == 7
        assert s.poll(a)["state"] == "cancelled" and s.poll(a)["frames_done"] < 200
        c = s.submit(job_scene(), 3)
        s.wait(c, 10000)
        s.release(c)
        with pytest.raises(AtxError):
            s.poll(c)


def test_injected_device_failure_fails_active_jobs_only():
    with Server(host_executor=True, pass_spp=1, host_fail_pass=3) as s:
        a = s.submit(job_scene(), 10)
        with pytest.raises(AtxError) as e:
            s.wait(a, 10000)
        assert e.value.status == 3
        assert s.poll(a)["state"] == "failed"
        b = s.submit(job_scene(), 2)              # the server keeps serving after the failure
        s.wait(b, 10000)
        assert s.poll(b)["state"] == "done"
        st = s.stats()
        assert st["failed"] == 1 and st["completed"] == 1 and st["device_bytes"] == 0


def test_concurrent_submitters_and_pass_slicing():
    ids = []
    lock = threading.Lock()
    with Server(host_executor=True, pass_spp=8, max_pass_paths=32 * 16 * 6) as s:
        def worker(k):
            for i in range(10):
                j = s.submit(job_scene(seed=(k * 10 + i) % 200), 1 + (i % 5) * 3)
                with lock:
                    ids.append((j, 1 + (i % 5) * 3))

        th = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for j, target in ids:
            s.wait(j, 20000)
            assert s.poll(j)["frames_done"] == target
        st = s.stats()
        assert st["completed"] == 40 and st["submitted"] == 40
        # pass slices were scaled down: never more than max_pass_paths per pass (or one frame per job)
        assert st["paths"] <= st["passes"] * max(32 * 16 * 6, 32 * 16 * 64)


def test_smallest_first_policy():
    """With one slot busy, queued jobs are admitted smallest first (arrival order by default)."""
    order = {}
    for policy in ("arrival", "smallest"):
        with Server(host_executor=True, max_active_jobs=1, pass_spp=64, policy=policy) as s:
            blocker = s.submit(job_scene(512, 512), 64)          # holds the slot for ~17 ms
            big = s.submit(job_scene(256, 256), 64)
            small = s.submit(job_scene(16, 16), 4)
            for j in (blocker, big, small):
                s.wait(j, 10000)
            order[policy] = s.poll(small)["done_s"] < s.poll(big)["done_s"]
    assert order == {"arrival": False, "smallest": True}


def test_camera_change_restarts_job():
    sc = job_scene(512, 512)                     # 0.26 ms of simulated device time per frame
    with Server(host_executor=True, pass_spp=1) as s:
        j = s.submit(sc, 40)
        while s.poll(j)["frames_done"] < 5:
            time.sleep(0.0005)
        cam = Camera(sc.fov, sc.near, sc.far, (1.0, 2.0, 3.0), sc.camera_direction)
        s.set_camera(j, cam)
        s.wait(j, 10000)
        info = s.poll(j)
        assert info["state"] == "done" and info["frames_done"] == 40
        assert np.all(s.image(j) == 40)          # every frame of the result is from after the change
        with pytest.raises(AtxError) as e:
            s.set_camera(j, cam)                 # finished: nothing to restart
        assert e.value.status == 5
