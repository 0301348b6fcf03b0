"""Host logic of the benchmark's double-buffered camera path (the viewer's
worker-thread cache update, realtime_viewer/src/application.cu:168-229),
run on the CPU with a fake renderer: a build starts when a frame's coverage
is below the threshold and no build is running, frames keep rendering
meanwhile, and the timed region ends after the last build."""
import os
import sys
import threading
import time
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class FakeRenderer:
    def __init__(self, build_s):
        self.build_s = build_s
        self.builds, self.renders, self.swaps = [], 0, 0
        self.lock = threading.Lock()
        self.current = 0  # the frame the current cache was built at

    def initCacheBlockwise(self, info):
        time.sleep(self.build_s)
        with self.lock:
            self.builds.append(info)

    def swapCache(self):
        with self.lock:
            self.swaps += 1
            self.current = self.builds[-1]

    def render_device(self, info, image=None, results=None):
        time.sleep(0.005)
        with self.lock:
            self.renders += 1
            self.last = info

    @property
    def _render_stats(self):
        with self.lock:
            age = self.last - self.current  # coverage falls as the camera moves away from the cache's pose
        return types.SimpleNamespace(n_cache_hits=100 if age <= 1 else 10, n_resamples=10)


def test_builds_overlap_frames_and_the_last_build_is_waited_for():
    sys.path.insert(0, ROOT)
    import bench
    fake_torch = types.SimpleNamespace(cuda=types.SimpleNamespace(synchronize=lambda dev: None))
    r = FakeRenderer(build_s=0.05)
    infos = list(range(40))

    def rebuild(info, record):
        r.initCacheBlockwise(info)
        r.swapCache()

    out = bench.run_double_buffered(fake_torch, None, r, infos, None, None, rebuild)
    assert out["error"] is None
    assert r.renders == len(infos)
    assert out["builds"] == len(r.builds) - 1 >= 2          # the initial build is not counted
    assert out["builds"] < len(infos)                      # frames rendered while builds ran
    assert r.swaps == len(r.builds)
    assert 0.0 < out["mean_coverage"] < 1.0
    assert out["value"] > 0 and out["ms_per_frame"] * len(infos) >= 1e3 * 0.05 * out["builds"] * 0.9
