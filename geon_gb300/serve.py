"""Serving engine (the geon_server_* entry points of include/geon_gpu.h).

Render, shadow-bisection and curvature requests from many callers run
together on one GPU: each is admitted while its buffers fit in the server's
device memory budget, its rays join the persistent kernels at the next launch,
and its result is the one the single-call API gives (render.render,
shadow.bisect with one bracket, curvature.grid), bit for bit.
"""
import ctypes

import numpy as np

from . import _ffi
from ._util import GeonError, check
from .geodesic import PRECISION
from .render import RenderConfig, RenderStats

JOB_RENDER, JOB_BISECT, JOB_CURVATURE = 0, 1, 2
QUEUED, RUNNING, DONE = 0, 1, 2


def _metric_fields(job, metric):
    job.metric_kind = int(metric.kind)
    job.nparams = len(metric.params)
    for i, v in enumerate(metric.params):
        job.metric_params[i] = float(v)


def _addr(a):
    return a.ctypes.data if a is not None else None


class Job:
    """A submitted request. `result()` waits and returns its outputs."""

    def __init__(self, server, jid, kind, struct, outputs):
        self.server = server
        self.id = jid
        self.kind = kind
        self._struct = struct      # keeps the request's output buffers alive
        self._out = outputs
        self.status = None

    def poll(self):
        return self.server._lib.geon_server_poll(self.server._h, self.id)

    def wait(self, timeout=None):
        rc = self.server._lib.geon_server_wait(self.server._h, self.id, -1.0 if timeout is None else float(timeout))
        if rc == _ffi.GEON_ERR_TIMEOUT and self.poll() != _ffi.GEON_ERR_TIMEOUT:
            raise TimeoutError(f"job {self.id} not finished within {timeout} s")
        self.status = rc
        return rc

    def cancel(self):
        check(self.server._lib.geon_server_cancel(self.server._h, self.id))

    def result(self, timeout=None):
        rc = self.wait(timeout)
        if rc != _ffi.GEON_OK:
            raise GeonError(rc, f"job {self.id} failed")
        o = self._out
        if self.kind == JOB_RENDER:
            st = o["stats"]
            stats = RenderStats(st.captured, st.escaped, st.diverged, st.max_null_residual, st.avg_steps,
                                st.total_steps)
            if "rgb8" in o:
                return o["rgb"], stats, o["cls"], o["steps"], o["rgb8"]
            return o["rgb"], stats, o["cls"], o["steps"]
        if self.kind == JOB_BISECT:
            return {"alpha_c": float(o["v"][0]), "lo": float(o["v"][1]), "hi": float(o["v"][2]),
                    "steps": int(o["steps"][0])}
        return o["einstein"], o["nec"]


class Server:
    """A serving engine with `budget_bytes` of device memory for requests."""

    def __init__(self, budget_bytes=64 << 30):
        self._lib = _ffi.load()
        h = ctypes.c_void_p()
        check(self._lib.geon_server_create(int(budget_bytes), ctypes.byref(h)))
        self._h = h

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.geon_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _submit(self, job, kind, outputs):
        jid = ctypes.c_uint64()
        check(self._lib.geon_server_submit(self._h, ctypes.byref(job), ctypes.byref(jid)))
        return Job(self, jid.value, kind, job, outputs)

    def submit_render(self, metric, camera, cfg=None, precision=None, deadline_s=0.0, with_u8=False):
        """render.render(metric, camera, cfg, with_classes=True) as a request
        (with_u8: also the tonemapped bytes of render_u8, returned fifth)."""
        cfg = cfg or RenderConfig()
        job = _ffi.GeonJob()
        job.type = JOB_RENDER
        _metric_fields(job, metric)
        job.precision = PRECISION[precision or cfg.precision]
        job.deadline_s = float(deadline_s)
        job.camera = camera.c_struct()
        job.render = cfg.c_struct()
        out = {"rgb": np.empty((camera.height, camera.width, 3), dtype=np.float32),
               "cls": np.empty((camera.height, camera.width), dtype=np.int32),
               "steps": np.empty((camera.height, camera.width), dtype=np.int64),
               "stats": _ffi.GeonRenderStats()}
        job.rgb = _addr(out["rgb"])
        job.pixel_class = _addr(out["cls"])
        job.pixel_steps = _addr(out["steps"])
        job.render_stats = ctypes.addressof(out["stats"])
        if with_u8:
            out["rgb8"] = np.empty((camera.height, camera.width, 3), dtype=np.uint8)
            job.rgb8 = _addr(out["rgb8"])
        return self._submit(job, JOB_RENDER, out)

    def submit_bisect(self, metric, r_obs, lo, hi, iters=60, step=0.01, max_steps=200000, precision="fp64",
                      rays_per_round=31, deadline_s=0.0):
        """One bracket of shadow.bisect (bin/validate_shadow.rs:70-77) as a request."""
        job = _ffi.GeonJob()
        job.type = JOB_BISECT
        _metric_fields(job, metric)
        job.precision = PRECISION[precision]
        job.deadline_s = float(deadline_s)
        job.r_obs, job.lo, job.hi, job.step = float(r_obs), float(lo), float(hi), float(step)
        job.max_steps = int(max_steps)
        job.iters = int(iters)
        job.rays_per_round = int(rays_per_round)
        out = {"v": np.zeros(3), "steps": np.zeros(1, dtype=np.int64)}
        base = out["v"].ctypes.data
        job.alpha_c, job.lo_out, job.hi_out = base, base + 8, base + 16
        job.steps_out = _addr(out["steps"])
        return self._submit(job, JOB_BISECT, out)

    def submit_curvature(self, metric, lo, hi, n, t=0.0, nk=16, seed=0x5EED, with_einstein=True, deadline_s=0.0):
        """curvature.grid(metric, lo, hi, n, t, nk, seed) as a request."""
        job = _ffi.GeonJob()
        job.type = JOB_CURVATURE
        _metric_fields(job, metric)
        job.deadline_s = float(deadline_s)
        for i in range(3):
            job.grid.lo[i] = float(lo[i])
            job.grid.hi[i] = float(hi[i])
            job.grid.n[i] = int(n[i])
        job.grid.t = float(t)
        job.nk = int(nk)
        job.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        npts = int(n[0]) * int(n[1]) * int(n[2])
        out = {"einstein": np.empty((npts, 4, 4)) if with_einstein else None,
               "nec": np.empty((npts, nk)) if nk else None}
        job.einstein = _addr(out["einstein"])
        job.nec = _addr(out["nec"])
        return self._submit(job, JOB_CURVATURE, out)

    def steps_per_launch(self, precision):
        return self._lib.geon_server_get_steps_per_launch(self._h, PRECISION[precision])

    def set_steps_per_launch(self, precision, steps):
        check(self._lib.geon_server_set_steps_per_launch(self._h, PRECISION[precision], int(steps)))

    def autotune(self):
        """Pick steps per launch per precision (geon_server_autotune) on an idle
        server; returns {precision: {"steps": s, "rates": {steps: ray-steps/s}}}."""
        rates = (ctypes.c_double * 10)()
        best = (ctypes.c_int * 2)()
        check(self._lib.geon_server_autotune(self._h, rates, best))
        cand = {"fp64": (32, 64, 128, 256, 512), "mixed": (1024, 2048, 4096, 8192, 16384)}
        out = {}
        for i, p in enumerate(("fp64", "mixed")):
            out[p] = {"steps": int(best[i]), "rates": {c: float(rates[5 * i + k]) for k, c in enumerate(cand[p])}}
        return out

    def wait_all(self, timeout=None):
        rc = self._lib.geon_server_wait_all(self._h, -1.0 if timeout is None else float(timeout))
        if rc == _ffi.GEON_ERR_TIMEOUT:
            raise TimeoutError("requests still running")
        check(rc)

    def stats(self):
        s = _ffi.GeonServerStats()
        check(self._lib.geon_server_stats_get(self._h, ctypes.byref(s)))
        names = ("render", "bisect", "curvature")
        return {
            "submitted": s.submitted, "completed": s.completed, "failed": s.failed,
            "queued": s.queued, "running": s.running,
            "p50_ms": s.p50_ms, "p99_ms": s.p99_ms, "mean_ms": s.mean_ms,
            "by_type": {names[t]: {"completed": s.completed_by_type[t], "p50_ms": s.p50_ms_by_type[t],
                                   "p99_ms": s.p99_ms_by_type[t]} for t in range(3)},
            "ray_steps": s.ray_steps, "grid_points": s.grid_points, "wall_s": s.wall_s,
            "launches": s.epochs, "ray_steps_unfinished": s.ray_steps_unfinished,
        }
