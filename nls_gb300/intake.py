"""Job intake in front of the serving pool, on schedulr's job contract.

The reference farms solves out through schedulr (schedulr/schedulr.py:48-154): clients POST a list
of JSON job descriptions to ``/api/jobs``; CPU workers (schedulr/workr.py:39-107) each GET one job
from ``/api/job``, build the model its description names (``solve_problem``: a 2-D model with a
Gaussian pump of the description's ``power``), solve it, store the ``.mat`` and POST the job back
as done.  Here the workers are replaced by the GPU serving pool: ``JobQueue`` keeps schedulr's job
table (pending, active, done) in process, ``run_jobs`` turns pending jobs into pool requests,
admits as many as the pool's HBM budget allows, keeps the pool fed and marks jobs done as their
solves finish, returning ``Solution`` objects (optionally stored as ``.mat`` like the worker).

A description is a JSON object.  ``power`` sets the pump power as in the reference worker; any
keyword of ``Problem().model`` given in it (``model``, ``dx``, ``dt``, ``order``, ``num_nodes``,
``num_iters``, ``u0``) replaces the worker's fixed choice (2-D, dx 0.2, dt 2e-3, u0 0.1, order 5,
200 x 200 nodes, 2000 steps, pump variation 5).

``serve_http(queue, port)`` optionally exposes the job table on 127.0.0.1 with the reference's
routes for submitting and listing jobs (``POST /api/jobs`` with ``{"jobs": [...]}``,
``GET /api/jobs``) and for an outside worker (``GET /api/job``, ``POST /api/job``); the GPU pool
consumes the same table in process.
"""

from __future__ import annotations

import json
import threading
from dataclasses import dataclass, field

import numpy as np

from .batch import Spec
from .model import Problem, Solution
from .pumping import GaussianPumping2D

# The reference worker's fixed problem (schedulr/workr.py:49-71), overridable per description.
WORKER_DEFAULTS = {"model": "2d", "dx": 2.0e-1, "dt": 2.0e-3, "t0": 0.0, "u0": 0.1, "order": 5,
                   "num_nodes": 200, "num_iters": 2000}
MODEL_KEYS = ("model", "dx", "dt", "t0", "u0", "order", "num_nodes", "num_iters")


def job_model(description: str):
    """The model a job description names (schedulr/workr.py:45-71 with per-job overrides)."""
    desc = json.loads(description)
    if not isinstance(desc, dict):
        raise ValueError("a job description must be a JSON object")
    kw = dict(WORKER_DEFAULTS)
    kw.update({k: desc[k] for k in MODEL_KEYS if k in desc})
    power = float(desc.get("power", 1.0))
    variation = float(desc.get("variation", 5.0))
    if kw["model"] == "2d":
        kw["pumping"] = GaussianPumping2D(power=power, variation=variation)
    else:
        from .pumping import GaussianPumping1D
        kw["pumping"] = GaussianPumping1D(power=power, variation=variation)
    return Problem().model(**kw)


def model_spec(model, dtype=np.complex128) -> Spec:
    """The pool request of a model: its pump on the model's grid, coefficients, initial state."""
    u0 = np.asarray(model.getInitialSolution())
    dim = u0.ndim
    return Spec(dim, model.getNumberOfNodes(), model.getApproximationOrder(), model.getTimeStep(),
                model.getSpatialStep(), np.asarray(model.getCoefficients(), dtype=np.float64),
                pumping=np.asarray(model.getPumping(), dtype=np.float64), u0=u0.astype(dtype))


@dataclass
class Job:
    job_id: int
    description: str
    state: str = "pending"          # pending -> active -> done
    worker_id: int | None = None
    solution: object = field(default=None, repr=False)


class JobQueue:
    """schedulr's job table, in process (thread-safe)."""

    def __init__(self):
        self._jobs = {}
        self._next = 1
        self._lock = threading.Lock()

    def post_jobs(self, descriptions):
        """Add jobs (schedulr.py post_jobs); returns their ids."""
        ids = []
        with self._lock:
            for d in descriptions:
                d = d if isinstance(d, str) else json.dumps(d)
                self._jobs[self._next] = Job(self._next, d)
                ids.append(self._next)
                self._next += 1
        return ids

    def get_job(self, worker_id: int):
        """Hand the first pending job to a worker (schedulr.py get_job); None when none is left."""
        with self._lock:
            for job in self._jobs.values():
                if job.state == "pending":
                    job.state, job.worker_id = "active", worker_id
                    return job
        return None

    def post_job(self, worker_id: int, job_id: int, solution=None) -> bool:
        """Mark a worker's job done (schedulr.py post_job)."""
        with self._lock:
            job = self._jobs.get(job_id)
            if job is None or job.worker_id != worker_id or job.state != "active":
                return False
            job.state, job.solution = "done", solution
            return True

    def active(self):
        """Jobs handed out and not done (schedulr.py get_jobs)."""
        with self._lock:
            return [j for j in self._jobs.values() if j.state == "active"]

    def pending(self) -> int:
        with self._lock:
            return sum(1 for j in self._jobs.values() if j.state == "pending")

    def job(self, job_id: int) -> Job:
        with self._lock:
            return self._jobs[job_id]


def run_jobs(queue: JobQueue, pool, dtype=np.complex128, store: bool = False, worker_id: int = 0):
    """Serve every pending job of ``queue`` on ``pool`` (a serve.Pool of the same dtype): admit
    jobs while the pool has room, keep chunks in flight, take finished states and mark their jobs
    done with a ``Solution``.  Returns {job_id: Solution}."""
    import time
    out = {}
    waiting = []       # (job, model, spec) not yet admitted
    running = {}       # job_id -> (job, model)

    def admit():
        while True:
            if not waiting:
                job = queue.get_job(worker_id)
                if job is None:
                    return
                model = job_model(job.description)
                waiting.append((job, model, model_spec(model, dtype)))
            job, model, spec = waiting[0]
            if pool.admit(spec, model.getNumberOfIterations(), job.job_id) is None:
                return
            waiting.pop(0)
            running[job.job_id] = (job, model, time.perf_counter())

    admit()
    while running or waiting:
        while pool.launch():
            pass
        if pool.info()[0]:
            pool.wait()
        while True:
            got = pool.take_with_state()
            if got is None:
                break
            tag, state = got
            job, model, t0 = running.pop(tag)
            sol = Solution(model, state)
            sol.setElapsedTime(time.perf_counter() - t0)
            if store:
                sol.store()
            queue.post_job(worker_id, job.job_id, sol)
            out[job.job_id] = sol
        admit()
        if waiting and not running and pool.info()[0] == 0:
            raise RuntimeError(f"job {waiting[0][0].job_id} does not fit the pool even when it is empty")
    return out


def serve_http(queue: JobQueue, port: int = 5000, host: str = "127.0.0.1"):
    """Start a background HTTP server on the job table (the reference's job routes); returns it
    (call ``shutdown()`` to stop)."""
    from http.server import BaseHTTPRequestHandler, ThreadingHTTPServer

    class Handler(BaseHTTPRequestHandler):
        def _body(self):
            n = int(self.headers.get("Content-Length") or 0)
            if not n:
                return None
            try:
                return json.loads(self.rfile.read(n))
            except ValueError:
                return None

        def _reply(self, code, payload=None):
            data = b"" if payload is None else json.dumps(payload).encode()
            self.send_response(code)
            self.send_header("Content-Type", "application/json")
            self.send_header("Content-Length", str(len(data)))
            self.end_headers()
            self.wfile.write(data)

        def log_message(self, *args):
            pass

        def do_GET(self):
            if self.path == "/api/jobs":
                rows = [{"id": j.job_id, "worker_id": j.worker_id, "description": j.description}
                        for j in queue.active()]
                return self._reply(200, {"columns": ["id", "worker_id", "description"], "jobs": rows})
            if self.path == "/api/job":
                body = self._body()
                if not body or "worker_id" not in body:
                    return self._reply(400)
                job = queue.get_job(int(body["worker_id"]))
                if job is None:
                    return self._reply(204)
                return self._reply(200, {"job_id": job.job_id, "description": job.description})
            return self._reply(404)

        def do_POST(self):
            body = self._body()
            if self.path == "/api/jobs":
                if not body or not isinstance(body.get("jobs"), list):
                    return self._reply(400)
                queue.post_jobs(body["jobs"])
                return self._reply(201)
            if self.path == "/api/job":
                if not body or "worker_id" not in body or "job_id" not in body:
                    return self._reply(400)
                ok = queue.post_job(int(body["worker_id"]), int(body["job_id"]))
                return self._reply(204 if ok else 404)
            return self._reply(404)

    server = ThreadingHTTPServer((host, port), Handler)
    threading.Thread(target=server.serve_forever, daemon=True).start()
    return server


__all__ = ["WORKER_DEFAULTS", "job_model", "model_spec", "Job", "JobQueue", "run_jobs", "serve_http"]
