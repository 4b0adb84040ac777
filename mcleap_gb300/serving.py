"""Serving: a request loop over meshes resident on the device, with continuous
batching.

Requests are kinetic updates (k diffusion-limited-aggregation steps of one
mesh) and query batches (fixed-radius neighbours or one-rings of a list of
vertices of one mesh).  The reference has no serving layer; its experiments
loop over one mesh (experiments/diffusion_limited_aggregation.cu:170-300).

* Residency and admission: meshes are admitted against an HBM budget (bytes
  estimated from the engine's per-vertex and per-edge arrays) and live in one
  device batch for the whole run; nothing is copied per request.
* Ordering: the requests of one mesh are served in arrival order (one in
  service at a time); requests of different meshes are independent.  A
  request's result therefore depends only on its own mesh's request sequence,
  not on what else is in flight, and is the same alone and in the mix.
* Continuous batching: every iteration takes the request in service of every
  mesh that has one; all step requests advance one step in ONE launch (the
  batch restricted to their meshes), all query requests run in one launch per
  query kind; requests that arrive meanwhile join at the next iteration.
* Plain form (for comparison): one request at a time in arrival order, one
  launch per step or query, the same kernels.

Motion per step (A19 of the reference's DLA experiment): free walkers take a
Gaussian step (sigma = sigma_frac x the mesh's spacing, clamped to its box),
coincident moves are settled, the mesh is stepped, then walkers within
contact_frac x spacing of a frozen vertex freeze.  Initially the even local
vertex ids are frozen (experiments/diffusion_limited_aggregation.cu:125-132).
"""
import dataclasses
import time

import numpy as np

from . import _lib as L
from .batch import MeshBatch, build_mesh

BOX_HI = float(np.nextafter(np.float32(8192), np.float32(0)))

# Device bytes per vertex and per edge of a resident mesh: the engine's arrays
# (positions x2, work lists, marks, reinsertion scratch; edge records, claims,
# stamps), the batch tables, the settle table and the server's own state.
BYTES_PER_VERTEX = 16 + 4 + 1 + 8 + 4 + 12 + 4 + 4 + 4 + 4 + 8 + 8 + 4 + 4 + 16 + 4 + 1 + 1 + 8
BYTES_PER_EDGE = 16 + 16 + 4 + 4 + 4 + 8 + 4 + 8 + 16


def mesh_bytes(n_points):
    V = n_points + 4
    E = 3 * n_points + 5
    return BYTES_PER_VERTEX * V + BYTES_PER_EDGE * E


class Admission:
    """HBM budget bookkeeping: a mesh is admitted when its bytes fit."""

    def __init__(self, budget_bytes):
        self.budget = int(budget_bytes)
        self.used = 0

    def try_admit(self, nbytes):
        if self.used + nbytes > self.budget:
            return False
        self.used += nbytes
        return True

    def release(self, nbytes):
        self.used = max(0, self.used - int(nbytes))


@dataclasses.dataclass
class Request:
    rid: int
    t_arrival: float
    mesh: int
    kind: str            # "step", "frnn" or "ring"
    k: int = 0           # steps (kind == "step")
    verts: np.ndarray = None  # local vertex ids (queries)
    # filled by the server
    remaining: int = 0
    t_done: float = None
    result: object = None


def poisson_requests(n_meshes, rate, duration, seed, step_frac=0.5, k_max=16, q_lo=1_000, q_hi=100_000,
                     mesh_sizes=None):
    """Open-loop Poisson arrivals: half step requests (k uniform in 1..k_max),
    half query batches of log-uniform size in [q_lo, q_hi] vertices (FRNN or
    one-ring, evenly), each on a uniformly chosen mesh."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            return out
        m = int(rng.integers(n_meshes))
        if rng.random() < step_frac:
            out.append(Request(len(out), t, m, "step", k=int(rng.integers(1, k_max + 1))))
        else:
            nq = int(np.exp(rng.uniform(np.log(q_lo), np.log(q_hi))))
            if mesh_sizes is not None:
                nq = min(nq, int(mesh_sizes[m]))
                verts = 4 + rng.choice(int(mesh_sizes[m]), nq, replace=False).astype(np.int32)
            else:
                verts = None
            out.append(Request(len(out), t, m, "frnn" if rng.random() < 0.5 else "ring", verts=verts))


class MeshServer:
    """Meshes resident in one device batch, served with continuous batching."""

    def __init__(self, point_sets, budget_bytes, seed=1, sigma_frac=0.1, contact_frac=1.0, frnn_frac=2.0,
                 max_frnn=32, max_ring=32, max_query_rows=1 << 22, stream=None):
        import torch

        self.torch = torch
        self.admission = Admission(budget_bytes)
        self.admitted, self.rejected = [], []
        handles = []
        for i, p in enumerate(point_sets):
            if self.admission.try_admit(mesh_bytes(len(p))):
                self.admitted.append(i)
                handles.append(build_mesh(np.ascontiguousarray(p, np.float32).copy()))
            else:
                self.rejected.append(i)
        if not handles:
            raise RuntimeError("no mesh fits the HBM budget")
        self.batch = MeshBatch.from_handles(handles)
        b = self.batch
        self.n = b.count
        self.sizes = (b.nv - 4).astype(np.int64)
        h = (8192.0 / np.sqrt(self.sizes)).astype(np.float32)
        dev = "cuda"
        self.sigma = torch.tensor(sigma_frac * h, device=dev)
        self.contact = torch.tensor(contact_frac * h, device=dev)
        self.radius = torch.tensor(frnn_frac * h, device=dev)
        self.counter = torch.zeros(self.n, dtype=torch.int64, device=dev)
        self.seed = int(seed)
        self.d = torch.zeros((b.V, 2), dtype=torch.float32, device=dev)
        frozen = np.zeros(b.V, np.uint8)
        for i in range(self.n):
            v0, nv = int(b.v0[i]), int(b.nv[i])
            frozen[v0 + 4:v0 + nv:2] = 1  # even local ids of the points (4, 6, ...)
        self.frozen = torch.from_numpy(frozen).to(dev)
        self.max_frnn, self.max_ring = max_frnn, max_ring
        self.max_query_rows = max_query_rows
        self.qout = torch.empty(max_query_rows * max(max_frnn, max_ring), dtype=torch.int32, device=dev)
        self.stream = stream or torch.cuda.Stream()
        self.steps_done = np.zeros(self.n, np.int64)
        self.point_steps = 0
        self.iterations = 0
        self.launches = 0

    # -- per-iteration work ---------------------------------------------------------
    def _step(self, meshes):
        b, s = self.batch, self.stream
        b.set_active(meshes, stream=s)
        b.walk(self.sigma, self.counter, self.d, seed=self.seed, frozen=self.frozen, hi=BOX_HI, stream=s)
        b.settle(self.d, stream=s, sync=False)
        L.check(L.lib().mcl_step(b.handle, L.ptr(self.d), s.cuda_stream, None))
        b.dla_freeze(self.contact, self.frozen, stream=s, sync=False)
        self.launches += 6  # walk + counter, settle, step, contact (2)
        for m in meshes:
            self.steps_done[m] += 1
            self.point_steps += int(self.sizes[m])

    def _queries(self, reqs, keep_results):
        torch, b, s = self.torch, self.batch, self.stream
        for kind in ("frnn", "ring"):
            group = [r for r in reqs if r.kind == kind]
            if not group:
                continue
            verts = np.concatenate([r.verts.astype(np.int32) + np.int32(b.v0[r.mesh]) for r in group])
            width = self.max_frnn if kind == "frnn" else self.max_ring
            out = self.qout[:len(verts) * width]
            with torch.cuda.stream(s):
                vd = torch.from_numpy(verts).to("cuda")  # ordered on the serving stream
                if kind == "frnn":
                    b.frnn_list(self.radius, vd, width, out, stream=s, sync=False)
                else:
                    b.one_ring_list(vd, width, out, stream=s, sync=False)
            self.launches += 1
            if keep_results:
                s.synchronize()
                rows = out.view(len(verts), width).cpu().numpy()
                off = 0
                for r in group:
                    n = len(r.verts)
                    r.result = rows[off:off + n].copy()
                    off += n

    # -- serving loops ------------------------------------------------------------------
    def serve(self, requests, batched=True, realtime=True, time_limit=None, keep_results=False):
        """Serve `requests` (sorted by arrival).  Returns the completed requests."""
        import collections

        t0 = time.perf_counter()
        queues = [collections.deque() for _ in range(self.n)]
        fifo = collections.deque()  # plain form: global arrival order
        nxt = 0
        pending = 0
        done = []
        for r in requests:
            r.remaining = r.k if r.kind == "step" else 1
            r.t_done = None
        while nxt < len(requests) or pending:
            now = time.perf_counter() - t0 if realtime else float("inf")
            if time_limit is not None and time.perf_counter() - t0 > time_limit:
                break
            while nxt < len(requests) and requests[nxt].t_arrival <= now:
                r = requests[nxt]
                queues[r.mesh].append(r)
                if not batched:
                    fifo.append(r)
                nxt += 1
                pending += 1
            if not pending:
                time.sleep(max(0.0, min(0.002, requests[nxt].t_arrival - now)))
                continue
            if batched:
                heads = [q[0] for q in queues if q]
                rows, qs = 0, []
                for r in heads:
                    if r.kind != "step" and rows + len(r.verts) <= self.max_query_rows:
                        qs.append(r)
                        rows += len(r.verts)
                stepping = [r for r in heads if r.kind == "step"]
            else:
                r = fifo[0]
                stepping = [r] if r.kind == "step" else []
                qs = [] if r.kind == "step" else [r]
            if stepping:
                self._step([r.mesh for r in stepping])
            if qs:
                self._queries(qs, keep_results)
            self.stream.synchronize()
            if stepping:
                self.batch.status(self.stream)  # raises if this iteration's step failed
            self.iterations += 1
            t_end = time.perf_counter() - t0
            for r in stepping + qs:
                r.remaining -= 1
                if r.remaining == 0:
                    r.t_done = t_end
                    queues[r.mesh].popleft()
                    if not batched:
                        fifo.popleft()
                    pending -= 1
                    done.append(r)
        self.batch.set_active(None, stream=self.stream)
        st = self.batch.status(self.stream)
        if st["status"] != 0:
            raise RuntimeError(f"engine status {st}")
        self.wall = time.perf_counter() - t0
        return done


def latency_summary(done, wall, point_steps, n_requests):
    lat = np.array([r.t_done - r.t_arrival for r in done]) if done else np.zeros(1)
    q = sum(len(r.verts) for r in done if r.kind != "step")
    return {
        "completed": len(done), "submitted": n_requests,
        "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "p999_ms": float(np.percentile(lat, 99.9) * 1e3), "max_ms": float(lat.max() * 1e3),
        "wall_s": wall, "pts_steps_per_s": point_steps / wall, "query_vertices_per_s": q / wall,
        "requests_per_s": len(done) / wall,
    }
