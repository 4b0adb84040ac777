"""Serving: a request loop over meshes resident on the device, with continuous
batching and admission against an HBM budget as memory frees up.

Requests are kinetic updates (k diffusion-limited-aggregation steps of one
mesh), query batches (fixed-radius neighbours or one-rings of a list of
vertices of one mesh), new meshes ("open", with their points) and the end of a
mesh ("close").  The reference has no serving layer; its experiments loop over
one mesh (experiments/diffusion_limited_aggregation.cu:170-300) or keep a fixed
set resident (experiments/dla_results_collection.cu:170-241).

* Residency and admission: every mesh gets an id when it is submitted (at
  construction or by an "open" request) and waits in a FIFO until its bytes
  (estimated from the engine's per-vertex and per-edge arrays) fit the HBM
  budget.  Meshes admitted together are built on the device and form one
  group (one device batch).  A closed mesh gives its bytes back when its group
  is freed (its last mesh closed) or compacted (its open meshes rebuilt into a
  new group without it, done when waiting meshes need the room); the waiting
  meshes are then admitted at the next iteration.  A mesh larger than the
  whole budget is rejected at submission.
* Ordering: the requests of one mesh are served in arrival order (one in
  service at a time); requests of a mesh not yet admitted wait with it.  A
  request's result depends only on its own mesh's request sequence: the walk
  draws of mesh g are keyed by (seed + g, its step counter, local vertex id)
  whatever group holds it, so results are the same alone and in the mix.
* Continuous batching: every iteration takes the request in service of every
  resident mesh that has one; per group, all step requests advance one step in
  ONE launch (the batch restricted to their meshes) and all query requests run
  in one launch per query kind; requests that arrive meanwhile join at the
  next iteration.
* Plain form (for comparison): one request at a time in arrival order, one
  launch per step or query, the same kernels.

Motion per step (A19 of the reference's DLA experiment): free walkers take a
Gaussian step (sigma = sigma_frac x the mesh's spacing, clamped to its box),
coincident moves are settled, the mesh is stepped, then walkers within
contact_frac x spacing of a frozen vertex freeze.  Initially the even local
vertex ids are frozen (experiments/diffusion_limited_aggregation.cu:125-132).
"""
import collections
import ctypes as C
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

    def fits(self, nbytes):
        return self.used + nbytes <= self.budget

    def try_admit(self, nbytes):
        if not self.fits(nbytes):
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
    kind: str            # "step", "frnn", "ring", "open" or "close"
    k: int = 0           # steps (kind == "step")
    verts: np.ndarray = None  # local vertex ids (queries)
    points: np.ndarray = None  # the new mesh's points (kind == "open")
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


class _Group:
    """Meshes admitted together, in one device batch, with their per-mesh
    motion state (sigma, contact and FRNN radii, walk keys and counters) and
    per-vertex frozen flags."""

    def __init__(self, torch, ids, handles, sizes, seed, fracs, counters=None, frozen=None):
        self.ids = list(ids)
        self.local = {g: i for i, g in enumerate(self.ids)}
        self.batch = MeshBatch.from_handles(handles)
        b = self.batch
        self.sizes = np.asarray(sizes, np.int64)
        self.nbytes = int(sum(mesh_bytes(int(n)) for n in self.sizes))
        self.closed = np.zeros(len(self.ids), bool)
        h = (8192.0 / np.sqrt(self.sizes)).astype(np.float32)
        dev = "cuda"
        sigma_frac, contact_frac, frnn_frac = fracs
        self.sigma = torch.tensor(sigma_frac * h, device=dev)
        self.contact = torch.tensor(contact_frac * h, device=dev)
        self.radius = torch.tensor(frnn_frac * h, device=dev)
        self.seeds = torch.tensor(np.asarray([seed + g for g in self.ids], np.uint64).view(np.int64), device=dev)
        cnt = np.zeros(len(self.ids), np.int64) if counters is None else np.asarray(counters, np.int64)
        self.counter = torch.tensor(cnt, device=dev)
        self.d = torch.zeros((b.V, 2), dtype=torch.float32, device=dev)
        if frozen is None:
            fz = np.zeros(b.V, np.uint8)
            for i in range(b.count):
                v0, nv = int(b.v0[i]), int(b.nv[i])
                fz[v0 + 4:v0 + nv:2] = 1  # even local ids of the points (4, 6, ...)
        else:
            fz = np.concatenate(frozen).astype(np.uint8)
        self.frozen = torch.from_numpy(fz).to(dev)

    def frozen_of(self, i):
        b = self.batch
        return self.frozen[int(b.v0[i]):int(b.v0[i] + b.nv[i])].cpu().numpy()

    def close(self):
        self.batch.close()


class MeshServer:
    """Meshes resident in device batches, served with continuous batching and
    admitted against an HBM budget as memory frees up."""

    def __init__(self, point_sets, budget_bytes, seed=1, sigma_frac=0.1, contact_frac=1.0, frnn_frac=2.0,
                 max_frnn=32, max_ring=32, max_query_rows=1 << 22, stream=None):
        import torch

        self.torch = torch
        self.admission = Admission(budget_bytes)
        self.seed = int(seed)
        self.fracs = (sigma_frac, contact_frac, frnn_frac)
        self.groups = []
        self.where = {}            # mesh id -> (group, local index)
        self.mesh_sizes = []       # points per submitted mesh
        self.status = []           # per mesh: "waiting", "resident", "closed" or "rejected"
        self.waiting = collections.deque()  # (id, points), admission order
        self.rejected = []
        self.max_frnn, self.max_ring = max_frnn, max_ring
        self.max_query_rows = max_query_rows
        self.qout = torch.empty(max_query_rows * max(max_frnn, max_ring), dtype=torch.int32, device="cuda")
        # query vertex lists of an iteration: written into pinned memory with
        # their batch offsets, copied in one transfer on the serving stream
        self.qstage = torch.empty(max_query_rows, dtype=torch.int32, pin_memory=True)
        self.qstage_np = self.qstage.numpy()
        self.qverts = torch.empty(max_query_rows, dtype=torch.int32, device="cuda")
        self.stream = stream or torch.cuda.Stream()
        self.point_steps = 0
        self.iterations = 0
        self.launches = 0
        self.admissions = 0        # admission events (groups built)
        self.profile = None        # set to {} for device seconds per launch kind (CUDA events)
        self._events = []
        self.compactions = 0
        for p in point_sets:
            self.submit_mesh(p)
        self.admit()
        if not self.where:
            raise RuntimeError("no mesh fits the HBM budget")

    # -- residency ----------------------------------------------------------------------
    def submit_mesh(self, points):
        """Queue a new mesh for admission; returns its id (rejected at once if
        it is larger than the whole budget)."""
        g = len(self.mesh_sizes)
        pts = np.ascontiguousarray(points, np.float32).copy()
        self.mesh_sizes.append(len(pts))
        if mesh_bytes(len(pts)) > self.admission.budget:
            self.status.append("rejected")
            self.rejected.append(g)
        else:
            self.status.append("waiting")
            self.waiting.append((g, pts))
        return g

    @property
    def admitted(self):
        return sorted(self.where)

    @property
    def n(self):
        return len(self.mesh_sizes)

    @property
    def sizes(self):
        return np.asarray(self.mesh_sizes, np.int64)

    def admit(self):
        """Admit the waiting meshes, in order, while they fit (compacting
        groups that hold closed meshes when that makes room); the meshes
        admitted together form one new group.  Returns their ids."""
        take = []
        need = 0
        while self.waiting:
            g, pts = self.waiting[0]
            nb = mesh_bytes(len(pts))
            if not self.admission.fits(need + nb) and not self._make_room(need + nb):
                break
            self.waiting.popleft()
            take.append((g, pts))
            need += nb
        if not take:
            return []
        self.admission.try_admit(need)
        handles = [build_mesh(p) for _, p in take]
        grp = _Group(self.torch, [g for g, _ in take], handles, [len(p) for _, p in take], self.seed, self.fracs)
        self._add_group(grp)
        self.admissions += 1
        return [g for g, _ in take]

    def _add_group(self, grp):
        self.groups.append(grp)
        for i, g in enumerate(grp.ids):
            self.where[g] = (grp, i)
            self.status[g] = "resident"

    def _make_room(self, nbytes):
        """Free or compact groups holding closed meshes until nbytes fit."""
        cands = sorted((grp for grp in self.groups if grp.closed.any()),
                       key=lambda grp: -sum(mesh_bytes(int(n)) for n in grp.sizes[grp.closed]))
        for grp in cands:
            if self.admission.fits(nbytes):
                break
            self._compact(grp)
        return self.admission.fits(nbytes)

    def _compact(self, grp):
        """Rebuild grp without its closed meshes (their positions, topology,
        frozen flags and walk counters carried over), then free it."""
        keep = [i for i in range(len(grp.ids)) if not grp.closed[i]]
        self.groups.remove(grp)
        if keep:
            b = grp.batch
            handles, frozen = [], []
            counters = grp.counter.cpu().numpy()
            for i in keep:
                pos, v, he, t = b.download(i)
                view = L.AosView(L.ptr(pos), L.ptr(v), L.ptr(he), L.ptr(t), len(pos), len(he), len(t))
                h = C.c_void_p()
                L.check(L.lib().mcl_mesh_create_from_aos(C.byref(view), C.byref(h)))
                handles.append(h)
                frozen.append(grp.frozen_of(i))
            new = _Group(self.torch, [grp.ids[i] for i in keep], handles, grp.sizes[keep], self.seed, self.fracs,
                         counters=counters[keep], frozen=frozen)
            self._add_group(new)
            self.admission.release(grp.nbytes - new.nbytes)
        else:
            self.admission.release(grp.nbytes)
        grp.close()
        self.compactions += 1

    def close_mesh(self, g):
        """End mesh g: its bytes return to the budget when its group is freed
        or compacted."""
        if self.status[g] == "waiting":
            self.waiting = collections.deque((i, p) for i, p in self.waiting if i != g)
            self.status[g] = "closed"
            return
        if self.status[g] != "resident":
            raise ValueError(f"mesh {g} is not resident")
        grp, i = self.where.pop(g)
        grp.closed[i] = True
        self.status[g] = "closed"
        if grp.closed.all():
            self.groups.remove(grp)
            self.admission.release(grp.nbytes)
            grp.close()

    def mesh_state(self, g):
        """(positions, sorted edges, frozen flags) of resident mesh g, local ids."""
        grp, i = self.where[g]
        return grp.batch.download(i)[0], grp.batch.edges(i), grp.frozen_of(i)

    def frozen_fraction(self):
        tot = sum(int(grp.frozen.sum().item()) for grp in self.groups)
        return tot / max(1, sum(int(grp.batch.V) for grp in self.groups))

    def close(self):
        for grp in self.groups:
            grp.close()
        self.groups = []
        self.where = {}

    # -- per-iteration work ---------------------------------------------------------
    def _mark(self, name):
        """With profiling on, a CUDA event after the work launched so far."""
        if self.profile is not None:
            ev = self.torch.cuda.Event(enable_timing=True)
            ev.record(self.stream)
            self._events.append((name, ev))

    def _step(self, grp, locals_):
        b, s = grp.batch, self.stream
        b.set_active(locals_, stream=s)
        self._mark(None)
        b.walk(grp.sigma, grp.counter, grp.d, frozen=grp.frozen, hi=BOX_HI, stream=s, seeds=grp.seeds)
        self._mark("walk")
        b.settle(grp.d, stream=s, sync=False)
        self._mark("settle")
        L.check(L.lib().mcl_step(b.handle, L.ptr(grp.d), s.cuda_stream, None))
        self._mark("step")
        b.dla_freeze(grp.contact, grp.frozen, stream=s, sync=False)
        self._mark("freeze")
        self.launches += 6  # walk + counter, settle, step, contact (2)
        for i in locals_:
            self.point_steps += int(grp.sizes[i])

    def _queries(self, grp, reqs, keep_results, at):
        """Launch this group's query requests; their vertex lists go to
        self.qstage from row `at` on.  Returns the next free row."""
        torch, b, s = self.torch, grp.batch, self.stream
        for kind in ("frnn", "ring"):
            group = [r for r in reqs if r.kind == kind]
            if not group:
                continue
            start = at
            for r in group:
                n = len(r.verts)
                np.add(r.verts, np.int32(b.v0[grp.local[r.mesh]]), out=self.qstage_np[at:at + n], casting="unsafe")
                at += n
            count = at - start
            width = self.max_frnn if kind == "frnn" else self.max_ring
            W = max(self.max_frnn, self.max_ring)  # row stride of qout's regions: kinds never overlap
            out = self.qout[start * W:start * W + count * width]
            vd = self.qverts[start:at]
            with torch.cuda.stream(s):
                vd.copy_(self.qstage[start:at], non_blocking=True)  # ordered on the serving stream
                if kind == "frnn":
                    b.frnn_list(grp.radius, vd, width, out, stream=s, sync=False)
                else:
                    b.one_ring_list(vd, width, out, stream=s, sync=False)
            self.launches += 1
            self._mark(kind)
            if keep_results:
                s.synchronize()
                rows = out.view(count, width).cpu().numpy()
                off = 0
                for r in group:
                    n = len(r.verts)
                    r.result = rows[off:off + n].copy()
                    off += n
        return at

    # -- serving loops ------------------------------------------------------------------
    def serve(self, requests, batched=True, realtime=True, time_limit=None, keep_results=False):
        """Serve `requests` (sorted by arrival).  Returns the completed requests.
        An "open" request submits its points as mesh `r.mesh` (the next id); a
        "close" request ends its mesh after the mesh's earlier requests."""
        t0 = time.perf_counter()
        self.wait_s = 0.0  # time spent waiting for the device at the end of iterations
        queues = collections.defaultdict(collections.deque)
        fifo = collections.deque()  # plain form: global arrival order
        nxt = 0
        pending = 0
        done = []
        failed0 = {id(grp): grp.batch.totals()["failed_launches"] for grp in self.groups}
        for r in requests:
            r.remaining = r.k if r.kind == "step" else 1
            r.t_done = None

        def finish(r, t_end):
            r.t_done = t_end
            done.append(r)

        while nxt < len(requests) or pending:
            now = time.perf_counter() - t0 if realtime else float("inf")
            if time_limit is not None and time.perf_counter() - t0 > time_limit:
                break
            while nxt < len(requests) and requests[nxt].t_arrival <= now:
                r = requests[nxt]
                nxt += 1
                if r.kind == "open":
                    g = self.submit_mesh(r.points)
                    if g != r.mesh:
                        raise ValueError(f"open request {r.rid} names mesh {r.mesh}, the next id is {g}")
                    finish(r, time.perf_counter() - t0)
                    continue
                queues[r.mesh].append(r)
                if not batched:
                    fifo.append(r)
                pending += 1
            admitted_now = []
            if self.waiting:
                admitted_now = self.admit_groups()
                for grp in admitted_now:
                    failed0[id(grp)] = 0
            if not pending:
                if nxt < len(requests):
                    time.sleep(max(0.0, min(0.002, requests[nxt].t_arrival - now)))
                continue
            if batched:
                heads = [q[0] for g, q in queues.items() if q and self.status[g] in ("resident", "closed")]
            else:
                heads = [fifo[0]] if self.status[fifo[0].mesh] in ("resident", "closed") else []
            # closing is host work: done at once, the budget frees for the next iteration
            closing = [r for r in heads if r.kind == "close" or self.status[r.mesh] == "closed"]
            heads = [r for r in heads if r not in closing]
            stepping = {}
            qs = {}
            rows = 0
            for r in heads:
                grp, i = self.where[r.mesh]
                if r.kind == "step":
                    stepping.setdefault(id(grp), (grp, []))[1].append(r)
                elif rows + len(r.verts) <= self.max_query_rows:
                    qs.setdefault(id(grp), (grp, []))[1].append(r)
                    rows += len(r.verts)
            for grp, rs in stepping.values():
                self._step(grp, [grp.local[r.mesh] for r in rs])
            at = 0
            if qs:
                self._mark(None)
            for grp, rs in qs.values():
                at = self._queries(grp, rs, keep_results, at)
            ran = [r for _, rs in stepping.values() for r in rs] + [r for _, rs in qs.values() for r in rs]
            if ran:
                tw = time.perf_counter()
                self.stream.synchronize()
                self.wait_s += time.perf_counter() - tw
                self.iterations += 1
                if self.profile is not None:
                    for (_, a), (name, b) in zip(self._events, self._events[1:]):
                        if name is not None:
                            self.profile[name] = self.profile.get(name, 0.0) + a.elapsed_time(b) / 1e3
                    self._events = []
            t_end = time.perf_counter() - t0
            for r in closing:
                if r.kind == "close" and self.status[r.mesh] == "resident":
                    self.close_mesh(r.mesh)
                r.remaining = 0
            for r in ran + closing:
                if r not in closing:
                    r.remaining -= 1
                if r.remaining == 0:
                    queues[r.mesh].popleft()
                    if not batched:
                        fifo.popleft()
                    pending -= 1
                    finish(r, t_end)
            if not ran and not closing and not admitted_now:
                # only requests of meshes that wait for room: nothing frees it
                # unless a later arrival closes a mesh
                if nxt >= len(requests):
                    break
                if realtime:
                    time.sleep(max(0.0, min(0.002, requests[nxt].t_arrival - (time.perf_counter() - t0))))
        for grp in self.groups:
            grp.batch.set_active(None, stream=self.stream)
            st = grp.batch.status(self.stream)
            if st["status"] != 0:
                raise RuntimeError(f"engine status {st}")
            if grp.batch.totals()["failed_launches"] != failed0.get(id(grp), 0):
                raise RuntimeError("a served step failed")
        self.wall = time.perf_counter() - t0
        return done

    def admit_groups(self):
        """admit(), returning the groups it built."""
        before = list(self.groups)
        self.admit()
        return [grp for grp in self.groups if grp not in before]


def latency_summary(done, wall, point_steps, n_requests):
    done = [r for r in done if r.kind in ("step", "frnn", "ring")]
    lat = np.array([r.t_done - r.t_arrival for r in done]) if done else np.zeros(1)
    q = sum(len(r.verts) for r in done if r.kind != "step")
    return {
        "completed": len(done), "submitted": n_requests,
        "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "p999_ms": float(np.percentile(lat, 99.9) * 1e3), "max_ms": float(lat.max() * 1e3),
        "wall_s": wall, "pts_steps_per_s": point_steps / wall, "query_vertices_per_s": q / wall,
        "requests_per_s": len(done) / wall,
    }
