"""Kinetic-step benchmark of the GB300 engine (Taylor-Green vortex, 1M points).

One "step" = one kinetic step of the hot path on one mesh: move every point by
its Taylor-Green displacement, untangle inverted faces, restore the Delaunay
property with parallel Lawson flips (a single persistent launch).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--n POINTS] [--impl ours|reference]

value: points x steps / device time of the K steps, displacements resident in
HBM, L2 flushed (256 MB write) before every step and excluded from the timing.
e2e:   the same steps through the C ABI with host displacement buffers
(mcl_step_host: pinned host -> device copy inside the timed region) and a
device -> host read of each step's counters.
--impl reference: the reference's CPU kinetic path (restated in oracle/, the
oracle the tests compare with) on all host cores, each worker stepping an independent bounded
sample of the same workload.

Multi-GPU: meshes are independent, so N GPUs run N replicas (weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "kinetic pts*steps/s (move + untangle + Delaunay restore), 1M pts Taylor-Green, plain single-mesh form"
UNIT = "pts*steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--e2e-steps", type=int, default=120, help="timed e2e steps (segments of 40)")
    ap.add_argument("--repair-steps", type=int, default=10, help="timed steps of the 1M random-walk repair run")
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--cpu-sample", type=int, default=0, help="points per CPU mesh (0: the workload's own size)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-queries", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-repair", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--workload", default="taylor-green",
                    choices=["taylor-green", "batched", "serving", "precision", "periodic", "repair"])
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--duration", type=float, default=10.0)
    ap.add_argument("--drain-limit", type=float, default=60.0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--meshes", type=int, default=4096)
    ap.add_argument("--plain-steps", type=int, default=3)
    return ap.parse_args()


# ---------------------------------------------------------------------------
def max_over_ranks(x, dist, device="cpu"):
    """The largest value of x over all ranks (x itself without a process group)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def clocks_start():
    """Sample SM clocks and throttle reasons every 200 ms while a timed region
    runs; the raw samples go to $MCL_CLOCKS_CSV when set."""
    try:
        f = open(os.environ.get("MCL_CLOCKS_CSV") or os.devnull, "w")
        p = subprocess.Popen(
            ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
             "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
            text=True)
        return p, f
    except Exception:
        return None, None


def clocks_stop(p, f, gpu_index=0):
    if p is None:
        return None
    time.sleep(0.25)
    p.terminate()
    try:
        out, _ = p.communicate(timeout=5)
    except Exception:
        p.kill()
        out = ""
    if f is not None:
        f.write(out)
        f.close()
    sm, mx, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in out.strip().splitlines():
        c = [x.strip() for x in line.split(",")]
        if len(c) < 9 or c[0] != str(gpu_index):
            continue
        try:
            sm.append(float(c[1]))
            mx = max(mx, float(c[2]))
        except ValueError:
            continue
        for nm, val in zip(names, c[5:9]):
            if val.lower() == "active":
                reasons.add(nm)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def cpu_reference(n, seconds, seed, workers, max_steps=0):
    """The reference CPU kinetic path (oracle port: movePoint, untangle until
    false, delonize restart-scan, FP64 predicates) on `workers` processes, each
    stepping an independent n-point Taylor-Green mesh (seeds seed, seed+1, ...)
    for about `seconds` (at least one step; at most `max_steps` when > 0).
    Returns the aggregate pts*steps/s over the slowest worker's wall time and
    the per-worker details."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        res = pool.starmap(_cpu_worker, [(n, seconds, seed + i, max_steps) for i in range(workers)])
    wall = max(r["wall_s"] for r in res)
    steps = sum(r["steps"] for r in res)
    return {"value": n * steps / wall, "wall_s": wall, "steps": steps,
            "flips": sum(r["flips"] for r in res), "capped": sum(r["capped"] for r in res),
            "s_per_step": float(np.median([s for r in res for s in r["step_s"]])),
            "build_s": float(np.median([r["build_s"] for r in res])),
            "final_mesh": {k: int(sum(r["final"][k] for r in res)) for k in res[0]["final"]}}


def _cpu_worker(n, seconds, seed, max_steps):
    sys.path.insert(0, ROOT)
    from mcleap_gb300 import workloads as W
    from oracle import oracle as O

    t0 = time.perf_counter()
    pts = O.morton_sort(W.uniform_points(n, seed))
    m = O.Mesh.build(pts, exact=False)  # the reference's own build (FP64)
    build_s = time.perf_counter() - t0
    pos = m.positions()
    t0 = time.perf_counter()
    steps = flips = capped = 0
    step_s = []
    while (time.perf_counter() - t0 < seconds or steps == 0) and (max_steps <= 0 or steps < max_steps):
        # the GPU workload's displacement: Taylor-Green, dt = 0.5 x mean spacing
        d = W.taylor_green_displacements(pos, n, 1, frac=0.5)[0]
        r = m.kinetic_step_ref(d)
        step_s.append(float(r["seconds"]))
        flips += r["untangle_flips"] + r["delonize_flips"]
        capped += r["capped"]
        pos = m.positions()
        steps += 1
    wall = time.perf_counter() - t0
    # what the reference's path left (exact predicates, untimed): its untangle
    # covers only two cases and its restart scan stops where no tangled quad tests
    # positive, so the mesh can stay inverted and non-Delaunay
    chk = m.check(exact=True)
    return {"steps": steps, "wall_s": wall, "flips": flips, "capped": capped,
            "step_s": step_s, "build_s": build_s, "final": chk}


def oracle_parity(dt, ht, n_points):
    """Checker, run outside every timed region: the GPU mesh after the timed
    steps against the oracle's exact Delaunay triangulation of the same
    positions (sorted edge sets, bit for bit), and the engine's predicate
    ladder on every live quad and face against the oracle's exact signs.
    Returns the parity record and the oracle rebuild time in seconds."""
    import torch

    from mcleap_gb300 import _lib as L
    from oracle import oracle as O

    dt.transferToHost()
    pos, he = ht.m_pos, ht.m_he
    t0 = time.perf_counter()
    exact = O.Mesh.build(pos[4:], exact=True)
    rebuild_s = time.perf_counter() - t0
    got, want = ht.edges(), exact.edges()
    edges_equal = bool(np.array_equal(got, want))
    diff = 0
    if not edges_equal:
        diff = len(set(map(tuple, got.tolist())) ^ set(map(tuple, want.tolist())))
    org, apex = he[:, 1], he[:, 3]
    inner = np.nonzero((apex[0::2] >= 0) & (apex[1::2] >= 0))[0]
    a, b, c, d = org[2 * inner], org[2 * inner + 1], apex[2 * inner], apex[2 * inner + 1]
    pts8 = np.stack([pos[a], pos[b], pos[c], pos[d]], 1).reshape(-1, 8).astype(np.float32)
    ids = np.stack([a, b, c, d], 1).astype(np.int32)
    h = np.nonzero(apex >= 0)[0]
    pts6 = np.stack([pos[org[h]], pos[org[h ^ 1]], pos[apex[h]]], 1).reshape(-1, 6).astype(np.float32)

    def dev(kind, pts, idx=None):
        dp = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
        di = torch.from_numpy(np.ascontiguousarray(idx)).cuda() if idx is not None else None
        sg = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
        stg = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
        L.check(L.lib().mcl_debug_predicates_device(kind, dp.data_ptr(), di.data_ptr() if di is not None else None,
                                                    len(pts), sg.data_ptr(), stg.data_ptr(), None))
        return sg.cpu().numpy()

    dis_in = int((dev(1, pts8) != O.incircle(pts8, mode=1)).sum())
    dis_sos = int((dev(2, pts8, ids) != O.incircle(pts8, mode=2, ids=ids)).sum())
    dis_or = int((dev(0, pts6) != O.orient2d(pts6, mode=1)).sum())
    return {"edges_equal": edges_equal, "edges": int(len(got)), "edge_differences": diff,
            "sign_disagreements": dis_in + dis_sos + dis_or,
            "quads_sampled": int(len(pts8)), "faces_sampled": int(len(pts6)),
            "what": f"final {n_points}-point mesh after the timed steps vs the oracle's exact Delaunay rebuild of "
                    "the same positions; incircle (exact and with symbolic perturbation) on every interior edge's "
                    "quad and orient2d on every face by the engine's predicate ladder vs the exact oracle"}, rebuild_s


def run_reference(args, rank, world):
    if rank != 0:
        return
    import oracle.oracle as O

    O.build()
    workers = max(1, os.cpu_count() or 1)
    sample = args.cpu_sample or args.n
    secs = max(3.0, args.cpu_seconds)
    t_all = time.perf_counter()
    r = cpu_reference(sample, secs, 2026, workers)
    value = r["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * r["s_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"taylor-green {args.n} pts, dt = 0.5 x mean spacing, periodic wrap",
                   "points": sample, "same_config": sample == args.n, "parallelism": "cpu processes"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                         "sample": f"{workers} independent Taylor-Green meshes of {sample} points (one per core), "
                                   f"about {secs:.0f} s of steps each ({r['steps']} steps in all, median "
                                   f"{r['s_per_step']:.2f} s per step, {r['capped']} stopped at the Lawson cap); "
                                   "reference kinetic step = movePoint + untangle until false + delonize "
                                   "(restart scan), FP64 predicates; mesh build untimed"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "flips_per_s": r["flips"] / r["wall_s"],
        "final_mesh_exact_check": r["final_mesh"],
        "wall_s": time.perf_counter() - t_all,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_ours(args, rank, world, dist):
    import ctypes as C

    import torch

    import mcleap_gb300 as M
    from mcleap_gb300 import _lib as L
    from mcleap_gb300 import build as B
    from mcleap_gb300 import workloads as W

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    B.build()
    n, K, Wm = args.n, args.steps, max(3, args.warmup)  # at least 3 untimed warm-up steps
    pts = W.uniform_points(n, 2026 + rank)
    t0 = time.perf_counter()
    ht = M.HostTriangulation()
    ht.addDelaunayPoints(pts)
    dt = M.DeviceTriangulation(ht)
    t_build = time.perf_counter() - t0
    V = dt.m_pos_size
    E = dt.m_he_size // 2
    # displacements for warm-up + timed + e2e steps (Taylor-Green, generated on
    # the device; the e2e ones are staged in pinned host memory)
    # e2e: segments of 40 steps, at least 3, whatever --steps is
    SEG = 40
    KE = 0 if args.no_e2e else SEG * max(3, -(-args.e2e_steps // SEG))
    KEW = min(20, KE)  # untimed warm-up steps of the host-displacement pipeline
    dev_disp = W.taylor_green_displacements_device(ht.m_pos, n, Wm + K + KEW + KE, device=f"cuda:{local}")
    host_e2e = [d.cpu().pin_memory() for d in dev_disp[Wm + K:]]
    dev_disp = dev_disp[:Wm + K]
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    lib = L.lib()
    # per-step queries on the moved mesh: one-ring of every vertex (column
    # layout, 32 slots) and FRNN with r = 3 x spacing on the torus (periodic
    # grid of 640 x 640 cells of 12.8 units = r / 1.92, the fastest of 256-1280
    # cells per side; minimum-image distances) over the N
    # moving points, answered in vertex-id order without permuting the mesh
    do_q = not args.no_queries
    RING_M, FRNN_MAX = 32, 64
    h = W.mean_spacing(n)
    r_q = 3.0 * h
    if do_q:
        ring = torch.empty(V * RING_M, dtype=torch.int32, device=f"cuda:{local}")
        qcounts = torch.empty(n, dtype=torch.int32, device=f"cuda:{local}")
        qids = torch.empty(n * FRNN_MAX, dtype=torch.int32, device=f"cuda:{local}")
        grid = M.GridCount2d(n, (0.0, 0.0), (8192.0 / 640, 8192.0 / 640), (640, 640), periodic=True)
    torch.cuda.synchronize()

    cp, cf = clocks_start()
    # warm-up (untimed), with stats to check the status
    for k in range(Wm):
        st = L.StepStats()
        L.check(lib.mcl_step(dt.handle, dev_disp[k].data_ptr(), sp, C.byref(st)))
    torch.cuda.synchronize()
    tot0 = dt.totals()

    def queries():
        L.check(lib.mcl_one_ring(dt.handle, L.LAYOUT_COLUMN, RING_M, ring.data_ptr(), sp, None))
        qa.record(stream)
        pos_pts = dt.m_pos + 8 * 4  # the N moving points (ids 4..)
        L.check(lib.mcl_grid_build(grid.handle, pos_pts, sp))
        L.check(lib.mcl_grid_frnn_ids(grid.handle, r_q, FRNN_MAX, qcounts.data_ptr(), qids.data_ptr(), sp, None))

    # timed region: K steps, device-resident inputs; each step is followed by
    # its queries (timed separately, not part of the kinetic value)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    q_ring = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    q_end = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(K):
            flush.fill_(k & 0xFF)  # L2 flush, outside the timed window
            starts[k].record(stream)
            L.check(lib.mcl_step(dt.handle, dev_disp[Wm + k].data_ptr(), sp, None))
            ends[k].record(stream)
            if do_q:
                qa = q_ring[k]
                queries()
                q_end[k].record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    step_ms = np.array([s.elapsed_time(e) for s, e in zip(starts, ends)])
    qinfo = None
    if do_q:
        ring_ms = np.array([e.elapsed_time(a) for e, a in zip(ends, q_ring)])
        frnn_ms = np.array([a.elapsed_time(b) for a, b in zip(q_ring, q_end)])
        trunc = C.c_int64()
        L.check(lib.mcl_one_ring(dt.handle, L.LAYOUT_COLUMN, RING_M, ring.data_ptr(), sp, C.byref(trunc)))
        ovf = grid.frnn_ids(r_q, FRNN_MAX, qcounts, qids, stream=stream)
        k_nb = int(qcounts.sum().item())
        q_s = float(ring_ms.sum() + frnn_ms.sum()) / 1e3
        ring_bytes, frnn_bytes = 52 * V, 28 * n + 4 * k_nb
        qinfo = {
            "one_ring": {"ms": float(ring_ms.mean()), "slots": RING_M, "truncated": trunc.value,
                         "alg_bytes": ring_bytes, "gbs": ring_bytes / (ring_ms.mean() / 1e3) / 1e9},
            "frnn": {"ms": float(frnn_ms.mean()), "r": r_q, "grid": "periodic 640x640 cells of 12.8",
                     "neighbours": k_nb, "overflow": ovf, "alg_bytes": frnn_bytes,
                     "gbs": frnn_bytes / (frnn_ms.mean() / 1e3) / 1e9},
            "ms_per_step": 1e3 * q_s / K,
            "pts_per_s": world * n * K / q_s,
            "total_pts_steps_per_s": world * n * K / (q_s + float(step_ms.sum()) / 1e3),
        }
    st = dt.status(stream)
    if st["status"] != 0:
        raise RuntimeError(f"engine status {st}")
    tot1 = dt.totals()
    if tot1["failed_launches"] != tot0["failed_launches"]:
        raise RuntimeError(f"{tot1['failed_launches'] - tot0['failed_launches']} timed steps failed")
    dev_s = max_over_ranks(float(step_ms.sum()) / 1e3, dist, f"cuda:{local}")
    value = world * n * K / dev_s
    flips = tot1["lawson_flips"] - tot0["lawson_flips"] + tot1["removal_flips"] - tot0["removal_flips"]
    wl_items = (tot1["incircle_tests"] - tot0["incircle_tests"]) - K * (E - 4)
    inverted = tot1["inverted_faces"] - tot0["inverted_faces"]
    removed = tot1["removed_vertices"] - tot0["removed_vertices"]

    # roofline of the step kernel: algorithmic bytes per step (move 24 B/vertex,
    # classification 16 B/edge + 8 B/vertex, 20 B per later work-list item,
    # 96 B per flip), per launch, over the measured launch duration
    alg_bytes = 24 * V + 16 * E + 8 * V + 20 * max(wl_items, 0) / K + 96 * flips / K
    achieved = alg_bytes / (dev_s / K) / 1e9
    peak, peak_kind = peaks()
    # DRAM traffic of one k_step launch measured by ncu on this workload
    # (dram__bytes_read.sum + dram__bytes_write.sum = 73.4 MB at 3,000,005
    # edges), scaled by the edge count for other sizes
    traffic = 73.42e6 * E / 3000005

    # e2e: pinned host displacements through the pipelined C-ABI call (the
    # host-to-device copy of step k+1 overlaps step k); every step's counters
    # are copied back and checked by the host two steps later
    e2e = None
    if not args.no_e2e:
        host_disp = host_e2e
        nstat = C.sizeof(L.StepStats)
        stats_pin = torch.empty(2 * nstat, dtype=torch.uint8, pin_memory=True)
        views = [L.StepStats.from_address(stats_pin.data_ptr() + j * nstat) for j in range(2)]
        done_ev = [torch.cuda.Event() for _ in range(2)]
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

        e2e_tot = {"lawson_flips": 0, "inverted_faces": 0, "removed_vertices": 0, "steps": 0}

        def check(j):
            done_ev[j].synchronize()
            if views[j].status != 0:
                raise RuntimeError(f"e2e step failed: {views[j].as_dict()}")
            for key in ("lawson_flips", "inverted_faces", "removed_vertices"):
                e2e_tot[key] += getattr(views[j], key)
            e2e_tot["steps"] += 1

        # timed in segments of SEG steps (the pipeline drained after each); the
        # median segment is reported, so that one host-side stall of a few
        # milliseconds does not stand for the whole run
        seg_s = []
        # the first KEW steps warm the pipeline up (host threads, clocks) untimed
        for s0 in [0] + list(range(KEW, KEW + KE - SEG + 1, SEG)):
            if s0 == 0 and KEW == 0:
                continue
            e0 = time.perf_counter()
            nseg = KEW if s0 == 0 else SEG
            for k in range(s0, s0 + nseg):
                j = k & 1
                if k >= s0 + 2:
                    check(j)  # step k-2 wrote this counter slot
                L.check(lib.mcl_step_host_async(dt.handle, host_disp[k].data_ptr(), sp,
                                                stats_pin.data_ptr() + j * nstat))
                done_ev[j].record(stream)
            for k in range(max(s0, s0 + nseg - 2), s0 + nseg):
                check(k & 1)
            t_seg = max_over_ranks(time.perf_counter() - e0, dist, f"cuda:{local}")
            if s0 > 0:
                seg_s.append(t_seg)
        e_s = float(np.median(seg_s))
        e2e = {"value": world * n * SEG / e_s, "unit": UNIT, "h2d_bytes_per_step": 8 * V,
               "d2h_bytes_per_step": nstat, "ms_per_step": 1e3 * e_s / SEG, "steps": SEG * len(seg_s),
               "segments_ms_per_step": [1e3 * x / SEG for x in seg_s],
               "per_step": {k: v / max(1, e2e_tot["steps"]) for k, v in e2e_tot.items() if k != "steps"},
               "path": "mcl_step_host_async (pinned host displacements, copy overlapped with the previous step); "
                       f"{KEW} untimed warm-up steps, then the median of {len(seg_s)} segments of {SEG} steps; "
                       "steps back to back as an application runs them (no L2 flush in between, unlike the "
                       "device-timed value)"}
    clocks = clocks_stop(cp, cf, local)

    # served vs plain on a short stream over 128 resident meshes (the serving
    # workload at a quarter of its 512 meshes and a fifth of its 10 s stream,
    # to keep the default run within a few minutes)
    served = None
    if not args.no_serving:
        sv, pl, info = serving_measure(128, 2000.0, 2.0, 10.0, 150.0, 5 + rank)
        served = {"workload": f"{info['meshes']} resident meshes ({info['points']} points), Poisson 2000 req/s "
                              "for 2 s, k-step aggregation updates and FRNN / one-ring batches",
                  "served": {k: sv[k] for k in ("p50_ms", "p99_ms", "p999_ms", "pts_steps_per_s", "completed",
                                                "submitted", "iterations")},
                  "plain": {k: pl[k] for k in ("p50_ms", "p99_ms", "p999_ms", "pts_steps_per_s", "completed",
                                               "submitted", "iterations")},
                  "capacity": info["capacity"]}

    cpu = parity = None
    if rank == 0 and not args.no_cpu_baseline:
        # the CPU leg: the oracle checks the timed mesh (edges and signs, outside
        # every timed region) and the reference's CPU kinetic path is timed on
        # one core on a mesh of the same workload
        from oracle import oracle as O

        O.build()
        parity, rebuild_s = oracle_parity(dt, ht, n)
        sample = args.cpu_sample or n
        r = cpu_reference(sample, args.cpu_seconds, 2026, 1)
        cpu = {"value": r["value"], "unit": UNIT, "cores": 1, "kind": "port", "points": sample,
               "same_config": sample == n, "s_per_step": r["s_per_step"],
               "oracle_rebuild_pts_per_s": n / rebuild_s, "final_mesh_exact_check": r["final_mesh"],
               "sample": f"1 core, Taylor-Green mesh of {sample} points (the workload's own size), {r['steps']} "
                         f"steps in {r['wall_s']:.1f} s ({r['capped']} stopped at the Lawson cap); reference kinetic "
                         "step = movePoint + untangle until false + delonize (restart scan), FP64 predicates; "
                         f"mesh build ({r['build_s']:.1f} s) untimed"}

    repair = None
    if not args.no_repair:
        repair = repair_measure(1_000_000, args.repair_steps, 3, 2026 + rank, local)

    # the batched form, scaled down to 512 meshes to keep the default run short
    batched = None
    if not args.no_batched:
        r = batched_measure(512, 10, 3, 2, 4 + rank, local)
        batched = {k: r[k] for k in ("meshes", "points", "steps", "kinetic_pts_steps_per_s", "ms_per_step",
                                     "flips_per_s", "pipeline_graph", "plain", "speedup_vs_plain",
                                     "speedup_vs_plain_launch_gaps_included", "same_as_plain", "autotune")}
        batched["workload"] = ("512 meshes, sizes log-uniform in [100, 1e5], Gaussian walk sigma = 0.1 x spacing, "
                               "FRNN r = 2 x spacing (the batched configuration at an eighth of its mesh count)")

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": Wm,
            "ms_per_step": 1e3 * dev_s / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"taylor-green {n} pts, dt = 0.5 x mean spacing, periodic wrap",
                       "points": n, "vertices": V, "edges": E, "parallelism": f"replicas x{world}",
                       "l2": "flushed (256 MB write) before every timed step"},
            "flips_per_s": world * flips / dev_s,
            "step_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                        "max": float(step_ms.max())},
            "per_step": {"flips": flips / K, "worklist_items": wl_items / K, "inverted_faces": inverted / K,
                         "removed_vertices": removed / K},
            "predicates": {k: tot1[k] - tot0[k] for k in ("incircle_tests", "incircle_fp64", "incircle_exact",
                                                          "orient_fp64", "orient_exact", "sos_decisions")},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "k_step", "alg_bytes_per_launch": alg_bytes},
            "queries": qinfo,
            "served_vs_plain": served,
            # sign disagreements of the engine's predicate ladder with the exact
            # oracle on every live quad and face of the final mesh (null
            # without the CPU leg); the edge set against the exact rebuild
            "predicate_errors": parity["sign_disagreements"] if parity else None,
            "parity": parity, "repair": repair, "batched": batched,
            "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks,
            # k_step per step, plus k_one_ring + 7 grid-build kernels + k_grid_frnn per step
            "gpu_launches": K * (10 if do_q else 1),
            "wall_s": wall, "build_s": t_build,
        }
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def repair_measure(n, K, Wm, seed, local):
    """The repair path at the headline size: an n-point mesh under a Gaussian
    random walk (sigma = 0.1 x mean spacing, clamped to the box, coincident
    moves settled), which inverts faces every step, so every step runs the
    untangle repair (send back, remove, Lawson, reinsert).  K timed steps of
    k_step (CUDA events on its stream, L2 flushed before each), with the
    phase split from the kernel's own %globaltimer marks."""
    import ctypes as C

    import torch

    from mcleap_gb300 import _lib as L
    from mcleap_gb300 import batch as MB
    from mcleap_gb300 import workloads as W

    dev = f"cuda:{local}"
    mesh = MB.MeshBatch(MB.build_mesh(W.uniform_points(n, seed)))
    V, E = mesh.V, mesh.E
    sigma = torch.tensor([0.1 * W.mean_spacing(n)], dtype=torch.float32, device=dev)
    counter = torch.zeros(1, dtype=torch.int64, device=dev)
    d = torch.zeros((V, 2), dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream()
    lib = L.lib()
    keys = ("inverted_faces", "reverted_vertices", "removed_vertices", "lawson_flips", "removal_flips",
            "insert_rounds", "lawson_rounds", "incircle_tests", "incircle_fp64", "incircle_exact", "orient_fp64",
            "orient_exact")
    tot = {k: 0 for k in keys}
    ms, phases, rounds = [], [], []
    tl = np.zeros(48, np.int64)
    cn = np.zeros(32, np.int64)
    trm = np.zeros(96, np.int64)
    tin = np.zeros(64, np.int64)
    last_rounds = None
    for k in range(Wm + K):
        mesh.walk(sigma, counter, d, seed=77, stream=stream)
        mesh.settle(d, stream=stream)
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        st = L.StepStats()
        a.record(stream)
        L.check(lib.mcl_step(mesh.handle, d.data_ptr(), stream.cuda_stream, None))
        b.record(stream)
        stream.synchronize()
        L.check(lib.mcl_mesh_last_status(mesh.handle, stream.cuda_stream, C.byref(st)))
        sd = st.as_dict()
        if sd["status"] != 0:
            raise RuntimeError(f"repair step {k} failed: {sd}")
        if k < Wm:
            continue
        ms.append(a.elapsed_time(b))
        for key in keys:
            tot[key] += sd[key]
        L.check(lib.mcl_debug_timeline(mesh.handle, L.ptr(tl)))
        t0 = tl[0]
        # start -> classified -> reverted -> removed -> reinserted -> Lawson -> end
        marks = [tl[1], tl[43], tl[44], tl[45], tl[46], tl[47]]
        phases.append(np.diff(np.array([t0] + marks, np.float64)) / 1e3)
        if lib.mcl_debug_counters(mesh.handle, L.ptr(cn), len(cn)) < 16:  # returns how many counters exist
            raise RuntimeError("mcl_debug_counters failed")
        rounds.append((cn[14], cn[15], sd["insert_rounds"], sd["lawson_rounds"]))
        # the last step's rounds: send-back passes, removal rounds (claim,
        # verify, remove), insertion rounds (locate, win, split), in us
        L.check(lib.mcl_debug_remove_timeline(mesh.handle, L.ptr(trm)))
        L.check(lib.mcl_debug_insert_timeline(mesh.handle, L.ptr(tin)))
        npass, nrem, nins = int(min(cn[14], 16)), int(min(cn[15], 16)), int(min(sd["insert_rounds"], 16))
        prev = tl[1]
        passes = []
        for p_ in range(npass):
            passes.append((trm[48 + p_] - prev) / 1e3)
            prev = trm[48 + p_]
        prev = tl[43]
        rem = []
        for r_ in range(nrem):
            m3 = [trm[4 * r_], trm[4 * r_ + 1], trm[4 * r_ + 2]]
            rem.append([round((m3[0] - prev) / 1e3, 1), round((m3[1] - m3[0]) / 1e3, 1), round((m3[2] - m3[1]) / 1e3, 1)])
            prev = m3[2]
        prev = tl[44]
        ins = []
        for r_ in range(nins):
            m3 = [tin[4 * r_], tin[4 * r_ + 1], tin[4 * r_ + 2]]
            ins.append([round((m3[0] - prev) / 1e3, 1), round((m3[1] - m3[0]) / 1e3, 1), round((m3[2] - m3[1]) / 1e3, 1)])
            prev = tin[4 * r_ + 3]
        last_rounds = {"send_back_pass_us": [round(x, 1) for x in passes], "removal_round_us": rem,
                       "insertion_round_us": ins,
                       "slowest_removal_cycles_spokes": [[int(trm[64 + r_]) >> 16, int(trm[64 + r_]) & 0xffff]
                                                         for r_ in range(nrem)],
                       "uncached_removals": [int(trm[80 + r_]) for r_ in range(nrem)]}
    ms = np.array(ms)
    ph = np.median(np.array(phases), 0)
    flips = tot["lawson_flips"] + tot["removal_flips"]
    wl_items = max(0, tot["incircle_tests"] - K * (E - 4))
    alg = 24 * V + 16 * E + 8 * V + 20 * wl_items / K + 96 * flips / K
    peak, peak_kind = peaks()
    mesh.close()
    return {"workload": f"{n} points uniform, Gaussian random walk sigma = 0.1 x mean spacing (clamped, coincident "
                        "moves settled); every step inverts faces and runs the repair",
            "steps": K, "ms_per_step": float(ms.mean()), "p50_ms": float(np.median(ms)),
            "p99_ms": float(np.percentile(ms, 99)), "pts_steps_per_s": n * K / (ms.sum() / 1e3),
            "flips_per_s": flips / (ms.sum() / 1e3),
            "per_step": {k: tot[k] / K for k in keys},
            "phase_us_median": {"classify": ph[0], "send_back": ph[1], "remove": ph[2], "reinsert": ph[3],
                                "lawson": ph[4], "tail": ph[5]},
            "rounds_median": dict(zip(("fixpoint_passes", "removal", "insertion", "flip"),
                                      np.median(np.array(rounds), 0).tolist())),
            "last_step_rounds": last_rounds,
            "roofline": {"bound": "hbm", "achieved": alg / (ms.mean() / 1e3) / 1e9, "peak": peak,
                         "frac": alg / (ms.mean() / 1e3) / 1e9 / peak, "peak_kind": peak_kind,
                         "alg_bytes_per_launch": alg, "kernel": "k_step (repair)"},
            "l2": "flushed (256 MB write) before every timed step"}


def run_repair(args, rank, world, dist):
    """The repair-path run alone (1M random walk), as its own JSON line."""
    import torch

    from mcleap_gb300 import build as B

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    B.build()
    cp, cf = clocks_start()
    rep = repair_measure(args.n, args.steps, max(3, args.warmup), 2026 + rank, local)
    clocks = clocks_stop(cp, cf, local)
    line = {"metric": "repair-path kinetic pts*steps/s (Gaussian random walk, every step untangles)",
            "value": world * rep["pts_steps_per_s"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": rep["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": rep["workload"], "points": args.n, "parallelism": f"replicas x{world}"},
            "repair": rep, "clocks": clocks, "gpu_launches": args.steps * 4}
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def batched_measure(nm, K, Wm, KP, seed, local, dist=None, tune=True):
    """Batched form: nm independent meshes (sizes log-uniform in [100, 1e5]),
    each with its own Gaussian walk (sigma = 0.1 x its spacing, clamped to its
    box) and FRNN at r = 2 x its spacing.  Kinetic steps of the whole batch in
    one launch each (CUDA events around the step launch), the whole per-step
    pipeline (walk, settle, step, FRNN) as the library's captured StepPipeline,
    and the plain form: the same meshes stepped one launch per mesh."""
    import torch

    from mcleap_gb300 import _lib as L
    from mcleap_gb300 import batch as MB
    from mcleap_gb300 import workloads as W

    dev = f"cuda:{local}"
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(100), np.log(1e5), nm)).astype(np.int64)
    t0 = time.perf_counter()
    handles = [MB.build_mesh(W.uniform_points(int(n), 40000 + i)) for i, n in enumerate(sizes)]
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch = MB.MeshBatch.from_handles(handles, destroy_inputs=False)
    verify = batch.clone()
    t_batch = time.perf_counter() - t0
    singles = [MB.MeshBatch(h) for h in handles]
    V, E, npts = batch.V, batch.E, int(sizes.sum())
    h = (8192.0 / np.sqrt(sizes)).astype(np.float32)
    sigma = torch.tensor(0.1 * h, dtype=torch.float32, device=dev)
    radius_host = (2.0 * h).astype(np.float32)
    radius = torch.tensor(radius_host, dtype=torch.float32, device=dev)
    F = 48
    d = torch.zeros((V, 2), dtype=torch.float32, device=dev)
    out = torch.empty(V * F, dtype=torch.int32, device=dev)
    counter = torch.zeros(nm, dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    lib = L.lib()
    SEED = 1234

    # the library's captured pipeline (autotuned on clones first); its own
    # walk counters, so the kinetic run below steps the same states
    t0 = time.perf_counter()
    pipe = MB.StepPipeline(batch.clone(), sigma, radius_host, radius, F, seed=SEED, steps_per_graph=2, stream=stream,
                           tune=tune)
    t_tune = time.perf_counter() - t0
    tuned = pipe.batch.tuning()
    batch.set_tuning(tuned["blocks_per_sm"], tuned["tail_items"], tuned["removal_tile"])

    def pipeline_step(m, ctr, dd, outp, s, with_events=None):
        m.walk(sigma, ctr, dd, seed=SEED, stream=s)
        m.settle(dd, stream=s, sync=False)
        if with_events:
            with_events[0].record(s)
        L.check(lib.mcl_step(m.handle, L.ptr(dd), s.cuda_stream, None))
        if with_events:
            with_events[1].record(s)
        m.frnn_grid(radius_host, radius, F, outp, stream=s, sync=False)
        if with_events:
            with_events[2].record(s)

    # warm-up, then K timed steps (inputs far larger than L2)
    for k in range(Wm):
        pipeline_step(batch, counter, d, out, stream)
    stream.synchronize()
    st = batch.status(stream)
    if st["status"] != 0:
        raise RuntimeError(f"batched warm-up failed: {st}")
    tot0 = batch.totals()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(K)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(K):
        pipeline_step(batch, counter, d, out, stream, evs[k])
    stream.synchronize()
    st = batch.status(stream)
    if st["status"] != 0:
        raise RuntimeError(f"batched step failed: {st}")
    tot1 = batch.totals()
    if tot1["failed_launches"] != tot0["failed_launches"]:
        raise RuntimeError(f"{tot1['failed_launches'] - tot0['failed_launches']} batched steps failed")
    step_ms = np.array([e[0].elapsed_time(e[1]) for e in evs])
    frnn_ms = np.array([e[1].elapsed_time(e[2]) for e in evs])
    kin_s = max_over_ranks(float(step_ms.sum()) / 1e3, dist, dev)
    flips = tot1["lawson_flips"] - tot0["lawson_flips"] + tot1["removal_flips"] - tot0["removal_flips"]
    wl_items = (tot1["incircle_tests"] - tot0["incircle_tests"]) - K * (E - 4 * nm)

    # the whole per-step pipeline, replayed from the captured graph (two steps per replay)
    for _ in range(max(1, Wm // 2)):
        pipe.replay()
    reps = max(1, K // 2)
    ge = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    with torch.cuda.stream(stream):
        for r in range(reps):
            ge[r][0].record(stream)
            pipe.replay()
            ge[r][1].record(stream)
    pipe.check()
    gms = np.array([a.elapsed_time(b) for a, b in ge]) / 2
    graph = {"ms_per_step": float(gms.mean()), "p50": float(np.median(gms)), "p99": float(np.percentile(gms, 99)),
             "pts_steps_per_s": npts / (gms.mean() / 1e3), "steps": 2 * reps,
             "contents": "mcleap_gb300.batch.StepPipeline: walk + settle + step + per-mesh grid FRNN, one CUDA "
                         "graph replay per two steps"}
    pipe.batch.close()

    # plain form: the same meshes, one launch per mesh (device time of the
    # steps only: host launch gaps are not counted against it)
    ctrs = torch.zeros(nm, dtype=torch.int64, device=dev)
    pe = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nm)]
          for _ in range(KP)]
    pw = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(KP)]
    v0 = batch.v0
    for i, m in enumerate(singles):  # first-call scratch allocation outside the timing
        m.settle(d[int(v0[i]):int(v0[i] + batch.nv[i])], stream=stream, sync=False)
    stream.synchronize()
    for k in range(KP):
        pw[k][0].record(stream)
        for i, m in enumerate(singles):
            di = d[int(v0[i]):int(v0[i] + batch.nv[i])]
            m.walk(sigma[i:i + 1], ctrs[i:i + 1], di, seed=SEED + i, stream=stream)
            m.settle(di, stream=stream, sync=False)
            pe[k][i][0].record(stream)
            L.check(lib.mcl_step(m.handle, L.ptr(di), sp, None))
            pe[k][i][1].record(stream)
            oi = out[int(v0[i]) * F:int(v0[i] + batch.nv[i]) * F]
            m.frnn(radius[i:i + 1], F, oi, stream=stream, sync=False)
        pw[k][1].record(stream)
    stream.synchronize()
    bad = [i for i, m in enumerate(singles) if m.totals()["failed_launches"] != 0]
    plain_step_s = sum(a.elapsed_time(b) for row in pe for a, b in row) / 1e3
    plain_wall_s = sum(a.elapsed_time(b) for a, b in pw) / 1e3

    # the same steps through the batch (verify clone, fresh counter) must
    # leave every mesh exactly as the plain form did
    vctr = torch.zeros(nm, dtype=torch.int64, device=dev)
    vd = torch.zeros_like(d)
    for k in range(KP):
        pipeline_step(verify, vctr, vd, out, stream)
    stream.synchronize()
    check = sorted(set([0, nm - 1, int(np.argmax(sizes)), int(np.argmin(sizes))] +
                       rng.choice(nm, size=min(nm, 12), replace=False).tolist()))
    same = all(np.array_equal(verify.edges(i), singles[i].edges(0)) for i in check)
    for m in singles:
        m.close()
    verify.close()
    batch.close()
    return {
        "meshes": nm, "points": npts, "vertices": V, "edges": E, "steps": K, "warmup": Wm,
        "kinetic_pts_steps_per_s": npts * K / kin_s, "ms_per_step": 1e3 * kin_s / K, "kin_s": kin_s,
        "flips_per_s": flips / kin_s,
        "step_ms": {"p50": float(np.median(step_ms)), "p99": float(np.percentile(step_ms, 99)),
                    "max": float(step_ms.max())},
        "per_step": {"flips": flips / K, "worklist_items": wl_items / K},
        "frnn": {"ms": float(frnn_ms.mean()), "max_nb": F, "pts_per_s": npts / (frnn_ms.mean() / 1e3),
                 "method": "per-mesh grids (mcl_batch_frnn_grid); the plain loop uses the mesh walk per mesh"},
        "pipeline_graph": graph,
        "plain": {"steps": KP, "kinetic_pts_steps_per_s": npts * KP / plain_step_s,
                  "launch_gaps_included_pts_steps_per_s": npts * KP / plain_wall_s,
                  "ms_per_step": 1e3 * plain_step_s / KP, "failed_meshes": bad},
        "speedup_vs_plain": (npts * K / kin_s) / (npts * KP / plain_step_s),
        "speedup_vs_plain_launch_gaps_included": (npts * K / kin_s) / (npts * KP / plain_wall_s),
        "same_as_plain": {"meshes_checked": len(check), "identical": same},
        "autotune": {"best": pipe.tuned, "seconds": t_tune},
        "predicates": {k: tot1[k] - tot0[k] for k in ("incircle_tests", "incircle_fp64", "incircle_exact",
                                                      "orient_fp64", "orient_exact", "sos_decisions")},
        "setup_s": {"build_meshes": t_build, "batch": t_batch},
    }


def run_batched(args, rank, world, dist):
    """The batched form at its full size (4096 meshes), one JSON line."""
    import torch

    from mcleap_gb300 import build as B

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    B.build()
    cp, cf = clocks_start()
    r = batched_measure(args.meshes, args.steps, max(3, args.warmup), args.plain_steps, 4 + rank, local, dist)
    clocks = clocks_stop(cp, cf, local)
    line = {
        "metric": "batched kinetic pts*steps/s (move + untangle + Delaunay restore), one launch per step",
        "value": world * r["kinetic_pts_steps_per_s"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": r["warmup"], "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched: {r['meshes']} meshes, sizes log-uniform in [100, 1e5] (seed 4), Gaussian "
                               "walk sigma = 0.1 x spacing clamped to each mesh's box, FRNN r = 2 x spacing",
                   "meshes": r["meshes"], "points": r["points"], "vertices": r["vertices"], "edges": r["edges"],
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
        "clocks": clocks,
        # per step: k_walk + k_advance, k_settle, k_step, and the grid FRNN
        # (k_bgrid_hash, 3 scan kernels, k_bgrid_scatter, k_grid_sort_cells,
        # k_gather, k_bgrid_frnn)
        "gpu_launches": args.steps * 12,
    }
    line.update({k: v for k, v in r.items() if k not in ("kin_s", "steps", "warmup", "meshes", "points", "vertices",
                                                        "edges", "ms_per_step")})
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def serving_measure(nm, rate, duration, drain, budget_gb, seed):
    """Serve an open-loop Poisson stream over nm resident meshes (sizes
    log-uniform in [1e3, 1e6]) with continuous batching, then the same stream
    in the plain one-request-at-a-time form."""
    from mcleap_gb300 import serving as S
    from mcleap_gb300 import workloads as W

    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(1e3), np.log(1e6), nm)).astype(np.int64)
    t0 = time.perf_counter()
    pts = [W.uniform_points(int(n), 60000 + i) for i, n in enumerate(sizes)]
    server = S.MeshServer(pts, budget_bytes=budget_gb * 1e9, seed=99)
    del pts
    t_setup = time.perf_counter() - t0
    sizes = server.sizes
    warm = S.poisson_requests(server.n, rate, 0.05, seed=1, mesh_sizes=sizes)
    server.serve(warm, batched=True, realtime=False)  # warm-up (not reported)
    server.point_steps = 0
    it0, l0 = server.iterations, server.launches
    reqs = S.poisson_requests(server.n, rate, duration, seed=seed + 72, mesh_sizes=sizes)
    done = server.serve(reqs, batched=True, realtime=True, time_limit=duration + drain)
    served = S.latency_summary(done, server.wall, server.point_steps, len(reqs))
    served["iterations"] = server.iterations - it0
    served["device_wait_s"] = server.wait_s
    launches = server.launches - l0
    server.point_steps = 0
    it1 = server.iterations
    reqs2 = S.poisson_requests(server.n, rate, duration, seed=seed + 72, mesh_sizes=sizes)
    done2 = server.serve(reqs2, batched=False, realtime=True, time_limit=duration + drain)
    plain = S.latency_summary(done2, server.wall, server.point_steps, len(reqs2))
    plain["iterations"] = server.iterations - it1
    # capacity: the same requests all submitted at once (closed loop), served
    # with continuous batching and in the plain form; work done / wall time
    cap = {}
    for mode, batched in (("served", True), ("plain", False)):
        server.point_steps = 0
        rq = S.poisson_requests(server.n, rate, duration, seed=seed + 72, mesh_sizes=sizes)
        for r in rq:
            r.t_arrival = 0.0
        it_c = server.iterations
        dn = server.serve(rq, batched=batched, realtime=False, time_limit=drain + duration)
        summ = S.latency_summary(dn, server.wall, server.point_steps, len(rq))
        summ["iterations"] = server.iterations - it_c
        summ["device_wait_s"] = server.wait_s
        cap[mode] = {k: summ[k] for k in ("completed", "submitted", "wall_s", "pts_steps_per_s",
                                          "query_vertices_per_s", "requests_per_s", "iterations", "device_wait_s")}
    cap["speedup_pts_steps"] = cap["served"]["pts_steps_per_s"] / max(cap["plain"]["pts_steps_per_s"], 1e-9)
    cap["speedup_requests"] = cap["served"]["requests_per_s"] / max(cap["plain"]["requests_per_s"], 1e-9)
    frozen = server.frozen_fraction()
    info = {"meshes": server.n, "points": int(sizes.sum()), "admitted": len(server.admitted),
            "rejected": len(server.rejected), "budget_used_gb": server.admission.used / 1e9,
            "rate": rate, "duration_s": duration, "setup_s": t_setup, "launches": launches,
            "capacity": cap, "frozen_fraction_at_end": frozen}
    server.close()
    return served, plain, info


def run_serving(args, rank, world, dist):
    """Serving: meshes resident against an HBM budget, an open-loop Poisson
    request stream (k-step aggregation updates and FRNN / one-ring query
    batches), continuous batching vs the plain one-request-at-a-time form."""
    import torch

    from mcleap_gb300 import build as B

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    B.build()
    nm = args.meshes if args.meshes != 4096 else 512
    cp, cf = clocks_start()
    served, plain, info = serving_measure(nm, args.rate, args.duration, args.drain_limit, args.budget_gb, 5 + rank)
    clocks = clocks_stop(cp, cf, local)
    capacity = info.pop("capacity")
    line = {
        "metric": "served kinetic pts*steps/s with p50/p99/p99.9 request latency (continuous batching)",
        "value": served["pts_steps_per_s"], "unit": UNIT, "n_gpus": world, "steps": served["iterations"],
        "warmup": 1, "ms_per_step": 1e3 * served["wall_s"] / max(1, served["iterations"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload=f"serving: {info['meshes']} resident meshes (sizes log-uniform in [1e3, 1e6]), "
                                f"Poisson arrivals at {args.rate:g} req/s for {args.duration:g} s, half k-step "
                                "aggregation updates (k in 1..16), half FRNN / one-ring batches of 1e3..1e5 "
                                f"vertices; HBM budget {args.budget_gb:g} GB",
                       parallelism=f"replicas x{world}", **info),
        "served": served, "plain": plain, "capacity": capacity,
        "speedup_vs_plain": served["pts_steps_per_s"] / max(plain["pts_steps_per_s"], 1e-9),
        "p50_latency_ratio_plain_over_served": plain["p50_ms"] / max(served["p50_ms"], 1e-9),
        "clocks": clocks, "gpu_launches": info["launches"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_precision(args, rank, world, dist):
    """Precision stress: 4M float32 points (half on a jittered lattice, 30% in
    tight clusters, 20% uniform), Gaussian walk sigma = 0.05 x spacing; the
    predicate ladder's stage rates per step."""
    import ctypes as C

    import torch

    from mcleap_gb300 import _lib as L
    from mcleap_gb300 import batch as MB
    from mcleap_gb300 import build as B
    from mcleap_gb300 import workloads as W

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    B.build()
    n = 4_000_000 if args.n == 1_000_000 else args.n
    K = min(args.steps, 200)
    t0 = time.perf_counter()
    pts = W.precision_points(n, 3 + rank)
    mesh = MB.MeshBatch(MB.build_mesh(pts))
    t_build = time.perf_counter() - t0
    V = mesh.V
    h = 8192.0 / np.sqrt(n)
    sigma = torch.tensor([0.05 * h], dtype=torch.float32, device="cuda")
    counter = torch.zeros(1, dtype=torch.int64, device="cuda")
    d = torch.zeros((V, 2), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    lib = L.lib()
    keys = ("incircle_tests", "incircle_fp64", "incircle_exact", "orient_fp64", "orient_exact", "sos_decisions",
            "lawson_flips", "inverted_faces", "removed_vertices")
    tot = {k: 0 for k in keys}

    cp, cf = clocks_start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    settled = 0
    for k in range(K):
        mesh.walk(sigma, counter, d, seed=21, stream=stream)
        settled += mesh.settle(d, stream=stream)
        ev[k][0].record(stream)
        st = L.StepStats()
        L.check(lib.mcl_step(mesh.handle, d.data_ptr(), stream.cuda_stream, C.byref(st)))
        ev[k][1].record(stream)
        sd = st.as_dict()
        if sd["status"] != 0:
            raise RuntimeError(f"precision step {k} failed: {sd}")
        for key in keys:
            tot[key] += sd[key]
    stream.synchronize()
    clocks = clocks_stop(cp, cf, local)
    ms = np.array([a.elapsed_time(b) for a, b in ev])
    inc = max(1, tot["incircle_tests"])
    line = {
        "metric": "precision stress: kinetic pts*steps/s and predicate stage rates",
        "value": n * K / (ms.sum() / 1e3), "unit": UNIT, "n_gpus": world, "steps": K, "warmup": 0,
        "ms_per_step": float(ms.mean()), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"precision: {n} points (50% jittered 2048x1024 lattice, 30% in 64 Gaussian "
                               "clusters sigma 1e-3, 20% uniform), Gaussian walk sigma = 0.05 x spacing",
                   "points": n, "parallelism": f"replicas x{world}"},
        "rates": {"incircle_fp32_undecided": tot["incircle_fp64"] / inc,
                  "incircle_fp64_undecided": tot["incircle_exact"] / inc,
                  "sos_per_incircle": tot["sos_decisions"] / inc,
                  "orient_fp32_undecided_per_step": tot["orient_fp64"] / K,
                  "orient_fp64_undecided_per_step": tot["orient_exact"] / K},
        "totals": tot, "settled_moves": settled,
        "sign_check": "tests/test_gpu_precision.py compares sampled live-mesh predicate signs with the exact oracle",
        "step_ms": {"p50": float(np.median(ms)), "p99": float(np.percentile(ms, 99))},
        "clocks": clocks, "gpu_launches": K * 5, "build_s": t_build,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def periodic_displacements_device(pos, steps, period, drift=(0.3, 0.2), frac=0.5):
    """Taylor-Green advection on the torus [2L, 3L)^2 plus a uniform drift (so
    points cross the sides), dt = frac x mean spacing; positions mirrored in
    float32 with the engine's move + wrap arithmetic.  Returns the (n, 2)
    float32 device displacements and the final mirrored positions."""
    import torch

    n = len(pos)
    lo, hi = np.float32(2 * period), np.float32(3 * period)
    dt = frac * period / np.sqrt(n)
    p = torch.as_tensor(pos, dtype=torch.float32, device="cuda").clone()
    two_pi = 2.0 * np.pi
    out = []
    for _ in range(steps):
        q = (p.double() - float(lo)) / period
        u = torch.sin(two_pi * q[:, 0]) * torch.cos(two_pi * q[:, 1]) + drift[0]
        v = -torch.cos(two_pi * q[:, 0]) * torch.sin(two_pi * q[:, 1]) + drift[1]
        d = (torch.stack([u, v], 1) * dt).float()
        new = p + d
        new = torch.where(new >= hi, new - np.float32(period), new)
        up = new + np.float32(period)
        up = torch.where(up >= hi, torch.full_like(up, float(lo)), up)
        new = torch.where(new < lo, up, new)
        out.append(d)
        p = new
    return out, p


def run_periodic(args, rank, world, dist):
    """Kinetic steps of a periodic (torus) mesh: 1M points on [2L, 3L)^2,
    Taylor-Green advection plus a uniform drift (points wrap every step),
    move + wrap + flip rounds on the GPU (mcl_periodic_step)."""
    import torch

    from mcleap_gb300 import build as B
    from mcleap_gb300 import periodic as MP

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    B.build()
    n, period = args.n, 8192.0
    K, Wm = args.steps, max(3, args.warmup)
    rng = np.random.default_rng(11 + rank)
    pts = (2 * period + rng.random((n, 2)) * period).astype(np.float32)
    pts[pts >= 3 * period] = np.nextafter(np.float32(3 * period), np.float32(0))
    pts = np.unique(pts, axis=0)
    pts = pts[rng.permutation(len(pts))]
    n = len(pts)
    t0 = time.perf_counter()
    pt = MP.PeriodicTriangulation(pts, period)
    t_build = time.perf_counter() - t0
    disp, mirror = periodic_displacements_device(pts, Wm + K, period)
    stream = torch.cuda.Stream()
    for k in range(Wm):
        pt.step(disp[k], stream=stream)
    stream.synchronize()
    cp, cf = clocks_start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    tot = {"lawson_flips": 0, "lawson_rounds": 0, "wrapped": 0, "inverted_faces": 0, "substep_vertices": 0,
           "removed_vertices": 0, "reverted_vertices": 0}
    for k in range(K):
        ev[k][0].record(stream)
        st = pt.step(disp[Wm + k], stream=stream)
        ev[k][1].record(stream)
        for key in tot:
            tot[key] += st[key]
    stream.synchronize()
    clocks = clocks_stop(cp, cf, local)
    ms = np.array([a.elapsed_time(b) for a, b in ev])
    pos = pt.download()[0]
    line = {
        "metric": "periodic kinetic pts*steps/s (torus, move + wrap + flips)",
        "value": n * K / (ms.sum() / 1e3), "unit": UNIT, "n_gpus": world, "steps": K, "warmup": Wm,
        "ms_per_step": float(ms.mean()), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"periodic: {n} points on the torus [2L, 3L)^2, L = 8192, Taylor-Green advection "
                               "plus drift (0.3, 0.2), dt = 0.5 x mean spacing; inputs > L2",
                   "points": n, "parallelism": f"replicas x{world}"},
        "totals": tot, "positions_match_mirror": bool(np.array_equal(pos, mirror.cpu().numpy())),
        "step_ms": {"p50": float(np.median(ms)), "p99": float(np.percentile(ms, 99))},
        # one cooperative launch per step (mcl_periodic_step)
        "clocks": clocks, "gpu_launches": K, "build_s": t_build,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist_mod

        if args.impl == "ours":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist_mod.init_process_group("nccl" if args.impl == "ours" else "gloo")
        dist = dist_mod
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        elif args.workload == "batched":
            run_batched(args, rank, world, dist)
        elif args.workload == "serving":
            run_serving(args, rank, world, dist)
        elif args.workload == "precision":
            run_precision(args, rank, world, dist)
        elif args.workload == "periodic":
            run_periodic(args, rank, world, dist)
        elif args.workload == "repair":
            run_repair(args, rank, world, dist)
        else:
            run_ours(args, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
