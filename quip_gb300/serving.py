"""Continuous-batching GAP service on one GPU.

Energy+force requests (independent structures) and resident MD replicas share the
device:
  * request workers (one libgapgpu context and CUDA stream each) take whatever has
    arrived from a shared queue, admit requests in arrival order while their estimated
    device memory (gapgpu_model_footprint) fits the worker's share of the budget,
    evaluate them as one batch (gapgpu_calc_batch) and complete them together; a request
    that arrives while batches are on the GPU joins the next batch a worker forms, so
    batches on different workers' streams overlap on the device;
  * the MD replicas advance in their own thread and stream (gapgpu_md_step), their
    positions, velocities and neighbour lists resident in HBM between steps.
Each request's latency is completion time minus arrival time.  A structure's results
do not depend on the batch it lands in (per-structure arithmetic is independent of its
position in a batch), so a request gives the same answer alone and in the mix.

ctypes releases the GIL around each library call, so the worker threads drive the GPU
concurrently.
"""
import collections
import threading
import time

import numpy as np

from ._lib import GapGpuError
from .potential import Potential


class Request:
    __slots__ = ("rid", "arrival", "atoms", "admitted", "done", "result")

    def __init__(self, rid, arrival, atoms):
        self.rid, self.arrival, self.atoms = rid, arrival, atoms
        self.admitted = self.done = None
        self.result = None


def admit_prefix(queue, footprint, share):
    """Pop from `queue` the longest arrival-order prefix whose summed footprint fits
    `share` bytes -- always at least one request, so that no request starves."""
    batch, used = [], 0
    while queue:
        f = footprint(queue[0])
        if batch and used + f > share:
            break
        batch.append(queue.popleft())
        used += f
    return batch


def poisson_arrivals(rate, count, seed=0):
    """Arrival times (s) of `count` requests of a Poisson process of `rate` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, count))


class Server:
    """Server(param_filename, precision="tf32", workers=2, budget_bytes=None, md=None,
    pair_tiles=False)

    ``md`` is an MDReplicas object whose replicas step alongside the requests (built on
    its own Potential, so on its own context and stream).

    ``pair_tiles=False`` (the default) runs every context the server drives, the
    workers' and the MD replicas', on single-CTA GEMM tiles (context option pairs=0; the
    fp16 form then computes its GEMMs in TF32).  With CTA-pair (cluster) GEMM tiles
    issued from several streams at once -- two workers and the MD stream -- the device
    stalled under load: a GEMM kernel stayed resident and never finished, at 1500-4000
    requests/s.  Single-CTA tiles ran the same loads without a stall."""

    def __init__(self, param_filename, precision="tf32", workers=2, budget_bytes=None, md=None, mean_neighbours=60.0,
                 pair_tiles=False):
        self.pots = [Potential(param_filename=param_filename, precision=precision) for _ in range(max(1, workers))]
        for p in self.pots:
            p.set_option("timing", 0)
            p.set_option("priority", 1)   # requests ahead of the background MD stream
            if not pair_tiles:
                p.set_option("pairs", 0)
        if md is not None and not pair_tiles:
            md.set_option("pairs", 0)
        self.md = md
        self.mean_neighbours = mean_neighbours
        if budget_bytes is None:
            budget_bytes = 16 << 30
        self.budget = int(budget_bytes)
        self.share = self.budget // len(self.pots)
        self._lock = threading.Lock()
        self._cv = threading.Condition(self._lock)

    def footprint(self, atoms):
        return self.pots[0].footprint(len(atoms), self.mean_neighbours)

    def admit(self, queue):
        return admit_prefix(queue, lambda r: self.footprint(r.atoms), self.share)

    def warmup(self, structures, max_atoms=None):
        """Run batches of doubling size (up to one worker's memory share) through every
        worker before serving: device buffers reach their final size and the GEMM
        autotuner has seen every row count, so no request later waits on an allocation
        (cudaMalloc/cudaFree synchronise the whole device) or a tuning run."""
        if not structures:
            return
        per_atom = max(1, self.pots[0].footprint(1 << 16, self.mean_neighbours) >> 16)
        cap = self.share // per_atom if max_atoms is None else max_atoms
        order = sorted(structures, key=len)
        target = 8
        while True:
            batch, n = [], 0
            for a in order:
                if n + len(a) > target:
                    break
                batch.append(a)
                n += len(a)
            if not batch:
                batch = order[:1]
            for p in self.pots:
                p.calc_batch(batch)
            if target >= cap or n >= sum(len(a) for a in order):
                break
            target = min(2 * target, cap)
            order = order[len(batch):] + order[:len(batch)]

    def run(self, structures, arrivals, md_steps_per_tick=1, timeout=600.0):
        """Serve requests for `structures` arriving at times `arrivals` (s, from start).
        Returns the completed requests and statistics."""
        reqs = [Request(i, float(t), a) for i, (t, a) in enumerate(zip(arrivals, structures))]
        pending = collections.deque(sorted(reqs, key=lambda r: r.arrival))
        queue = collections.deque()
        state = {"left": len(reqs), "error": None, "batches": 0, "batch_atoms": []}
        stop = threading.Event()
        t0 = time.perf_counter()

        def clock():
            return time.perf_counter() - t0

        def feeder():
            while pending and not stop.is_set():
                dt = pending[0].arrival - clock()
                if dt > 0:
                    time.sleep(min(dt, 0.002))
                    continue
                with self._cv:
                    while pending and pending[0].arrival <= clock():
                        queue.append(pending.popleft())
                    self._cv.notify_all()

        def evaluate(pot, batch):
            """The batch in one pass; if that fails (a structure the library rejects:
            overlapping atoms, NaN positions, ...), each request alone, so that only
            the bad ones fail -- their result is {"error": message}.  Once the run's
            deadline has passed, the requests not yet retried fail with
            {"error": "deadline"} instead of being evaluated."""
            try:
                return pot.calc_batch([r.atoms for r in batch])
            except GapGpuError:
                out = []
                for r in batch:
                    if stop.is_set():
                        out.append({"error": "deadline"})
                        continue
                    try:
                        out.append(pot.calc_batch([r.atoms])[0])
                    except GapGpuError as e:
                        out.append({"error": str(e)})
                return out

        def worker(pot):
            try:
                while not stop.is_set():
                    with self._cv:
                        while not queue and state["left"] > 0 and not stop.is_set():
                            self._cv.wait(0.01)
                        if state["left"] <= 0 or stop.is_set():
                            return
                        batch = self.admit(queue)
                    if not batch:
                        continue
                    ta = clock()
                    res = evaluate(pot, batch)
                    td = clock()
                    with self._cv:
                        for r, x in zip(batch, res):
                            r.admitted, r.done, r.result = ta, td, x
                        state["left"] -= len(batch)
                        state["batches"] += 1
                        state["batch_atoms"].append(sum(len(r.atoms) for r in batch))
                        self._cv.notify_all()
            except Exception as e:  # surfaced to the caller after the threads stop
                state["error"] = e
                stop.set()

        md_info = {"steps": 0}

        def md_loop():
            try:
                while not stop.is_set() and state["left"] > 0:
                    self.md.step(md_steps_per_tick)
                    md_info["steps"] += md_steps_per_tick
            except Exception as e:
                state["error"] = e
                stop.set()

        threads = [threading.Thread(target=feeder, daemon=True)]
        threads += [threading.Thread(target=worker, args=(p,), daemon=True) for p in self.pots]
        if self.md is not None:
            threads.append(threading.Thread(target=md_loop, daemon=True))
        for t in threads:
            t.start()
        deadline = time.perf_counter() + timeout
        while any(t.is_alive() for t in threads) and time.perf_counter() < deadline:
            time.sleep(0.01)
        stop.set()
        # after the deadline a thread only finishes the library call it is in
        for t in threads:
            t.join(timeout=max(1.0, 0.1 * timeout))
        stuck = sum(1 for t in threads if t.is_alive())
        wall = clock()
        if state["error"] is not None:
            raise state["error"]
        done = [r for r in reqs if r.done is not None and "error" not in r.result]
        lat = np.array([r.done - r.arrival for r in done]) if done else np.zeros(1)
        atoms = sum(len(r.atoms) for r in done)
        stats = {"requests": len(done), "failed": sum(1 for r in reqs if r.result is not None and "error" in r.result),
                 "wall_s": wall, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                 "p99_ms": 1e3 * float(np.percentile(lat, 99)), "mean_ms": 1e3 * float(lat.mean()),
                 "atom_evals_per_s": atoms / wall if wall > 0 else 0.0, "batches": state["batches"],
                 "mean_batch_atoms": float(np.mean(state["batch_atoms"])) if state["batch_atoms"] else 0.0,
                 "md_steps": md_info["steps"], "unfinished": sum(1 for r in reqs if r.done is None),
                 "deadline_hit": bool(state["left"] > 0), "threads_still_running": stuck}
        if self.md is not None:
            n_md = int(self.md.n_atoms.sum())
            stats["md_atom_steps_per_s"] = md_info["steps"] * n_md / wall if wall > 0 else 0.0
        return reqs, stats
