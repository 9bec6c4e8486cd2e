"""Continuous-batching serving of kMC trajectories on one GPU.

A request asks for N kMC steps of one model on one lattice with given rate constants
and returns the trajectory's final TOFs (from procstat and from integ_rates),
coverages, kmc_time and step count.  The server keeps every admitted trajectory
resident in the pool's HBM arena and advances all of them together, one *quantum* (a
persistent launch per model, each trajectory taking min(remaining, quantum) steps) at a
time.  Between quanta it retires finished trajectories (one gathered read-back) and
admits waiting requests while the arena has room for them — admission by free HBM.
Requests that arrive while a quantum runs join the next one, so their work overlaps on
the device with the requests already running.

Each trajectory's random stream is Philox keyed by (seed, trajectory id), so a request's
result is the same alone and in any mix.

Sessions: requests naming the same ``session`` continue one trajectory.  After a
session's request finishes, its trajectory stays resident (lattice, tables, rates, clock
and random stream) for the next request of that session, which may bring new rate
constants (a new temperature or pressure: ``kmc_pool_set_rates``) and runs on from the
same state; a session's requests run one after the other.  Idle sessions are the first
moved to host memory when admission needs room.  A request with ``keep=False`` ends its
session.  Results report the request's own interval (TOFs from the procstat and
integ_rates differences over its kmc_time) beside the trajectory's totals.

Sampled results: a request with ``samples > 0`` also gets get_std_sampled_data's
averages (kmos/run/__init__.py:865-966) over its steps, split into ``samples`` batches:
the server ends a quantum at each batch boundary and takes the sample on the device
(``kmc_pool_sample``: occupation weighted by kmc_time_step), so no lattice is copied
back; the request's result carries ``sampled`` = TOFs from procstat and from
integ_rates over the sampled time, the mean occupation, total and simulated time and
steps.  A sampling request is not evicted while it runs.

Scheduling policy: "fifo" admits in arrival order.  "srpt" (shortest remaining
processing time) admits the waiting request with the fewest remaining steps first and,
when the arena or the slot table is full, evicts the resident trajectory with the most
remaining steps if it has more than ``evict_ratio`` times the head's: its state image
(kmc_pool_save_state, a compact copy of lattice, tables, counters, clock and random
stream) goes to host memory and the request back to the queue, to be restored
(kmc_pool_restore_state) and continued bit for bit later.  Short requests then no longer
wait behind long ones.

kmos has no counterpart (it runs one model per process; ``ModelRunner``,
kmos/run/__init__.py:1991-2368, forks one process per parameter set).
"""
from __future__ import annotations

import collections
import heapq
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import engine as E
from .program import Program


@dataclass
class Request:
    model: str                      # key of a registered model
    size: Sequence[int]             # system size per axis
    rates: Optional[Sequence[float]]  # rate constant per process (None: a session's current rates)
    steps: int                      # kMC steps to run
    seed: int = 1
    traj_id: int = 0                # Philox key word: a request's stream identity
    rid: int = 0
    arrival: float = 0.0            # seconds, on the server's clock
    # filled in by the server
    slot: int = -1
    remaining: int = 0
    admitted: float = -1.0
    done: float = -1.0
    result: Optional[dict] = None
    error: Optional[str] = None
    image: Optional[bytes] = None   # state while evicted to host memory
    evictions: int = 0
    session: Optional[str] = None   # requests of one session continue one trajectory
    keep: bool = True               # with a session: keep its trajectory after this request
    start: Optional[tuple] = None   # (procstat, integ_rates, kmc_time) when the request began
    samples: int = 0                # > 0: get_std_sampled_data averages over this many batches
    to_sample: int = 0              # steps left to the next sample boundary


@dataclass
class Session:
    model: str
    size: Tuple[int, ...]
    slot: int = -1                  # resident and idle when >= 0 and not busy
    image: Optional[bytes] = None   # state while evicted to host memory
    busy: bool = False              # a request of this session is queued or running
    queue: collections.deque = field(default_factory=collections.deque)
    last_used: float = 0.0


@dataclass
class ModelEntry:
    program: Program
    model_id: int
    nproc: int
    nspecies: int
    spuck: int
    tof_matrix: np.ndarray          # [n_tof, nproc]
    tof_names: List[str] = field(default_factory=list)


class Server:
    """Continuous-batching server over one pool."""

    def __init__(self, arena_bytes: int, max_slots: int = 8192, quantum: int = 20000, device: int = 0,
                 policy: str = "fifo", evict_ratio: float = 4.0, max_evict: int = 64):
        if policy not in ("fifo", "srpt"):
            raise ValueError("policy must be fifo or srpt")
        self.pool = E.Pool(arena_bytes=arena_bytes, max_slots=max_slots, device=device)
        self.max_slots = max_slots
        self.quantum = int(quantum)
        self.policy = policy
        self.evict_ratio = float(evict_ratio)
        self.max_evict = int(max_evict)
        self.models: Dict[str, ModelEntry] = {}
        self.waiting = _Queue(policy)
        self.active: Dict[int, Request] = {}
        self.finished: List[Request] = []
        self.t0 = time.perf_counter()
        self.kmc_steps = 0
        self.quanta = 0
        self.evicted = 0
        self.sessions: Dict[str, Session] = {}

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def add_model(self, key: str, program: Program) -> None:
        m = program.model
        tofs = m.tof_names()
        mat = np.zeros((len(tofs), program.nproc))
        for j, p in enumerate(m.processes):
            for name, factor in (p.tof_count or {}).items():
                mat[tofs.index(name), j] += factor
        self.models[key] = ModelEntry(program, self.pool.add_model(program), program.nproc,
                                      len(m.species), m.spuck, mat, tofs)

    def submit(self, req: Request) -> None:
        if req.model not in self.models:
            raise KeyError("unknown model %r" % req.model)
        continuing = req.session is not None and req.session in self.sessions
        if req.rates is None and not continuing:
            raise ValueError("request %d: rates are needed to start a trajectory" % req.rid)
        if req.rates is not None and len(req.rates) != self.models[req.model].nproc:
            raise ValueError("request %d: %d rates for %d processes" % (req.rid, len(req.rates),
                                                                       self.models[req.model].nproc))
        if req.samples > 0:
            # samples batches of int(steps / samples) steps, as do_steps(sample_size / samples)
            req.steps = req.samples * int(req.steps / req.samples)
        req.remaining = int(req.steps)
        if req.session is not None:
            sess = self.sessions.get(req.session)
            if sess is None:
                self.sessions[req.session] = Session(req.model, tuple(req.size), busy=True)
            else:
                if sess.model != req.model or tuple(sess.size) != tuple(req.size):
                    raise ValueError("request %d: session %r runs model %r on %s" % (req.rid, req.session, sess.model,
                                                                                    sess.size))
                if sess.busy:
                    sess.queue.append(req)  # after the session's current request
                    return
                sess.busy = True
        self.waiting.push(req)

    def close_session(self, name: str) -> None:
        """Drops a session's trajectory (resident or in host memory)."""
        sess = self.sessions.pop(name, None)
        if sess is not None and sess.slot >= 0 and not sess.busy:
            self.pool.release(sess.slot)

    # ------------------------------------------------------------------ scheduling
    def _need(self, req: Request) -> int:
        extra = 4096 if req.samples > 0 else 0  # the on-device sampling record
        sess = self.sessions.get(req.session) if req.session is not None else None
        if sess is not None and sess.slot >= 0:
            return extra  # continues a resident trajectory
        return self.pool.slot_bytes(self.models[req.model].model_id, req.size) + extra

    def _resident(self) -> int:
        """Slots in use: running requests and resident session trajectories waiting for
        their next request."""
        return len(self.active) + sum(1 for x in self.sessions.values() if x.slot >= 0)

    def _evict_idle(self, need: int) -> None:
        """Moves idle resident sessions (least recently used first) to host memory until
        ``need`` bytes are free or none is left."""
        idle = sorted((s for s in self.sessions.values() if s.slot >= 0 and not s.busy), key=lambda s: s.last_used)
        free = self.pool.free_bytes()[0]
        for sess in idle:
            if need <= free and self._resident() < self.max_slots:
                break
            sess.image = self.pool.save_state(sess.slot)
            free += self.pool.slot_bytes(self.models[sess.model].model_id, sess.size)
            self.pool.release(sess.slot)
            sess.slot = -1
            self.evicted += 1

    def _evict(self) -> int:
        """srpt: while the queue's head does not fit and a resident trajectory has far
        more steps left, move that trajectory's state to host memory."""
        if self.policy != "srpt" or not self.waiting or not self.active:
            return 0
        n = 0
        victims = sorted((r for r in self.active.values() if r.samples == 0), key=lambda r: -r.remaining)
        free = self.pool.free_bytes()[0]
        head = self.waiting.peek()
        need = self._need(head)
        for v in victims:
            if n >= self.max_evict:
                break
            fits = len(self.active) < self.max_slots and need <= free
            if fits or v.remaining <= self.evict_ratio * head.remaining:
                break
            v.image = self.pool.save_state(v.slot)
            free += self._need(v)
            self.pool.release(v.slot)
            del self.active[v.slot]
            v.slot = -1
            v.evictions += 1
            self.waiting.push(v)
            n += 1
        self.evicted += n
        return n

    def _admit(self) -> int:
        """Admits waiting requests in policy order while the arena and the slot table
        have room (admission by free HBM); evicted requests are restored from their
        images."""
        batch: List[Request] = []
        restored = 0
        started: List[Request] = []
        if self.waiting:
            head = self.waiting.peek()
            self._evict_idle(self._need(head))
        free, _largest = self.pool.free_bytes()
        budget = free
        while self.waiting and self._resident() + len(batch) < self.max_slots:
            req = self.waiting.peek()
            need = self._need(req)
            if need > budget:
                break
            self.waiting.pop()
            sess = self.sessions.get(req.session) if req.session is not None else None
            if sess is not None and (sess.slot >= 0 or sess.image is not None):
                # a session's next request: its trajectory runs on, with the new rates
                if sess.slot < 0:
                    try:
                        sess.slot = self.pool.restore_state(self.models[req.model].model_id, sess.image)
                    except E.KMCError as err:
                        if err.code != 6:
                            raise
                        self.waiting.push(req)
                        break
                    sess.image = None
                    budget = self.pool.free_bytes()[0]
                if req.rates is not None:
                    self.pool.set_rates(sess.slot, req.rates)
                req.slot, req.admitted = sess.slot, self.now()
                sess.slot = -1  # the running request owns the trajectory until it retires
                self.active[req.slot] = req
                started.append(req)
                restored += 1
                continue
            if req.image is not None:
                try:
                    s = self.pool.restore_state(self.models[req.model].model_id, req.image)
                except E.KMCError as err:
                    if err.code != 6:
                        raise
                    self.waiting.push(req)  # fragmentation: try again next quantum
                    break
                req.image, req.slot = None, s
                self.active[s] = req
                restored += 1
                budget = self.pool.free_bytes()[0]
                continue
            budget -= need
            batch.append(req)
        self._snapshot(started)
        self._begin_sampling([r for r in started if r.samples > 0])
        if not batch:
            return restored
        try:
            slots = self.pool.admit_many([self.models[r.model].model_id for r in batch], [r.size for r in batch],
                                         [r.rates for r in batch], seeds=[r.seed for r in batch],
                                         rng=E.RNG_PHILOX, trajs=[r.traj_id for r in batch])
        except E.KMCError as err:
            if err.code != 6:
                raise
            # fragmentation: fall back to one at a time
            slots = []
            for r in batch:
                try:
                    slots.append(self.pool.admit(self.models[r.model].model_id, r.size, r.rates, seed=r.seed,
                                                 rng=E.RNG_PHILOX, traj=r.traj_id))
                except E.KMCError as e2:
                    if e2.code != 6:
                        raise
                    slots.append(None)
        t = self.now()
        for r, s in zip(batch, slots):
            if s is None:
                self.waiting.push(r)
                continue
            r.slot, r.admitted = s, t
            r.start = None  # a fresh trajectory starts from zero counters
            self.active[s] = r
        self._begin_sampling([r for r, s in zip(batch, slots) if s is not None and r.samples > 0])
        return restored + len([s for s in slots if s is not None])

    def _begin_sampling(self, reqs: List[Request]) -> None:
        if not reqs:
            return
        self.pool.sample_begin([r.slot for r in reqs])
        for r in reqs:
            r.to_sample = max(1, int(r.steps / r.samples))  # do_steps(sample_size / samples)

    def _snapshot(self, reqs: List[Request]) -> None:
        """Counters and clock of continued trajectories when their request begins."""
        by_model: Dict[str, List[Request]] = collections.defaultdict(list)
        for r in reqs:
            by_model[r.model].append(r)
        for key, rs in by_model.items():
            ps, ig, times, _k, _st = self.pool.results([r.slot for r in rs], self.models[key].nproc)
            for i, r in enumerate(rs):
                r.start = (ps[i].copy(), ig[i].copy(), float(times[i]))

    def _retire(self, reqs: List[Request]) -> None:
        if not reqs:
            return
        by_model: Dict[str, List[Request]] = collections.defaultdict(list)
        for r in reqs:
            by_model[r.model].append(r)
        t = self.now()
        for key, rs in by_model.items():
            entry = self.models[key]
            slots = [r.slot for r in rs]
            ps, ig, times, steps, status = self.pool.results(slots, entry.nproc)
            occ = self.pool.occupation_counts(slots, entry.nspecies * entry.spuck)
            sampled = {}
            smp = [r for r in rs if r.samples > 0]
            if smp:
                out = self.pool.sample_end([r.slot for r in smp])
                for j, r in enumerate(smp):
                    cells = float(np.prod(r.size))
                    dt = out["times"][j, 0]
                    with np.errstate(divide="ignore", invalid="ignore"):
                        tof = entry.tof_matrix @ (out["dprocstat"][j, :entry.nproc] / dt / cells)
                        tofi = entry.tof_matrix @ (out["dinteg"][j, :entry.nproc] / dt / cells)
                    sampled[id(r)] = {
                        "tof": dict(zip(entry.tof_names, tof)), "tof_integ": dict(zip(entry.tof_names, tofi)),
                        "occupation": out["occ"][j, :entry.nspecies * entry.spuck].reshape(entry.nspecies,
                                                                                          entry.spuck),
                        "total_time": float(dt), "simulated_time": float(out["times"][j, 1]),
                        "kmc_steps": int(out["steps"][j])}
            for i, r in enumerate(rs):
                cells = int(np.prod(r.size))
                if status[i] not in (0, 3):
                    r.error = "status %d" % status[i]
                ps0, ig0, t0 = r.start if r.start is not None else (0, 0.0, 0.0)
                dt = times[i] - t0
                tt = dt if dt > 0 else np.inf
                r.result = {
                    "kmc_time": float(times[i]), "kmc_step": int(steps[i]), "status": int(status[i]),
                    "procstat": ps[i], "integ_rates": ig[i], "interval_time": float(dt),
                    "tof": dict(zip(entry.tof_names, entry.tof_matrix @ (ps[i] - ps0) / tt / cells)),
                    "tof_integ": dict(zip(entry.tof_names, entry.tof_matrix @ (ig[i] - ig0) / tt / cells)),
                    "coverage": occ[i].reshape(entry.nspecies, entry.spuck) / cells,
                }
                if id(r) in sampled:
                    r.result["sampled"] = sampled[id(r)]
                r.done = t
                del self.active[r.slot]
                self.finished.append(r)
                sess = self.sessions.get(r.session) if r.session is not None else None
                if sess is not None and r.keep and status[i] in (0, 3):
                    sess.slot, sess.busy, sess.last_used = r.slot, False, t
                    if sess.queue:  # the session's next request
                        nxt = sess.queue.popleft()
                        sess.busy = True
                        self.waiting.push(nxt)
                    continue
                if sess is not None:
                    self.sessions.pop(r.session, None)
                    for nxt in sess.queue:
                        nxt.error = "session %r ended" % r.session
                        self.finished.append(nxt)
                self.pool.release(r.slot)

    def run_quantum(self) -> None:
        """One persistent launch advancing every active trajectory."""
        if not self.active:
            return
        slots = list(self.active)
        steps = []
        for s in slots:
            r = self.active[s]
            n = min(r.remaining, self.quantum)
            if r.samples > 0:
                n = min(n, r.to_sample)  # end the quantum at the next sample boundary
            steps.append(n)
        before = self.pool.results(slots, 1)[3]
        self.pool.run(slots, steps, sync=True)
        self.quanta += 1
        _ps, _ig, _t, after, statuses = self.pool.results(slots, 1)
        done, sample_now = [], []
        for s, n, k0, k1, st in zip(slots, steps, before, after, statuses):
            r = self.active[s]
            self.kmc_steps += int(k1 - k0)
            r.remaining -= n
            if r.samples > 0:
                r.to_sample -= n
                if r.to_sample <= 0:
                    sample_now.append(s)
                    r.to_sample = max(1, int(r.steps / r.samples))
            # a trajectory that found no process (absorbing state) ends early, as the
            # reference stops there
            if r.remaining <= 0 or st != 0:
                r.remaining = 0
                done.append(r)
        if sample_now:
            self.pool.sample(sample_now)
        self._retire(done)

    def serve(self, arrivals: Sequence[Request], until_empty: bool = True, deadline: float = float("inf")):
        """Feeds ``arrivals`` (sorted by arrival time, server clock) and runs quanta
        until every request finished (or ``deadline`` seconds passed)."""
        pending = collections.deque(sorted(arrivals, key=lambda r: r.arrival))
        self.t0 = time.perf_counter()
        while pending or self.waiting or self.active or any(s.queue for s in self.sessions.values()):
            t = self.now()
            if t > deadline:
                break
            while pending and pending[0].arrival <= t:
                self.submit(pending.popleft())
            self._evict()
            self._admit()
            if self.active:
                self.run_quantum()
            elif pending:
                time.sleep(max(0.0, min(0.01, pending[0].arrival - self.now())))
            if not until_empty and not pending:
                break
        return self.finished

    def close(self):
        self.pool.close()


class _Queue:
    """Waiting requests: arrival order (fifo) or fewest remaining steps first (srpt)."""

    def __init__(self, policy: str):
        self.policy = policy
        self.items: list = []
        self.fifo: collections.deque = collections.deque()
        self.n = 0

    def push(self, r: Request) -> None:
        if self.policy == "srpt":
            heapq.heappush(self.items, (r.remaining, r.arrival, r.rid, self.n, r))
            self.n += 1
        else:
            self.fifo.append(r)

    def peek(self) -> Request:
        return self.items[0][-1] if self.policy == "srpt" else self.fifo[0]

    def pop(self) -> Request:
        return heapq.heappop(self.items)[-1] if self.policy == "srpt" else self.fifo.popleft()

    def __len__(self) -> int:
        return len(self.items) if self.policy == "srpt" else len(self.fifo)

    def __bool__(self) -> bool:
        return len(self) > 0


def latency_stats(reqs: Sequence[Request]) -> dict:
    lat = np.array([r.done - r.arrival for r in reqs if r.done >= 0])
    if len(lat) == 0:
        return {"completed": 0}
    return {"completed": int(len(lat)), "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean())}


def main(argv=None):
    """Configuration 5 on one GPU: ``python -m kmos_gb300.serving [--rate R] [--duration S]
    [--steps-scale F]``; prints one JSON line with p50/p99 latency and steps/s."""
    import argparse
    import json
    from . import configs
    ap = argparse.ArgumentParser()
    ap.add_argument("--rate", type=float, default=500.0)
    ap.add_argument("--duration", type=float, default=60.0)
    ap.add_argument("--steps-scale", type=float, default=1.0)
    ap.add_argument("--quantum", type=int, default=20000)
    ap.add_argument("--arena-gb", type=float, default=64.0)
    ap.add_argument("--deadline", type=float, default=float("inf"))
    ap.add_argument("--policy", default="fifo", choices=["fifo", "srpt"])
    ap.add_argument("--max-slots", type=int, default=16384)
    a = ap.parse_args(argv)
    reqs, progs = configs.serving_requests(rate=a.rate, duration=a.duration, steps_scale=a.steps_scale)
    srv = Server(arena_bytes=int(a.arena_gb * (1 << 30)), max_slots=a.max_slots, quantum=a.quantum,
                 policy=a.policy)
    for k, p in progs.items():
        srv.add_model(k, p)
    t0 = time.perf_counter()
    done = srv.serve(reqs, deadline=a.deadline)
    wall = time.perf_counter() - t0
    stats = latency_stats(done)
    offered = sum(r.steps for r in reqs)
    line = {"metric": "serving p50/p99 request latency", "requests": len(reqs), "rate_per_s": a.rate,
            "duration_s": a.duration, "steps_scale": a.steps_scale, "quantum": a.quantum,
            "offered_steps": offered, "served_steps": srv.kmc_steps, "wall_s": wall,
            "steps_per_s": srv.kmc_steps / wall, "quanta": srv.quanta, "policy": a.policy,
            "max_slots": a.max_slots, "evictions": srv.evicted, **stats}
    srv.close()
    print(json.dumps(line))
    return line


if __name__ == "__main__":
    main()
