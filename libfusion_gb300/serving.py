"""Continuous-batching server over a FusionBatch.

The reference runs one map and one camera per process (src/system.cpp:40-114,
src/data_struct/map_struct.cu:10); serving many reconstruction sessions on one
GPU is this library's own layer.  Requests (a camera that will stream N frames
at a frame rate) arrive over time and wait in a queue.  A request is admitted
when a batch slot is free and the device memory budget has room for its
session arena (gbf_session_bytes: block pool, hash table, images).  Once
admitted its camera starts streaming; every tick fuses, in the same launches,
one frame of each session that has a frame waiting (continuous batching: a
tick takes the frames that have arrived, whichever sessions they belong to).
A session whose last frame is fused is evicted: its slot empties and its arena
is reset (gbf_session_reset keeps the device memory) and cached for a later
request of the same configuration, so admission allocates only when the cache
has no arena of that configuration; cached arenas of other configurations are
freed when the budget needs their room.

Latency of a frame: from the moment its camera produced it (admission time +
index / fps) to the moment its pose is on the host.  The wait for admission is
reported separately, per request.

Block garbage collection (optional): every `collect_every` fused frames of a
session, `collect(session, pose, stream)` runs between two ticks with the pose
its last frame tracked -- typically gbf_map_prune_async around the camera,
stream-ordered with the batch's launches and with no host synchronisation.

Parking (optional): a camera may pause (Request.pauses: after frame k, no frame
for that many seconds).  A session whose next frame is more than `park_after`
seconds away is snapshotted to host memory (`snapshot(session)`, e.g.
gbf_session_snapshot), and its slot and arena are freed for other requests;
when its next frame arrives it is resumed -- ahead of new requests -- into a
free slot and an arena of its configuration (`restore(session, snapshot)`,
e.g. gbf_session_restore) and continues bit for bit.

The clock, the batch and the session factory are parameters, so the scheduling
is testable without a GPU.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass


@dataclass
class Request:
    """A camera asking for a reconstruction session."""
    sid: int
    arrival: float                 # seconds after the server starts
    frames: int                    # frames the camera will stream
    key: tuple                     # session configuration (arena reuse key)
    nbytes: int                    # device bytes of its session (gbf_session_bytes)
    pose0: object = None           # initial camera -> world pose
    source: object = None          # frame k -> (depth device pointer, rgb device pointer)
    fps: float = 30.0
    pauses: dict = None            # frame k -> seconds without frames after frame k


@dataclass
class _Live:
    req: Request
    session: object
    admitted: float
    next_frame: int = 0
    fused: int = 0
    failed: int = 0
    delay: float = 0.0             # pauses before next_frame
    snapshot: object = None        # while parked


class WallClock:
    def now(self) -> float:
        return time.perf_counter()

    def sleep_until(self, t: float) -> None:
        d = t - time.perf_counter()
        if d > 0:
            time.sleep(d)


class ArenaCache:
    """Device memory accounting for admission.  Every arena counts against the
    budget while it exists, serving or cached for reuse."""

    def __init__(self, budget: int, make, destroy, reset):
        self.budget = budget
        self._make, self._destroy, self._reset = make, destroy, reset
        self.free: dict[tuple, deque] = {}
        self.live_bytes = 0          # bytes of every existing arena
        self.peak_bytes = 0
        self.created = self.reused = self.freed = 0

    def _cached_bytes(self) -> list[tuple[tuple, int]]:
        return [(k, nb) for k, q in self.free.items() for (_, nb) in q]

    def fits(self, nbytes: int, key: tuple) -> bool:
        """Would an arena of `key` be available without exceeding the budget?"""
        if self.free.get(key):
            return True
        reclaimable = sum(nb for k, nb in self._cached_bytes() if k != key)
        return self.live_bytes - reclaimable + nbytes <= self.budget

    def acquire(self, key: tuple, nbytes: int):
        """A reset session of configuration `key`, or None if the budget has no room."""
        q = self.free.get(key)
        if q:
            s, _ = q.popleft()
            self.reused += 1
            return s
        # free cached arenas of other configurations, oldest first, until it fits
        while self.live_bytes + nbytes > self.budget:
            victim = next((k for k, q in self.free.items() if q and k != key), None)
            if victim is None:
                return None
            s, nb = self.free[victim].popleft()
            self._destroy(s)
            self.live_bytes -= nb
            self.freed += 1
        s = self._make(key)
        self.live_bytes += nbytes
        self.peak_bytes = max(self.peak_bytes, self.live_bytes)
        self.created += 1
        return s

    def release(self, key: tuple, nbytes: int, session) -> None:
        self._reset(session)
        self.free.setdefault(key, deque()).append((session, nbytes))

    def close(self) -> None:
        for q in self.free.values():
            while q:
                s, nb = q.popleft()
                self._destroy(s)
                self.live_bytes -= nb


def _pct(xs, q):
    if not xs:
        return None
    s = sorted(xs)
    return s[min(len(s) - 1, max(0, int(math.ceil(q * len(s))) - 1))]


class Server:
    """Admission, continuous batching and eviction over `batch` (a
    FusionBatch-like object: set(slot, session), set_inputs(slot, depth, rgb),
    process(active, use_graph, stream), results(back) -> (poses, tracked,
    status, frame_index)).  `look_ahead`: how many queued requests admission
    may look past a head that does not fit in memory."""

    def __init__(self, batch, slots: int, cache: ArenaCache, clock=None, set_pose=None, stream=None,
                 use_graph: bool = True, look_ahead: int = 8, record_poses: bool = False, collect=None,
                 collect_every: int = 0, park_after: float | None = None, snapshot=None, restore=None):
        self.batch, self.slots, self.cache = batch, slots, cache
        self.collect, self.collect_every = collect, collect_every
        self.collections = 0
        self.park_after, self.snapshot, self.restore = park_after, snapshot, restore
        self.parked: list[_Live] = []             # snapshotted, waiting for their next frame
        self.parks = self.resumes = 0
        self.snapshot_bytes = 0
        self.park_s = self.resume_s = 0.0
        self.clock = clock or WallClock()
        self.set_pose = set_pose or (lambda s, T: s.set_pose(T))
        self.stream, self.use_graph, self.look_ahead = stream, use_graph, look_ahead
        self.pending: list[Request] = []          # not yet arrived, by arrival time
        self.queue: deque[Request] = deque()      # arrived, waiting for admission
        self.live: list[_Live | None] = [None] * slots
        self.latency_ms: list[float] = []
        self.queue_wait_s: list[float] = []
        self.deferred_memory: set[int] = set()
        self.deferred_slots: set[int] = set()
        self.completed = 0
        self.ticks = 0
        self.active_per_tick: list[int] = []
        self.concurrency_peak = 0
        self.failed_frames = 0
        self.t0 = None
        self.poses = {} if record_poses else None  # (request id, frame) -> camera -> world pose

    def submit(self, req: Request) -> None:
        self.pending.append(req)
        self.pending.sort(key=lambda r: r.arrival)

    # ---------------------------------------------------------------- scheduling
    def _arrive(self, now: float) -> None:
        while self.pending and self.t0 + self.pending[0].arrival <= now:
            self.queue.append(self.pending.pop(0))

    def _resume(self, now: float) -> None:
        """Parked sessions whose next frame has arrived, back into free slots."""
        for x in sorted(self.parked, key=lambda x: self._frame_time(x, x.next_frame)):
            if self._frame_time(x, x.next_frame) > now:
                break
            free = [i for i, y in enumerate(self.live) if y is None]
            if not free or not self.cache.fits(x.req.nbytes, x.req.key):
                break
            s = self.cache.acquire(x.req.key, x.req.nbytes)
            if s is None:
                break
            t = time.perf_counter()
            self.restore(s, x.snapshot)
            self.resume_s += time.perf_counter() - t
            x.session, x.snapshot = s, None
            self.parked.remove(x)
            slot = free[0]
            self.batch.set(slot, s)
            self.live[slot] = x
            self.resumes += 1

    def _park(self, now: float) -> None:
        """Snapshot the sessions whose next frame is more than park_after away."""
        for slot, x in enumerate(self.live):
            if x is None or self._frame_time(x, x.next_frame) - now <= self.park_after:
                continue
            t = time.perf_counter()
            x.snapshot = self.snapshot(x.session)
            self.park_s += time.perf_counter() - t
            self.snapshot_bytes += len(x.snapshot)
            self.batch.set(slot, None)
            self.cache.release(x.req.key, x.req.nbytes, x.session)
            x.session = None
            self.live[slot] = None
            self.parked.append(x)
            self.parks += 1

    def _admit(self, now: float) -> None:
        while self.queue:
            free = [i for i, x in enumerate(self.live) if x is None]
            if not free:
                for r in self.queue:
                    self.deferred_slots.add(r.sid)
                return
            pick = None
            for j, r in enumerate(list(self.queue)[:self.look_ahead]):
                if self.cache.fits(r.nbytes, r.key):
                    pick = j
                    break
                self.deferred_memory.add(r.sid)
            if pick is None:
                return
            r = self.queue[pick]
            del self.queue[pick]
            s = self.cache.acquire(r.key, r.nbytes)
            if s is None:  # a guard: acquire() agrees with fits() above
                self.queue.appendleft(r)
                return
            if r.pose0 is not None:
                self.set_pose(s, r.pose0)
            slot = free[0]
            self.batch.set(slot, s)
            self.live[slot] = _Live(r, s, now)
            self.queue_wait_s.append(now - (self.t0 + r.arrival))
            n = sum(1 for x in self.live if x is not None)
            self.concurrency_peak = max(self.concurrency_peak, n)

    def _frame_time(self, x: _Live, k: int) -> float:
        """Capture time of frame k >= next_frame - 1 (pauses before next_frame counted)."""
        return x.admitted + k / x.req.fps + x.delay

    def _evict(self, slot: int) -> None:
        x = self.live[slot]
        self.batch.set(slot, None)
        self.cache.release(x.req.key, x.req.nbytes, x.session)
        self.live[slot] = None
        self.completed += 1

    def next_event(self) -> float | None:
        """The earliest time something can happen: an arrival or a frame."""
        ts = [self._frame_time(x, x.next_frame) for x in self.live if x is not None]
        ts += [self._frame_time(x, x.next_frame) for x in self.parked]
        if self.pending:
            ts.append(self.t0 + self.pending[0].arrival)
        return min(ts) if ts else None

    def step(self) -> bool:
        """One round: arrivals, admissions, then one tick over the sessions with
        a frame waiting.  Returns whether a tick ran.  The first call starts
        the server's clock, from which request arrivals count."""
        now = self.clock.now()
        if self.t0 is None:
            self.t0 = now
        self._arrive(now)
        if self.parked:
            self._resume(now)
        self._admit(now)
        ready = [i for i, x in enumerate(self.live)
                 if x is not None and self._frame_time(x, x.next_frame) <= now]
        if not ready:
            return False
        for i in ready:
            x = self.live[i]
            d, c = x.req.source(x.next_frame)
            self.batch.set_inputs(i, d, c)
        active = [False] * self.slots
        for i in ready:
            active[i] = True
        self.batch.process(active, use_graph=self.use_graph, stream=self.stream)
        poses, tracked, _, _ = self.batch.results(back=0)
        done = self.clock.now()
        self.ticks += 1
        self.active_per_tick.append(len(ready))
        for i in ready:
            x = self.live[i]
            self.latency_ms.append((done - self._frame_time(x, x.next_frame)) * 1e3)
            if self.poses is not None:
                self.poses[(x.req.sid, x.next_frame)] = poses[i]
            if x.next_frame > 0 and not tracked[i]:
                x.failed += 1
                self.failed_frames += 1
            if x.req.pauses and x.next_frame in x.req.pauses:
                x.delay += x.req.pauses[x.next_frame]
            x.next_frame += 1
            x.fused += 1
            if x.next_frame >= x.req.frames:
                self._evict(i)
            elif self.collect is not None and self.collect_every > 0 and x.fused % self.collect_every == 0:
                self.collect(x.session, poses[i], self.stream)
                self.collections += 1
        if self.park_after is not None:
            self._park(self.clock.now())
        return True

    def run(self, until: float) -> None:
        """Serve until `until` seconds after the first call (server clock)."""
        if self.t0 is None:
            self.t0 = self.clock.now()
        end = self.t0 + until
        while self.clock.now() < end:
            if not self.step():
                t = self.next_event()
                self.clock.sleep_until(min(end, t) if t is not None else end)
        self.wall = self.clock.now() - self.t0

    # ---------------------------------------------------------------- report
    def report(self) -> dict:
        live = sum(1 for x in self.live if x is not None)
        frames = len(self.latency_ms)
        wall = getattr(self, "wall", None)
        return {
            "requests_arrived": self.completed + live + len(self.queue) + len(self.parked),
            "admitted": len(self.queue_wait_s), "completed": self.completed, "still_serving": live,
            "still_queued": len(self.queue),
            "deferred_by_memory": len(self.deferred_memory), "deferred_by_slots": len(self.deferred_slots),
            "queue_wait_s": {"p50": _pct(self.queue_wait_s, 0.5), "p95": _pct(self.queue_wait_s, 0.95),
                             "p99": _pct(self.queue_wait_s, 0.99),
                             "max": max(self.queue_wait_s) if self.queue_wait_s else None},
            "concurrency_peak": self.concurrency_peak,
            "active_per_tick_mean": (sum(self.active_per_tick) / len(self.active_per_tick))
            if self.active_per_tick else 0.0,
            "ticks": self.ticks, "frames": frames,
            "frames_per_s": frames / wall if wall else None,
            "latency_ms": {"p50": _pct(self.latency_ms, 0.5), "p95": _pct(self.latency_ms, 0.95),
                           "p99": _pct(self.latency_ms, 0.99),
                           "max": max(self.latency_ms) if self.latency_ms else None},
            "tracking_failed_frames": self.failed_frames,
            "collections": self.collections,
            "parking": {"parked": self.parks, "resumed": self.resumes, "still_parked": len(self.parked),
                        "snapshot_bytes": self.snapshot_bytes, "snapshot_s": self.park_s,
                        "restore_s": self.resume_s},
            "memory": {"budget_bytes": self.cache.budget, "peak_bytes": self.cache.peak_bytes,
                       "arenas_created": self.cache.created, "arenas_reused": self.cache.reused,
                       "arenas_freed": self.cache.freed},
            "wall_s": wall,
        }
