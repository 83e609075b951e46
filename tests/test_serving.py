"""The continuous-batching server's scheduling (libfusion_gb300/serving.py) on
the host, with a simulated clock, a stand-in batch whose ticks take simulated
time, and stand-in arenas: admission by memory and by slots, arena reuse and
reclaim, eviction, frame pacing, latency accounting, continuous batching."""
import pytest

from libfusion_gb300.serving import ArenaCache, Request, Server


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def now(self):
        return self.t

    def sleep_until(self, t):
        self.t = max(self.t, t)


class FakeBatch:
    """A tick takes base + per_frame seconds per active slot on the clock."""

    def __init__(self, clock, slots, base=0.002, per_frame=0.0002):
        self.clock, self.base, self.per_frame = clock, base, per_frame
        self.slots = [None] * slots
        self.inputs = {}
        self.ticks = []

    def set(self, slot, s):
        self.slots[slot] = s

    def set_inputs(self, slot, d, c):
        self.inputs[slot] = (d, c)

    def process(self, active, use_graph=True, stream=None):
        n = sum(1 for a in active if a)
        assert all(self.slots[i] is not None for i, a in enumerate(active) if a), "tick on an empty slot"
        self.ticks.append([i for i, a in enumerate(active) if a])
        self.clock.t += self.base + self.per_frame * n

    def results(self, back=0):
        # each slot's "pose": a translation by (slot, ticks so far)
        poses = []
        for i in range(len(self.slots)):
            T = [[1.0, 0, 0, float(i)], [0, 1.0, 0, float(len(self.ticks))], [0, 0, 1.0, 0], [0, 0, 0, 1.0]]
            poses.append(T)
        return poses, [1] * len(self.slots), None, None


class Arena:
    n = 0

    def __init__(self, key):
        Arena.n += 1
        self.key, self.id, self.resets, self.closed = key, Arena.n, 0, False


def make_cache(budget):
    return ArenaCache(budget, make=lambda key: Arena(key), destroy=lambda a: setattr(a, "closed", True),
                      reset=lambda a: setattr(a, "resets", a.resets + 1))


def req(sid, t, frames, key=("a",), nbytes=10, fps=30.0):
    return Request(sid=sid, arrival=t, frames=frames, key=key, nbytes=nbytes, source=lambda k: (k, k), fps=fps)


def server(slots, budget, **kw):
    clock = FakeClock()
    batch = FakeBatch(clock, slots, **kw)
    return Server(batch, slots, make_cache(budget), clock=clock, set_pose=lambda s, T: None), clock, batch


def test_admission_waits_for_memory_and_reuses_the_arena():
    srv, clock, _ = server(slots=8, budget=20)
    for i in range(3):
        srv.submit(req(i, 0.0, frames=30))
    srv.run(0.5)
    r = srv.report()
    assert r["deferred_by_memory"] == 1 and r["deferred_by_slots"] == 0
    # two fit; the third waits for one of them to finish its 30 frames (1 s at 30 fps)
    assert r["admitted"] == 2 and r["still_queued"] == 1
    srv.run(2.0)
    r = srv.report()
    assert r["admitted"] == 3 and r["completed"] == 3
    assert r["memory"]["arenas_created"] == 2 and r["memory"]["arenas_reused"] == 1
    assert r["memory"]["peak_bytes"] <= 20
    assert r["queue_wait_s"]["max"] >= 29 / 30.0  # it waited for a whole session


def test_cached_arenas_of_another_configuration_are_freed_for_room():
    srv, clock, _ = server(slots=4, budget=25)
    srv.submit(req(0, 0.0, frames=3, key=("small",), nbytes=10))
    srv.submit(req(1, 0.5, frames=3, key=("big",), nbytes=20))
    srv.run(1.0)
    r = srv.report()
    assert r["completed"] == 2
    # the first session's cached arena had to go for the second one to fit
    assert r["memory"]["arenas_freed"] == 1 and r["memory"]["arenas_created"] == 2


def test_slots_bound_concurrency():
    srv, clock, _ = server(slots=2, budget=10 ** 9)
    for i in range(5):
        srv.submit(req(i, 0.0, frames=10))
    srv.run(0.1)
    r = srv.report()
    assert r["concurrency_peak"] == 2 and r["deferred_by_slots"] == 3 and r["deferred_by_memory"] == 0
    srv.run(5.0)
    assert srv.report()["completed"] == 5


def test_a_head_that_does_not_fit_does_not_block_smaller_requests_behind_it():
    srv, clock, _ = server(slots=4, budget=30)
    srv.submit(req(0, 0.0, frames=60, nbytes=20))
    srv.submit(req(1, 0.1, frames=60, key=("big",), nbytes=25))   # does not fit while 0 runs
    srv.submit(req(2, 0.2, frames=60, key=("s",), nbytes=10))     # fits
    srv.run(0.3)
    r = srv.report()
    assert r["admitted"] == 2 and r["still_queued"] == 1 and r["deferred_by_memory"] == 1


def test_every_frame_is_fused_once_in_order_and_paced_by_the_camera():
    srv, clock, batch = server(slots=4, budget=100)
    srv.submit(req(0, 0.0, frames=45))
    srv.submit(req(1, 0.01, frames=30))
    srv.run(3.0)
    r = srv.report()
    assert r["frames"] == 75 and r["completed"] == 2
    # a tick fuses only the sessions whose camera has produced their next frame
    assert max(len(t) for t in batch.ticks) <= 2 and min(len(t) for t in batch.ticks) >= 1
    # nothing waits longer than a tick or two: the GPU is idle between frames
    assert r["latency_ms"]["max"] < 2 * (2.0 + 0.4)
    assert r["frames_per_s"] == pytest.approx(75 / 3.0, rel=0.05)


def test_continuous_batching_under_load_groups_frames_of_many_sessions():
    # a tick of 5 ms + 0.5 ms per frame: 40 sessions at 30 fps (1,200 frames/s)
    # keep it busy, so the frames that arrive during a tick share the next one
    # (steady state about 15 frames per 12.5 ms tick)
    srv, clock, batch = server(slots=40, budget=10 ** 9, base=0.005, per_frame=0.0005)
    for i in range(40):
        srv.submit(req(i, 0.001 * i, frames=60))
    srv.run(3.0)
    r = srv.report()
    assert r["completed"] == 40 and r["frames"] == 40 * 60
    assert r["active_per_tick_mean"] > 3
    assert r["latency_ms"]["p99"] < 40.0


def test_eviction_empties_the_slot_and_resets_the_arena():
    srv, clock, batch = server(slots=1, budget=10)
    srv.submit(req(0, 0.0, frames=5))
    srv.submit(req(1, 0.0, frames=5))
    srv.run(1.0)
    r = srv.report()
    assert r["completed"] == 2 and r["memory"]["arenas_created"] == 1 and r["memory"]["arenas_reused"] == 1
    assert batch.slots[0] is None
    arena = srv.cache.free[("a",)][0][0]
    assert arena.resets == 2  # reset when each session was evicted


def test_arrivals_count_from_the_server_start():
    """Request arrival times are seconds after the server starts, whatever the
    clock reads then."""
    srv, clock, _ = server(slots=4, budget=100)
    clock.t = 1000.0
    srv.submit(req(0, 0.0, frames=3))
    srv.submit(req(1, 5.0, frames=3))
    srv.run(1.0)
    r = srv.report()
    assert r["admitted"] == 1 and r["requests_arrived"] == 1
    srv.run(6.0)
    r = srv.report()
    assert r["admitted"] == 2 and r["queue_wait_s"]["max"] < 0.1


def test_collection_runs_every_n_frames_between_ticks_with_the_tracked_pose():
    clock = FakeClock()
    batch = FakeBatch(clock, 2)
    calls = []

    def collect(session, pose, stream):
        calls.append((session.id, len(batch.ticks), pose[0][3], pose[1][3], stream))

    srv = Server(batch, 2, make_cache(100), clock=clock, set_pose=lambda s, T: None, stream="st",
                 collect=collect, collect_every=4)
    srv.submit(req(0, 0.0, frames=10))
    srv.run(2.0)
    r = srv.report()
    assert r["frames"] == 10 and r["completed"] == 1
    # after its 4th and 8th frames (not after the last: the session leaves), with
    # the pose of the tick that fused that frame, on the server's stream
    assert r["collections"] == 2
    assert [c[1] for c in calls] == [4, 8]
    assert [c[3] for c in calls] == [4.0, 8.0] and all(c[2] == 0.0 and c[4] == "st" for c in calls)


def test_a_paused_camera_parks_its_session_and_resumes_it_in_a_freed_slot():
    clock = FakeClock()
    batch = FakeBatch(clock, 1)
    restored = []

    def snapshot(s):
        return bytes(10)

    srv = Server(batch, 1, make_cache(100), clock=clock, set_pose=lambda s, T: None, park_after=0.2,
                 snapshot=snapshot, restore=lambda s, snap: restored.append((s.id, len(snap))))
    paused = req(0, 0.0, frames=6)
    paused.pauses = {2: 1.0}  # after its third frame the camera stops for a second
    srv.submit(paused)
    srv.submit(req(1, 0.2, frames=10))  # arrives during the pause: takes the freed slot
    srv.run(0.6)
    r = srv.report()
    assert r["parking"]["parked"] == 1 and r["parking"]["still_parked"] == 1
    assert r["admitted"] == 2 and r["completed"] == 1 and r["frames"] == 3 + 10
    srv.run(3.0)
    r = srv.report()
    assert r["completed"] == 2 and r["frames"] == 16
    assert r["parking"]["resumed"] == 1 and r["parking"]["snapshot_bytes"] == 10 and len(restored) == 1
    # the resumed frames were fused when they arrived (a free slot was waiting)
    assert r["latency_ms"]["max"] < 10.0
    # only one slot: request 1 ran while request 0 was parked, never beside it
    assert all(len(t) == 1 for t in batch.ticks)
