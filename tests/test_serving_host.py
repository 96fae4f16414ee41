"""Host-side logic of the server: the arena allocator, the request stream, the
stall rule and the memory accounting (no GPU needed)."""

import math

import numpy as np

from astrea_gb300 import initial
from astrea_gb300.serving import ARENA_COPIES, Arena, arena_copies, make_requests, stalled


def test_arena_first_fit_and_merge():
    a = Arena(100)
    x, y, z = a.alloc(30), a.alloc(30), a.alloc(30)
    assert (x, y, z) == (0, 30, 60)
    assert a.alloc(20) is None  # only 10 left
    a.release(y, 30)
    assert a.alloc(20) == 30  # first fit into the hole
    a.release(30, 20)
    a.release(x, 30)
    a.release(z, 30)
    assert a.free == [(0, 100)]  # every hole merged back


def test_arena_never_hands_out_overlapping_ranges():
    rng = np.random.default_rng(1)
    a = Arena(1000)
    live = {}
    for _ in range(2000):
        if live and rng.uniform() < .5:
            off = list(live)[rng.integers(len(live))]
            a.release(off, live.pop(off))
        else:
            n = int(rng.integers(1, 80))
            off = a.alloc(n)
            if off is not None:
                live[off] = n
        spans = sorted(live.items())
        for (o1, n1), (o2, _) in zip(spans, spans[1:]):
            assert o1 + n1 <= o2
        assert all(0 <= o and o + n <= 1000 for o, n in spans)


def test_request_stream_is_seeded_and_follows_the_mix():
    a = make_requests(400, rate=100.0, seed=5)
    b = make_requests(400, rate=100.0, seed=5)
    assert [(r.arrival, r.n, r.scheme, r.solver, r.t_end) for r in a] == \
           [(r.arrival, r.n, r.scheme, r.solver, r.t_end) for r in b]
    arrivals = np.array([r.arrival for r in a])
    assert np.all(np.diff(arrivals) > 0)
    assert abs(arrivals[-1] / len(a) - 1 / 100.0) < .2 / 100.0  # Poisson arrivals at the rate
    frac_1d = np.mean([r.dim == 1 for r in a])
    assert .3 < frac_1d < .5
    for r in a:
        lo, hi = (256, 65536) if r.dim == 1 else (128, 2048)
        assert lo - 2 <= r.n <= hi and r.n % 2 == 0
        assert r.solver in ("llf", "hlld" if r.mhd else "hllc")
        assert .05 <= r.t_end <= .3


def test_request_ic_carries_the_host_initial_state():
    for r in make_requests(20, rate=100.0, seed=8, n1d=(16, 64), n2d=(8, 32)):
        w = r.initial_state()
        ic = r.ic()
        st = r.states()
        assert ic.dim == r.dim and ic.n == r.n and ic.shock == .5
        if r.dim == 1:
            assert ic.kind == initial.SPLIT
            assert list(ic.left) == list(st[0]) and list(ic.right) == list(st[1])
            assert np.array_equal(w[0], st[0]) and np.array_equal(w[-1], st[1])
        else:
            assert ic.kind == initial.QUADRANT
            assert np.array_equal(w[0, 0], st[0]) and np.array_equal(w[0, -1], st[1])
            assert np.array_equal(w[-1, 0], st[2]) and np.array_equal(w[-1, -1], st[3])


def test_stall_rule():
    # no limit: never
    assert not stalled(10 ** 9, 0.0, 1e-12, 1.0, None)
    # past the limit: always
    assert stalled(50001, .2, 1e-3, .3, 50000)
    # early steps are never judged by their projection
    assert not stalled(10, 0.0, 1e-12, 1.0, 50000)
    # after the check point: projected total against the limit
    assert stalled(2000, .01, 1e-7, .3, 50000)       # 2.9e6 more steps needed
    assert not stalled(2000, .01, 1e-4, .3, 50000)   # 2900 more steps
    assert stalled(2000, .01, 0.0, .3, 50000)        # a zero step never arrives
    assert stalled(2000, .01, math.nan, .3, 50000)


def test_arena_copies_count_the_cell_average_arenas():
    assert arena_copies(1, 32) == ARENA_COPIES and arena_copies(1, 64) == ARENA_COPIES
    assert arena_copies(2, 32) == ARENA_COPIES + 1
    assert arena_copies(2, 64) == ARENA_COPIES + 2


def test_poll_size_follows_the_nearest_completion():
    from astrea_gb300.serving import Request, Server
    srv = Server.__new__(Server)  # the poll rule only, no device
    srv.steps_per_poll, srv.max_steps_per_poll = 8, 32
    cls = (2, 4)
    h = 2.0 ** -10  # binary fractions keep the step counts exact
    r1 = Request(rid=1, arrival=0, dim=2, n=64, mhd=False, scheme="ppm", solver="hllc", t_end=.5, seed=1)
    r2 = Request(rid=2, arrival=0, dim=2, n=64, mhd=False, scheme="ppm", solver="hllc", t_end=.125, seed=2)
    srv.active = {cls: {0: (r1, 0, 1), 1: (r2, 1, 1)}}
    srv.last_clk = {}
    assert srv._poll_steps(cls) == 8  # no clock reading yet
    clk = {"t": np.array([.25, .125 - 10 * h]), "dt": np.array([16 * h, h]), "steps": np.array([10, 90]),
           "done": np.array([0, 0])}
    srv.last_clk = {cls: (clk, {0: 1, 1: 2})}
    assert srv._poll_steps(cls) == 10  # r2 needs 10 more steps
    clk["t"][1] = .125 - h / 2
    assert srv._poll_steps(cls) == 1  # the rounded-up remainder
    clk["dt"][1] = 0.
    assert srv._poll_steps(cls) == 1  # a zero step: poll every step (the stall rule retires it)
    clk["t"][1], clk["dt"][1] = 0., 2.0 ** -20
    assert srv._poll_steps(cls) == 16  # r1's 16 steps come first
    clk["t"][0] = 0.
    assert srv._poll_steps(cls) == 32  # both far off: the cap
    srv.active[cls][1] = (Request(rid=3, arrival=0, dim=2, n=64, mhd=False, scheme="plm", solver="llf",
                                  t_end=.2, seed=3), 1, 1)
    assert srv._poll_steps(cls) == 8  # slot 1 holds a new request without a clock reading
