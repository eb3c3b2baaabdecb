"""Host bookkeeping of CompactSolver's graph replay (no GPU): which steps
step() replays from the captured graph and which it launches one by one,
and when it sets the device step clock.  The device calls are replaced by
recorders."""


class FakeBuffer:
    def __init__(self, ptr):
        self.ptr = ptr

    def data_ptr(self):
        return self.ptr


class FakeClock:
    def __init__(self, log):
        self.log = log

    def __getitem__(self, i):
        log = self.log

        class Slot:
            def fill_(self, v):
                log.append(("clock", i, v))

        return Slot()


class FakeGraph:
    def __init__(self, solver, log):
        self.solver, self.log = solver, log

    def replay(self):
        self.log.append(("replay", self.solver.step_count + 1))


def make(log, graph_steps=4, cur0=0, first=1):
    from mpf3d.solver import CompactSolver
    s = CompactSolver.__new__(CompactSolver)
    s.step_count, s.cur = first - 1, cur0
    s.buf = [(FakeBuffer(0x100),), (FakeBuffer(0x200),)]
    s.clock = FakeClock(log)
    s._clock_next = first

    def launch_step(i):
        log.append(("eager", i))
        s.cur = 1 - s.cur
        s._clock_next = i + 1

    s.launch_step = launch_step
    s.graph, s.graph_steps = FakeGraph(s, log), graph_steps
    s._graph_at = (cur0, first & 1, s.buf[cur0][0].data_ptr())
    return s


def test_replays_where_the_graph_fits_and_launches_the_rest():
    log = []
    s = make(log)
    s.step(10, check=False)
    assert log == [("replay", 1), ("replay", 5), ("eager", 9), ("eager", 10)]
    assert s.step_count == 10 and s._clock_next == 11


def test_an_odd_eager_step_shifts_the_parity_and_the_graph_waits():
    log = []
    s = make(log)
    s.step(1, check=False)        # eager: the graph needs 4 steps
    s.step(4, check=False)        # step 2 has the other parity; after it only 3 steps are left
    assert log == [("eager", 1), ("eager", 2), ("eager", 3), ("eager", 4), ("eager", 5)]
    s.step(5, check=False)        # one eager step (6) lines buffers and parity up again
    assert log[-2:] == [("eager", 6), ("replay", 7)]
    assert s.step_count == 10


def test_the_clock_is_set_before_a_replay_after_the_index_jumped():
    log = []
    s = make(log)
    s._clock_next = 42            # e.g. after a tuning trial moved the device clock
    s.step(4, check=False)
    assert log == [("clock", 1, 1), ("replay", 1)]
    assert s._clock_next == 5


def test_no_graph_means_eager_steps():
    log = []
    s = make(log)
    s.graph = None
    s.step(3, check=False)
    assert log == [("eager", 1), ("eager", 2), ("eager", 3)]
