"""Scheduler logic of the serving loop on the CPU (a fake executor stands in
for the device): FIFO admission under the HBM budget, batching by launch
shape in groups of at most QMC_MAX_BATCH jobs, slice bookkeeping of the
Metropolis step counters, retirement and budget release."""
import pytest

from qmctorch_gb300.serving import MAX_BATCH, Request, Scheduler, hydrogen_chain


class Token:
    def __init__(self, polls):
        self.left = polls

    def tick(self):
        self.left -= 1


class FakeExecutor:
    def __init__(self, bytes_per_walker=1000, delay=1):
        self.bpw = bytes_per_walker
        self.delay = delay
        self.tokens = []
        self.slices = []       # (rids, offsets, steps)
        self.admitted = []
        self.live = set()
        self.max_live_bytes = 0
        self.live_bytes = 0

    def footprint(self, req):
        return req.nwalkers * self.bpw

    def admit(self, req):
        self.admitted.append(req.rid)
        self.live.add(req.rid)
        self.live_bytes += self.footprint(req)
        self.max_live_bytes = max(self.max_live_bytes, self.live_bytes)
        n = req.atoms.count("H")
        return {"req": req, "offsets": []}, ("H", n, req.precision)

    def _token(self):
        t = Token(self.delay)
        self.tokens.append(t)
        return t

    def launch_slice(self, handles, offsets, steps, sid):
        self.slices.append(([h["req"].rid for h in handles], list(offsets), list(steps)))
        for h, o in zip(handles, offsets):
            h["offsets"].append(o)
        return self._token()

    def launch_energy(self, h, sid):
        return self._token()

    def launch_epoch(self, h, epoch, sid):
        h.setdefault("epochs", []).append(epoch)
        return self._token()

    def ready(self, token):
        token.tick()
        return token.left <= 0

    def stats(self, h):
        r = h["req"]
        energies = [float(e) for e in h.get("epochs", [])] if r.kind == "run" else None
        return (float(r.seed), float(r.nwalkers), float(r.nstep), energies)

    def release(self, h):
        r = h["req"]
        self.live.discard(r.rid)
        self.live_bytes -= self.footprint(r)


def req(n, nw, nstep, seed=0):
    return Request(atoms=hydrogen_chain(n, 0.74), nwalkers=nw, nstep=nstep, seed=seed)


def test_every_request_gets_its_result():
    ex = FakeExecutor()
    s = Scheduler(ex, hbm_budget=10 ** 9, slice_steps=64)
    rids = [s.submit(req(2 * (i % 3 + 1), 100 + i, 100 + 37 * i, seed=i)) for i in range(10)]
    out = s.run(sleep=0)
    assert sorted(r.rid for r in out) == rids
    for r in out:
        assert r.energy == float(r.rid) and r.nstep == 100 + 37 * r.rid
        assert r.latency >= 0 and r.admitted >= r.arrival


def test_step_offsets_cover_each_chain_once():
    ex = FakeExecutor()
    s = Scheduler(ex, hbm_budget=10 ** 9, slice_steps=50)
    s.submit(req(4, 10, 175))
    s.submit(req(4, 10, 60))
    s.run(sleep=0)
    per = {}
    for rids, offs, steps in ex.slices:
        for r, o, n in zip(rids, offs, steps):
            per.setdefault(r, []).append((o, n))
    assert per[0] == [(0, 50), (50, 50), (100, 50), (150, 25)]
    assert per[1] == [(0, 50), (50, 10)]


def test_budget_limits_resident_jobs_and_admission_is_fifo():
    ex = FakeExecutor(bytes_per_walker=1000)
    s = Scheduler(ex, hbm_budget=2500 * 1000, slice_steps=10)
    for i in range(6):
        s.submit(req(2, 1000, 30, seed=i))
    s.run(sleep=0)
    assert ex.max_live_bytes <= 2500 * 1000
    assert ex.admitted == list(range(6))
    assert len(s.results) == 6 and s.used == 0


def test_head_of_line_waits_for_budget():
    ex = FakeExecutor(bytes_per_walker=1)
    s = Scheduler(ex, hbm_budget=1000, slice_steps=10)
    s.submit(req(2, 800, 20))
    s.submit(req(2, 700, 20))   # does not fit next to the first
    s.submit(req(2, 100, 20))   # would fit, but waits behind the head (FIFO)
    s.poll()
    assert ex.admitted == [0]
    s.run(sleep=0)
    assert ex.admitted == [0, 1, 2]


def test_oversized_request_is_rejected():
    s = Scheduler(FakeExecutor(bytes_per_walker=1), hbm_budget=100)
    with pytest.raises(ValueError):
        s.submit(req(2, 1000, 10))


def test_batches_group_by_shape_and_respect_the_batch_limit():
    ex = FakeExecutor()
    s = Scheduler(ex, hbm_budget=10 ** 12, slice_steps=1000)
    n6 = MAX_BATCH + 5
    for i in range(n6):
        s.submit(req(6, 10, 100, seed=i))
    for i in range(3):
        s.submit(req(8, 10, 100, seed=100 + i))
    s.poll()
    sizes = sorted(len(rids) for rids, _, _ in ex.slices)
    assert sizes == [3, 5, MAX_BATCH]
    for rids, _, _ in ex.slices:  # one launch shape per launch
        assert len({r >= n6 for r in rids}) == 1


def test_jobs_arriving_later_start_while_others_run():
    """Continuous batching: a job submitted while another job is sampling is
    admitted and launched at the next pass, before the running job ends."""
    ex = FakeExecutor(delay=3)
    s = Scheduler(ex, hbm_budget=10 ** 9, slice_steps=10)
    s.submit(req(4, 10, 100))
    s.poll()
    s.submit(req(4, 10, 30))
    s.poll()
    assert [rids for rids, _, _ in ex.slices] == [[0], [1]]
    assert 0 not in s.results
    s.run(sleep=0)
    assert set(s.results) == {0, 1}


def test_run_jobs_alternate_gradient_and_resampling():
    """kind="run": initial sampling, then nepoch x (gradient, nstep_update
    resampling steps), then the final energy; single points run alongside."""
    ex = FakeExecutor()
    s = Scheduler(ex, hbm_budget=10 ** 9, slice_steps=40)
    r = req(4, 10, 100)
    r.kind, r.nepoch, r.nstep_update = "run", 3, 25
    s.submit(r)
    s.submit(req(4, 10, 60))
    s.run(sleep=0)
    res = s.results[0]
    assert res.energies == [0.0, 1.0, 2.0]
    per = [(o, n) for rids, offs, steps in ex.slices for rr, o, n in zip(rids, offs, steps)
           if rr == 0]
    assert per == [(0, 40), (40, 40), (80, 20), (100, 25), (125, 25), (150, 25)]
    assert s.results[1].energies is None


def test_unknown_request_kind_is_rejected():
    s = Scheduler(FakeExecutor(), hbm_budget=10 ** 9)
    r = req(2, 10, 10)
    r.kind = "optimise"
    with pytest.raises(ValueError):
        s.submit(r)
