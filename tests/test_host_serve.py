"""The served loop's host logic (serve.serve, serve.sustained) against a fake
batch: no GPU, no library.  The fake finishes a job after a fixed number of
ticks, makes a result ticket ready one poll after it was begun, holds at
most fvc.BATCH_RESULT_SLOTS tickets and refuses to release a job whose
ticket is held -- the rules of fvc_batch_result_* and fvc_batch_release."""
import numpy as np

import fvc
import serve


class FakeBatch:
    def __init__(self, ticks_needed=3):
        self.ticks_needed = ticks_needed
        self.jobs = {}        # jid -> dict(kind, n, ticks, released)
        self.tickets = {}     # ticket -> [jid, polls]
        self.next_ticket = 0
        self.max_held = 0
        self.order = []       # jids in release order

    def _add(self, kind, n):
        jid = len(self.jobs)
        self.jobs[jid] = dict(kind=kind, n=n, ticks=0, released=False)
        return jid

    def submit_ftle(self, grid, t0, t1):
        return self._add("ftle", int(grid[6]) * int(grid[7]) * int(grid[8]))

    def submit_tracers(self, seeds, t0, t1, residence=False):
        return self._add("residence" if residence else "tracers", len(seeds))

    def tick(self):
        for j in self.jobs.values():
            if not j["released"] and j["ticks"] < self.ticks_needed:
                j["ticks"] += 1
        return sum(1 for j in self.jobs.values() if j["ticks"] < self.ticks_needed)

    def poll(self, jid):
        j = self.jobs[jid]
        if j["released"]:
            return fvc.BATCH_RELEASED
        return fvc.BATCH_DONE if j["ticks"] >= self.ticks_needed else fvc.BATCH_RUNNING

    def result_begin(self, jid):
        assert self.poll(jid) == fvc.BATCH_DONE
        if len(self.tickets) >= fvc.BATCH_RESULT_SLOTS:
            raise fvc.FvcError(fvc.FVC_ERR_STATE, "all result blocks held")
        t = self.next_ticket
        self.next_ticket += 1
        self.tickets[t] = [jid, 0]
        self.max_held = max(self.max_held, len(self.tickets))
        return t

    def result_ready(self, t):
        self.tickets[t][1] += 1
        return self.tickets[t][1] > 1

    def result_get(self, t):
        jid = self.tickets[t][0]
        j = self.jobs[jid]
        n = j["n"]
        if j["kind"] == "ftle":
            return {"wT": np.full(n, float(jid)), "wN": np.full(n, -float(jid))}
        return {"X": np.full((n, 3), float(jid)), "eid": np.arange(n, dtype=np.int32),
                "left": np.zeros(n, np.int32), "ldt": np.zeros(n), "rt": np.full(n, 0.5)}

    def result_release(self, t):
        del self.tickets[t]

    def job_stats(self, jid):
        j = self.jobs[jid]
        return {"steps_main": 10 * j["n"] * j["ticks"], "steps_early": j["n"] if j["kind"] == "ftle" else 0}

    def release(self, jid):
        if any(v[0] == jid for v in self.tickets.values()):
            raise fvc.FvcError(fvc.FVC_ERR_STATE, "ticket held")
        self.jobs[jid]["released"] = True
        self.order.append(jid)


class FakeSite:
    def __init__(self, batch):
        self.batch = batch


def requests(n):
    out = []
    for k in range(n):
        kind = ("tracers", "ftle", "residence")[k % 3]
        if kind == "ftle":
            job = ("ftle", (0, 1, 0, 1, 0, 1, 3, 3, 3), 0.0, 1.0)
        else:
            job = (kind, (lambda m=5 + k: np.zeros((m, 3))), 0.0, 1.0)
        out.append(serve.Request(t_arrive=0.0, site="a" if k % 2 else "b", job=job, kind=kind,
                                 npts=27 if kind == "ftle" else 5 + k))
    return out


def test_serve_collects_every_result_through_tickets():
    sites = {"a": FakeSite(FakeBatch()), "b": FakeSite(FakeBatch())}
    reqs = requests(40)  # more finished jobs than result blocks at once
    s = serve.serve(sites, reqs, keep_results=True, time_limit=60.0)
    assert s["requests"] == 40
    for site in sites.values():
        b = site.batch
        assert b.max_held <= fvc.BATCH_RESULT_SLOTS
        assert not b.tickets and all(j["released"] for j in b.jobs.values())
    expect = 0
    for r in reqs:
        b = sites[r.site].batch
        j = b.jobs[r.jid]
        expect += 10 * j["n"] * b.ticks_needed + (j["n"] if r.kind == "ftle" else 0)
        assert r.t_done is not None and r.t_done >= r.t_arrive
        if r.kind == "ftle":
            wT, wN = r.result
            assert np.all(wT == r.jid) and np.all(wN == -r.jid)
        elif r.kind == "residence":
            assert np.all(r.result == 0.5) and len(r.result) == r.npts
        else:
            assert r.result["X"].shape == (r.npts, 3) and np.all(r.result["X"] == r.jid)
    assert s["steps"] == expect
    assert s["p50_ms"] <= s["p99_ms"]


def test_serve_stops_at_its_time_limit():
    class Never(FakeBatch):
        def poll(self, jid):
            return fvc.BATCH_RUNNING
    sites = {"a": FakeSite(Never()), "b": FakeSite(Never())}
    reqs = requests(6)
    s = serve.serve(sites, reqs, time_limit=0.05, censor=True)
    assert s["requests"] == 0 and s["requests_unfinished"] == 6
    assert s["steps"] > 0  # the running jobs' completed ticks are counted


def test_sustained_criterion():
    reqs = [serve.Request(t_arrive=t, site="a", job=None, kind="tracers", npts=1) for t in np.linspace(0, 15, 60)]
    for r in reqs:
        r.t_done = r.t_arrive + 0.02
    summary = {"wall_s": 15.1, "p99_ms": 20.0}
    assert serve.sustained(summary, reqs, 15.0)
    # light load: a late third twice as slow as the early one, still far under the limit
    for r in reqs[40:]:
        r.t_done = r.t_arrive + 0.1
    assert serve.sustained(dict(summary, p99_ms=100.0), reqs, 15.0)
    # a growing queue: the late third waits seconds
    for k, r in enumerate(reqs):
        r.t_done = r.t_arrive + 0.05 * k
    assert not serve.sustained(dict(summary, wall_s=18.0, p99_ms=2950.0), reqs, 15.0)
    assert not serve.sustained(dict(summary, requests_unfinished=3), reqs, 15.0)
